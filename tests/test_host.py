"""Host-side pieces and the C ABI surface (CPU only, no GPU calls).

The host library keeps the reference's formats byte for byte: its checkpoint
writer and VTK writer are compared with the files the reference itself wrote
(tests/golden/ckpt_4x5x6.dat, tests/golden/vtk/), fed with states the oracle
reproduces bitwise.
"""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from cbns3d_cart_mpi_gb300._abi import (CBNS_ERR_FORMAT, CBNS_ERR_IO, NG, CbnsParams, tgv_params)

pytestmark = pytest.mark.usefixtures("built")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions(name):
    """Function names declared in include/<name>."""
    text = open(os.path.join(ROOT, "include", name)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cbns_\w+)\s*\(", text)))


def exported(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_gpu_library_exports_every_declared_symbol():
    from cbns3d_cart_mpi_gb300 import _lib
    names = header_functions("cbns_gpu.h")
    assert "cbns_create" in names and "cbns_step" in names
    syms = exported(_lib.GPU_LIB)
    missing = [n for n in names if n not in syms]
    assert not missing, missing
    lib = _lib.gpu()  # loads without a GPU
    for n in names:
        assert hasattr(lib, n)
    assert set(names) <= set(_lib.GPU_API), "ctypes table misses %s" % (set(names) - set(_lib.GPU_API))


def test_host_library_exports_every_declared_symbol():
    from cbns3d_cart_mpi_gb300 import _lib
    names = header_functions("cbns_host.h")
    syms = exported(_lib.HOST_LIB)
    assert not [n for n in names if n not in syms]
    assert set(names) <= set(_lib.HOST_API)


def test_create_without_device_fails_cleanly():
    """No GPU in this container: cbns_create must fail with a status, not crash."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from cbns3d_cart_mpi_gb300.solver import CbnsError, Solver
    with pytest.raises(CbnsError):
        Solver(tgv_params(8))


def test_params_derive_matches_reference_formulas():
    from cbns3d_cart_mpi_gb300 import _lib
    p = tgv_params(32, Re=1234.5, Mach=0.17)
    q = CbnsParams()
    ctypes.memmove(ctypes.byref(q), ctypes.byref(p), ctypes.sizeof(p))
    q.Mach2 = q.Re_inv = q.C_dt_v = 0.0
    assert _lib.gpu().cbns_params_derive(ctypes.byref(q)) == 0
    for f in ("Mach2", "Re_inv", "Pr_inv", "gam1", "gM2", "gam1_inv", "p_inf", "C_T_inf", "C_dt_v"):
        assert getattr(q, f) == getattr(p, f), f


def test_ini_to_input_txt_and_read_input(tmp_path):
    from cbns3d_cart_mpi_gb300.params import ini_to_input_txt, read_input
    from cbns3d_cart_mpi_gb300.solver import read_input as read_input_cpp
    ini = tmp_path / "case.ini"
    ini.write_text("[string]\ncheckpoint_fname = ckpt\n\n[real]\nCFL = 0.5\nt_cur = 0.0\nt_end = 20.0\n"
                   "Pr = 0.71\ngamma = 1.4\nMach = 0.1\nRe = 1600.0\nT_inf = 255.556\nL = 1.0\n\n"
                   "[integer]\nIM = 64\nJM = 48\nKM = 32\nnstep_max = 100\ncheckpoint_freq = 5000\n"
                   "num_output = 10\n\n[bool]\nis_restart = 1\n")
    out = tmp_path / "input.txt"
    pairs = ini_to_input_txt(str(ini), str(out))
    assert [k for k, _ in pairs][:3] == ["checkpoint_fname", "CFL", "t_cur"]
    assert out.read_text().split("\n")[:4] == ["ckpt", "0.5", "0.0", "20.0"]
    a = read_input(str(out))
    b = read_input_cpp(str(out))
    for name, _ in CbnsParams._fields_:
        assert getattr(a, name) == getattr(b, name), name
    assert (a.IM, a.JM, a.KM, a.nstep_max, a.is_restart) == (64, 48, 32, 100, 1)
    assert a.C_T_inf == 110.5 / 255.556


def test_read_input_errors(tmp_path):
    """The reference's read_input never reports a bad file (its try/catch is dead,
    src/read_input.cpp:19-97); this one does."""
    from cbns3d_cart_mpi_gb300.solver import CbnsError, read_input
    with pytest.raises(CbnsError) as e:
        read_input(str(tmp_path / "missing.txt"))
    assert e.value.status == CBNS_ERR_IO
    short = tmp_path / "short.txt"
    short.write_text("ckpt\n0.5\n0.0\n")
    with pytest.raises(CbnsError) as e:
        read_input(str(short))
    assert e.value.status == CBNS_ERR_FORMAT
    bad = tmp_path / "bad.txt"
    bad.write_text("ckpt 0.5 0.0 20 0.71 1.4 0.1 abc 255 1 8 8 8 10 10 1 1\n")
    with pytest.raises(CbnsError):
        read_input(str(bad))


def _golden_state(golden_dir, key):
    g = np.load(os.path.join(golden_dir, "tgv_min.npz"))
    from oracle.oracle import OracleBlock
    p = tgv_params(4, JM=5, KM=6)
    Q = np.zeros((6 + 2 * NG, 5 + 2 * NG, 4 + 2 * NG, 5))
    Q[NG:-NG, NG:-NG, NG:-NG] = g[key]
    o = OracleBlock(p)
    o.set_Q(Q, 0.0)
    return p, o, g


def test_checkpoint_bytes_match_reference(golden_dir, tmp_path):
    from cbns3d_cart_mpi_gb300.solver import output_bin, read_bin
    p, o, g = _golden_state(golden_dir, "Q2")
    ref = open(os.path.join(golden_dir, "ckpt_4x5x6.dat"), "rb").read()
    path = tmp_path / "ck.dat"
    output_bin(str(path), float(g["t"][1]), o.get_Q(), 4, 5, 6)
    assert path.read_bytes() == ref
    t, Q = read_bin(os.path.join(golden_dir, "ckpt_4x5x6.dat"), 4, 5, 6)
    assert t == g["t"][1] and np.array_equal(Q, o.get_Q())


def test_checkpoint_errors(golden_dir, tmp_path):
    from cbns3d_cart_mpi_gb300.solver import CbnsError, read_bin
    with pytest.raises(CbnsError) as e:  # "The dimensions do not match." (src/Block3d.cpp:334-338)
        read_bin(os.path.join(golden_dir, "ckpt_4x5x6.dat"), 4, 5, 7)
    assert e.value.status == CBNS_ERR_FORMAT
    trunc = tmp_path / "t.dat"
    trunc.write_bytes(open(os.path.join(golden_dir, "ckpt_4x5x6.dat"), "rb").read()[:1000])
    with pytest.raises(CbnsError) as e:
        read_bin(str(trunc), 4, 5, 6)
    assert e.value.status == CBNS_ERR_FORMAT
    with pytest.raises(CbnsError) as e:
        read_bin(str(tmp_path / "none.dat"), 4, 5, 6)
    assert e.value.status == CBNS_ERR_IO


@pytest.mark.parametrize("which,key", [("vtk_init", "Q0"), ("vtk_final", "Q2")])
def test_vtk_text_matches_reference(golden_dir, tmp_path, which, key):
    from cbns3d_cart_mpi_gb300.solver import output_vtk_xml
    p, o, g = _golden_state(golden_dir, key)
    output_vtk_xml(str(tmp_path), "output", p, o.get_prims())
    for f in ("output000.vtr", "output.vtm"):
        ref = open(os.path.join(golden_dir, "vtk", which + "_" + f)).read()
        assert (tmp_path / f).read_text() == ref, f


def _cell_text(values):
    """The lines of one cell-data array as the reference prints them
    (src/Block3d.cpp:416-424), built with Python's %e: both are correctly rounded."""
    out = ["        "]
    for c, v in enumerate(values):
        out.append("%e " % v)
        if c % 5 == 4:
            out.append("\n        ")
    if len(values) % 5:
        out.append("\n")
    return "".join(out)


def _wide_ranging_fields(shape, seed):
    """Five padded fields whose values test a %e formatter: typical densities,
    magnitudes from 1e-300 to 1e300, random bit patterns, decimal near-ties and
    exact binary ties, powers of ten and their neighbours, signed zeros,
    subnormals and infinities."""
    rng = np.random.default_rng(seed)
    n = int(np.prod(shape))
    rho = 1.0 + 1e-3 * rng.standard_normal(n)
    u = rng.standard_normal(n) * 10.0 ** rng.integers(-300, 300, n).astype(float)
    v = rng.integers(0, 2**64, n, dtype=np.uint64).view(np.float64).copy()
    v[~np.isfinite(v)] = 0.0
    digits = rng.integers(1_000_000, 10_000_000, n).astype(float)
    w = (digits + 0.5) * 10.0 ** rng.integers(-290, 290, n).astype(float)
    for _ in range(3):
        step = rng.integers(-1, 2, n)
        w = np.where(step > 0, np.nextafter(w, np.inf), np.where(step < 0, np.nextafter(w, 0.0), w))
    w[::7] = digits[::7] + 0.5                      # exact binary ties: half to even
    w[3::7] = (digits[3::7] + 0.5) * 2.0 ** -20
    pw = 10.0 ** rng.integers(-300, 300, n).astype(float)
    p = np.where(rng.random(n) < 0.5, np.nextafter(pw, np.inf), np.nextafter(pw, 0.0))
    p[::11] = 9.9999995 * 10.0 ** rng.integers(-20, 20, p[::11].size).astype(float)
    special = [0.0, -0.0, 5e-324, -1e-310, 2.2250738585072014e-308, 1e-290, 1.0000001e-290, 9.999999e289,
               1e290, 1.7976931348623157e308, np.inf, -np.inf, 0.5, 1.0, 9.9999995, 1234567.5, 1234568.5]
    p[:len(special)] = special
    return [a.reshape(shape) for a in (rho, u, v, w, p)]


@pytest.mark.parametrize("threads", ["1", "3", None])
def test_vtk_text_of_wide_ranging_values(tmp_path, monkeypatch, threads):
    """The writer formats the numbers itself, in chunks spread over host threads;
    over a grid of several chunks per array and values of every kind, the text is
    printf's "%e " in the reference's line layout, whatever the thread count."""
    from cbns3d_cart_mpi_gb300.solver import output_vtk_xml
    if threads is None:
        monkeypatch.delenv("CBNS_HOST_THREADS", raising=False)
    else:
        monkeypatch.setenv("CBNS_HOST_THREADS", threads)
    IM, JM, KM = 37, 41, 23
    p = tgv_params(IM, JM=JM, KM=KM)
    fields = _wide_ranging_fields((KM + 2 * NG, JM + 2 * NG, IM + 2 * NG), seed=3)
    names = ("rho", "u", "v", "w", "p")
    output_vtk_xml(str(tmp_path), "output", p, dict(zip(names, fields)))
    text = (tmp_path / "output000.vtr").read_text()
    for name, a in zip(names, fields):
        got = text.split('<DataArray type="Float64" Name="%s" format="ascii">\n' % name)[1]
        got = got.split("      </DataArray>")[0]
        assert got == _cell_text(a[NG:-NG, NG:-NG, NG:-NG].ravel()), name


def test_initial_condition_matches_reference(golden_dir):
    from cbns3d_cart_mpi_gb300.solver import initial_condition
    for name, dims in (("tgv16.npz", (16, 16, 16)), ("tgv_odd.npz", (12, 16, 20))):
        g = np.load(os.path.join(golden_dir, name))
        IM, JM, KM = dims
        Q = initial_condition(tgv_params(IM, JM=JM, KM=KM))
        np.testing.assert_allclose(Q[NG:-NG, NG:-NG, NG:-NG], g["Q0"], rtol=4e-16, atol=0)


def test_perturbation_is_solenoidal_and_seeded():
    from cbns3d_cart_mpi_gb300.solver import initial_condition, initial_condition_perturbed
    p = tgv_params(32, Re=800.0, Mach=0.2)
    a = initial_condition_perturbed(p, seed=5, amp=1e-3)
    b = initial_condition_perturbed(p, seed=5, amp=1e-3)
    c = initial_condition_perturbed(p, seed=6, amp=1e-3)
    base = initial_condition(p)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    ai, bi = a[NG:-NG, NG:-NG, NG:-NG], base[NG:-NG, NG:-NG, NG:-NG]
    du = ai[..., 1:4] / ai[..., :1] - bi[..., 1:4] / bi[..., :1]
    amp = np.abs(du).max()
    assert 1e-4 < amp <= 1.01e-3
    # Spectral divergence of the perturbation is zero to rounding.
    k = np.fft.fftfreq(32, 1.0 / 32)
    div = sum(np.fft.ifftn(1j * np.meshgrid(k, k, k, indexing="ij")[2 - d] * np.fft.fftn(du[..., d])).real
              for d in range(3))
    assert np.abs(div).max() < 1e-12


def test_opcount_constants_match_record(golden_dir):
    from cbns3d_cart_mpi_gb300 import workload as w
    rec = {}
    for line in open(os.path.join(golden_dir, "opcount.txt")):
        parts = line.split()
        if len(parts) == 2:
            rec[parts[0]] = float(parts[1])
    assert rec["rec_riemann_x_per_face"] == w.FLOPS_PER_FACE
    assert round(rec["calc_viscous_terms_per_ring_point"]) == w.FLOPS_VISC_TERMS_PER_RING
    assert rec["calc_viscous_flux_per_ring_point"] == w.FLOPS_VISC_FLUX_PER_RING
    assert round(rec["viscous_divergence_per_cell"]) == w.FLOPS_VISC_DIV_PER_CELL
    assert rec["update_rk3_per_cell"] == w.FLOPS_UPDATE_PER_CELL
    assert rec["calc_primitive_per_padded_cell"] == w.FLOPS_PRIM_PER_PADDED
    assert round(rec["calc_dt_per_cell"]) == w.FLOPS_DT_PER_CELL
    assert abs(w.flops_per_step(256, 256, 256) / 256 ** 3 - 15198.25) < 0.1


def test_block_size_limit_follows_memory_not_a_31_bit_index():
    """Offsets are 64-bit, so a block is limited by device memory (cbns_create
    compares cbns_footprint's arena size with the free bytes) and by the 16-bit
    tile coordinates, not by 5 (N+8)^3 < 2^31 (N ~ 745).  The arena of a 768^3
    block fits the 280 GB a GB300 offers in every precision, 1024^3 does not."""
    from cbns3d_cart_mpi_gb300.solver import CbnsError, footprint
    hbm = 280e9
    per_cell = {}
    for prec in ("fp64", "fp32_mixed", "fp64_ff"):
        fp768 = footprint(768, 768, 768, prec)
        assert fp768 < hbm, (prec, fp768)
        assert footprint(1024, 1024, 1024, prec) > hbm
        per_cell[prec] = fp768 / 776 ** 3
        # grows with the padded volume: about 380 bytes per padded cell (about 555
        # with the float-float copies and packed layouts; 768^3 is then 259 GB)
        assert 300 < per_cell[prec] < 600, per_cell
    # Float-float solves add float-float copies of Q and Q_p and of six
    # primitives (16 pairs of binary32, 128 bytes, per padded cell), and pack the
    # face fluxes (48 instead of 40 bytes per interior cell and direction) and the
    # viscous terms (96 instead of 72 bytes per ring point).
    extra = footprint(256, 256, 256, "fp64_ff") - footprint(256, 256, 256, "fp64")
    assert abs(extra - (128 * 264 ** 3 + 24 * 256 ** 3 + 24 * 260 ** 3)) < 4096, extra
    # 745^3 and 746^3 straddle the old 31-bit limit; both are accepted now.
    assert footprint(746, 746, 746) > footprint(745, 745, 745)
    # Tile coordinates are 16-bit: 65535 - 2 NG cells along an axis is the most.
    footprint(65527, 4, 4)
    with pytest.raises(CbnsError):
        footprint(65528, 4, 4)
    with pytest.raises(CbnsError):
        footprint(4, 4, 70000)


def test_create_rejects_block_extents_other_than_the_grid():
    """One GPU holds the whole periodic grid: cbns_create takes the spacing from
    p->IM/JM/KM and the periodic images from the block's extents, so the two must
    agree.  The check runs before any device call, so it answers on a host
    without a GPU too."""
    from cbns3d_cart_mpi_gb300 import _lib
    from cbns3d_cart_mpi_gb300._abi import CBNS_ERR_BAD_DIMS
    p = tgv_params(16, JM=12, KM=20)
    h = ctypes.c_void_p()
    st = _lib.gpu().cbns_create(ctypes.byref(p), 16, 12, 21, 0, ctypes.byref(h))
    assert st == CBNS_ERR_BAD_DIMS and not h.value
    assert "whole periodic grid" in _lib.last_error()
