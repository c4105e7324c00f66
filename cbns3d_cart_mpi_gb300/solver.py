"""Python face of the C ABI: a Block3d-like solve on the GPU, and the host pieces.

Mirrors the reference's Block3d public interface (include/Block3d.h:126-163):
``calc_dt``, the three-stage step, ``get_Q``/``get_Q_p``, the primitive arrays,
``output_bin``/``read_bin``/``output_vtk_xml`` — each call goes through the
native libraries; nothing here computes the solution.
"""
import ctypes

import numpy as np

from . import _lib
from ._abi import CBNS_FINISHED, CBNS_FP32_MIXED, CBNS_FP64, CBNS_OK, NEQ, NG, STATUS_NAMES, CbnsParams


class CbnsError(RuntimeError):
    def __init__(self, status, where):
        self.status = status
        msg = "%s failed: %s (%s)" % (where, STATUS_NAMES.get(status, status), _lib.last_error())
        super().__init__(msg)


def _check(st, where):
    if st < 0:
        raise CbnsError(st, where)
    return st


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


PRECISIONS = {"fp64": CBNS_FP64, "fp32_mixed": CBNS_FP32_MIXED}


class Solver:
    """One periodic block on the GPU (a Block3d whose stage block runs on sm_103a)."""

    def __init__(self, params, IM=None, JM=None, KM=None, precision="fp64"):
        self.params = params
        self.IM = int(IM or params.IM)
        self.JM = int(JM or params.JM)
        self.KM = int(KM or params.KM)
        self.precision = precision
        h = ctypes.c_void_p()
        _check(_lib.gpu().cbns_create(ctypes.byref(params), self.IM, self.JM, self.KM, PRECISIONS[precision],
                                      ctypes.byref(h)), "cbns_create")
        self._h = h

    @property
    def shape(self):
        return (self.KM + 2 * NG, self.JM + 2 * NG, self.IM + 2 * NG, NEQ)

    @property
    def prim_shape(self):
        return self.shape[:3]

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.gpu().cbns_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # --- state -------------------------------------------------------------
    def upload_Q(self, Q, t=None):
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        if Q.size != int(np.prod(self.shape)):
            raise ValueError("Q has %d values, %d expected" % (Q.size, int(np.prod(self.shape))))
        _check(_lib.gpu().cbns_upload_Q(self._h, _ptr(Q), self.params.t_cur if t is None else t), "cbns_upload_Q")

    def download_Q(self, out=None):
        out = np.empty(self.shape) if out is None else out
        _check(_lib.gpu().cbns_download_Q(self._h, _ptr(out)), "cbns_download_Q")
        return out

    def download_Q_p(self, out=None):
        out = np.empty(self.shape) if out is None else out
        _check(_lib.gpu().cbns_download_Q_p(self._h, _ptr(out)), "cbns_download_Q_p")
        return out

    def download_prims(self):
        arrs = [np.empty(self.prim_shape) for _ in range(6)]
        _check(_lib.gpu().cbns_download_prims(self._h, *[_ptr(a) for a in arrs]), "cbns_download_prims")
        return dict(zip(["rho", "u", "v", "w", "p", "T"], arrs))

    # --- stepping ----------------------------------------------------------
    def calc_dt(self):
        dt = ctypes.c_double()
        _check(_lib.gpu().cbns_calc_dt(self._h, ctypes.byref(dt)), "cbns_calc_dt")
        return dt.value

    def stage(self, dt, stage):
        _check(_lib.gpu().cbns_stage(self._h, float(dt), int(stage)), "cbns_stage")

    def step(self, t_end=None):
        """One time-loop iteration; returns (dt, t_cur), or None once finished."""
        dt, t = ctypes.c_double(), ctypes.c_double()
        te = self.params.t_end if t_end is None else t_end
        st = _check(_lib.gpu().cbns_step(self._h, te, ctypes.byref(dt), ctypes.byref(t)), "cbns_step")
        return None if st == CBNS_FINISHED else (dt.value, t.value)

    def run(self, nsteps, t_end=None):
        done = ctypes.c_uint32()
        te = self.params.t_end if t_end is None else t_end
        _check(_lib.gpu().cbns_run(self._h, int(nsteps), te, ctypes.byref(done)), "cbns_run")
        return done.value

    def time(self):
        t, dt = ctypes.c_double(), ctypes.c_double()
        _check(_lib.gpu().cbns_get_time(self._h, ctypes.byref(t), ctypes.byref(dt)), "cbns_get_time")
        return t.value, dt.value

    def diagnostics(self):
        ke, en = ctypes.c_double(), ctypes.c_double()
        _check(_lib.gpu().cbns_diagnostics(self._h, ctypes.byref(ke), ctypes.byref(en)), "cbns_diagnostics")
        return ke.value, en.value

    def check_state(self):
        return _check(_lib.gpu().cbns_check_state(self._h), "cbns_check_state") == CBNS_OK

    def profile_begin(self):
        """Time every kernel this solve launches until profile_end (CUDA events)."""
        _check(_lib.gpu().cbns_profile_begin(self._h), "cbns_profile_begin")

    def profile_end(self):
        """{kernel name: (launches, total ms)} since profile_begin."""
        recs = (_lib.KernelTime * 32)()
        n = ctypes.c_int()
        _check(_lib.gpu().cbns_profile_end(self._h, recs, 32, ctypes.byref(n)), "cbns_profile_end")
        return {recs[i].name.decode(): (recs[i].launches, recs[i].total_ms) for i in range(n.value)}

    @property
    def stream(self):
        return _lib.gpu().cbns_stream(self._h)

    def info(self):
        dims = (ctypes.c_uint32 * 3)()
        nbytes, prec = ctypes.c_uint64(), ctypes.c_int()
        _check(_lib.gpu().cbns_get_info(self._h, dims, ctypes.byref(nbytes), ctypes.byref(prec)), "cbns_get_info")
        return {"dims": tuple(dims), "device_bytes": nbytes.value, "precision": prec.value}


def probe_peak(fp64=True):
    """Measured FMA throughput of the current GPU, TFLOP/s (2 FLOPs per FMA)."""
    tf = ctypes.c_double()
    _check(_lib.gpu().cbns_probe_peak(1 if fp64 else 0, ctypes.byref(tf)), "cbns_probe_peak")
    return tf.value


# --- host pieces (include/cbns_host.h) ----------------------------------------

def read_input(path="input.txt"):
    p = CbnsParams()
    _check(_lib.host().cbns_host_read_input(str(path).encode(), ctypes.byref(p)), "cbns_host_read_input")
    return p


def gen_mesh(params, IM=None, JM=None, KM=None, origin=(0, 0, 0)):
    IM, JM, KM = IM or params.IM, JM or params.JM, KM or params.KM
    x, y, z = np.empty(IM + 1), np.empty(JM + 1), np.empty(KM + 1)
    _check(_lib.host().cbns_host_gen_mesh(ctypes.byref(params), IM, JM, KM, *origin, _ptr(x), _ptr(y), _ptr(z)),
           "cbns_host_gen_mesh")
    return x, y, z


def initial_condition(params, IM=None, JM=None, KM=None, origin=(0, 0, 0)):
    """Taylor-Green state Q (ghosts zero) of Block3d::initial_condition + calc_conservative."""
    IM, JM, KM = IM or params.IM, JM or params.JM, KM or params.KM
    Q = np.empty((KM + 2 * NG, JM + 2 * NG, IM + 2 * NG, NEQ))
    _check(_lib.host().cbns_host_initial_condition(ctypes.byref(params), IM, JM, KM, *origin, _ptr(Q)),
           "cbns_host_initial_condition")
    return Q


def initial_condition_perturbed(params, seed, amp=1e-3, nmodes=16, kmax=4):
    """Taylor-Green state plus a solenoidal random-Fourier velocity perturbation
    (project-defined, |k| <= kmax, total amplitude amp)."""
    IM, JM, KM = params.IM, params.JM, params.KM
    Q = np.empty((KM + 2 * NG, JM + 2 * NG, IM + 2 * NG, NEQ))
    _check(_lib.host().cbns_host_initial_condition_perturbed(ctypes.byref(params), IM, JM, KM, int(seed), float(amp),
                                                             int(nmodes), int(kmax), _ptr(Q)),
           "cbns_host_initial_condition_perturbed")
    return Q


def output_bin(fname, t_cur, Q, IM, JM, KM):
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    _check(_lib.host().cbns_host_output_bin(str(fname).encode(), float(t_cur), IM, JM, KM, _ptr(Q)),
           "cbns_host_output_bin")


def read_bin(fname, IM, JM, KM):
    Q = np.empty((KM + 2 * NG, JM + 2 * NG, IM + 2 * NG, NEQ))
    t = ctypes.c_double()
    _check(_lib.host().cbns_host_read_bin(str(fname).encode(), IM, JM, KM, _ptr(Q), ctypes.byref(t)),
           "cbns_host_read_bin")
    return t.value, Q


def output_vtk_xml(dir_path, fname, params, prims, rank=0, num_blocks=1):
    IM, JM, KM = params.IM, params.JM, params.KM
    x, y, z = gen_mesh(params)
    arrs = [np.ascontiguousarray(prims[k], dtype=np.float64) for k in ("rho", "u", "v", "w", "p")]
    _check(_lib.host().cbns_host_output_vtk_xml(str(dir_path).encode(), str(fname).encode(), rank, num_blocks,
                                                IM, JM, KM, _ptr(x), _ptr(y), _ptr(z), *[_ptr(a) for a in arrs]),
           "cbns_host_output_vtk_xml")
