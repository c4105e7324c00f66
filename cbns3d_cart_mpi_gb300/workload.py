"""Algorithmic work of the hot path, pinned by counting the reference's own operations.

The per-unit figures are FLOPs (each +, -, *, / and sqrt on a binary64 value, as
written in the reference's source) that the reference executes per unit of
each hot-path function.  They were counted by compiling the reference's
sources with value_type replaced by an op-counting type (oracle/opcount/) and
are recorded in tests/golden/opcount.txt; a test checks these constants
against that record.
"""
FLOPS_PER_FACE = 1570            # rec_riemann_x/y/z, per face (src/Block3d.cpp:555-748)
FLOPS_VISC_TERMS_PER_RING = 129  # calc_viscous_terms incl. 4 calc_gradient, per NGV-ring point
FLOPS_VISC_FLUX_PER_RING = 18    # calc_viscous_flux, per NGV-ring point
FLOPS_VISC_DIV_PER_CELL = 104    # divergence in calc_viscous_flux_contribution, per cell
FLOPS_UPDATE_PER_CELL = 54       # update_rk3, per cell
FLOPS_PRIM_PER_PADDED = 14       # calc_primitive, per padded cell
FLOPS_DT_PER_CELL = 31           # calc_dt, per cell (plus a data-dependent re-add)

NG, NGV = 4, 2


def faces_per_direction(IM, JM, KM, d, periodic=False):
    """Faces per direction.  The reference computes (IM+1)*JM*KM for x (faces
    -1/2 .. IM-1/2), etc.; on a periodic grid the last face is the first, so the
    distinct faces (what the GPU computes) are IM*JM*KM (periodic=True)."""
    ext = [IM, JM, KM]
    if not periodic:
        ext[d] += 1
    return ext[0] * ext[1] * ext[2]


def kernel_flops(name, IM, JM, KM, periodic=True):
    """Algorithmic FLOPs of one launch of the named kernel (one solve): the
    reference's op count per unit times the units, with the distinct periodic
    faces by default (periodic=False counts the faces the reference computes)."""
    cells = IM * JM * KM
    ring = (IM + 2 * NGV) * (JM + 2 * NGV) * (KM + 2 * NGV)
    padded = (IM + 2 * NG) * (JM + 2 * NG) * (KM + 2 * NG)
    if name.startswith("inviscid_"):
        d = "xyz".index(name[-1])
        return FLOPS_PER_FACE * faces_per_direction(IM, JM, KM, d, periodic)
    if name == "viscous":
        return (FLOPS_VISC_TERMS_PER_RING + FLOPS_VISC_FLUX_PER_RING) * ring
    if name == "update":
        return (FLOPS_VISC_DIV_PER_CELL + FLOPS_UPDATE_PER_CELL) * cells + FLOPS_PRIM_PER_PADDED * padded
    if name == "dt_reduce":
        return FLOPS_DT_PER_CELL * cells
    return 0


def flops_per_step(IM, JM, KM):
    """Algorithmic FLOPs of one RK3 step (3 stages + calc_dt), as the reference
    executes it (its (N+1) N^2 faces per direction)."""
    stage = sum(kernel_flops(n, IM, JM, KM, periodic=False)
                for n in ("inviscid_x", "inviscid_y", "inviscid_z", "viscous", "update"))
    return 3 * stage + kernel_flops("dt_reduce", IM, JM, KM)


def state_bytes_per_step(IM, JM, KM):
    """Minimum HBM traffic of one step: read Q, write Q_p (stage 1); read Q, Q_p,
    write one (stages 2, 3) -> 320 B per cell (binary64, 5 fields)."""
    return 320 * IM * JM * KM


# Compulsory HBM bytes per interior cell of the FP32-mixed update kernel, by stage:
# reads Q (5 binary64: 40 B), Q_p (40 B, stages 2-3 only), the 15 binary32 face fluxes
# (60 B; the neighbours' are their own cells'), the viscous terms on the NGV ring,
# grouped by differencing direction as 3 x 4 binary32 (48 B x 1.047 ring/interior at
# 256^3); writes the binary64 state (40 B), the binary32 perturbation state (20 B) and
# 8 binary32 primitives (32 B), plus the periodic ghost images of those writes (9.7% of
# the cells at 256^3, 9 B).
MIXED_UPDATE_BYTES_PER_CELL = {1: 251, 2: 291, 3: 291}


def mixed_update_bytes(IM, JM, KM):
    """Average compulsory bytes of one FP32-mixed update launch over the three stages."""
    return sum(MIXED_UPDATE_BYTES_PER_CELL.values()) / 3.0 * IM * JM * KM



def probe_peak(fp64=True):
    """Measured FMA throughput of the current GPU, TFLOP/s (2 FLOPs per FMA): the
    pipe peak the roofline divides by (libcbns_probe.so, built beside the product
    library but not part of it)."""
    import ctypes
    from . import _lib
    tf = ctypes.c_double()
    st = _lib.probe().cbns_probe_peak(1 if fp64 else 0, ctypes.byref(tf))
    if st != 0:
        raise RuntimeError("cbns_probe_peak failed with status %d" % st)
    return tf.value
