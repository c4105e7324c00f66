"""Python face of the C ABI: a Block3d-like solve on the GPU, and the host pieces.

Mirrors the reference's Block3d public interface (include/Block3d.h:126-163):
``calc_dt``, the three-stage step, ``get_Q``/``get_Q_p``, the primitive arrays,
``output_bin``/``read_bin``/``output_vtk_xml`` — each call goes through the
native libraries; nothing here computes the solution.
"""
import ctypes
import os

import numpy as np

from . import _lib
from ._abi import (CBNS_FINISHED, CBNS_FP32_MIXED, CBNS_FP64, CBNS_FP64_FF, CBNS_OK, NEQ, NG, STATUS_NAMES,
                   CbnsParams)


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


PRECISIONS = {"fp64": CBNS_FP64, "fp32_mixed": CBNS_FP32_MIXED, "fp64_ff": CBNS_FP64_FF}


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

    def init_tgv(self, seed=0, amp=0.0, nmodes=0, kmax=4, t=None):
        """Build the Taylor-Green state (plus the seeded perturbation when nmodes > 0)
        on the device, then the start-up fill (cbns_init_tgv)."""
        _check(_lib.gpu().cbns_init_tgv(self._h, int(seed), float(amp), int(nmodes), int(kmax),
                                        self.params.t_cur if t is None else t), "cbns_init_tgv")

    def _out_state(self, out):
        """A buffer the library may write a padded state into: float64, C-contiguous,
        exactly one state long."""
        if out is None:
            return np.empty(self.shape)
        if out.dtype != np.float64 or not out.flags.c_contiguous or out.size != int(np.prod(self.shape)):
            raise ValueError("out must be a C-contiguous float64 array of %d values" % int(np.prod(self.shape)))
        return out

    def download_Q(self, out=None):
        out = self._out_state(out)
        _check(_lib.gpu().cbns_download_Q(self._h, _ptr(out)), "cbns_download_Q")
        return out

    def download_Q_p(self, out=None):
        out = self._out_state(out)
        _check(_lib.gpu().cbns_download_Q_p(self._h, _ptr(out)), "cbns_download_Q_p")
        return out

    def load_checkpoint(self, path):
        """Restart from a checkpoint file in the reference's output_bin format,
        streamed to the device (cbns_load_checkpoint); returns the file's t_cur."""
        t = ctypes.c_double()
        _check(_lib.gpu().cbns_load_checkpoint(self._h, os.fsencode(path), ctypes.byref(t)), "cbns_load_checkpoint")
        return t.value

    def save_checkpoint(self, path):
        """Write Q and t_cur in the reference's output_bin format (cbns_save_checkpoint)."""
        _check(_lib.gpu().cbns_save_checkpoint(self._h, os.fsencode(path)), "cbns_save_checkpoint")

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

    # Asynchronous forms (cbns_*_async): each call enqueues and returns; the host
    # arrays must stay alive and untouched until wait().  Page-locked arrays
    # (pinned_state) let the copies overlap the kernels.
    def upload_Q_async(self, Q, t=None):
        if not (isinstance(Q, np.ndarray) and Q.dtype == np.float64 and Q.flags.c_contiguous):
            raise ValueError("upload_Q_async needs a C-contiguous float64 array that stays alive until wait()")
        if Q.size != int(np.prod(self.shape)):
            raise ValueError("Q has %d values, %d expected" % (Q.size, int(np.prod(self.shape))))
        _check(_lib.gpu().cbns_upload_Q_async(self._h, _ptr(Q), self.params.t_cur if t is None else t),
               "cbns_upload_Q_async")

    def step_async(self, t_end=None):
        te = self.params.t_end if t_end is None else t_end
        _check(_lib.gpu().cbns_step_async(self._h, te), "cbns_step_async")

    def download_Q_async(self, out):
        if not (isinstance(out, np.ndarray) and out.dtype == np.float64 and out.flags.c_contiguous
                and out.size == int(np.prod(self.shape))):
            raise ValueError("download_Q_async needs a C-contiguous float64 array of the state's size")
        _check(_lib.gpu().cbns_download_Q_async(self._h, _ptr(out)), "cbns_download_Q_async")

    def wait(self):
        """Wait for everything enqueued; returns (dt, t_cur), or None once finished."""
        dt, t = ctypes.c_double(), ctypes.c_double()
        st = _check(_lib.gpu().cbns_wait(self._h, ctypes.byref(dt), ctypes.byref(t)), "cbns_wait")
        return None if st == CBNS_FINISHED else (dt.value, t.value)

    def poll(self):
        done = ctypes.c_int()
        _check(_lib.gpu().cbns_poll(self._h, ctypes.byref(done)), "cbns_poll")
        return bool(done.value)

    def pinned_state(self):
        """A page-locked host array of the state's shape (torch's pinned allocator;
        the solver keeps the owning tensor alive as long as itself)."""
        import torch
        t = torch.empty(int(np.prod(self.shape)), dtype=torch.float64, pin_memory=True)
        if not hasattr(self, "_pins"):
            self._pins = []
        self._pins.append(t)
        return t.numpy().reshape(self.shape)

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


class Batch:
    """Many independent solves stepped together (include/cbns_gpu.h, cbns_batch_*):
    one launch per kernel over the flattened tiles of every solve, a batch step
    replayed as one CUDA graph, each solve stopping at its own t_end."""

    def __init__(self, solvers):
        self.solvers = list(solvers)
        arr = (ctypes.c_void_p * len(self.solvers))(*[s._h.value for s in self.solvers])
        b = ctypes.c_void_p()
        _check(_lib.gpu().cbns_batch_create(arr, len(self.solvers), ctypes.byref(b)), "cbns_batch_create")
        self._b = b

    def close(self):
        if getattr(self, "_b", None) is not None and self._b.value:
            _lib.gpu().cbns_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, nsteps):
        """nsteps batch steps; returns the steps each solve has taken since creation."""
        out = (ctypes.c_uint32 * len(self.solvers))()
        _check(_lib.gpu().cbns_batch_run(self._b, int(nsteps), out), "cbns_batch_run")
        return list(out)

    @property
    def config(self):
        c = _lib.LaunchConfig()
        _check(_lib.gpu().cbns_batch_get_config(self._b, ctypes.byref(c)), "cbns_batch_get_config")
        return {"tile_rows": c.tile_rows, "ctas_per_sm": c.ctas_per_sm}

    def set_config(self, tile_rows=4, ctas_per_sm=0):
        c = _lib.LaunchConfig(tile_rows, ctas_per_sm)
        _check(_lib.gpu().cbns_batch_set_config(self._b, ctypes.byref(c)), "cbns_batch_set_config")

    def autotune(self, reps=2):
        """Time every candidate launch shape over `reps` steps, keep the fastest, and
        restore the solves' state; returns [(tile_rows, ctas_per_sm, ms/step)]."""
        ms = (ctypes.c_double * 64)()
        n = ctypes.c_int()
        _check(_lib.gpu().cbns_batch_autotune(self._b, int(reps), ms, 64, ctypes.byref(n)), "cbns_batch_autotune")
        cands = [(r, c) for r in (2, 4, 8) for c in (0, 2, 4, 8)]
        return [(r, c, ms[i]) for i, (r, c) in enumerate(cands[:n.value])]

    @property
    def stream(self):
        return _lib.gpu().cbns_batch_stream(self._b)


def footprint(IM, JM, KM, precision="fp64"):
    """Device bytes a solve of these extents holds (cbns_footprint)."""
    b = ctypes.c_uint64()
    _check(_lib.gpu().cbns_footprint(IM, JM, KM, PRECISIONS[precision], ctypes.byref(b)), "cbns_footprint")
    return b.value


class Server:
    """Continuous-batching request loop (include/cbns_gpu.h, cbns_server_*)."""

    def __init__(self, precision="fp64", memory_budget_bytes=0, max_active=0, steps_per_round=10, tile_rows=0,
                 ctas_per_sm=0):
        opts = _lib.ServerOpts(PRECISIONS[precision], int(memory_budget_bytes), int(max_active),
                               int(steps_per_round), int(tile_rows), int(ctas_per_sm))
        sv = ctypes.c_void_p()
        _check(_lib.gpu().cbns_server_create(ctypes.byref(opts), ctypes.byref(sv)), "cbns_server_create")
        self._s = sv
        self._shapes = {}  # request id -> padded state shape
        self.precision = precision

    def close(self):
        if getattr(self, "_s", None) is not None and self._s.value:
            _lib.gpu().cbns_server_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _track(self, rid, params):
        self._shapes[rid] = (params.KM + 2 * NG, params.JM + 2 * NG, params.IM + 2 * NG, NEQ)
        return rid

    def submit(self, params, Q0, keep_state=False):
        rid = ctypes.c_uint64()
        Q0 = np.ascontiguousarray(Q0, dtype=np.float64)
        n = NEQ * (params.IM + 2 * NG) * (params.JM + 2 * NG) * (params.KM + 2 * NG)
        if Q0.size != n:
            raise ValueError("Q0 has %d values, %d expected" % (Q0.size, n))
        _check(_lib.gpu().cbns_server_submit(self._s, ctypes.byref(params), params.IM, params.JM, params.KM,
                                             _ptr(Q0), int(keep_state), ctypes.byref(rid)), "cbns_server_submit")
        return self._track(rid.value, params)

    def submit_tgv(self, params, seed=0, amp=0.0, nmodes=0, kmax=4, keep_state=False):
        rid = ctypes.c_uint64()
        _check(_lib.gpu().cbns_server_submit_tgv(self._s, ctypes.byref(params), params.IM, params.JM, params.KM,
                                                 int(seed), float(amp), int(nmodes), int(kmax), int(keep_state),
                                                 ctypes.byref(rid)), "cbns_server_submit_tgv")
        return self._track(rid.value, params)

    def submit_checkpoint(self, params, path, keep_state=False):
        """A request that starts from a checkpoint file, read by the worker at admission."""
        rid = ctypes.c_uint64()
        _check(_lib.gpu().cbns_server_submit_checkpoint(self._s, ctypes.byref(params), params.IM, params.JM,
                                                        params.KM, os.fsencode(path), int(keep_state),
                                                        ctypes.byref(rid)), "cbns_server_submit_checkpoint")
        return self._track(rid.value, params)

    def cancel(self, rid):
        _check(_lib.gpu().cbns_server_cancel(self._s, int(rid)), "cbns_server_cancel")

    def wait(self, rid, timeout=-1.0):
        """Block until the request finishes; returns its info dict (status included)."""
        info = _lib.RequestInfo()
        st = _lib.gpu().cbns_server_wait(self._s, int(rid), float(timeout), ctypes.byref(info))
        out = {f: getattr(info, f) for f, _ in _lib.RequestInfo._fields_}
        out["status"] = st
        return out

    def result(self, rid, shape=None):
        """The kept final state of a request (padded, get_idx_Q layout).  The buffer
        is sized from the request's own extents; a given shape must match them."""
        own = self._shapes.get(int(rid))
        if own is None:
            raise ValueError("unknown request %d" % int(rid))
        if shape is not None and tuple(shape) != own:
            raise ValueError("request %d has shape %s, not %s" % (int(rid), own, tuple(shape)))
        Q = np.empty(own)
        _check(_lib.gpu().cbns_server_result(self._s, int(rid), _ptr(Q)), "cbns_server_result")
        return Q

    def release(self, rid):
        _check(_lib.gpu().cbns_server_release(self._s, int(rid)), "cbns_server_release")

    def stats(self):
        st = _lib.ServerStats()
        _check(_lib.gpu().cbns_server_get_stats(self._s, ctypes.byref(st)), "cbns_server_get_stats")
        return {f: getattr(st, f) for f, _ in _lib.ServerStats._fields_}


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
    if Q.size != NEQ * (IM + 2 * NG) * (JM + 2 * NG) * (KM + 2 * NG):
        raise ValueError("Q has %d values, not one padded %dx%dx%d state" % (Q.size, IM, JM, KM))
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
