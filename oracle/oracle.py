"""ctypes wrapper of the oracle's CPU restatement (``oracle/cbns_oracle.c``).

TEST INFRASTRUCTURE: imported only by tests, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline leg, as the checker or the timed CPU baseline.
"""
import ctypes
import os

import numpy as np

from cbns3d_cart_mpi_gb300._abi import NEQ, NG, CbnsParams, padded_shape

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def lib():
    global _lib
    if _lib is None:
        from oracle.build import build_port
        path = build_port()
        L = ctypes.CDLL(path)
        vp, d, dp, L_ = ctypes.c_void_p, ctypes.c_double, ctypes.POINTER(ctypes.c_double), ctypes.c_long
        L.oracle_create.restype = vp
        L.oracle_create.argtypes = [ctypes.POINTER(CbnsParams), L_, L_, L_]
        L.oracle_destroy.argtypes = [vp]
        L.oracle_initial_condition.argtypes = [vp]
        L.oracle_start.argtypes = [vp]
        L.oracle_step.argtypes = [vp, dp, dp]
        L.oracle_step.restype = ctypes.c_int
        L.oracle_stage.argtypes = [vp, d, ctypes.c_int]
        L.oracle_calc_dt.argtypes = [vp]
        L.oracle_calc_dt.restype = d
        L.oracle_set_Q.argtypes = [vp, ctypes.c_void_p, d]
        L.oracle_get_Q.argtypes = [vp, ctypes.c_void_p]
        L.oracle_get_Q_p.argtypes = [vp, ctypes.c_void_p]
        L.oracle_get_prims.argtypes = [vp] + [ctypes.c_void_p] * 7
        L.oracle_get_time.argtypes = [vp]
        L.oracle_get_time.restype = d
        L.oracle_get_spacing.argtypes = [vp, ctypes.c_void_p]
        L.oracle_diagnostics.argtypes = [ctypes.c_void_p, L_, L_, L_, d, d, d, dp, dp]
        L.oracle_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class OracleBlock:
    """One reference Block3d restated on the CPU (single periodic block)."""

    def __init__(self, params, IM=None, JM=None, KM=None):
        self.params = params
        self.IM = IM or params.IM
        self.JM = JM or params.JM
        self.KM = KM or params.KM
        self._h = lib().oracle_create(ctypes.byref(params), self.IM, self.JM, self.KM)
        if not self._h:
            raise ValueError("oracle_create failed for %s" % ((self.IM, self.JM, self.KM),))

    def close(self):
        if self._h:
            lib().oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def shape(self):
        return padded_shape(self.IM, self.JM, self.KM)

    def initial_condition(self):
        """Block3d::initial_condition + calc_conservative + the start-up ghost fill."""
        lib().oracle_initial_condition(self._h)
        lib().oracle_start(self._h)

    def set_Q(self, Q, t=0.0):
        Q = np.ascontiguousarray(Q, dtype=np.float64).reshape(self.shape)
        lib().oracle_set_Q(self._h, _ptr(Q), t)
        lib().oracle_start(self._h)

    def get_Q(self):
        Q = np.empty(self.shape)
        lib().oracle_get_Q(self._h, _ptr(Q))
        return Q

    def get_Q_p(self):
        Q = np.empty(self.shape)
        lib().oracle_get_Q_p(self._h, _ptr(Q))
        return Q

    def get_prims(self):
        n = self.shape[:3]
        arrs = [np.empty(n) for _ in range(7)]
        lib().oracle_get_prims(self._h, *[_ptr(a) for a in arrs])
        return dict(zip(["rho", "u", "v", "w", "p", "T", "mu"], arrs))

    def calc_dt(self):
        return lib().oracle_calc_dt(self._h)

    def stage(self, dt, stage):
        lib().oracle_stage(self._h, dt, stage)

    def step(self):
        dt, t = ctypes.c_double(), ctypes.c_double()
        fin = lib().oracle_step(self._h, ctypes.byref(dt), ctypes.byref(t))
        return (None, None) if fin else (dt.value, t.value)

    @property
    def t(self):
        return lib().oracle_get_time(self._h)

    def spacing(self):
        d = np.empty(3)
        lib().oracle_get_spacing(self._h, _ptr(d))
        return tuple(d)

    def diagnostics(self, Q=None):
        Q = self.get_Q() if Q is None else np.ascontiguousarray(Q, dtype=np.float64)
        return diagnostics(Q, self.IM, self.JM, self.KM, *self.spacing())


def diagnostics(Q, IM, JM, KM, dx, dy, dz):
    """Kinetic energy and enstrophy (project-defined) of a ghost-filled state."""
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    ke, en = ctypes.c_double(), ctypes.c_double()
    lib().oracle_diagnostics(_ptr(Q), IM, JM, KM, dx, dy, dz, ctypes.byref(ke), ctypes.byref(en))
    return ke.value, en.value


def num_threads():
    return lib().oracle_num_threads()


def read_state(path):
    """Read a state written in Block3d::output_bin's format (src/Block3d.cpp:964-987):
    t (f64), IM_G, JM_G, KM_G (u32), then Q (f64, get_idx_Q order, ghosts included)."""
    with open(path, "rb") as f:
        t = np.frombuffer(f.read(8), dtype=np.float64)[0]
        dims = np.frombuffer(f.read(12), dtype=np.uint32)
        Q = np.frombuffer(f.read(), dtype=np.float64)
    IM_G, JM_G, KM_G = (int(x) for x in dims)
    return float(t), Q.reshape(KM_G, JM_G, IM_G, NEQ).copy()


def write_state(path, Q, t):
    """Write a state in Block3d::output_bin's format."""
    KM_G, JM_G, IM_G, _ = Q.shape
    with open(path, "wb") as f:
        f.write(np.float64(t).tobytes())
        f.write(np.array([IM_G, JM_G, KM_G], dtype=np.uint32).tobytes())
        f.write(np.ascontiguousarray(Q, dtype=np.float64).tobytes())
