"""ctypes mirror of the C ABI types declared in ``include/cbns_gpu.h``.

``CbnsParams`` is ``cbns_params``: the fields of the reference's
``SimulationParams`` (include/simulation_params.h:15-53) in the order
``read_input`` reads them (src/read_input.cpp:24-72), then the derived
constants of src/read_input.cpp:78-90.
"""
import ctypes

NEQ = 5
NG = 4
NGV = 2

CBNS_OK = 0
CBNS_FINISHED = 1
CBNS_ERR_INVALID_ARG = -1
CBNS_ERR_BAD_DIMS = -2
CBNS_ERR_CUDA = -3
CBNS_ERR_OUT_OF_MEMORY = -4
CBNS_ERR_NONPHYSICAL = -5
CBNS_ERR_TIMEOUT = -6
CBNS_ERR_NO_DEVICE = -7
CBNS_ERR_IO = -8
CBNS_ERR_FORMAT = -9
CBNS_ERR_CANCELLED = -10
CBNS_ERR_BOUNDS = -11

STATUS_NAMES = {
    0: "CBNS_OK", 1: "CBNS_FINISHED", -1: "CBNS_ERR_INVALID_ARG", -2: "CBNS_ERR_BAD_DIMS",
    -3: "CBNS_ERR_CUDA", -4: "CBNS_ERR_OUT_OF_MEMORY", -5: "CBNS_ERR_NONPHYSICAL",
    -6: "CBNS_ERR_TIMEOUT", -7: "CBNS_ERR_NO_DEVICE", -8: "CBNS_ERR_IO", -9: "CBNS_ERR_FORMAT", -10: "CBNS_ERR_CANCELLED",
    -11: "CBNS_ERR_BOUNDS",
}

CBNS_FP64 = 0
CBNS_FP32_MIXED = 1
CBNS_FP64_FF = 2


class CbnsParams(ctypes.Structure):
    _fields_ = [
        ("checkpoint_fname", ctypes.c_char * 256),
        ("CFL", ctypes.c_double),
        ("t_cur", ctypes.c_double),
        ("t_end", ctypes.c_double),
        ("Pr", ctypes.c_double),
        ("gamma", ctypes.c_double),
        ("Mach", ctypes.c_double),
        ("Re", ctypes.c_double),
        ("T_inf", ctypes.c_double),
        ("L", ctypes.c_double),
        ("IM", ctypes.c_uint32),
        ("JM", ctypes.c_uint32),
        ("KM", ctypes.c_uint32),
        ("nstep_max", ctypes.c_uint32),
        ("checkpoint_freq", ctypes.c_uint32),
        ("num_output", ctypes.c_uint32),
        ("is_restart", ctypes.c_int32),
        ("Mach2", ctypes.c_double),
        ("Re_inv", ctypes.c_double),
        ("Pr_inv", ctypes.c_double),
        ("gam1", ctypes.c_double),
        ("gM2", ctypes.c_double),
        ("gam1_inv", ctypes.c_double),
        ("p_inf", ctypes.c_double),
        ("C_T_inf", ctypes.c_double),
        ("C_dt_v", ctypes.c_double),
    ]

    def derive(self):
        """Derived constants, src/read_input.cpp:78-90 (same binary64 operations)."""
        self.Mach2 = self.Mach * self.Mach
        self.Re_inv = 1.0 / self.Re
        self.Pr_inv = 1.0 / self.Pr
        self.gam1 = self.gamma - 1.0
        self.gM2 = self.gamma * self.Mach2
        self.gam1_inv = 1.0 / self.gam1
        self.p_inf = 1.0 / self.gM2
        self.C_T_inf = 110.5 / self.T_inf
        a, g = 4.0 / 3.0, self.gamma * self.Pr_inv
        self.C_dt_v = (g if a < g else a) * self.Re_inv
        return self

    def as_dict(self):
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = v.decode() if isinstance(v, bytes) else v
        return out


def tgv_params(N, Re=1600.0, Mach=0.1, CFL=0.5, t_end=20.0, nstep_max=1000000,
               gamma=1.4, Pr=0.71, T_inf=255.556, JM=None, KM=None):
    """Parameters of the Taylor-Green case file python/taylor_green.ini:1-27 with the
    grid, Reynolds and Mach numbers, CFL and end time overridable."""
    p = CbnsParams()
    p.checkpoint_fname = b"checkpoint"
    p.CFL = CFL
    p.t_cur = 0.0
    p.t_end = t_end
    p.Pr = Pr
    p.gamma = gamma
    p.Mach = Mach
    p.Re = Re
    p.T_inf = T_inf
    p.L = 1.0
    p.IM = N
    p.JM = N if JM is None else JM
    p.KM = N if KM is None else KM
    p.nstep_max = nstep_max
    p.checkpoint_freq = 5000
    p.num_output = 10
    p.is_restart = 1
    return p.derive()


def padded_shape(IM, JM, KM):
    """numpy shape (KM_G, JM_G, IM_G, NEQ) of the reference's Q array."""
    return (KM + 2 * NG, JM + 2 * NG, IM + 2 * NG, NEQ)
