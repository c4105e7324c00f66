"""ctypes bindings of the two native libraries (include/cbns_gpu.h, include/cbns_host.h).

The GPU library is the only compute path: if it is not built, loading fails
with an error that says so; nothing falls back to a CPU implementation.
"""
import ctypes
import os

from ._abi import CbnsParams

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(PKG, "lib")
GPU_LIB = os.path.join(LIB_DIR, "libcbns_gpu.so")
HOST_LIB = os.path.join(LIB_DIR, "libcbns_host.so")
PROBE_LIB = os.path.join(LIB_DIR, "libcbns_probe.so")

_gpu = None
_probe = None


class ServerOpts(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("memory_budget_bytes", ctypes.c_uint64),
                ("max_active", ctypes.c_uint32), ("steps_per_round", ctypes.c_uint32),
                ("tile_rows", ctypes.c_int), ("ctas_per_sm", ctypes.c_int)]


class RequestInfo(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("steps", ctypes.c_uint32), ("t_final", ctypes.c_double),
                ("ke", ctypes.c_double), ("enstrophy", ctypes.c_double), ("submit_s", ctypes.c_double),
                ("admit_s", ctypes.c_double), ("done_s", ctypes.c_double), ("device_bytes", ctypes.c_uint64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("rounds", ctypes.c_uint64), ("batch_builds", ctypes.c_uint64), ("cell_steps", ctypes.c_uint64),
                ("peak_active", ctypes.c_uint32), ("queued", ctypes.c_uint32),
                ("budget_bytes", ctypes.c_uint64), ("used_bytes", ctypes.c_uint64), ("clock_s", ctypes.c_double)]


class LaunchConfig(ctypes.Structure):
    _fields_ = [("tile_rows", ctypes.c_int), ("ctas_per_sm", ctypes.c_int)]


class KernelTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 32), ("launches", ctypes.c_uint32), ("total_ms", ctypes.c_double)]
_host = None

c_int, c_u32, c_u64, c_d, c_vp = ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_double, ctypes.c_void_p
c_dp = ctypes.POINTER(ctypes.c_double)
P_params = ctypes.POINTER(CbnsParams)

# name -> (restype, argtypes); every entry point include/cbns_gpu.h declares.
GPU_API = {
    "cbns_params_derive": (c_int, [P_params]),
    "cbns_create": (c_int, [P_params, c_u32, c_u32, c_u32, c_int, ctypes.POINTER(c_vp)]),
    "cbns_destroy": (c_int, [c_vp]),
    "cbns_upload_Q": (c_int, [c_vp, c_vp, c_d]),
    "cbns_download_Q": (c_int, [c_vp, c_vp]),
    "cbns_download_Q_p": (c_int, [c_vp, c_vp]),
    "cbns_download_prims": (c_int, [c_vp] + [c_vp] * 6),
    "cbns_load_checkpoint": (c_int, [c_vp, ctypes.c_char_p, c_dp]),
    "cbns_save_checkpoint": (c_int, [c_vp, ctypes.c_char_p]),
    "cbns_calc_dt": (c_int, [c_vp, c_dp]),
    "cbns_stage": (c_int, [c_vp, c_d, c_int]),
    "cbns_step": (c_int, [c_vp, c_d, c_dp, c_dp]),
    "cbns_run": (c_int, [c_vp, c_u32, c_d, ctypes.POINTER(c_u32)]),
    "cbns_upload_Q_async": (c_int, [c_vp, c_vp, c_d]),
    "cbns_step_async": (c_int, [c_vp, c_d]),
    "cbns_download_Q_async": (c_int, [c_vp, c_vp]),
    "cbns_wait": (c_int, [c_vp, c_dp, c_dp]),
    "cbns_poll": (c_int, [c_vp, ctypes.POINTER(c_int)]),
    "cbns_get_time": (c_int, [c_vp, c_dp, c_dp]),
    "cbns_diagnostics": (c_int, [c_vp, c_dp, c_dp]),
    "cbns_check_state": (c_int, [c_vp]),
    "cbns_stream": (c_vp, [c_vp]),
    "cbns_get_info": (c_int, [c_vp, ctypes.POINTER(c_u32), ctypes.POINTER(c_u64), ctypes.POINTER(c_int)]),
    "cbns_init_tgv": (c_int, [c_vp, c_u64, c_d, c_int, c_int, c_d]),
    "cbns_footprint": (c_int, [c_u32, c_u32, c_u32, c_int, ctypes.POINTER(c_u64)]),
    "cbns_server_create": (c_int, [c_vp, ctypes.POINTER(c_vp)]),
    "cbns_server_destroy": (c_int, [c_vp]),
    "cbns_server_submit": (c_int, [c_vp, P_params, c_u32, c_u32, c_u32, c_vp, c_int, ctypes.POINTER(c_u64)]),
    "cbns_server_submit_tgv": (c_int, [c_vp, P_params, c_u32, c_u32, c_u32, c_u64, c_d, c_int, c_int, c_int,
                                       ctypes.POINTER(c_u64)]),
    "cbns_server_submit_checkpoint": (c_int, [c_vp, P_params, c_u32, c_u32, c_u32, ctypes.c_char_p, c_int,
                                              ctypes.POINTER(c_u64)]),
    "cbns_server_cancel": (c_int, [c_vp, c_u64]),
    "cbns_server_wait": (c_int, [c_vp, c_u64, c_d, c_vp]),
    "cbns_server_result": (c_int, [c_vp, c_u64, c_vp]),
    "cbns_server_release": (c_int, [c_vp, c_u64]),
    "cbns_server_get_stats": (c_int, [c_vp, c_vp]),
    "cbns_batch_create": (c_int, [ctypes.POINTER(c_vp), c_int, ctypes.POINTER(c_vp)]),
    "cbns_batch_destroy": (c_int, [c_vp]),
    "cbns_batch_run": (c_int, [c_vp, c_u32, ctypes.POINTER(c_u32)]),
    "cbns_batch_set_config": (c_int, [c_vp, c_vp]),
    "cbns_batch_get_config": (c_int, [c_vp, c_vp]),
    "cbns_batch_autotune": (c_int, [c_vp, c_int, c_dp, c_int, ctypes.POINTER(c_int)]),
    "cbns_batch_stream": (c_vp, [c_vp]),
    "cbns_profile_begin": (c_int, [c_vp]),
    "cbns_profile_end": (c_int, [c_vp, c_vp, c_int, ctypes.POINTER(c_int)]),
    "cbns_diagnostics_noalloc": (c_int, [c_vp, c_u32, c_u32, c_u32, c_d, c_d, c_d, c_vp, c_vp]),
    "cbns_last_error": (ctypes.c_char_p, []),
    "cbns_version": (ctypes.c_char_p, []),
}

HOST_API = {
    "cbns_host_read_input": (c_int, [ctypes.c_char_p, P_params]),
    "cbns_host_gen_mesh": (c_int, [P_params, c_u32, c_u32, c_u32, c_u32, c_u32, c_u32, c_vp, c_vp, c_vp]),
    "cbns_host_initial_condition": (c_int, [P_params, c_u32, c_u32, c_u32, c_u32, c_u32, c_u32, c_vp]),
    "cbns_host_initial_condition_perturbed": (c_int, [P_params, c_u32, c_u32, c_u32, c_u64, c_d, c_int, c_int,
                                                      c_vp]),
    "cbns_host_output_bin": (c_int, [ctypes.c_char_p, c_d, c_u32, c_u32, c_u32, c_vp]),
    "cbns_host_read_bin": (c_int, [ctypes.c_char_p, c_u32, c_u32, c_u32, c_vp, c_dp]),
    "cbns_host_output_vtk_xml": (c_int, [ctypes.c_char_p, ctypes.c_char_p, c_int, c_u32, c_u32, c_u32, c_u32]
                                 + [c_vp] * 8),
}


def _bind(lib, table):
    for name, (res, args) in table.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def gpu():
    """The GPU library; raises if it has not been built (no fallback exists).
    CBNS_GPU_LIB may name another build of it (the bounds-checked test build)."""
    global _gpu
    if _gpu is None:
        path = os.environ.get("CBNS_GPU_LIB") or GPU_LIB
        if not os.path.exists(path):
            raise RuntimeError("%s is not built; run cbns3d_cart_mpi_gb300.build.build() "
                               "or __graft_entry__.build()" % path)
        _gpu = _bind(ctypes.CDLL(path), GPU_API)
    return _gpu


def host():
    global _host
    if _host is None:
        if not os.path.exists(HOST_LIB):
            raise RuntimeError("libcbns_host.so is not built (%s); run cbns3d_cart_mpi_gb300.build.build()"
                               % HOST_LIB)
        _host = _bind(ctypes.CDLL(HOST_LIB), HOST_API)
    return _host


def probe():
    """The FMA-throughput probe library that bench.py uses for roofline peaks."""
    global _probe
    if _probe is None:
        if not os.path.exists(PROBE_LIB):
            raise RuntimeError("libcbns_probe.so is not built (%s); run cbns3d_cart_mpi_gb300.build.build()"
                               % PROBE_LIB)
        _probe = ctypes.CDLL(PROBE_LIB)
        _probe.cbns_probe_peak.restype = c_int
        _probe.cbns_probe_peak.argtypes = [c_int, c_dp]
        _probe.cbns_probe_rcp64.restype = c_int
        _probe.cbns_probe_rcp64.argtypes = [c_vp, c_vp, c_vp, ctypes.c_longlong]
        _probe.cbns_probe_ff.restype = c_int
        _probe.cbns_probe_ff.argtypes = [c_vp, c_vp, c_vp, ctypes.c_longlong]
    return _probe


def last_error():
    return gpu().cbns_last_error().decode(errors="replace")
