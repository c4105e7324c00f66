"""Build the native parts in-tree, with nvcc and g++ only (no CMake).

  lib/libcbns_gpu.so   CUDA kernels + C ABI of include/cbns_gpu.h (sm_103a only)
  lib/libcbns_probe.so FMA-throughput probe, the roofline denominator bench.py
                       measures (not part of the product library)
  lib/libcbns_host.so  host C++ of include/cbns_host.h (input.txt, IC, checkpoint, VTK)
  lib/cbns3d_gb300     the Block3d-style driver executable

Translation units compile in parallel and are skipped when up to date, so a
rebuild on the GPU machine takes about a minute from scratch.
"""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "lib")
INCLUDE = os.path.join(ROOT, "include")

GPU_SOURCES = ["cbns_kernels.cu", "cbns_ff_kernels.cu", "cbns_api.cu", "cbns_noalloc.cu", "cbns_serve.cu",
               "cbns_ckpt.cu"]
PROBE_SOURCE = "cbns_probe.cu"
HOST_SOURCES = ["host/cbns_host.cpp"]
DRIVER_SOURCE = "host/cbns3d_gb300.cpp"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without contracting a*b+c into fused multiply-adds
# (-ffp-contract=off): g++ contracts by default on aarch64 but cannot on x86-64's
# base ISA, so without it the initial condition and the per-solve constants
# would differ in the last bit between the two hosts and from the reference.
# Device code keeps nvcc's contraction.
HOST_FP = ["-ffp-contract=off"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", HOST_FP[0],
              "--expt-relaxed-constexpr"]

GPU_LIB = os.path.join(LIB, "libcbns_gpu.so")
# The same library with every kernel index checked against its array
# (-DCBNS_BOUNDS_CHECK): a test build, loaded through CBNS_GPU_LIB.
CHECKED_GPU_LIB = os.path.join(LIB, "libcbns_gpu_checked.so")
PROBE_LIB = os.path.join(LIB, "libcbns_probe.so")
HOST_LIB = os.path.join(LIB, "libcbns_host.so")
DRIVER = os.path.join(LIB, "cbns3d_gb300")


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.isdir(c):
            return c
    nvcc = shutil.which("nvcc")
    return os.path.dirname(os.path.dirname(nvcc)) if nvcc else "/usr/local/cuda"


def _nvcc():
    return shutil.which("nvcc") or os.path.join(_cuda_home(), "bin", "nvcc")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n  %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def _headers():
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _atomic(cmd_fn, target):
    tmp = target + ".tmp%d" % os.getpid()
    _run(cmd_fn(tmp))
    os.replace(tmp, target)


def build(verbose=False, extra_nvcc=()):
    """Compile everything that is out of date; returns the paths built."""
    os.makedirs(LIB, exist_ok=True)
    objdir = os.path.join(LIB, "obj")
    os.makedirs(objdir, exist_ok=True)
    hdrs = _headers()
    nvcc = _nvcc()
    extra = list(extra_nvcc)

    def cu_obj(src):
        path = os.path.join(CSRC, src)
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        if _stale(obj, [path] + hdrs + [__file__]):
            _atomic(lambda out: [nvcc] + ARCH + NVCC_FLAGS + extra + ["-c", path, "-o", out], obj)
        return obj

    def cpp_obj(src):
        path = os.path.join(CSRC, src)
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        if _stale(obj, [path] + hdrs + [__file__]):
            _atomic(lambda out: ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-pthread"] + HOST_FP +
                    ["-c", path, "-o", out], obj)
        return obj

    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        gpu_f = [ex.submit(cu_obj, s) for s in GPU_SOURCES]
        probe_f = ex.submit(cu_obj, PROBE_SOURCE)
        host_f = [ex.submit(cpp_obj, s) for s in HOST_SOURCES]
        drv_f = ex.submit(cpp_obj, DRIVER_SOURCE)
        gpu_objs = [f.result() for f in gpu_f]
        host_objs = [f.result() for f in host_f]
        drv_obj = drv_f.result()
        probe_obj = probe_f.result()

    cudalib = os.path.join(_cuda_home(), "lib64")
    if _stale(GPU_LIB, gpu_objs):
        _atomic(lambda out: [nvcc] + ARCH + ["-shared", "-o", out] + gpu_objs + ["-lcudart"], GPU_LIB)
    if _stale(PROBE_LIB, [probe_obj]):
        _atomic(lambda out: [nvcc] + ARCH + ["-shared", "-o", out, probe_obj, "-lcudart"], PROBE_LIB)
    if _stale(HOST_LIB, host_objs):
        _atomic(lambda out: ["g++", "-shared", "-o", out] + host_objs, HOST_LIB)
    if _stale(DRIVER, [drv_obj, GPU_LIB, HOST_LIB]):
        _atomic(lambda out: ["g++", "-o", out, drv_obj, "-L" + LIB, "-lcbns_gpu", "-lcbns_host",
                             "-L" + cudalib, "-lcudart", "-pthread", "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + cudalib],
                DRIVER)
    if verbose:
        for p in (GPU_LIB, PROBE_LIB, HOST_LIB, DRIVER):
            print(p)
    return GPU_LIB, HOST_LIB, DRIVER


def build_checked():
    """The bounds-checked GPU library (every global index of the kernels checked
    against its array; misses reported as CBNS_ERR_BOUNDS, never a trap)."""
    os.makedirs(LIB, exist_ok=True)
    objdir = os.path.join(LIB, "obj_checked")
    os.makedirs(objdir, exist_ok=True)
    hdrs = _headers()
    nvcc = _nvcc()
    flags = ARCH + NVCC_FLAGS + ["-DCBNS_BOUNDS_CHECK"]

    def cu_obj(src):
        path = os.path.join(CSRC, src)
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        if _stale(obj, [path] + hdrs + [__file__]):
            _atomic(lambda out: [nvcc] + flags + ["-c", path, "-o", out], obj)
        return obj

    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        objs = [f.result() for f in [ex.submit(cu_obj, s) for s in GPU_SOURCES]]
    if _stale(CHECKED_GPU_LIB, objs):
        _atomic(lambda out: [nvcc] + ARCH + ["-shared", "-o", out] + objs + ["-lcudart"], CHECKED_GPU_LIB)
    return CHECKED_GPU_LIB


if __name__ == "__main__":
    build(verbose=True)
