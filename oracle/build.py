"""Build recipes for the oracle (test infrastructure only).

``build_port()`` compiles the CPU restatement ``oracle/cbns_oracle.c`` into
``oracle/liboracle.so`` (-O3, OpenMP, no fused multiply-add), on any host.

``build_ref()`` compiles the reference solver's own sources into ``oracle/_ref/``
when they are present on this machine.  The reference (chenbei102/cbns3d_cart_mpi) is C++17
built by CMake against MPI (CMakeLists.txt:1-38).  This recipe does not run that
build: it compiles the reference's solver sources where they lie, unmodified,
with g++ and the reference's Release flags (-O3, C++17; CMakeLists.txt:11,14),
against the project-written single-rank MPI shim in ``oracle/mpi_shim/``, and
links them with ``oracle/ref_harness.cpp`` (a replacement for src/cbns3d.cpp's
``main`` that dumps states) and, separately, with the op-counting harness.

``-ffp-contract=off`` keeps the binary free of fused multiply-adds on every
host; on x86-64 at the default ISA level g++ emits none anyway, so the result
is the reference's own arithmetic.

Outputs (git-ignored): ``oracle/_ref/ref_harness`` and ``oracle/_ref/opcount``.
Usage: ``python oracle/build.py [reference_dir]``.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
DEFAULT_REF = "/root/reference"

# The solver's translation units; src/cbns3d.cpp (main + MPI topology) is replaced
# by the harness.
REF_SOURCES = [
    "Block3d.cpp", "boundary_condition.cpp", "calc_gradient.cpp",
    "eigenvectors_roe.cpp", "lf_flux.cpp", "output_vtk_xml.cpp",
    "read_input.cpp", "weno.cpp",
]
# The op-counting build swaps value_type for a counting type, so the I/O-only
# translation units (and read_input's std::max on mixed types) stay out of it.
OPCOUNT_SOURCES = [
    "Block3d.cpp", "boundary_condition.cpp", "calc_gradient.cpp",
    "eigenvectors_roe.cpp", "lf_flux.cpp", "weno.cpp",
]
CXXFLAGS = ["-O3", "-std=c++17", "-ffp-contract=off", "-w"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_ref(ref_dir=None, quiet=True):
    """Build ``ref_harness`` and ``opcount``; returns their paths, or None if the
    reference sources are not present on this machine."""
    ref_dir = ref_dir or os.environ.get("CBNS_REFERENCE_DIR", DEFAULT_REF)
    src = os.path.join(ref_dir, "src")
    inc = os.path.join(ref_dir, "include")
    if not os.path.isdir(src):
        return None
    os.makedirs(OUT, exist_ok=True)
    shim = os.path.join(HERE, "mpi_shim")
    incs = ["-I" + shim, "-I" + inc]

    def compile_obj(path, tag, extra):
        obj = os.path.join(OUT, tag + "_" + os.path.basename(path) + ".o")
        deps = [path, os.path.join(shim, "mpi.h"), os.path.join(HERE, "opcount", "count_types.h")]
        deps = [d for d in deps if os.path.exists(d)]
        if _newer(obj, deps):
            _run(["g++"] + CXXFLAGS + extra + incs + ["-c", path, "-o", obj])
        return obj

    count_hdr = os.path.join(HERE, "opcount", "count_types.h")
    jobs = []
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        ref_objs = [ex.submit(compile_obj, os.path.join(src, s), "ref", []) for s in REF_SOURCES]
        ref_objs.append(ex.submit(compile_obj, os.path.join(HERE, "ref_harness.cpp"), "ref", []))
        ref_objs.append(ex.submit(compile_obj, os.path.join(shim, "mpi_shim.cpp"), "ref", []))
        cnt_objs = [ex.submit(compile_obj, os.path.join(src, s), "cnt", ["-include", count_hdr])
                    for s in OPCOUNT_SOURCES]
        cnt_objs.append(ex.submit(compile_obj, os.path.join(HERE, "opcount", "opcount_harness.cpp"),
                                  "cnt", ["-include", count_hdr]))
        cnt_objs.append(ex.submit(compile_obj, os.path.join(shim, "mpi_shim.cpp"), "cnt", []))
        ref_objs = [f.result() for f in ref_objs]
        cnt_objs = [f.result() for f in cnt_objs]
    harness = os.path.join(OUT, "ref_harness")
    if _newer(harness, ref_objs):
        _run(["g++", "-O3", "-o", harness] + ref_objs)
    opcount = os.path.join(OUT, "opcount")
    if _newer(opcount, cnt_objs):
        _run(["g++", "-O3", "-o", opcount] + cnt_objs)
    if not quiet:
        print(harness)
        print(opcount)
    return harness, opcount


PORT_SRC = os.path.join(HERE, "cbns_oracle.c")
PORT_LIB = os.path.join(HERE, "liboracle.so")


def build_port(quiet=True):
    """Compile the CPU restatement into ``oracle/liboracle.so``; returns its path."""
    hdr = os.path.join(os.path.dirname(HERE), "include", "cbns_gpu.h")
    if _newer(PORT_LIB, [PORT_SRC, hdr]):
        tmp = PORT_LIB + ".tmp%d" % os.getpid()
        _run(["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
              "-fno-fast-math", PORT_SRC, "-o", tmp, "-lm"])
        os.replace(tmp, PORT_LIB)
    if not quiet:
        print(PORT_LIB)
    return PORT_LIB


if __name__ == "__main__":
    build_port(quiet=False)
    res = build_ref(sys.argv[1] if len(sys.argv) > 1 else None, quiet=False)
    if res is None:
        print("reference sources not found; oracle/_ref not built")
