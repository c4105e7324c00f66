"""Per-core speed of the oracle's C restatement against the reference itself
(test infrastructure: the CPU baseline's fairness check).

Both run the Taylor-Green vortex at 64^3 (Re 1600, Ma 0.1, CFL 0.5) for
`steps` RK3 steps on one host thread:
  * the reference: oracle/_ref/ref_harness, the reference's own solver sources
    compiled unmodified by oracle/build.py (needs them on this machine), timed
    as a whole process minus a zero-step run of the same binary (start-up);
  * the port: oracle/cbns_oracle.c through oracle.oracle.OracleBlock with
    OMP_NUM_THREADS=1, timed around its step loop.

  python oracle/time_vs_reference.py [N] [steps]
"""
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)


def main(N=64, steps=10):
    from cbns3d_cart_mpi_gb300._abi import tgv_params
    from cbns3d_cart_mpi_gb300.params import write_input_txt
    from oracle.build import build_port, build_ref
    if build_ref() is None:
        sys.exit("the reference's sources are not on this machine")
    build_port()
    harness = os.path.join(HERE, "_ref", "ref_harness")
    wd = tempfile.mkdtemp(prefix="cbns_timing_")
    write_input_txt(tgv_params(N, t_end=20.0), os.path.join(wd, "input.txt"))
    env = dict(os.environ, OMP_NUM_THREADS="1")

    def run_ref(n):
        t0 = time.perf_counter()
        subprocess.run([harness, wd, str(n), str(n + 1)], env=env, check=True, capture_output=True)
        return time.perf_counter() - t0

    ref = min(run_ref(steps) for _ in range(2)) - min(run_ref(0) for _ in range(2))
    code = ("import sys, time; sys.path.insert(0, %r)\n"
            "from cbns3d_cart_mpi_gb300._abi import tgv_params\n"
            "from oracle.oracle import OracleBlock\n"
            "b = OracleBlock(tgv_params(%d, t_end=20.0)); b.initial_condition()\n"
            "t0 = time.perf_counter()\n"
            "for _ in range(%d): b.step()\n"
            "print(time.perf_counter() - t0)\n") % (ROOT, N, steps)
    port = min(float(subprocess.run([sys.executable, "-c", code], env=env, check=True, capture_output=True,
                                    text=True).stdout) for _ in range(2))
    cells = N ** 3 * steps
    print("%d^3, %d steps, one thread: reference %.3f s/step (%.3g cell-RK3-steps/s), port %.3f s/step "
          "(%.3g cell-RK3-steps/s); port/reference speed %.3f" % (
              N, steps, ref / steps, cells / ref, port / steps, cells / port, ref / port))


if __name__ == "__main__":
    main(*[int(a) for a in sys.argv[1:3]])
