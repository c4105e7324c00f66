"""A fixed number of RK3 steps of one solve, for kernel profilers (ncu).

  python -m cbns3d_cart_mpi_gb300.profile_step [--N 256] [--precision fp64|fp32_mixed|fp64_ff] [--steps 2]

Builds the Taylor-Green state on the device (cbns_init_tgv), then takes
`steps` steps through cbns_step, whose kernels are launched one by one: per
step the time-step reduction, then per stage the x, y and z face kernels, the
viscous-term kernel and the update.  Prints nothing but the final time, so a
profiler's launch list and captures are the whole output.  Holds one solve
(6.4-6.8 GB at 256^3).
"""
import argparse

from ._abi import tgv_params
from .solver import Solver


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--N", type=int, default=256)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32_mixed", "fp64_ff"])
    ap.add_argument("--steps", type=int, default=2)
    args = ap.parse_args()
    s = Solver(tgv_params(args.N, t_end=2.0), precision=args.precision)
    s.init_tgv()
    t = 0.0
    for _ in range(args.steps):
        t = s.step()[1]
    s.close()
    print("profile_step: %d^3 %s, %d steps, t = %.6f" % (args.N, args.precision, args.steps, t))


if __name__ == "__main__":
    main()
