/*
 * Op-counting harness (test infrastructure): runs the reference's hot-path
 * functions once each on a TGV block of the given size, with value_type swapped
 * for CountedDouble (count_types.h), and prints the FLOPs each executed divided by
 * the units it iterates over:
 *   rec_riemann_x/y/z           per face   ((N+1)*N*N faces per direction)
 *   calc_viscous_terms           per ring point  ((N+2*NGV)^3), incl. 4 calc_gradient
 *   calc_viscous_flux            per ring point
 *   divergence part of calc_viscous_flux_contribution   per interior cell
 *   update_rk3                   per interior cell
 *   calc_primitive               per padded cell ((N+2*NG)^3)
 *   calc_dt                      per interior cell
 * and the per-cell-RK3-step total for each N given on the command line.
 *   opcount <N> [N2 ...]
 * FLOP = each +, -, *, / and sqrt executed on a value_type (comparisons, abs and
 * negation are listed apart).  The loops have no data-dependent arithmetic, so the
 * per-unit figures are exact integers independent of N.
 */
#include <mpi.h>

#include <cstdio>
#include <cstdlib>
#include <string>

#include "Block3d.h"

OpCounts g_ops;
void boundary_condition(Block3d* blk, value_type* Q);

static void reset() { g_ops = OpCounts{0, 0, 0, 0, 0, 0}; }
static unsigned long long flops() {
  return g_ops.add + g_ops.mul + g_ops.div + g_ops.sqrt;
}

int main(int argc, char** argv) {
  const unsigned N = 16;  // the per-unit figures do not depend on N
  SimulationParams sp;
  sp.checkpoint_fname = "unused";
  sp.CFL = 0.5; sp.t_cur = 0.0; sp.t_end = 20.0;
  sp.Pr = 0.71; sp.gamma = 1.4; sp.Mach = 0.1; sp.Re = 1600.0;
  double T_inf = 255.556;
  sp.L = 1.0; sp.IM = sp.JM = sp.KM = N;
  sp.nstep_max = 1; sp.checkpoint_freq = 1000; sp.num_output = 1; sp.is_restart = true;
  sp.Mach2 = sp.Mach * sp.Mach;
  sp.Re_inv = 1.0 / sp.Re;
  sp.Pr_inv = 1.0 / sp.Pr;
  sp.gam1 = sp.gamma - 1.0;
  sp.gM2 = sp.gamma * sp.Mach2;
  sp.gam1_inv = 1.0 / sp.gam1;
  sp.p_inf = 1.0 / sp.gM2;
  sp.C_T_inf = 110.5 / T_inf;
  sp.C_dt_v = ((4.0 / 3.0 > (sp.gamma * sp.Pr_inv).v) ? CountedDouble(4.0 / 3.0)
                                                      : sp.gamma * sp.Pr_inv) * sp.Re_inv;

  ProcessInfo pi;
  pi.comm = MPI_COMM_WORLD; pi.rank = 0;
  pi.coords[0] = pi.coords[1] = pi.coords[2] = 0;
  pi.left = pi.right = pi.down = pi.up = pi.back = pi.front = 0;
  Block3d b(&pi, &sp, N, N, N);
  b.gen_mesh(0, 0, 0);
  b.initial_condition();
  b.calc_conservative(b.get_Q());
  boundary_condition(&b, b.get_Q());
  b.calc_primitive(b.get_Q());
  b.init_Q_p();

  const double faces = (double)(N + 1) * N * N;
  const double ring = (double)(N + 4) * (N + 4) * (N + 4);
  const double cells = (double)N * N * N;
  const double padded = (double)(N + 8) * (N + 8) * (N + 8);

  reset(); b.calc_dt();                     double f_dt = flops() / cells;
  reset(); b.rec_riemann_x(b.get_Q());      double f_rx = flops() / faces;
  OpCounts rx = g_ops;
  reset(); b.rec_riemann_y(b.get_Q());      double f_ry = flops() / faces;
  reset(); b.rec_riemann_z(b.get_Q());      double f_rz = flops() / faces;
  reset(); b.calc_viscous_terms();          double f_vt = flops() / ring;
  reset(); b.calc_viscous_flux();           double f_vf = flops() / ring;
  reset(); b.calc_viscous_flux_contribution();
  double f_vc_total = (double)flops();
  double f_vd = (f_vc_total - f_vt * ring - f_vf * ring) / cells;
  reset(); b.update_rk3(1e-4, 1);           double f_up = flops() / cells;
  reset(); boundary_condition(&b, b.get_Q_p()); double f_bc = flops();
  reset(); b.calc_primitive(b.get_Q_p());   double f_pr = flops() / padded;

  std::printf("# FLOPs per unit, counted on the reference's own source (N=%u)\n", N);
  std::printf("rec_riemann_x_per_face %.6f\n", f_rx);
  std::printf("rec_riemann_y_per_face %.6f\n", f_ry);
  std::printf("rec_riemann_z_per_face %.6f\n", f_rz);
  std::printf("riemann_x_breakdown add %llu mul %llu div %llu sqrt %llu cmp %llu other %llu\n",
              rx.add, rx.mul, rx.div, rx.sqrt, rx.cmp, rx.other);
  std::printf("calc_viscous_terms_per_ring_point %.6f\n", f_vt);
  std::printf("calc_viscous_flux_per_ring_point %.6f\n", f_vf);
  std::printf("viscous_divergence_per_cell %.6f\n", f_vd);
  std::printf("update_rk3_per_cell %.6f\n", f_up);
  std::printf("boundary_condition_total %.0f\n", f_bc);
  std::printf("calc_primitive_per_padded_cell %.6f\n", f_pr);
  std::printf("calc_dt_per_cell %.6f\n", f_dt);
  for (int a = 1; a < argc; ++a) {
    double n = std::atof(argv[a]);
    double fc = (n + 1) * n * n, rc = (n + 4) * (n + 4) * (n + 4), cc = n * n * n,
           pc = (n + 8) * (n + 8) * (n + 8);
    double stage = fc * (f_rx + f_ry + f_rz) + rc * (f_vt + f_vf) + cc * (f_vd + f_up) + pc * f_pr;
    double step = 3 * stage + cc * f_dt;
    std::printf("N %.0f flops_per_cell_rk3_step %.3f flops_per_step %.6e\n", n, step / cc, step);
  }
  return 0;
}
