/*
 * Oracle harness (test infrastructure, never product code).
 *
 * Drives the reference solver's own Block3d, compiled unmodified from its
 * sources, through the time loop of src/cbns3d.cpp:136-241 on one rank, and dumps
 * states in the reference's checkpoint format (Block3d::output_bin,
 * src/Block3d.cpp:964-987) so tests can compare the GPU path with it.
 *
 *   ref_harness <workdir> <nsteps> <dump_every> [--inject FILE] [--stage1] [--vtk] [--ckpt]
 *
 * <workdir> holds input.txt (read by the reference's read_input(),
 * src/read_input.cpp:15-103).  Outputs, all in <workdir>:
 *   q_NNNNNN.bin  state Q (ghosts included) after step NNNNNN, every <dump_every>
 *                 steps and after the last one (step 0 = after the start-up ghost fill)
 *   steps.txt     one line per step: n_t dt t_cur, printed with %.17e
 *   qp_stage1.bin (--stage1) Q_p after stage 1 of the first step; the run stops there
 *   vtk_init/, vtk_final/  (--vtk) the reference's VTK XML output at start and end
 *   checkpoint_ref.dat  (--ckpt) Block3d::output_bin's own file after the last step
 * --inject FILE follows the reference's restart branch (read_bin) but calls
 * initial_condition() first, so mu holds the value the fresh-start branch gives it
 * (read_bin alone leaves mu unset for the first calc_dt, src/Block3d.cpp:535).
 */
#include <mpi.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <unistd.h>

#include "Block3d.h"
#include "output_vtk_xml.h"
#include "process_info.h"
#include "read_input.h"

void boundary_condition(Block3d* blk, value_type* Q);

static void dump_state(const char* fname, double t, const SimulationParams& sp,
                       const value_type* arr) {
  const unsigned ng = constant::NG;
  unsigned dims[3] = {sp.IM + 2 * ng, sp.JM + 2 * ng, sp.KM + 2 * ng};
  FILE* fh = std::fopen(fname, "wb");
  if (!fh) {
    std::fprintf(stderr, "cannot write %s\n", fname);
    std::exit(3);
  }
  std::fwrite(&t, sizeof(double), 1, fh);
  std::fwrite(dims, sizeof(unsigned), 3, fh);
  size_t n = (size_t)constant::NEQ * dims[0] * dims[1] * dims[2];
  std::fwrite(arr, sizeof(value_type), n, fh);
  std::fclose(fh);
}

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: ref_harness <workdir> <nsteps> <dump_every> "
                         "[--inject FILE] [--stage1] [--vtk]\n");
    return 1;
  }
  MPI_Init(&argc, &argv);
  if (chdir(argv[1]) != 0) {
    std::perror("chdir");
    return 1;
  }
  const long nsteps = std::atol(argv[2]);
  const long dump_every = std::atol(argv[3]);
  std::string inject;
  bool stage1 = false, vtk = false, ckpt = false;
  for (int a = 4; a < argc; ++a) {
    if (!std::strcmp(argv[a], "--inject") && a + 1 < argc) inject = argv[++a];
    else if (!std::strcmp(argv[a], "--stage1")) stage1 = true;
    else if (!std::strcmp(argv[a], "--vtk")) vtk = true;
    else if (!std::strcmp(argv[a], "--ckpt")) ckpt = true;
  }

  SimulationParams sp;
  if (0 != read_input(sp)) return 1;

  ProcessInfo pi;
  pi.comm = MPI_COMM_WORLD;
  pi.rank = 0;
  pi.coords[0] = pi.coords[1] = pi.coords[2] = 0;
  pi.left = pi.right = pi.down = pi.up = pi.back = pi.front = 0;

  Block3d block(&pi, &sp, sp.IM, sp.JM, sp.KM);
  block.gen_mesh(0, 0, 0);

  if (!inject.empty()) {
    block.initial_condition();
    if (0 != block.read_bin(inject)) return 2;
  } else {
    block.initial_condition();
    block.calc_conservative(block.get_Q());
  }
  boundary_condition(&block, block.get_Q());
  block.calc_primitive(block.get_Q());
  block.init_Q_p();

  if (vtk) {
    mkdir("vtk_init", 0755);
    if (0 != output_vtk_xml(&block, 0, 1, "vtk_init", "output")) return 4;
  }
  dump_state("q_000000.bin", sp.t_cur, sp, block.get_Q());

  FILE* steps = std::fopen("steps.txt", "w");
  char name[64];
  for (long n_t = 0; n_t < nsteps; n_t++) {
    if (block.is_finished()) break;
    value_type dt_local = block.calc_dt();
    value_type dt = 0.0;
    MPI_Allreduce(&dt_local, &dt, 1, MPI_DOUBLE, MPI_MIN, MPI_COMM_WORLD);
    if (sp.t_end - sp.t_cur < dt) dt = sp.t_end - sp.t_cur;
    sp.t_cur += dt;
    std::fprintf(steps, "%ld %.17e %.17e\n", n_t, dt, sp.t_cur);

    block.rec_riemann_x(block.get_Q());
    block.rec_riemann_y(block.get_Q());
    block.rec_riemann_z(block.get_Q());
    block.calc_viscous_flux_contribution();
    block.update_rk3(dt, 1);
    boundary_condition(&block, block.get_Q_p());
    block.calc_primitive(block.get_Q_p());
    if (stage1) {
      dump_state("qp_stage1.bin", sp.t_cur, sp, block.get_Q_p());
      break;
    }

    block.rec_riemann_x(block.get_Q_p());
    block.rec_riemann_y(block.get_Q_p());
    block.rec_riemann_z(block.get_Q_p());
    block.calc_viscous_flux_contribution();
    block.update_rk3(dt, 2);
    boundary_condition(&block, block.get_Q_p());
    block.calc_primitive(block.get_Q_p());

    block.rec_riemann_x(block.get_Q_p());
    block.rec_riemann_y(block.get_Q_p());
    block.rec_riemann_z(block.get_Q_p());
    block.calc_viscous_flux_contribution();
    block.update_rk3(dt, 3);
    boundary_condition(&block, block.get_Q());
    block.calc_primitive(block.get_Q());

    if ((n_t + 1) % dump_every == 0 || n_t + 1 == nsteps) {
      std::snprintf(name, sizeof name, "q_%06ld.bin", n_t + 1);
      dump_state(name, sp.t_cur, sp, block.get_Q());
    }
  }
  std::fclose(steps);
  if (ckpt && 0 != block.output_bin("checkpoint_ref.dat")) return 5;
  if (vtk) {
    mkdir("vtk_final", 0755);
    if (0 != output_vtk_xml(&block, 0, 1, "vtk_final", "output")) return 4;
  }
  MPI_Finalize();
  return 0;
}
