// cbns3d_gb300 — the solver's driver on one GB300: the time loop of the
// reference's main (src/cbns3d.cpp:27-308) with its stage block replaced by the
// GPU library (include/cbns_gpu.h).  Parameters come from ./input.txt through
// the same .ini -> parser -> input.txt flow; output is the reference's VTK XML
// directories output000 .. and its checkpoint file format.
//
//   cbns3d_gb300 <dimX> <dimY> <dimZ>
//
// One GPU holds the whole grid, so the process count dimX*dimY*dimZ must be 1
// (the reference checks the same product against its MPI world size,
// src/cbns3d.cpp:45-53).
#include <sys/stat.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "../../../include/cbns_gpu.h"
#include "../../../include/cbns_host.h"

// Output staging: the primitives of the current state are downloaded once
// (cbns_download_prims), then the ASCII VTK writer (1.3 GB of text at 256^3,
// formatted on every host core) runs on a host thread while the GPU keeps
// stepping.  One writer at a time; the next output waits for the previous one
// before reusing the buffers.
class OutputStager {
 public:
  explicit OutputStager(const cbns_params& sp) : sp_(sp) {
    const size_t n = (size_t)(sp.IM + 2 * CBNS_NG) * (sp.JM + 2 * CBNS_NG) * (sp.KM + 2 * CBNS_NG);
    for (auto& a : f_) a.resize(n);
    x_.resize(sp.IM + 1);
    y_.resize(sp.JM + 1);
    z_.resize(sp.KM + 1);
    cbns_host_gen_mesh(&sp, sp.IM, sp.JM, sp.KM, 0, 0, 0, x_.data(), y_.data(), z_.data());
  }
  ~OutputStager() { wait(); }

  // Returns 0, or -1 if the download failed; a failed write is reported by wait().
  int submit(cbns_handle* h, unsigned cnt) {
    if (wait() != 0) return -1;
    if (cbns_download_prims(h, f_[0].data(), f_[1].data(), f_[2].data(), f_[3].data(), f_[4].data(), nullptr) !=
        CBNS_OK)
      return -1;
    std::ostringstream dir;
    dir << "output" << std::setw(3) << std::setfill('0') << cnt;
    writer_ = std::thread([this, d = dir.str()] {
      status_ = cbns_host_output_vtk_xml(d.c_str(), "output", 0, 1, sp_.IM, sp_.JM, sp_.KM, x_.data(), y_.data(),
                                         z_.data(), f_[0].data(), f_[1].data(), f_[2].data(), f_[3].data(),
                                         f_[4].data());
    });
    return 0;
  }

  int wait() {
    if (writer_.joinable()) writer_.join();
    if (status_ != CBNS_OK) {
      std::cerr << "Unable to open the .vtr file by process 0\n";
      return -1;
    }
    return 0;
  }

 private:
  cbns_params sp_;
  std::vector<double> f_[5], x_, y_, z_;
  std::thread writer_;
  cbns_status status_ = CBNS_OK;
};

int main(int argc, char** argv) {
  if (4 > argc) {
    std::cout << "Usage: program <dimX> <dimY> <dimZ>\n";
    return 1;
  }
  int dims[3] = {std::atoi(argv[1]), std::atoi(argv[2]), std::atoi(argv[3])};
  if (dims[0] * dims[1] * dims[2] != 1) {
    std::cerr << "Error: Number of processes must equal dimX * dimY * dimZ (one GPU: 1 1 1).\n";
    return 1;
  }
  cbns_params sp;
  cbns_status st = cbns_host_read_input("input.txt", &sp);
  if (st != CBNS_OK) {
    std::cerr << "Exception opening/reading file input.txt\n";
    return 1;
  }
  std::cout << "checkpoint_fname : " << sp.checkpoint_fname << "\nCFL : " << sp.CFL << "\nt_cur : " << sp.t_cur
            << "\nt_end : " << sp.t_end << "\nPr : " << sp.Pr << "\ngamma : " << sp.gamma << "\nMach : " << sp.Mach
            << "\nRe : " << sp.Re << "\nT_inf : " << sp.T_inf << "\nL : " << sp.L << "\nIM : " << sp.IM
            << "\nJM : " << sp.JM << "\nKM : " << sp.KM << "\nnstep_max : " << sp.nstep_max
            << "\ncheckpoint_freq : " << sp.checkpoint_freq << "\nnum_output : " << sp.num_output
            << "\nis_restart : " << sp.is_restart << std::endl;
  for (unsigned i = 0; i <= sp.num_output; i++) {
    char name[20];
    std::snprintf(name, sizeof name, "output%.3i", i);
    mkdir(name, 0755);
  }
  const uint32_t IM = sp.IM, JM = sp.JM, KM = sp.KM;
  std::string ckpt = std::string(sp.checkpoint_fname) + "000.dat";
  // The command line stays the reference's; the environment variable
  // CBNS_PRECISION picks the arithmetic: fp64 (default), fp64_ff or fp32_mixed.
  int precision = CBNS_FP64;
  if (const char* pe = std::getenv("CBNS_PRECISION")) {
    const std::string ps(pe);
    if (ps == "fp64_ff") {
      precision = CBNS_FP64_FF;
    } else if (ps == "fp32_mixed") {
      precision = CBNS_FP32_MIXED;
    } else if (ps != "fp64") {
      std::cerr << "Error: CBNS_PRECISION must be fp64, fp64_ff or fp32_mixed\n";
      return 1;
    }
  }
  cbns_handle* h = nullptr;
  if ((st = cbns_create(&sp, IM, JM, KM, precision, &h)) != CBNS_OK) {
    std::cerr << "cbns_create failed: " << cbns_last_error() << "\n";
    return 1;
  }
  if (sp.is_restart) {
    // The reference's initial condition on the host (its libm sin/cos), uploaded.
    std::vector<double> Q((size_t)CBNS_NEQ * (IM + 2 * CBNS_NG) * (JM + 2 * CBNS_NG) * (KM + 2 * CBNS_NG));
    cbns_host_initial_condition(&sp, IM, JM, KM, 0, 0, 0, Q.data());
    if ((st = cbns_upload_Q(h, Q.data(), sp.t_cur)) != CBNS_OK) {
      std::cerr << "cbns_upload_Q failed: " << cbns_last_error() << "\n";
      return 1;
    }
  } else {
    // The checkpoint streams from the file to the device.
    double t0 = sp.t_cur;
    if (cbns_load_checkpoint(h, ckpt.c_str(), &t0) != CBNS_OK) {
      std::cerr << "Unable to open the checkpoint file by process 0\n" << cbns_last_error() << "\n";
      return 1;
    }
    sp.t_cur = t0;
  }
  unsigned cnt_out = 0;
  OutputStager out(sp);
  if (out.submit(h, cnt_out) != 0) return 1;
  double dt_out = sp.t_end / sp.num_output;
  double t_out = ((int)(sp.t_cur / dt_out) + 1) * dt_out;

  auto start = std::chrono::high_resolution_clock::now();
  for (uint32_t n_t = 0; n_t < sp.nstep_max; n_t++) {
    double dt = 0.0, t = 0.0;
    st = cbns_step(h, sp.t_end, &dt, &t);
    if (st == CBNS_FINISHED) {
      std::cout << "Finished!\n";
      break;
    }
    if (st != CBNS_OK) {
      std::cerr << "cbns_step failed: " << cbns_last_error() << "\n";
      return 1;
    }
    sp.t_cur = t;
    std::cout << n_t << ", " << dt << ", " << sp.t_cur << std::endl;
    if (0 == (n_t + 1) % sp.checkpoint_freq) {
      if (cbns_save_checkpoint(h, ckpt.c_str()) != CBNS_OK) {
        std::cerr << "Unable to save the checkpoint file by process 0\n";
        return 1;
      }
    }
    if (t_out < sp.t_cur) {
      cnt_out++;
      if (out.submit(h, cnt_out) != 0) return 1;
      t_out += dt_out;
    }
  }
  auto end = std::chrono::high_resolution_clock::now();
  double wall = std::chrono::duration<double>(end - start).count();
  std::cout << "  Wall time: " << wall << " seconds\n"
            << "  CPU time: " << wall << " seconds\n";
  cnt_out++;
  if (out.submit(h, cnt_out) != 0 || out.wait() != 0) return 1;
  cbns_destroy(h);
  return 0;
}
