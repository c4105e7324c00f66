// cbns_prof.h — optional per-launch CUDA-event timing of the library's kernels.
//
// When a handle's profiler is on, every kernel launch is bracketed by two events
// recorded on the launching stream, and launches are issued directly (not through
// a step graph).  Results are summed per kernel name.
#pragma once

#include <cuda_runtime.h>

#include <vector>

namespace cbns {

enum KernelId {
  KID_DT_REDUCE = 0,
  KID_DT_FINALIZE,
  KID_INVISCID_X,
  KID_INVISCID_Y,
  KID_INVISCID_Z,
  KID_VISCOUS,
  KID_UPDATE,
  KID_PREPARE,
  KID_LAYOUT,
  KID_DIAG,
  KID_COUNT
};

inline const char* kernel_name(int id) {
  static const char* names[KID_COUNT] = {"dt_reduce", "dt_finalize", "inviscid_x", "inviscid_y", "inviscid_z",
                                         "viscous",   "update",      "prepare",    "layout",     "diagnostics"};
  return (id >= 0 && id < KID_COUNT) ? names[id] : "?";
}

struct Profiler {
  bool on = false;
  struct Rec {
    int id;
    cudaEvent_t a, b;
  };
  std::vector<Rec> recs;
  std::vector<cudaEvent_t> pool;
  size_t used = 0;

  cudaEvent_t take() {
    if (used == pool.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      pool.push_back(e);
    }
    return pool[used++];
  }
  void before(int id, cudaStream_t st) {
    if (!on) return;
    Rec r{id, take(), nullptr};
    cudaEventRecord(r.a, st);
    recs.push_back(r);
  }
  void after(cudaStream_t st) {
    if (!on || recs.empty()) return;
    recs.back().b = take();
    cudaEventRecord(recs.back().b, st);
  }
  void reset() {
    recs.clear();
    used = 0;
  }
  ~Profiler() {
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
  }
};

}  // namespace cbns
