// cbns_internal.h — definitions shared by the library's host-side translation
// units (the C ABI, batches, the serving loop).  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/cbns_gpu.h"
#include "cbns_device.cuh"
#include "cbns_prof.h"

namespace cbns {
void set_last_error(const std::string& msg);
}  // namespace cbns

struct cbns_handle;
namespace cbns {
// Helpers shared by the translation units of the library (cbns_api.cu).
cbns_status enter(cbns_handle* h, const char* fn);           // null check, cudaSetDevice
cbns_status cuda_error(cudaError_t e, const char* what);     // records the error text
cbns_status adopt_staged(cbns_handle* h, double t);          // staged AoS state -> the solve's state
cbns_status stage_state(cbns_handle* h);                     // Q -> staged AoS (enqueued)
}  // namespace cbns

struct cbns_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  int precision = CBNS_FP64;
  cbns_params params{};
  uint32_t IM = 0, JM = 0, KM = 0;
  char* arena = nullptr;
  size_t arena_bytes = 0;
  cbns::SolveDev desc{};
  cbns::SolveDev* d_desc = nullptr;
  cbns::SolveCtl* d_ctl = nullptr;
  cbns::TileRef* d_tiles_int = nullptr;
  cbns::TileRef* d_tiles_ring = nullptr;
  cbns::TileRef* d_tiles_pad = nullptr;
  int n_int = 0, n_ring = 0, n_pad = 0;
  double* d_stage = nullptr;
  double* d_partials = nullptr;
  int nparts = 0;
  double* d_out = nullptr;  // small device results (diagnostics, raw dt)
  cbns::SolveCtl* h_ctl = nullptr;  // pinned
  double* h_out = nullptr;    // pinned
  char* h_chunk[2] = {nullptr, nullptr};           // pinned checkpoint chunks (cbns_ckpt.cu)
  cudaEvent_t ev_chunk[2] = {nullptr, nullptr};
  // Asynchronous entry points (cbns_*_async): an upload and a download stream
  // beside the compute stream and a second staging buffer, so one state's host
  // copies overlap another's kernels.  Created on the first asynchronous call.
  cudaStream_t up_stream = nullptr;
  cudaStream_t down_stream = nullptr;
  double* d_stage_out = nullptr;
  cudaEvent_t ev_in_ready = nullptr, ev_in_free = nullptr, ev_out_ready = nullptr, ev_out_free = nullptr;
  cudaGraphExec_t step_graph = nullptr;
  double graph_t_end = 0.0;
  cbns::Profiler prof;
  cbns::Profiler* pf() { return prof.on ? &prof : nullptr; }
};

struct cbns_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<cbns_handle*> handles;
  bool mixed = false;
  int precision = CBNS_FP64;
  char* arena = nullptr;
  cbns::SolveDev* d_descs = nullptr;
  cbns::TileRef* d_int[3] = {nullptr, nullptr, nullptr};
  cbns::TileRef* d_ring[3] = {nullptr, nullptr, nullptr};
  int n_int[3] = {0, 0, 0};
  int n_ring[3] = {0, 0, 0};
  int sm_count = 0;
  cbns::LaunchCfg cfg;  // tile_rows, max_ctas (= ctas_per_sm * sm_count, 0 = one CTA per tile)
  int ctas_per_sm = 0;
  cudaGraphExec_t graph = nullptr;
  int graph_rows = 0, graph_ctas = -1;
  cbns::SolveCtl* h_ctl = nullptr;  // pinned, one per solve
  std::vector<unsigned> start_steps;
};
