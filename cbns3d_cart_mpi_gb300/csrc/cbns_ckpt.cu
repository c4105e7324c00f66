// cbns_ckpt.cu — checkpoints streamed between a file and the device, in the
// reference's format (Block3d::read_bin, src/Block3d.cpp:318-357, and
// Block3d::output_bin, src/Block3d.cpp:964-987):
//   t_cur (binary64), IM_G, JM_G, KM_G (32-bit unsigned: the padded extents),
//   then Q in get_idx_Q order (AoS, ghosts included), native byte order.
// The state moves through two pinned chunk buffers owned by the handle, so the
// file read (write) of one chunk overlaps the copy of the other and the whole
// state never sits in host memory.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/cbns_gpu.h"
#include "cbns_internal.h"

namespace {

constexpr size_t kChunk = size_t(8) << 20;  // bytes per pinned buffer

cbns_status ckpt_fail(cbns_status st, const std::string& msg) {
  cbns::set_last_error(msg);
  return st;
}

cbns_status ensure_chunks(cbns_handle* h) {
  for (int b = 0; b < 2; ++b) {
    if (!h->h_chunk[b]) {
      cudaError_t e = cudaMallocHost(&h->h_chunk[b], kChunk);
      if (e != cudaSuccess) return cbns::cuda_error(e, "cudaMallocHost(checkpoint chunk)");
    }
    if (!h->ev_chunk[b]) {
      cudaError_t e = cudaEventCreateWithFlags(&h->ev_chunk[b], cudaEventDisableTiming);
      if (e != cudaSuccess) return cbns::cuda_error(e, "cudaEventCreate(checkpoint chunk)");
    }
  }
  return CBNS_OK;
}

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

}  // namespace

extern "C" {

cbns_status cbns_load_checkpoint(cbns_handle* h, const char* path, double* t_out) {
  cbns_status st = cbns::enter(h, "cbns_load_checkpoint");
  if (st != CBNS_OK) return st;
  if (!path) return ckpt_fail(CBNS_ERR_INVALID_ARG, "cbns_load_checkpoint: null path");
  File fh;
  fh.f = std::fopen(path, "rb");
  if (!fh.f) return ckpt_fail(CBNS_ERR_IO, std::string("cbns_load_checkpoint: cannot open ") + path);
  double t = 0.0;
  uint32_t dims[3] = {0, 0, 0};
  if (std::fread(&t, sizeof(double), 1, fh.f) != 1 || std::fread(dims, sizeof(uint32_t), 3, fh.f) != 3)
    return ckpt_fail(CBNS_ERR_FORMAT, "cbns_load_checkpoint: truncated header");
  const cbns::SolveDev& s = h->desc;
  if (dims[0] != (uint32_t)s.nx || dims[1] != (uint32_t)s.ny || dims[2] != (uint32_t)s.nz)
    return ckpt_fail(CBNS_ERR_FORMAT, "cbns_load_checkpoint: the dimensions do not match");
  if ((st = ensure_chunks(h)) != CBNS_OK) return st;
  const size_t total = sizeof(double) * CBNS_NEQ * (size_t)s.V;
  char* dst = reinterpret_cast<char*>(h->d_stage);
  cudaError_t e = cudaSuccess;
  size_t off = 0;
  for (int c = 0; off < total; ++c) {
    const int b = c & 1;
    const size_t n = total - off < kChunk ? total - off : kChunk;
    // Buffer b is free once the copy that last read it has completed.
    if ((e = cudaEventSynchronize(h->ev_chunk[b])) != cudaSuccess) return cbns::cuda_error(e, "cudaEventSynchronize");
    if (std::fread(h->h_chunk[b], 1, n, fh.f) != n) {
      cudaStreamSynchronize(h->stream);
      return ckpt_fail(CBNS_ERR_FORMAT, "cbns_load_checkpoint: truncated state");
    }
    if ((e = cudaMemcpyAsync(dst + off, h->h_chunk[b], n, cudaMemcpyHostToDevice, h->stream)) != cudaSuccess ||
        (e = cudaEventRecord(h->ev_chunk[b], h->stream)) != cudaSuccess)
      return cbns::cuda_error(e, "cudaMemcpyAsync(checkpoint chunk)");
    off += n;
  }
  // The staged state replaces the solve's state only after the whole file has
  // been read, so a failed load leaves the solve unchanged.
  if ((st = cbns::adopt_staged(h, t)) != CBNS_OK) return st;
  if (t_out) *t_out = t;
  return CBNS_OK;
}

cbns_status cbns_save_checkpoint(cbns_handle* h, const char* path) {
  cbns_status st = cbns::enter(h, "cbns_save_checkpoint");
  if (st != CBNS_OK) return st;
  if (!path) return ckpt_fail(CBNS_ERR_INVALID_ARG, "cbns_save_checkpoint: null path");
  double t = 0.0;
  if ((st = cbns_get_time(h, &t, nullptr)) != CBNS_OK) return st;
  if ((st = ensure_chunks(h)) != CBNS_OK) return st;
  if ((st = cbns::stage_state(h)) != CBNS_OK) return st;
  File fh;
  fh.f = std::fopen(path, "wb");
  if (!fh.f) {
    cudaStreamSynchronize(h->stream);
    return ckpt_fail(CBNS_ERR_IO, std::string("cbns_save_checkpoint: cannot open ") + path);
  }
  const cbns::SolveDev& s = h->desc;
  const uint32_t dims[3] = {(uint32_t)s.nx, (uint32_t)s.ny, (uint32_t)s.nz};
  bool ok = std::fwrite(&t, sizeof(double), 1, fh.f) == 1 && std::fwrite(dims, sizeof(uint32_t), 3, fh.f) == 3;
  const size_t total = sizeof(double) * CBNS_NEQ * (size_t)s.V;
  const char* src = reinterpret_cast<const char*>(h->d_stage);
  cudaError_t e = cudaSuccess;
  // Chunk c is copied into buffer c & 1 while the host writes chunk c - 1 from
  // the other buffer.
  size_t off = 0, prev_n = 0;
  int c = 0;
  for (; off < total; ++c) {
    const int b = c & 1;
    const size_t n = total - off < kChunk ? total - off : kChunk;
    if ((e = cudaMemcpyAsync(h->h_chunk[b], src + off, n, cudaMemcpyDeviceToHost, h->stream)) != cudaSuccess ||
        (e = cudaEventRecord(h->ev_chunk[b], h->stream)) != cudaSuccess)
      return cbns::cuda_error(e, "cudaMemcpyAsync(checkpoint chunk)");
    if (c > 0) {
      if ((e = cudaEventSynchronize(h->ev_chunk[b ^ 1])) != cudaSuccess)
        return cbns::cuda_error(e, "cudaEventSynchronize");
      ok = ok && std::fwrite(h->h_chunk[b ^ 1], 1, prev_n, fh.f) == prev_n;
    }
    prev_n = n;
    off += n;
  }
  if (c > 0) {
    const int b = (c - 1) & 1;
    if ((e = cudaEventSynchronize(h->ev_chunk[b])) != cudaSuccess) return cbns::cuda_error(e, "cudaEventSynchronize");
    ok = ok && std::fwrite(h->h_chunk[b], 1, prev_n, fh.f) == prev_n;
  }
  const bool closed = std::fclose(fh.f) == 0;
  fh.f = nullptr;
  if (!ok || !closed) return ckpt_fail(CBNS_ERR_IO, std::string("cbns_save_checkpoint: write failed: ") + path);
  return CBNS_OK;
}

}  // extern "C"
