// cbns_noalloc.cu — kinetic energy and enstrophy of a caller-held device state,
// computed without allocating any memory.
//
// Who needs this: code that must not call cudaMalloc while it runs — an in-situ
// monitor invoked from inside another solver's time loop that may not change the
// device's memory footprint, a host framework whose caching allocator owns the
// whole device budget, or a real-time loop where an allocation's latency and
// possible implicit synchronisation are not allowed.  Such callers already hold
// the state and a place for the result in their own device memory; they pass
// both, and the reduction's scratch lives in a fixed static device array.
//
// Scratch: g_noalloc_partials, NOALLOC_MAX_CTAS slots of 4 doubles (128 KiB),
// declared at file scope, so every GPU that loads the library holds it until the
// process exits.  Each CTA of the partial-sum kernel reduces a fixed chunk of
// NOALLOC_CELLS_PER_CTA cells into its own slot and writes that slot on every
// call; the finishing kernel reads only the slots of the current call, so no
// slot has to start at zero.  All calls share the one array: two calls whose
// kernels overlap on the GPU (different streams, no ordering) race on it.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/cbns_gpu.h"

namespace cbns {
void set_last_error(const std::string& msg);  // cbns_api.cu: the text cbns_last_error() returns
}  // namespace cbns

namespace {

constexpr int NOALLOC_THREADS = 256;
constexpr int NOALLOC_CELLS_PER_THREAD = 64;
constexpr long long NOALLOC_CELLS_PER_CTA = (long long)NOALLOC_THREADS * NOALLOC_CELLS_PER_THREAD;
constexpr int NOALLOC_MAX_CTAS = 4096;
constexpr int NG = CBNS_NG;
constexpr int NEQ = CBNS_NEQ;
constexpr int MAX_DEVICES = 64;

static __device__ __align__(256) double g_noalloc_partials[4 * NOALLOC_MAX_CTAS];

// Device address of g_noalloc_partials per device.  Every call made while its
// stream is not being captured looks the address up again (with the device
// current), so a context destroyed and recreated in between (cudaDeviceReset)
// leaves no stale pointer behind; a call inside a stream capture uses the
// address the last uncaptured call on that device found.
double* g_scratch_ptr[MAX_DEVICES] = {nullptr};
std::mutex g_scratch_mu;

struct Pair {
  double s, e;
};

__device__ __forceinline__ Pair pair_add(Pair a, Pair b) {
  // Two-sum: s + e carries the exact sum of the inputs' leading parts.
  double t = a.s + b.s;
  double z = t - a.s;
  double err = (a.s - (t - z)) + (b.s - z);
  return Pair{t, a.e + b.e + err};
}

__device__ __forceinline__ Pair warp_pair(Pair v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    Pair w{__shfl_down_sync(0xffffffffu, v.s, o), __shfl_down_sync(0xffffffffu, v.e, o)};
    v = pair_add(v, w);
  }
  return v;
}

#ifdef CBNS_BOUNDS_CHECK
// Bounds-checked build: accesses outside an array counted here (and sent to
// element 0 instead); the entry point reads and clears the count after its
// kernels.
static __device__ unsigned long long g_noalloc_misses;
#endif

// Element i of an array of n elements (plain indexing unless CBNS_BOUNDS_CHECK).
template <class T>
__device__ __forceinline__ T& elem(T* base, long long n, long long i) {
#ifdef CBNS_BOUNDS_CHECK
  if (i < 0 || i >= n) {
    atomicAdd(&g_noalloc_misses, 1ull);
    i = 0;
  }
#endif
  return base[i];
}

// Q in the reference's layout: Q[n + 5*((NG+i) + IM_G*((NG+j) + JM_G*(NG+k)))],
// nQ values in all.
__device__ __forceinline__ double velocity(const double* Q, long long nQ, long long c, int n) {
  return elem(Q, nQ, NEQ * c + n) / elem(Q, nQ, NEQ * c);
}

__device__ __forceinline__ double ddir(const double* Q, long long nQ, long long c, long long st, int n,
                                       double inv_h) {
  const double c12 = 1.0 / 12.0, c23 = 2.0 / 3.0;
  return ((velocity(Q, nQ, c - 2 * st, n) - velocity(Q, nQ, c + 2 * st, n)) * c12 +
          (velocity(Q, nQ, c + st, n) - velocity(Q, nQ, c - st, n)) * c23) * inv_h;
}

__global__ void __launch_bounds__(NOALLOC_THREADS)
    k_noalloc_partials(const double* __restrict__ Q, int IM, int JM, int KM, double inv_dx, double inv_dy,
                       double inv_dz, double* __restrict__ partials) {
  __shared__ Pair red[2][NOALLOC_THREADS / 32];
  const long long ncell = (long long)IM * JM * KM;
  const long long IM_G = IM + 2 * NG, JM_G = JM + 2 * NG;
  const long long sy = IM_G, sz = IM_G * JM_G;
  const long long nQ = NEQ * IM_G * JM_G * (long long)(KM + 2 * NG);
  Pair ke{0.0, 0.0}, en{0.0, 0.0};
  const long long first = (long long)blockIdx.x * NOALLOC_CELLS_PER_CTA;
  for (int r = 0; r < NOALLOC_CELLS_PER_THREAD; ++r) {
    const long long q = first + (long long)r * NOALLOC_THREADS + threadIdx.x;
    if (q >= ncell) break;
    const int i = (int)(q % IM);
    const int j = (int)((q / IM) % JM);
    const int k = (int)(q / ((long long)IM * JM));
    const long long c = (NG + i) + IM_G * ((NG + j) + JM_G * (long long)(NG + k));
    const double rho = elem(Q, nQ, NEQ * c);
    const double u = velocity(Q, nQ, c, 1), v = velocity(Q, nQ, c, 2), w = velocity(Q, nQ, c, 3);
    const double ox = ddir(Q, nQ, c, sy, 3, inv_dy) - ddir(Q, nQ, c, sz, 2, inv_dz);
    const double oy = ddir(Q, nQ, c, sz, 1, inv_dz) - ddir(Q, nQ, c, 1, 3, inv_dx);
    const double oz = ddir(Q, nQ, c, 1, 2, inv_dx) - ddir(Q, nQ, c, sy, 1, inv_dy);
    ke = pair_add(ke, Pair{0.5 * rho * (u * u + v * v + w * w), 0.0});
    en = pair_add(en, Pair{0.5 * rho * (ox * ox + oy * oy + oz * oz), 0.0});
  }
  ke = warp_pair(ke);
  en = warp_pair(en);
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = ke;
    red[1][threadIdx.x >> 5] = en;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    Pair a = red[0][0], b = red[1][0];
    for (int t = 1; t < NOALLOC_THREADS / 32; ++t) {
      a = pair_add(a, red[0][t]);
      b = pair_add(b, red[1][t]);
    }
    const long long np = 4 * NOALLOC_MAX_CTAS;
    elem(partials, np, 4 * blockIdx.x + 0) = a.s;
    elem(partials, np, 4 * blockIdx.x + 1) = a.e;
    elem(partials, np, 4 * blockIdx.x + 2) = b.s;
    elem(partials, np, 4 * blockIdx.x + 3) = b.e;
  }
}

__global__ void __launch_bounds__(1024)
    k_noalloc_finish(const double* __restrict__ partials, int nparts, double inv_n, double* __restrict__ out) {
  __shared__ Pair red[2][32];
  Pair ke{0.0, 0.0}, en{0.0, 0.0};
  for (int q = threadIdx.x; q < nparts; q += blockDim.x) {
    const long long np = 4 * NOALLOC_MAX_CTAS;
    ke = pair_add(ke, Pair{elem(partials, np, 4 * q), elem(partials, np, 4 * q + 1)});
    en = pair_add(en, Pair{elem(partials, np, 4 * q + 2), elem(partials, np, 4 * q + 3)});
  }
  ke = warp_pair(ke);
  en = warp_pair(en);
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = ke;
    red[1][threadIdx.x >> 5] = en;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    Pair a = red[0][0], b = red[1][0];
    for (int t = 1; t < (int)(blockDim.x / 32); ++t) {
      a = pair_add(a, red[0][t]);
      b = pair_add(b, red[1][t]);
    }
    out[0] = (a.s + a.e) * inv_n;
    out[1] = (b.s + b.e) * inv_n;
  }
}

cbns_status noalloc_fail(cbns_status st, const std::string& msg) {
  cbns::set_last_error(msg);
  return st;
}

}  // namespace

extern "C" cbns_status cbns_diagnostics_noalloc(const double* Q_dev, uint32_t IM, uint32_t JM, uint32_t KM,
                                                double dx, double dy, double dz, double* out_dev, void* stream) {
  if (!Q_dev || !out_dev) return noalloc_fail(CBNS_ERR_INVALID_ARG, "cbns_diagnostics_noalloc: null pointer");
  if (!(dx > 0.0) || !(dy > 0.0) || !(dz > 0.0))
    return noalloc_fail(CBNS_ERR_INVALID_ARG, "cbns_diagnostics_noalloc: grid spacings must be > 0");
  if (IM < (uint32_t)NG || JM < (uint32_t)NG || KM < (uint32_t)NG)
    return noalloc_fail(CBNS_ERR_BAD_DIMS, "cbns_diagnostics_noalloc: every extent must be >= 4 (NG)");
  const long long ncell = (long long)IM * JM * KM;
  const long long nctas = (ncell + NOALLOC_CELLS_PER_CTA - 1) / NOALLOC_CELLS_PER_CTA;
  if (nctas > NOALLOC_MAX_CTAS || (double)(IM + 2 * NG) * (JM + 2 * NG) * (KM + 2 * NG) * NEQ > 9.0e15) {
    return noalloc_fail(CBNS_ERR_BAD_DIMS, "cbns_diagnostics_noalloc: IM*JM*KM = " + std::to_string(ncell) +
                                               " exceeds the static scratch capacity of " +
                                               std::to_string((long long)NOALLOC_MAX_CTAS * NOALLOC_CELLS_PER_CTA) +
                                               " cells");
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return noalloc_fail(CBNS_ERR_CUDA, std::string("cbns_diagnostics_noalloc: cudaGetDevice: ") +
                                           cudaGetErrorString(e));
  if (dev < 0 || dev >= MAX_DEVICES)
    return noalloc_fail(CBNS_ERR_NO_DEVICE, "cbns_diagnostics_noalloc: device index out of range");
  cudaStream_t st = (cudaStream_t)stream;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
    cudaGetLastError();
    cap = cudaStreamCaptureStatusActive;  // unknown: keep to the address already found
  }
  double* scratch = nullptr;
  {
    // Set-up on this device (the device is current): the host-side name
    // g_noalloc_partials is not a device address, so look the address up.
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev] || cap == cudaStreamCaptureStatusNone) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_partials);
      if (e != cudaSuccess)
        return noalloc_fail(CBNS_ERR_CUDA, std::string("cbns_diagnostics_noalloc: cudaGetSymbolAddress: ") +
                                               cudaGetErrorString(e));
      g_scratch_ptr[dev] = (double*)p;
    }
    scratch = g_scratch_ptr[dev];
  }
  k_noalloc_partials<<<(int)nctas, NOALLOC_THREADS, 0, st>>>(Q_dev, (int)IM, (int)JM, (int)KM, 1.0 / dx, 1.0 / dy,
                                                             1.0 / dz, scratch);
  k_noalloc_finish<<<1, 1024, 0, st>>>(scratch, (int)nctas, 1.0 / (double)ncell, out_dev);
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return noalloc_fail(CBNS_ERR_CUDA, std::string("cbns_diagnostics_noalloc: launch: ") + cudaGetErrorString(e));
#ifdef CBNS_BOUNDS_CHECK
  // Bounds-checked build only: wait for the kernels and report any access that
  // left its array.
  unsigned long long misses = 0;
  const unsigned long long zero = 0;
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess ||
      (e = cudaMemcpyFromSymbol(&misses, g_noalloc_misses, sizeof misses)) != cudaSuccess ||
      (e = cudaMemcpyToSymbol(g_noalloc_misses, &zero, sizeof zero)) != cudaSuccess)
    return noalloc_fail(CBNS_ERR_CUDA, std::string("cbns_diagnostics_noalloc: ") + cudaGetErrorString(e));
  if (misses)
    return noalloc_fail(CBNS_ERR_BOUNDS, "cbns_diagnostics_noalloc: " + std::to_string(misses) +
                                             " accesses outside their arrays");
#endif
  return CBNS_OK;
}
