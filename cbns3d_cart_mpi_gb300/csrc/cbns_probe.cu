// cbns_probe.cu — pipe-throughput probes used as roofline denominators.
// Built as its own library (lib/libcbns_probe.so) for the benchmark; the
// product library does not contain it.
//
// The binary64 stencil kernels are bound by the FP64 pipe, whose peak no
// vendor table gives for this part, so it is measured here: each thread runs
// eight independent FMA chains for a fixed count, on 8 CTAs of 256 threads per
// SM, timed with CUDA events.  FLOPs count 2 per FMA.
#include <cuda_runtime.h>

#include "../../include/cbns_gpu.h"
#include "cbns_device.cuh"
#include "cbns_ff.cuh"

namespace {

template <typename T>
__global__ void k_fma_chains(T* out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x * (T)1e-3, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
  for (int it = 0; it < iters; ++it) {
    x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
    x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
cbns_status probe(int iters, double* tflops) {
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return CBNS_ERR_CUDA;
  const int blocks = prop.multiProcessorCount * 8, threads = 256;
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * blocks * threads) != cudaSuccess) return CBNS_ERR_OUT_OF_MEMORY;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    k_fma_chains<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return CBNS_ERR_CUDA;
  *tflops = 2.0 * 8.0 * (double)blocks * threads * iters / (best * 1e-3) * 1e-12;
  return CBNS_OK;
}

}  // namespace

// Measured FMA throughput of the current device in TFLOP/s (2 FLOPs per FMA),
// binary64 when fp64 != 0 else binary32.
extern "C" cbns_status cbns_probe_peak(int fp64, double* tflops) {
  if (!tflops) return CBNS_ERR_INVALID_ARG;
  return fp64 ? probe<double>(4096, tflops) : probe<float>(65536, tflops);
}

namespace {
__global__ void k_rcp64(const double* __restrict__ x, double* __restrict__ y, double* __restrict__ ref, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    y[i] = cbns::rcp64(x[i]);
    ref[i] = 1.0 / x[i];
  }
}
}  // namespace

// The face kernel's reciprocal and the IEEE division 1.0/x of n device values
// (test of its accuracy); device pointers, synchronous.
extern "C" cbns_status cbns_probe_rcp64(const double* x, double* y, double* ref, long long n) {
  if (!x || !y || !ref || n < 0) return CBNS_ERR_INVALID_ARG;
  if (n == 0) return CBNS_OK;
  k_rcp64<<<1024, 256>>>(x, y, ref, n);
  return cudaDeviceSynchronize() == cudaSuccess ? CBNS_OK : CBNS_ERR_CUDA;
}

namespace {
__global__ void k_ff(const double* __restrict__ x, const double* __restrict__ y, double* __restrict__ out,
                     long long n) {
  using namespace cbns;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float2 a2 = ff_split(x[i]), b2 = ff_split(y[i]);
    const ff a{a2.x, a2.y}, b{b2.x, b2.y};
    double* o = out + 6 * i;
    o[0] = ff_to_double(a);
    o[1] = ff_to_double(ff_rcp(a));
    o[2] = ff_to_double(ff_rsqrt(a));
    o[3] = ff_to_double(a * b);
    o[4] = ff_to_double(a + b);
    o[5] = ff_to_double(ff_fma(a, b, a));
  }
}
}  // namespace

// The float-float building blocks of the CBNS_FP64_FF face kernel on n device
// value pairs (x, y): out[6 i .. 6 i + 5] = the binary64 value of split(x),
// 1/x, 1/sqrt(x), x*y, x+y and x*y + x, each evaluated in float-float from the
// splits (test of their accuracy); device pointers, synchronous.
extern "C" cbns_status cbns_probe_ff(const double* x, const double* y, double* out, long long n) {
  if (!x || !y || !out || n < 0) return CBNS_ERR_INVALID_ARG;
  if (n == 0) return CBNS_OK;
  k_ff<<<1024, 256>>>(x, y, out, n);
  return cudaDeviceSynchronize() == cudaSuccess ? CBNS_OK : CBNS_ERR_CUDA;
}
