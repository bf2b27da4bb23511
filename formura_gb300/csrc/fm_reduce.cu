// fm_reduce.cu — deterministic FP64 sums for the conserved-total checks
// (mass and energy drift), and FP64/FP32 pipe probes used to measure the
// arithmetic roofline the stencil kernels are measured against.
//
// The sum is a fixed two-level tree whose shape depends only on n: stage 1
// gives each of G blocks a contiguous chunk (thread-strided, then a shared
// memory tree), stage 2 folds the G partials in one block.  The same n always
// gives the same bits, on any GPU.
#include <algorithm>

#include "fm_common.cuh"

namespace {

constexpr int kSumThreads = 256;
constexpr int kSumMaxBlocks = 1024;

__device__ __forceinline__ double block_tree_sum(double v) {
  __shared__ double sh[kSumThreads];
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int w = kSumThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + w];
    __syncthreads();
  }
  return sh[0];
}

__global__ void __launch_bounds__(kSumThreads)
    sum_stage1(int64_t n, int64_t chunk, const double *__restrict__ a, double *partials) {
  const int64_t lo = (int64_t)blockIdx.x * chunk;
  const int64_t hi = min(lo + chunk, n);
  double acc = 0.0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += kSumThreads) acc = acc + __ldg(a + i);
  const double s = block_tree_sum(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kSumThreads)
    sum_stage1_f32(int64_t n, int64_t chunk, const float *__restrict__ a, double *partials) {
  const int64_t lo = (int64_t)blockIdx.x * chunk;
  const int64_t hi = min(lo + chunk, n);
  double acc = 0.0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += kSumThreads) acc = acc + (double)__ldg(a + i);
  const double s = block_tree_sum(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kSumThreads)
    sum_stage2(int g, const double *__restrict__ partials, double *out) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < g; i += kSumThreads) acc = acc + partials[i];
  const double s = block_tree_sum(acc);
  if (threadIdx.x == 0) *out = s;
}

int sum_blocks(int64_t n) {
  const int64_t b = (n + 4095) / 4096;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, kSumMaxBlocks));
}

// FP64 / FP32 FMA pipe probes: 8 independent dependency chains per thread.
__global__ void probe_fma_f64(double *sink, int iters, double seed) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = seed + threadIdx.x * 1e-9 + k;
  const double m = 1.0000000001, c = 1e-12;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], m, c);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == 12345.678) sink[blockIdx.x] = s;  // never true; keeps the chains live
}

__global__ void probe_fma_f32(float *sink, int iters, float seed) {
  float a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = seed + threadIdx.x * 1e-6f + k;
  const float m = 1.000001f, c = 1e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], m, c);
  }
  float s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == 12345.678f) sink[blockIdx.x] = s;
}

}  // namespace

extern "C" size_t fm_sum_f64_scratch_elems(int64_t n) {
  return n <= 0 ? 1 : (size_t)sum_blocks(n);
}

extern "C" int fm_sum_f64(int64_t n, const double *a, double *partials, double *out_device,
                          void *stream) {
  FM_CHECK_ARG(out_device && partials, "fm_sum_f64: NULL argument");
  FM_CHECK_ARG(n >= 0 && (n == 0 || a), "fm_sum_f64: bad input");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (n == 0) {
    FM_TRY_CUDA(cudaMemsetAsync(out_device, 0, sizeof(double), s));
    return FM_OK;
  }
  const int g = sum_blocks(n);
  const int64_t chunk = (n + g - 1) / g;
  sum_stage1<<<g, kSumThreads, 0, s>>>(n, chunk, a, partials);
  sum_stage2<<<1, kSumThreads, 0, s>>>(g, partials, out_device);
  FM_TRY_CUDA(cudaGetLastError());
  return FM_OK;
}

extern "C" int fm_sum_f32_as_f64(int64_t n, const float *a, double *partials,
                                 double *out_device, void *stream) {
  FM_CHECK_ARG(out_device && partials, "fm_sum_f32_as_f64: NULL argument");
  FM_CHECK_ARG(n >= 0 && (n == 0 || a), "fm_sum_f32_as_f64: bad input");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (n == 0) {
    FM_TRY_CUDA(cudaMemsetAsync(out_device, 0, sizeof(double), s));
    return FM_OK;
  }
  const int g = sum_blocks(n);
  const int64_t chunk = (n + g - 1) / g;
  sum_stage1_f32<<<g, kSumThreads, 0, s>>>(n, chunk, a, partials);
  sum_stage2<<<1, kSumThreads, 0, s>>>(g, partials, out_device);
  FM_TRY_CUDA(cudaGetLastError());
  return FM_OK;
}

extern "C" int fm_probe_fma(int fp64, int blocks, int threads, int iters, void *sink,
                            void *stream) {
  FM_CHECK_ARG(sink && blocks > 0 && threads > 0 && threads <= 1024 && iters > 0,
               "fm_probe_fma: bad arguments");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (fp64)
    probe_fma_f64<<<blocks, threads, 0, s>>>((double *)sink, iters, 0.5);
  else
    probe_fma_f32<<<blocks, threads, 0, s>>>((float *)sink, iters, 0.5f);
  FM_TRY_CUDA(cudaGetLastError());
  return FM_OK;
}
