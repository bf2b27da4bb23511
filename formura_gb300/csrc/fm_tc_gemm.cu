// fm_tc_gemm.cu — BF16 GEMM on the tcgen05 tensor cores, FP32 accumulation in
// tensor memory: C[M x N] = A[M x K] * B[N x K]^T (A, B row-major bf16,
// C row-major fp32).  The building block of the surrogate's convolutions,
// exposed as fm_tc_gemm_bf16 so that the descriptor and layout conventions of
// fm_tc.cuh are tested on their own.
//
// CTA = 128 threads, output tile 128 x 64 (UMMA M = 128, N = 64, K = 16),
// 64 TMEM columns.  Per 64-wide K chunk: all threads stage the A and B chunks
// into shared memory in the K-major core-matrix layout, fence to the async
// proxy, thread 0 issues four MMAs and commits them to an mbarrier, all wait.
// The shared-memory stage is double-buffered so that staging chunk k+1
// overlaps the MMAs of chunk k.
#include <algorithm>

#include "fm_common.cuh"
#include "fm_tc.cuh"

namespace {

using namespace fm::tc;

constexpr int kTM = 128, kTN = 64, kKC = 64;
constexpr int kABytes = kTM * kKC * 2, kBBytes = kTN * kKC * 2;

__global__ void __launch_bounds__(128)
    tc_gemm_bf16(const __nv_bfloat16 *__restrict__ A, const __nv_bfloat16 *__restrict__ B,
                 float *__restrict__ C, int M, int N, int K, int *err) {
  extern __shared__ __align__(1024) uint8_t dsm[];
  // A buffers at dsm + b*kABytes, B buffers after both A buffers
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t s_tmem;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int m0 = blockIdx.y * kTM, n0 = blockIdx.x * kTN;
  if (warp == 0) tmem_alloc(&s_tmem, 64);
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = s_tmem;
  const uint32_t idesc = idesc_bf16_f32(kTM, kTN);
  const int nk = K / kKC;
  uint32_t phase[2] = {0u, 0u};
  bool ok = true;
  for (int kc = 0; kc < nk; ++kc) {
    const int b = kc & 1;
    // before overwriting buffer b, the MMAs that read it (chunk kc-2) must be done
    if (kc >= 2) {
      if (!mbar_wait(&bar[b], phase[b])) ok = false;
      phase[b] ^= 1u;
    }
    // stage A chunk: 128 rows x 64 k (16-byte vectors of 8 bf16)
    const int k0 = kc * kKC;
    for (int v = tid; v < kTM * (kKC / 8); v += 128) {
      const int r = v / (kKC / 8), kk = (v % (kKC / 8)) * 8;
      const uint4 val = *reinterpret_cast<const uint4 *>(A + (size_t)(m0 + r) * K + k0 + kk);
      *reinterpret_cast<uint4 *>(dsm + b * kABytes + kmajor_off(r, kk, kKC)) = val;
    }
    for (int v = tid; v < kTN * (kKC / 8); v += 128) {
      const int r = v / (kKC / 8), kk = (v % (kKC / 8)) * 8;
      const uint4 val = *reinterpret_cast<const uint4 *>(B + (size_t)(n0 + r) * K + k0 + kk);
      *reinterpret_cast<uint4 *>(dsm + 2 * kABytes + b * kBBytes + kmajor_off(r, kk, kKC)) = val;
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      fence_after_sync();
      const uint32_t a0 = smem_u32(dsm + b * kABytes), b0 = smem_u32(dsm + 2 * kABytes + b * kBBytes);
#pragma unroll
      for (int s = 0; s < kKC / 16; ++s) {
        const uint64_t ad = smem_desc(a0 + s * 256, 128, (kKC / 8) * 128);
        const uint64_t bd = smem_desc(b0 + s * 256, 128, (kKC / 8) * 128);
        mma_bf16(tmem, ad, bd, idesc, (kc | s) != 0);
      }
      mma_commit(&bar[b]);
    }
  }
  // drain: wait for the last one or two chunks
  for (int kc = (nk > 2 ? nk - 2 : 0); kc < nk; ++kc) {
    const int b = kc & 1;
    if (!mbar_wait(&bar[b], phase[b])) ok = false;
    phase[b] ^= 1u;
  }
  fence_after_sync();
  if (ok) {
    // epilogue: warp w owns TMEM lanes 32w..32w+31 = rows of the tile
    const int row = m0 + warp * 32 + (tid & 31);
#pragma unroll
    for (int c = 0; c < kTN; c += 16) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
      if (row < M) {
        float *dst = C + (size_t)row * N + n0 + c;
#pragma unroll
        for (int i = 0; i < 16; ++i) dst[i] = v[i];
      }
    }
  } else {
    if (tid == 0) atomicExch(err, 1);
    // give in-flight MMAs a second bounded chance to finish before the
    // tensor memory they write is released
    for (int b = 0; b < 2; ++b) mbar_wait(&bar[b], phase[b]);
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 64);
}

}  // namespace

extern "C" int fm_tc_gemm_bf16(int M, int N, int K, const void *A, const void *B, float *C,
                               int *err_device, void *stream) {
  FM_CHECK_ARG(A && B && C && err_device, "fm_tc_gemm_bf16: NULL argument");
  FM_CHECK_ARG(M > 0 && N > 0 && K > 0 && M % kTM == 0 && N % kTN == 0 && K % kKC == 0,
               "fm_tc_gemm_bf16: need M %% 128 == 0, N %% 64 == 0, K %% 64 == 0 (got %d,%d,%d)",
               M, N, K);
  FM_CHECK_ARG(((uintptr_t)A & 15) == 0 && ((uintptr_t)B & 15) == 0,
               "fm_tc_gemm_bf16: A and B must be 16-byte aligned");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int smem = 2 * (kABytes + kBBytes);
  FM_TRY_CUDA(cudaFuncSetAttribute(tc_gemm_bf16, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  tc_gemm_bf16<<<dim3(N / kTN, M / kTM), 128, smem, s>>>(
      reinterpret_cast<const __nv_bfloat16 *>(A), reinterpret_cast<const __nv_bfloat16 *>(B), C,
      M, N, K, err_device);
  FM_TRY_CUDA(cudaGetLastError());
  return FM_OK;
}
