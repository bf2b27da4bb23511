// fm_conv.cu — 3x3 periodic convolutions on the tcgen05 tensor cores (BF16
// operands, FP32 accumulation in tensor memory): the layers of the learned
// 16-step surrogate.
//
// Activation layout: NHWC bf16 with a one-pixel periodic halo,
// [B][H+2][W+2][C]; the halo always holds the wrapped-around border, so a
// 3x3 tap is a plain shifted read.  Weights: [Cout][9][Cin] bf16, tap
// t = (dy+1)*3 + (dx+1).
//
// conv3x3_fwd<NT>: implicit GEMM.  M = 128 consecutive pixels (row-major over
// B*H*W), N = Cout = NT (32 or 64), K = 9 taps x 64 input channels.  For each
// tap the CTA gathers the 128 shifted pixel rows (128 B each) and the tap's
// NT x 64 weight block into shared memory (K-major core-matrix layout, two
// stages), thread 0 issues four K=16 MMAs and commits them to the stage's
// mbarrier.  The fused epilogue reads the 128 x NT accumulator from TMEM:
//   v = acc (+ bias) (* gelu'(gate)) (+ residual);  z_out <- v;
//   y <- act(v) stored bf16 into the padded output (halo included) and/or
//   fp32 unpadded.
// One kernel thereby serves the forward layers and, with flipped/transposed
// weights, the data gradients (see the host entry points).
//
// conv3x3_wgrad<NT>: dW[t][co][ci] = sum_p dY[p][co] * X[p + t][ci] as a
// split-K GEMM: M = (tap, ci) rows (576, in 5 tiles of 128), N = co,
// K = pixels; each CTA accumulates a pixel range in TMEM and adds its tile
// to the fp32 gradient with atomics.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

// threads of the weight-resident convolution kernels: 128 per TMEM lane-quarter
// group, each group taking 64 / (threads / 128) of the 64 output channels
// (512 measured 0.653 against 0.640 ms per 8 x 512^2 network jump)
#ifndef FM_CONV_THREADS
#define FM_CONV_THREADS 256
#endif

#include "fm_common.cuh"
#include "fm_tc.cuh"
#include "fm_tune.h"

namespace {

using namespace fm::tc;
typedef __nv_bfloat16 bf16;

constexpr int CIN = 64;
constexpr int kTM = 128;

// erf(z) by Abramowitz & Stegun, Handbook of Mathematical Functions, 7.1.26
// (|error| <= 1.5e-7, far below the bf16 rounding of the activations): one
// reciprocal, a degree-5 polynomial and one exponential, without the range
// branches of a full-precision erff.  `e` returns exp(-z^2), which the GELU
// derivative reuses.
__device__ __forceinline__ float erf_as(float z, float &e) {
  const float az = fabsf(z);
  const float t = __fdividef(1.0f, fmaf(0.3275911f, az, 1.0f));
  const float poly =
      t * fmaf(t, fmaf(t, fmaf(t, fmaf(t, 1.061405429f, -1.453152027f), 1.421413741f),
                       -0.284496736f),
               0.254829592f);
  e = __expf(-az * az);
  return copysignf(fmaf(-poly, e, 1.0f), z);
}
// GELU(x) = x * Phi(x) = 0.5 x (1 + erf(x / sqrt 2)); GELU'(x) = Phi(x) + x phi(x)
__device__ __forceinline__ float gelu(float x) {
  float e;
  return 0.5f * x * (1.0f + erf_as(x * 0.70710678118654752f, e));
}
__device__ __forceinline__ float gelu_grad(float x) {
  float e;  // exp(-x^2 / 2)
  const float cdf = 0.5f * (1.0f + erf_as(x * 0.70710678118654752f, e));
  return cdf + x * (0.39894228040143268f * e);
}

struct ConvArgs {
  const bf16 *x;      // [B][H+2][W+2][64]
  const bf16 *w;      // [NT][9][64]
  const float *bias;  // [NT] or null
  const bf16 *gate;   // padded [..][NT]: multiply by gelu'(gate) (or null)
  const bf16 *resid;  // padded [..][NT]: add (or null)
  bf16 *z_out;        // padded [..][NT] pre-activation (or null)
  bf16 *y_out;        // padded [..][NT] (or null)
  float *y_f32;       // [B][H][W][NT] (or null)
  int B, H, W, act;   // act: 0 none, 1 GELU
  int *err;
};

__device__ __forceinline__ size_t pad_index(int b, int py, int px, int H, int W) {
  return ((size_t)b * (H + 2) + py) * (W + 2) + px;
}

template <int NT>
__global__ void __launch_bounds__(128) conv3x3_fwd(ConvArgs a) {
  constexpr int kABytes = kTM * CIN * 2, kBBytes = NT * CIN * 2;
  constexpr int kStage = kABytes + kBBytes;
  extern __shared__ __align__(1024) uint8_t dsm[];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t s_tmem;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int H = a.H, W = a.W;
  const int hw = H * W;
  const long long p0 = (long long)blockIdx.x * kTM;
  if (warp == 0) tmem_alloc(&s_tmem, NT < 32 ? 32 : NT);
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = s_tmem;
  const uint32_t idesc = idesc_bf16_f32(kTM, NT);
  uint32_t ph0 = 0u, ph1 = 0u;
  bool ok = true;
  for (int t = 0; t < 9; ++t) {
    const int st = t & 1;
    if (t >= 2) {
      if (!mbar_wait(&bar[st], st ? ph1 : ph0)) ok = false;
      if (st) ph1 ^= 1u; else ph0 ^= 1u;
    }
    const int dy = t / 3 - 1, dx = t % 3 - 1;
    uint8_t *sa = dsm + st * kStage;
    uint8_t *sb = sa + kABytes;
    // A: 128 shifted pixel rows x 64 channels
    for (int v = tid; v < kTM * 8; v += 128) {
      const int r = v >> 3, kk = (v & 7) * 8;
      const long long p = p0 + r;
      const int b = (int)(p / hw), rem = (int)(p % hw);
      const int y = rem / W, xx = rem % W;
      const bf16 *src = a.x + pad_index(b, y + 1 + dy, xx + 1 + dx, H, W) * CIN + kk;
      *reinterpret_cast<uint4 *>(sa + kmajor_off(r, kk, CIN)) =
          *reinterpret_cast<const uint4 *>(src);
    }
    // B: the tap's NT x 64 weights
    for (int v = tid; v < NT * 8; v += 128) {
      const int r = v >> 3, kk = (v & 7) * 8;
      *reinterpret_cast<uint4 *>(sb + kmajor_off(r, kk, CIN)) =
          *reinterpret_cast<const uint4 *>(a.w + ((size_t)r * 9 + t) * CIN + kk);
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      fence_after_sync();
      const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
#pragma unroll
      for (int s = 0; s < CIN / 16; ++s)
        mma_bf16(tmem, smem_desc(a0 + s * 256, 128, (CIN / 8) * 128),
                 smem_desc(b0 + s * 256, 128, (CIN / 8) * 128), idesc, (t | s) != 0);
      mma_commit(&bar[st]);
    }
  }
  // the last two taps (7 -> stage 1, 8 -> stage 0)
  if (!mbar_wait(&bar[1], ph1)) ok = false;
  if (!mbar_wait(&bar[0], ph0)) ok = false;
  fence_after_sync();
  if (ok) {
    const long long p = p0 + warp * 32 + (tid & 31);
    const int b = (int)(p / hw), rem = (int)(p % hw);
    const int y = rem / W, xx = rem % W;
    // padded positions this pixel occupies: interior + periodic halo copies
    int pys[2] = {y + 1, -1}, pxs[2] = {xx + 1, -1};
    if (y == 0) pys[1] = H + 1;
    if (y == H - 1) pys[1] = 0;
    if (xx == 0) pxs[1] = W + 1;
    if (xx == W - 1) pxs[1] = 0;
    const size_t pin = pad_index(b, y + 1, xx + 1, H, W);
#pragma unroll
    for (int c0 = 0; c0 < NT; c0 += 16) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (a.bias) {
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] += __ldg(a.bias + c0 + i);
      }
      if (a.gate) {
        const bf16 *g = a.gate + pin * NT + c0;
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] *= gelu_grad(__bfloat162float(g[i]));
      }
      if (a.resid) {
        const bf16 *rr = a.resid + pin * NT + c0;
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] += __bfloat162float(rr[i]);
      }
      __align__(16) bf16 zb[16], yb[16];
      if (a.z_out) {
#pragma unroll
        for (int i = 0; i < 16; ++i) zb[i] = __float2bfloat16_rn(v[i]);
      }
      if (a.act == 1) {
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = gelu(v[i]);
      }
#pragma unroll
      for (int i = 0; i < 16; ++i) yb[i] = __float2bfloat16_rn(v[i]);
#pragma unroll
      for (int iy = 0; iy < 2; ++iy) {
        if (pys[iy] < 0) continue;
#pragma unroll
        for (int ix = 0; ix < 2; ++ix) {
          if (pxs[ix] < 0) continue;
          const size_t q = pad_index(b, pys[iy], pxs[ix], H, W) * NT + c0;
          if (a.z_out) {
            reinterpret_cast<uint4 *>(a.z_out + q)[0] = reinterpret_cast<const uint4 *>(zb)[0];
            reinterpret_cast<uint4 *>(a.z_out + q)[1] = reinterpret_cast<const uint4 *>(zb)[1];
          }
          if (a.y_out) {
            reinterpret_cast<uint4 *>(a.y_out + q)[0] = reinterpret_cast<const uint4 *>(yb)[0];
            reinterpret_cast<uint4 *>(a.y_out + q)[1] = reinterpret_cast<const uint4 *>(yb)[1];
          }
        }
      }
      if (a.y_f32) {
        float *dst = a.y_f32 + (size_t)p * NT + c0;
#pragma unroll
        for (int i = 0; i < 16; ++i) dst[i] = v[i];
      }
    }
  } else {
    if (tid == 0) atomicExch(a.err, 1);
    mbar_wait(&bar[0], ph0 ^ 1u);
    mbar_wait(&bar[1], ph1 ^ 1u);
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, NT < 32 ? 32 : NT);
}

// ---------------------------------------------------------------------------
// The epilogue of one tile of the weight-resident kernels, for this warp's 32
// positions (its TMEM lane quarter) and kCh channels (its channel group):
//   v = acc + bias (* gelu'(gate)) (+ residual);  z_out <- v;  y <- act(v)
// stored bf16 into the padded output (with the periodic halo copies of border
// cells) and/or fp32 unpadded.  `tacc` is the accumulator's TMEM address,
// `res_rows` the tile's staged residual rows (128-byte swizzled) or null;
// `valid` false only loads the accumulator (the TMEM load is warp-collective).
constexpr int kConvThreads = FM_CONV_THREADS;
constexpr int kCh = 64 / (kConvThreads / 128);  // channels per epilogue warp
__device__ __forceinline__ void conv_tile_epilogue(const ConvArgs &a, int b, long long j0,
                                                   uint32_t tacc, const uint8_t *res_rows,
                                                   const float *s_bias, int quarter, int chalf,
                                                   bool valid) {
  constexpr int NT = 64;
  const int lane = threadIdx.x & 31;
  const int H = a.H, W = a.W, Wp = W + 2;
  const long long img = (long long)(H + 2) * Wp;
  const long long j = j0 + quarter * 32 + lane;
  const int py = (int)(j / Wp), px = (int)(j % Wp);
  const bool interior = valid && py >= 1 && py <= H && px >= 1 && px <= W;
  const int y = py - 1, xx = px - 1;
  int pys[2] = {py, -1}, pxs[2] = {px, -1};
  if (y == 0) pys[1] = H + 1;
  if (y == H - 1) pys[1] = 0;
  if (xx == 0) pxs[1] = W + 1;
  if (xx == W - 1) pxs[1] = 0;
  const size_t pin = (size_t)b * img + (size_t)j;
  // this thread's channels of the gate and residual inputs, loaded as 16-byte
  // vectors before the accumulator is read so that their latency overlaps
  uint4 gv[kCh / 8], rv[kCh / 8];
  if (interior && a.gate) {
    const uint4 *g4 = reinterpret_cast<const uint4 *>(a.gate + pin * NT + chalf * kCh);
#pragma unroll
    for (int q = 0; q < kCh / 8; ++q) gv[q] = __ldg(g4 + q);
  }
  if (interior && res_rows) {
    const int p = quarter * 32 + lane;
    const uint4 *r4 = reinterpret_cast<const uint4 *>(res_rows);
#pragma unroll
    for (int q = 0; q < kCh / 8; ++q) rv[q] = r4[p * 8 + ((chalf * (kCh / 8) + q) ^ (p & 7))];
  }
  float vv[kCh];
  const uint32_t tcol = tacc + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(chalf * kCh);
  if constexpr (kCh == 32)
    tmem_ld32(tcol, *reinterpret_cast<float(*)[32]>(vv));
  else
    tmem_ld16(tcol, *reinterpret_cast<float(*)[16]>(vv));
#pragma unroll
  for (int cc = 0; cc < kCh; cc += 16) {
    const int c0 = chalf * kCh + cc;
    float *v = vv + cc;
    if (!interior) continue;
    if (a.bias) {
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] += s_bias[c0 + i];
    }
    if (a.gate) {
      const bf16 *g = reinterpret_cast<const bf16 *>(&gv[cc / 8]);
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] *= gelu_grad(__bfloat162float(g[i]));
    }
    if (res_rows) {
      const bf16 *rr = reinterpret_cast<const bf16 *>(&rv[cc / 8]);
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] += __bfloat162float(rr[i]);
    }
    __align__(16) bf16 zb[16], yb[16];
    if (a.z_out) {
#pragma unroll
      for (int i = 0; i < 16; ++i) zb[i] = __float2bfloat16_rn(v[i]);
    }
    if (a.act == 1) {
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = gelu(v[i]);
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) yb[i] = __float2bfloat16_rn(v[i]);
#pragma unroll
    for (int iy = 0; iy < 2; ++iy) {
      if (pys[iy] < 0) continue;
#pragma unroll
      for (int ix = 0; ix < 2; ++ix) {
        if (pxs[ix] < 0) continue;
        const size_t q = (((size_t)b * (H + 2) + pys[iy]) * Wp + pxs[ix]) * NT + c0;
        if (a.z_out) {
          reinterpret_cast<uint4 *>(a.z_out + q)[0] = reinterpret_cast<const uint4 *>(zb)[0];
          reinterpret_cast<uint4 *>(a.z_out + q)[1] = reinterpret_cast<const uint4 *>(zb)[1];
        }
        if (a.y_out) {
          reinterpret_cast<uint4 *>(a.y_out + q)[0] = reinterpret_cast<const uint4 *>(yb)[0];
          reinterpret_cast<uint4 *>(a.y_out + q)[1] = reinterpret_cast<const uint4 *>(yb)[1];
        }
      }
    }
    if (a.y_f32) {
      float *dst = a.y_f32 + (((size_t)b * H + y) * W + xx) * NT + c0;
#pragma unroll
      for (int i = 0; i < 16; ++i) dst[i] = v[i];
    }
  }
}

// ---------------------------------------------------------------------------
// conv3x3_fwd_res: the persistent, weight-resident form for cout = 64.
//
// Output positions are indexed in the FLATTENED PADDED image,
// j = py*(W+2) + px; the 3x3 tap (dy,dx) of position j reads position
// j + dy*(W+2) + dx.  A tile of 128 consecutive positions therefore reads one
// contiguous region [j0 - (W+3), j0 + 128 + (W+3)).  That region is staged
// into shared memory as eight "channel-group planes" (8 channels = 16 B per
// position, positions consecutive, plane stride PL): in the K-major
// no-swizzle descriptor this is SBO = 128 B between 8-row groups and
// LBO = PL between K-adjacent core matrices, so the A operand of every tap is
// the SAME region at start offset ((W+3) + dy*(W+2) + dx)*16 — no per-tap
// gather.  Halo positions of the tile are computed and discarded.
//   * the 9 taps' weights (72 KB) are loaded once per CTA and stay resident;
//   * regions are double-buffered with cp.async (prefetch of tile i+1 while the
//     tensor core works on tile i);
//   * two TMEM accumulators (2 x 64 columns): the epilogue of tile i-1 runs
//     while the MMAs of tile i are in flight;
//   * eight warps: warp w reads TMEM lanes 32*(w%4).. (its 32 positions) and
//     columns 32*(w/4).. (its 32 channels), so the epilogue, which bounds the
//     kernel, is spread over twice the warps of the four TMEM lane quarters.
constexpr int kResThreads = kConvThreads;

__host__ __device__ __forceinline__ int res_region_len(int Wp) { return kTM + 2 * (Wp + 1); }

__global__ void __launch_bounds__(kResThreads, 1) conv3x3_fwd_res(ConvArgs a, int ntile_img,
                                                                  int ntiles, int plane) {
  constexpr int NT = 64;
  constexpr int kWBytes = 9 * NT * CIN * 2;  // 72 KB, tap tiles of 8 KB
  extern __shared__ __align__(1024) uint8_t dsm[];
  uint8_t *sw = dsm;                          // weights
  uint8_t *sreg = dsm + kWBytes;              // 2 region buffers of 8*plane bytes
  // 3 buffers of a tile's residual input (when there is one), 128 positions x
  // 8 chunks of 16 B, chunk q of position p at slot p*8 + (q ^ (p & 7))
  // (conflict-free 16-byte reads); tile t uses buffer t % 3
  uint8_t *sres = sreg + 2 * 8 * (size_t)plane;
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t s_tmem;
  __shared__ float s_bias[NT];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int quarter = warp & 3, chalf = warp >> 2;  // TMEM lane quarter, channel group
  if (tid < NT) s_bias[tid] = a.bias ? a.bias[tid] : 0.0f;
  const int H = a.H, W = a.W, Wp = W + 2;
  const int rlen = res_region_len(Wp);
  const long long img = (long long)(H + 2) * Wp;  // positions per padded image
  if (warp == 0) tmem_alloc(&s_tmem, 128);
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
  }
  // weights -> resident K-major tiles (one cp.async group)
  for (int v = tid; v < 9 * NT * 8; v += kResThreads) {
    const int tap = v / (NT * 8), rem = v % (NT * 8);
    const int r = rem >> 3, kk = (rem & 7) * 8;
    cp_async16(sw + tap * (NT * CIN * 2) + kmajor_off(r, kk, CIN),
               a.w + ((size_t)r * 9 + tap) * CIN + kk, true);
  }
  cp_async_commit();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = s_tmem;
  const uint32_t idesc = idesc_bf16_f32(kTM, NT);

  auto stage = [&](int it, int buf) {
    const int tile = blockIdx.x + it * gridDim.x;
    const int b = tile / ntile_img, tl = tile % ntile_img;
    const long long j0 = (long long)(Wp + 1) + (long long)tl * kTM;
    const long long r0 = j0 - (Wp + 1);
    const bf16 *base = a.x + (size_t)b * img * CIN;
    uint8_t *dst = sreg + (size_t)buf * 8 * plane;
    for (int v = tid; v < rlen * 8; v += kResThreads) {
      const int pos = v >> 3, kg = v & 7;
      const long long j = r0 + pos;
      const bool ok = j < img;
      cp_async16(dst + kg * plane + pos * 16, base + (size_t)(ok ? j : 0) * CIN + kg * 8, ok);
    }
    cp_async_commit();
  };
  // the residual rows of tile `it` (its own cp.async group); issued after the
  // barrier of an iteration, so its buffer's previous reader (the epilogue of
  // tile it-3, two iterations earlier) has finished
  auto stage_res = [&](int it) {
    const int tile = blockIdx.x + it * gridDim.x;
    const int b = tile / ntile_img, tl = tile % ntile_img;
    const long long j0 = (long long)(Wp + 1) + (long long)tl * kTM;
    const bf16 *rbase = a.resid + (size_t)b * img * NT;
    uint8_t *rdst = sres + (size_t)(it % 3) * kTM * NT * 2;
    for (int v = tid; v < kTM * 8; v += kResThreads) {
      const int pos = v >> 3, q = v & 7;
      const long long j = j0 + pos;
      const bool ok = j < img;
      cp_async16(rdst + (pos * 8 + (q ^ (pos & 7))) * 16, rbase + (size_t)(ok ? j : 0) * NT + q * 8,
                 ok);
    }
    cp_async_commit();
  };

  auto epilogue = [&](int it, int acc) {
    const int tile = blockIdx.x + it * gridDim.x;
    const long long j0 = (long long)(Wp + 1) + (long long)(tile % ntile_img) * kTM;
    conv_tile_epilogue(a, tile / ntile_img, j0, tmem + (uint32_t)(acc * 64),
                       a.resid ? sres + (size_t)(it % 3) * kTM * NT * 2 : nullptr, s_bias, quarter,
                       chalf, true);
  };

  const int my_tiles = ntiles > (int)blockIdx.x ? (ntiles - 1 - (int)blockIdx.x) / gridDim.x + 1 : 0;
  uint32_t ph[2] = {0u, 0u};
  bool ok = true;
  if (my_tiles > 0) {
    stage(0, 0);
    if (a.resid) stage_res(0);
  }
  for (int it = 0; it < my_tiles; ++it) {
    const int buf = it & 1;
    if (it >= 1) {
      // MMAs of tile it-1 read region buffer buf^1 and write accumulator buf^1
      if (!mbar_wait(&bar[buf ^ 1], ph[buf ^ 1])) ok = false;
      ph[buf ^ 1] ^= 1u;
    }
    if (it + 1 < my_tiles) {
      stage(it + 1, buf ^ 1);
      cp_async_wait<1>();  // weights and region `it` have landed
    } else {
      cp_async_wait<0>();
    }
    fence_proxy_async_smem();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (tid == 0) {
      const uint32_t reg = smem_u32(sreg + (size_t)buf * 8 * plane);
      const uint32_t wbase = smem_u32(sw);
#pragma unroll 1
      for (int tap = 0; tap < 9; ++tap) {
        const int dy = tap / 3 - 1, dx = tap % 3 - 1;
        const uint32_t a_off = (uint32_t)((Wp + 1) + dy * Wp + dx) * 16u;
#pragma unroll
        for (int s = 0; s < CIN / 16; ++s) {
          const uint64_t ad = smem_desc(reg + a_off + (uint32_t)(2 * s) * (uint32_t)plane,
                                        (uint32_t)plane, 128);
          const uint64_t bd = smem_desc(wbase + tap * (NT * CIN * 2) + s * 256, 128,
                                        (CIN / 8) * 128);
          mma_bf16(tmem + (uint32_t)(buf * 64), ad, bd, idesc, (tap | s) != 0);
        }
      }
      mma_commit(&bar[buf]);
    }
    if (a.resid && it + 1 < my_tiles) stage_res(it + 1);
    if (it >= 1 && ok) epilogue(it - 1, buf ^ 1);
  }
  if (my_tiles > 0) {
    const int last = (my_tiles - 1) & 1;
    if (!mbar_wait(&bar[last], ph[last])) ok = false;
    fence_after_sync();
    if (ok) epilogue(my_tiles - 1, last);
  }
  if (!ok && tid == 0) atomicExch(a.err, 1);
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 128);
}

// ---------------------------------------------------------------------------
// conv3x3_fwd_tma: conv3x3_fwd_res with its staging on TMA and its steps
// chained by mbarriers instead of CTA-wide barriers.
//   * a tile's region (8 channel-group planes, as above) arrives by 16 tiled
//     TMA copies (a plane per channel group, in two boxes of at most 256
//     positions), its residual rows by one TMA copy with the 128-byte swizzle
//     (position p's 16-byte chunk q lands at chunk q ^ (p % 8): conflict-free
//     reads); each completes on its buffer's mbarrier by transaction count;
//   * thread 0 issues a tile's MMAs as soon as its region has landed and the
//     epilogue of the tile two back has released the accumulator (acc_empty,
//     one arrival per warp), so the MMAs of tile t+1 run under the epilogue of
//     tile t, and the region of tile t+2 is requested as soon as the MMAs of
//     tile t have finished reading region buffer t % 2;
//   * weights stay resident (loaded once with cp.async), two TMEM accumulators.
// Same MMA sequence and epilogue as conv3x3_fwd_res: identical results.
__global__ void __launch_bounds__(kResThreads, 1)
    conv3x3_fwd_tma(ConvArgs a, int ntile_img, int ntiles, int plane, int rlen, int r1,
                    const __grid_constant__ CUtensorMap tm_x1,
                    const __grid_constant__ CUtensorMap tm_x2,
                    const __grid_constant__ CUtensorMap tm_r) {
  constexpr int NT = 64;
  constexpr int kWBytes = 9 * NT * CIN * 2;
  constexpr uint32_t kResBytes = kTM * NT * 2;  // 16 KB of residual rows per tile
  extern __shared__ __align__(1024) uint8_t dsm[];
  uint8_t *sw = dsm;
  uint8_t *sreg = dsm + kWBytes;
  uint8_t *sres = dsm + (((size_t)kWBytes + 16 * (size_t)plane + 1023) & ~(size_t)1023);
  __shared__ __align__(8) uint64_t full_x[2], full_r[2], mma_done[2], acc_empty[2];
  __shared__ uint32_t s_tmem;
  __shared__ float s_bias[NT];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quarter = warp & 3, chalf = warp >> 2;  // TMEM lane quarter, channel group
  if (tid < NT) s_bias[tid] = a.bias ? a.bias[tid] : 0.0f;
  const int Wp = a.W + 2;
  if (warp == 0) tmem_alloc(&s_tmem, 128);
  if (tid == 0) {
    for (int b = 0; b < 2; ++b) {
      mbar_init(&full_x[b], 1);
      mbar_init(&full_r[b], 1);
      mbar_init(&mma_done[b], 1);
      mbar_init(&acc_empty[b], kResThreads / 32);
    }
  }
  for (int v = tid; v < 9 * NT * 8; v += kResThreads) {
    const int tap = v / (NT * 8), rem = v % (NT * 8);
    const int r = rem >> 3, kk = (rem & 7) * 8;
    cp_async16(sw + tap * (NT * CIN * 2) + kmajor_off(r, kk, CIN),
               a.w + ((size_t)r * 9 + tap) * CIN + kk, true);
  }
  cp_async_commit();
  cp_async_wait<0>();
  fence_proxy_async_smem();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = s_tmem;
  const uint32_t idesc = idesc_bf16_f32(kTM, NT);
  const int my_tiles =
      ntiles > (int)blockIdx.x ? (ntiles - 1 - (int)blockIdx.x) / gridDim.x + 1 : 0;

  auto tile_pos = [&](int it, int &b, long long &j0) {
    const int tile = blockIdx.x + it * gridDim.x;
    b = tile / ntile_img;
    j0 = (long long)(Wp + 1) + (long long)(tile % ntile_img) * kTM;
  };
  // (thread 0) region of tile `it` into region buffer it % 2
  auto issue_x = [&](int it) {
    int b;
    long long j0;
    tile_pos(it, b, j0);
    const int r0 = (int)(j0 - (Wp + 1));
    uint64_t *bar = &full_x[it & 1];
    uint8_t *dst = sreg + (size_t)(it & 1) * 8 * plane;
    mbar_arrive_expect_tx(bar, (uint32_t)(8 * rlen * 16));
    for (int kg = 0; kg < 8; ++kg) {
      tma_load_3d(dst + (size_t)kg * plane, &tm_x1, kg * 8, r0, b, bar);
      if (rlen > r1) tma_load_3d(dst + (size_t)kg * plane + (size_t)r1 * 16, &tm_x2, kg * 8, r0 + r1, b, bar);
    }
  };
  // (thread 0) residual rows of tile `it` into residual buffer it % 2
  auto issue_r = [&](int it) {
    int b;
    long long j0;
    tile_pos(it, b, j0);
    uint64_t *bar = &full_r[it & 1];
    mbar_arrive_expect_tx(bar, kResBytes);
    tma_load_3d(sres + (size_t)(it & 1) * kResBytes, &tm_r, 0, (int)j0, b, bar);
  };

  bool ok = true;
  // bookkeeping for the clean-up: the last tile issued per buffer (-1: none)
  int last_x[2] = {-1, -1}, last_r[2] = {-1, -1}, last_mma[2] = {-1, -1};
  if (tid == 0) {
    for (int it = 0; it < 2 && it < my_tiles; ++it) {
      issue_x(it);
      last_x[it & 1] = it;
      if (a.resid) {
        issue_r(it);
        last_r[it & 1] = it;
      }
    }
  }

  auto epilogue = [&](int t) {
    const int bt = t & 1;
    const uint32_t pt = (uint32_t)(t >> 1) & 1u;
    __syncwarp();
    bool good = mbar_wait(&mma_done[bt], pt);
    fence_after_sync();
    // region buffer bt is free: request tile t+2's region
    if (tid == 0 && good && ok && t + 2 < my_tiles) {
      issue_x(t + 2);
      last_x[bt] = t + 2;
    }
    if (a.resid && good) good = mbar_wait(&full_r[bt], pt);
    ok = __all_sync(0xffffffffu, ok && good);  // warp-uniform from here on
    int b;
    long long j0;
    tile_pos(t, b, j0);
    conv_tile_epilogue(a, b, j0, tmem + (uint32_t)(bt * 64),
                       a.resid ? sres + (size_t)bt * kResBytes : nullptr, s_bias, quarter, chalf, ok);
    // this warp is done with accumulator bt and residual buffer bt
    fence_before_sync();
    __syncwarp();
    if (lane == 0) mbar_arrive(&acc_empty[bt]);
    if (tid == 0 && ok && a.resid && t + 2 < my_tiles) {
      if (!mbar_wait(&acc_empty[bt], pt)) ok = false;
      if (ok) {
        issue_r(t + 2);
        last_r[bt] = t + 2;
      }
    }
  };

  for (int it = 0; it < my_tiles && ok; ++it) {
    const int bb = it & 1;
    if (tid == 0) {
      if (!mbar_wait(&full_x[bb], (uint32_t)(it >> 1) & 1u)) ok = false;
      if (ok && it >= 2 && !mbar_wait(&acc_empty[bb], (uint32_t)((it - 2) >> 1) & 1u)) ok = false;
      fence_after_sync();
      if (ok) {
        const uint32_t reg = smem_u32(sreg + (size_t)bb * 8 * plane);
        const uint32_t wbase = smem_u32(sw);
#pragma unroll 1
        for (int tap = 0; tap < 9; ++tap) {
          const int dy = tap / 3 - 1, dx = tap % 3 - 1;
          const uint32_t a_off = (uint32_t)((Wp + 1) + dy * Wp + dx) * 16u;
#pragma unroll
          for (int s = 0; s < CIN / 16; ++s) {
            const uint64_t ad = smem_desc(reg + a_off + (uint32_t)(2 * s) * (uint32_t)plane,
                                          (uint32_t)plane, 128);
            const uint64_t bd = smem_desc(wbase + tap * (NT * CIN * 2) + s * 256, 128,
                                          (CIN / 8) * 128);
            mma_bf16(tmem + (uint32_t)(bb * 64), ad, bd, idesc, (tap | s) != 0);
          }
        }
        mma_commit(&mma_done[bb]);
        last_mma[bb] = it;
      }
    }
    if (it >= 1) epilogue(it - 1);
    // a failed wait of thread 0 stops its whole warp at the same point (the
    // epilogue's TMEM loads are warp-collective)
    ok = __all_sync(0xffffffffu, ok);
  }
  if (my_tiles > 0 && ok) epilogue(my_tiles - 1);
  // clean-up: nothing may still be writing shared memory or TMEM when the CTA
  // ends — wait (bounded) for the last TMA copies and MMAs issued per buffer
  if (tid == 0) {
    for (int b = 0; b < 2; ++b) {
      if (last_x[b] >= 0) mbar_wait(&full_x[b], (uint32_t)(last_x[b] >> 1) & 1u);
      if (last_r[b] >= 0) mbar_wait(&full_r[b], (uint32_t)(last_r[b] >> 1) & 1u);
      if (last_mma[b] >= 0) mbar_wait(&mma_done[b], (uint32_t)(last_mma[b] >> 1) & 1u);
    }
    if (!ok) atomicExch(a.err, 1);
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == 0) tmem_dealloc(tmem, 128);
}

// ---------------------------------------------------------------------------
struct WgradArgs {
  const bf16 *x;   // [B][H+2][W+2][64]
  const bf16 *dy;  // padded [B][H+2][W+2][NT]
  float *dwt;      // [9][64][NT] fp32 accumulators (dW transposed)
  int B, H, W;
  int chunks_per_cta;  // 64-pixel K chunks per CTA
  int *err;
};

template <int NT>
__global__ void __launch_bounds__(128) conv3x3_wgrad(WgradArgs a) {
  constexpr int kKC = 64;                        // pixels per K chunk
  constexpr int kABytes = kTM * kKC * 2;         // (tap,ci) x pixels
  constexpr int kBBytes = NT * kKC * 2;          // co x pixels
  constexpr int kStage = kABytes + kBBytes;
  extern __shared__ __align__(1024) uint8_t dsm[];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t s_tmem;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int H = a.H, W = a.W, hw = H * W;
  const long long npix = (long long)a.B * hw;
  const int mt = blockIdx.y;  // rows 128*mt .. : taps 2mt, 2mt+1
  const long long k_begin = (long long)blockIdx.x * a.chunks_per_cta * kKC;
  const long long k_lim = k_begin + (long long)a.chunks_per_cta * kKC;
  const long long k_end = npix < k_lim ? npix : k_lim;
  const int nchunks = (int)((k_end - k_begin + kKC - 1) / kKC);
  if (warp == 0) tmem_alloc(&s_tmem, NT < 32 ? 32 : NT);
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = s_tmem;
  const uint32_t idesc = idesc_bf16_f32(kTM, NT);
  uint32_t ph0 = 0u, ph1 = 0u;
  bool ok = true;
  for (int c = 0; c < nchunks; ++c) {
    const int st = c & 1;
    if (c >= 2) {
      if (!mbar_wait(&bar[st], st ? ph1 : ph0)) ok = false;
      if (st) ph1 ^= 1u; else ph0 ^= 1u;
    }
    uint8_t *sa = dsm + st * kStage;
    uint8_t *sb = sa + kABytes;
    const long long kb = k_begin + (long long)c * kKC;
    // A[(tl, ci)][k] = X[p_k + tap(2mt+tl)][ci]: each thread reads 8 channels of
    // one pixel and scatters them down the column k of rows ci..ci+7.
    for (int v = tid; v < 2 * kKC * 8; v += 128) {
      const int tl = v / (kKC * 8);
      const int rem = v % (kKC * 8);
      const int k = rem >> 3, ci0 = (rem & 7) * 8;
      const int tap = 2 * mt + tl;
      const long long p = kb + k;
      __align__(16) bf16 vals[8];
      if (tap < 9 && p < k_end) {
        const int b = (int)(p / hw), r2 = (int)(p % hw);
        const int y = r2 / W, xx = r2 % W;
        const int dy = tap / 3 - 1, dx = tap % 3 - 1;
        *reinterpret_cast<uint4 *>(vals) = *reinterpret_cast<const uint4 *>(
            a.x + pad_index(b, y + 1 + dy, xx + 1 + dx, H, W) * CIN + ci0);
      } else {
        *reinterpret_cast<uint4 *>(vals) = make_uint4(0, 0, 0, 0);
      }
#pragma unroll
      for (int i = 0; i < 8; ++i)
        *reinterpret_cast<bf16 *>(sa + kmajor_off(tl * 64 + ci0 + i, k, kKC)) = vals[i];
    }
    // B[co][k] = dY[p_k][co]
    for (int v = tid; v < kKC * (NT / 8); v += 128) {
      const int k = v / (NT / 8), co0 = (v % (NT / 8)) * 8;
      const long long p = kb + k;
      __align__(16) bf16 vals[8];
      if (p < k_end) {
        const int b = (int)(p / hw), r2 = (int)(p % hw);
        const int y = r2 / W, xx = r2 % W;
        *reinterpret_cast<uint4 *>(vals) = *reinterpret_cast<const uint4 *>(
            a.dy + pad_index(b, y + 1, xx + 1, H, W) * NT + co0);
      } else {
        *reinterpret_cast<uint4 *>(vals) = make_uint4(0, 0, 0, 0);
      }
#pragma unroll
      for (int i = 0; i < 8; ++i)
        *reinterpret_cast<bf16 *>(sb + kmajor_off(co0 + i, k, kKC)) = vals[i];
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      fence_after_sync();
      const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
#pragma unroll
      for (int s = 0; s < kKC / 16; ++s)
        mma_bf16(tmem, smem_desc(a0 + s * 256, 128, (kKC / 8) * 128),
                 smem_desc(b0 + s * 256, 128, (kKC / 8) * 128), idesc, (c | s) != 0);
      mma_commit(&bar[st]);
    }
  }
  // wait for the outstanding chunks
  if (nchunks >= 2) {
    const int s_last = (nchunks - 1) & 1, s_prev = (nchunks - 2) & 1;
    if (!mbar_wait(&bar[s_prev], s_prev ? ph1 : ph0)) ok = false;
    if (s_prev) ph1 ^= 1u; else ph0 ^= 1u;
    if (!mbar_wait(&bar[s_last], s_last ? ph1 : ph0)) ok = false;
  } else if (nchunks == 1) {
    if (!mbar_wait(&bar[0], ph0)) ok = false;
  }
  fence_after_sync();
  if (ok && nchunks > 0) {
    const int row = warp * 32 + (tid & 31);  // (tl, ci)
    const int tap = 2 * mt + (row >> 6), ci = row & 63;
#pragma unroll
    for (int c0 = 0; c0 < NT; c0 += 16) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (tap < 9) {
        float *dst = a.dwt + ((size_t)tap * 64 + ci) * NT + c0;
#pragma unroll
        for (int i = 0; i < 16; ++i) atomicAdd(dst + i, v[i]);
      }
    }
  } else if (!ok) {
    if (tid == 0) atomicExch(a.err, 1);
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, NT < 32 ? 32 : NT);
}

template <int NT>
int launch_fwd(const ConvArgs &a, cudaStream_t s) {
  const int smem = 2 * (kTM * CIN * 2 + NT * CIN * 2);
  FM_TRY_CUDA(cudaFuncSetAttribute(conv3x3_fwd<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   smem));
  const long long npix = (long long)a.B * a.H * a.W;
  conv3x3_fwd<NT><<<(unsigned)(npix / kTM), 128, smem, s>>>(a);
  FM_TRY_CUDA(cudaGetLastError());
  return FM_OK;
}

template <int NT>
int launch_wgrad(WgradArgs a, cudaStream_t s) {
  const int smem = 2 * (kTM * 64 * 2 + NT * 64 * 2);
  FM_TRY_CUDA(cudaFuncSetAttribute(conv3x3_wgrad<NT>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  int sms = 0;
  int st = fm::device_sm_count(&sms);
  if (st) return st;
  const long long npix = (long long)a.B * a.H * a.W;
  const long long nch = (npix + 63) / 64;
  // about 4 CTAs per SM over the 5 row tiles
  const long long want = std::max<long long>(1, (long long)sms * 4 / 5);
  a.chunks_per_cta = (int)std::max<long long>(1, (nch + want - 1) / want);
  const long long gx = (nch + a.chunks_per_cta - 1) / a.chunks_per_cta;
  conv3x3_wgrad<NT><<<dim3((unsigned)gx, 5), 128, smem, s>>>(a);
  FM_TRY_CUDA(cudaGetLastError());
  return FM_OK;
}

}  // namespace

namespace {
int launch_fwd_res(const ConvArgs &a, cudaStream_t s) {
  const int Wp = a.W + 2;
  const int rlen = res_region_len(Wp);
  const int plane = ((rlen * 16 + 127) / 128) * 128;
  const size_t smem = (size_t)9 * 64 * CIN * 2 + 2 * 8 * (size_t)plane +
                      (a.resid ? 3 * (size_t)kTM * 64 * 2 : 0);
  int dev = 0, optin = 0;
  FM_TRY_CUDA(cudaGetDevice(&dev));
  FM_TRY_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (smem > (size_t)optin || plane / 16 >= (1 << 14)) return FM_ERR_UNSUPPORTED;
  FM_TRY_CUDA(cudaFuncSetAttribute(conv3x3_fwd_res, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
  int sms = 0;
  int st = fm::device_sm_count(&sms);
  if (st) return st;
  // positions Wp+1 .. (H+1)*Wp - 2 of each padded image hold every interior cell
  const long long span = (long long)a.H * Wp - 2;
  const int ntile_img = (int)((span + kTM - 1) / kTM);
  const long long ntiles = (long long)ntile_img * a.B;
  if (ntiles > (1ll << 30)) return FM_ERR_UNSUPPORTED;
  const int grid = (int)std::min<long long>(ntiles, sms);
  conv3x3_fwd_res<<<grid, kResThreads, smem, s>>>(a, ntile_img, (int)ntiles, plane);
  FM_TRY_CUDA(cudaGetLastError());
  return FM_OK;
}
}  // namespace

namespace {
// cuTensorMapEncodeTiled through the runtime's driver entry point (no -lcuda)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
  }
  return fn;
}

// A 3D tiled tensor map over a padded NHWC bf16 tensor viewed as
// [B][(H+2)*(W+2) positions][64 channels]; box = {bc channels, bp positions, 1}.
bool encode_positions_map_uncached(CUtensorMap *m, const void *base, long long img, int B, int bc,
                                   int bp, bool swizzle128) {
  auto enc = tensor_map_encoder();
  if (!enc || ((uintptr_t)base & 15u)) return false;
  cuuint64_t dims[3] = {64, (cuuint64_t)img, (cuuint64_t)B};
  cuuint64_t strides[2] = {128, (cuuint64_t)img * 128};
  cuuint32_t box[3] = {(cuuint32_t)bc, (cuuint32_t)bp, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void *>(base), dims, strides, box,
             estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The encoded maps of recent (buffer, shape, box) combinations: a network step
// runs the same layers on the same buffers, and encoding costs microseconds of
// host time per map.
bool encode_positions_map(CUtensorMap *m, const void *base, long long img, int B, int bc, int bp,
                          bool swizzle128) {
  struct Entry {
    const void *base;
    long long img;
    int B, bc, bp;
    bool sw;
    CUtensorMap map;
  };
  constexpr int kEntries = 64;
  static Entry cache[kEntries];
  static int used = 0, next = 0;
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  for (int i = 0; i < used; ++i) {
    const Entry &e = cache[i];
    if (e.base == base && e.img == img && e.B == B && e.bc == bc && e.bp == bp && e.sw == swizzle128) {
      *m = e.map;
      return true;
    }
  }
  if (!encode_positions_map_uncached(m, base, img, B, bc, bp, swizzle128)) return false;
  Entry &e = cache[next];
  e = Entry{base, img, B, bc, bp, swizzle128, *m};
  next = (next + 1) % kEntries;
  used = used < kEntries ? used + 1 : kEntries;
  return true;
}

int launch_fwd_tma(const ConvArgs &a, cudaStream_t s) {
  const int Wp = a.W + 2;
  const int rlen = res_region_len(Wp);
  const int r1 = std::min(rlen, 192);  // first box: a multiple of 8 positions (128-byte aligned)
  if (rlen - r1 > 256) return FM_ERR_UNSUPPORTED;
  const int plane = ((rlen * 16 + 127) / 128) * 128;
  const size_t smem = (((size_t)9 * 64 * CIN * 2 + 16 * (size_t)plane + 1023) & ~(size_t)1023) +
                      2 * (size_t)kTM * 64 * 2;
  int dev = 0, optin = 0;
  FM_TRY_CUDA(cudaGetDevice(&dev));
  FM_TRY_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (smem > (size_t)optin) return FM_ERR_UNSUPPORTED;
  const long long img = (long long)(a.H + 2) * Wp;
  CUtensorMap tx1, tx2, tr;
  if (!encode_positions_map(&tx1, a.x, img, a.B, 8, r1, false)) return FM_ERR_UNSUPPORTED;
  if (!encode_positions_map(&tx2, a.x, img, a.B, 8, rlen > r1 ? rlen - r1 : 8, false))
    return FM_ERR_UNSUPPORTED;
  tr = tx1;
  if (a.resid && !encode_positions_map(&tr, a.resid, img, a.B, 64, kTM, true))
    return FM_ERR_UNSUPPORTED;
  FM_TRY_CUDA(cudaFuncSetAttribute(conv3x3_fwd_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
  int sms = 0;
  int st = fm::device_sm_count(&sms);
  if (st) return st;
  const long long span = (long long)a.H * Wp - 2;
  const int ntile_img = (int)((span + kTM - 1) / kTM);
  const long long ntiles = (long long)ntile_img * a.B;
  if (ntiles > (1ll << 30) || img * (long long)a.B > (1ll << 31)) return FM_ERR_UNSUPPORTED;
  const int grid = (int)std::min<long long>(ntiles, sms);
  conv3x3_fwd_tma<<<grid, kResThreads, smem, s>>>(a, ntile_img, (int)ntiles, plane, rlen, r1, tx1,
                                                  tx2, tr);
  FM_TRY_CUDA(cudaGetLastError());
  return FM_OK;
}
}  // namespace

extern "C" int fm_conv3x3_fwd_bf16(int B, int H, int W, int cout, const void *x_pad,
                                   const void *w, const float *bias, const void *gate_pad,
                                   const void *resid_pad, int act, void *z_pad_out,
                                   void *y_pad_out, float *y_f32_out, int *err_device,
                                   void *stream) {
  FM_CHECK_ARG(x_pad && w && err_device, "fm_conv3x3_fwd_bf16: NULL input");
  FM_CHECK_ARG(B >= 1 && H >= 2 && W >= 2, "fm_conv3x3_fwd_bf16: need H, W >= 2");
  FM_CHECK_ARG(cout == 32 || cout == 64, "fm_conv3x3_fwd_bf16: cout must be 32 or 64");
  FM_CHECK_ARG(act == 0 || act == 1, "fm_conv3x3_fwd_bf16: act must be 0 or 1");
  FM_CHECK_ARG(z_pad_out || y_pad_out || y_f32_out, "fm_conv3x3_fwd_bf16: no output");
  ConvArgs a;
  a.x = (const bf16 *)x_pad;
  a.w = (const bf16 *)w;
  a.bias = bias;
  a.gate = (const bf16 *)gate_pad;
  a.resid = (const bf16 *)resid_pad;
  a.z_out = (bf16 *)z_pad_out;
  a.y_out = (bf16 *)y_pad_out;
  a.y_f32 = y_f32_out;
  a.B = B;
  a.H = H;
  a.W = W;
  a.act = act;
  a.err = err_device;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int kern = fm::tune_get("conv.kernel", 1);
  if (cout == 64 && kern == 2) {
    const int st = launch_fwd_tma(a, s);
    if (st != FM_ERR_UNSUPPORTED) return st;
  }
  if (cout == 64 && kern >= 1) {
    const int st = launch_fwd_res(a, s);
    if (st != FM_ERR_UNSUPPORTED) return st;
  }
  FM_CHECK_ARG(((long long)B * H * W) % kTM == 0,
               "fm_conv3x3_fwd_bf16: this shape needs B*H*W %% 128 == 0 (got %d*%d*%d)", B, H, W);
  return cout == 64 ? launch_fwd<64>(a, s) : launch_fwd<32>(a, s);
}

extern "C" int fm_conv3x3_wgrad_bf16(int B, int H, int W, int cout, const void *x_pad,
                                     const void *dy_pad, float *dwt, int *err_device,
                                     void *stream) {
  FM_CHECK_ARG(x_pad && dy_pad && dwt && err_device, "fm_conv3x3_wgrad_bf16: NULL input");
  FM_CHECK_ARG(B >= 1 && H >= 2 && W >= 2, "fm_conv3x3_wgrad_bf16: need H, W >= 2");
  FM_CHECK_ARG(cout == 32 || cout == 64, "fm_conv3x3_wgrad_bf16: cout must be 32 or 64");
  WgradArgs a;
  a.x = (const bf16 *)x_pad;
  a.dy = (const bf16 *)dy_pad;
  a.dwt = dwt;
  a.B = B;
  a.H = H;
  a.W = W;
  a.chunks_per_cta = 1;
  a.err = err_device;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  return cout == 64 ? launch_wgrad<64>(a, s) : launch_wgrad<32>(a, s);
}
