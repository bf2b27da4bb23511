// fm_surrogate.cu — the non-convolution kernels of the learned 16-step
// surrogate of 2D Gray-Scott: packing the state into the network's latent
// grid, unpacking its prediction, the training loss gradient, bias gradients,
// the weight flip used by data gradients, and Adam.
//
// Latent layout: a periodic N x N field is folded 4x4 into an (N/4) x (N/4)
// grid of 64 channels (space-to-depth): channel c = q*16 + (sy*4 + sx) holds
// quantity q at sub-pixel (sy, sx); inputs q = U, V, F', k' (F' = (F-0.04)*50,
// k' = (k-0.06)*100), outputs q = dU, dV (channels 0..31; 32..63 unused).
// Latent tensors are NHWC bf16 with a one-pixel periodic halo.
#include <cuda_bf16.h>

#include "fm_common.cuh"

namespace {

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ size_t pidx(int b, int py, int px, int n) {
  return ((size_t)b * (n + 2) + py) * (n + 2) + px;
}

// One thread per (instance, latent pixel incl. halo, channel group of 16).
__global__ void sur_pack(const float *__restrict__ U, const float *__restrict__ V,
                         const float *__restrict__ F, const float *__restrict__ K, bf16 *xpad,
                         int B, int N) {
  const int n = N / 4;
  const long long total = (long long)B * (n + 2) * (n + 2) * 4;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int q = (int)(i & 3);
  long long r = i >> 2;
  const int px = (int)(r % (n + 2));
  r /= (n + 2);
  const int py = (int)(r % (n + 2));
  const int b = (int)(r / (n + 2));
  const int ly = (py - 1 + n) % n, lx = (px - 1 + n) % n;  // halo wraps periodically
  __align__(16) bf16 v[16];
  for (int sub = 0; sub < 16; ++sub) {
    const int y = ly * 4 + sub / 4, x = lx * 4 + sub % 4;
    float val;
    if (q == 0) val = U[((size_t)b * N + y) * N + x];
    else if (q == 1) val = V[((size_t)b * N + y) * N + x];
    else if (q == 2) val = (F[b] - 0.04f) * 50.0f;
    else val = (K[b] - 0.06f) * 100.0f;
    v[sub] = __float2bfloat16_rn(val);
  }
  uint4 *dst = reinterpret_cast<uint4 *>(xpad + pidx(b, py, px, n) * 64 + q * 16);
  dst[0] = reinterpret_cast<const uint4 *>(v)[0];
  dst[1] = reinterpret_cast<const uint4 *>(v)[1];
}

// state += scale * latent prediction (channels 0..15 -> dU, 16..31 -> dV)
__global__ void sur_unpack(const float *__restrict__ y, float *U, float *V, int B, int N,
                           float scale) {
  const long long total = (long long)B * N * N;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int x = (int)(i % N), yy = (int)((i / N) % N), b = (int)(i / ((long long)N * N));
  const int n = N / 4;
  const size_t lp = ((size_t)b * n + yy / 4) * n + x / 4;
  const int sub = (yy % 4) * 4 + (x % 4);
  U[i] += scale * y[lp * 64 + sub];
  V[i] += scale * y[lp * 64 + 16 + sub];
}

// MSE on the latent increments: target t = (S_target - S_in)/scale.
// Writes dL/dy (bf16, padded, halo filled, channels 32..63 = 0) and adds the
// per-block loss partials into *loss.
__global__ void sur_loss_grad(const float *__restrict__ y, const float *__restrict__ U0,
                              const float *__restrict__ V0, const float *__restrict__ U1,
                              const float *__restrict__ V1, bf16 *dy_pad, float *loss, int B,
                              int N, float scale, float grad_scale) {
  __shared__ float sh[256];
  const int n = N / 4;
  const long long total = (long long)B * (n + 2) * (n + 2);
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float acc = 0.0f;
  if (i < total) {
    const int px = (int)(i % (n + 2)), py = (int)((i / (n + 2)) % (n + 2));
    const int b = (int)(i / ((long long)(n + 2) * (n + 2)));
    const int ly = (py - 1 + n) % n, lx = (px - 1 + n) % n;
    const bool interior = px >= 1 && px <= n && py >= 1 && py <= n;
    const size_t lp = ((size_t)b * n + ly) * n + lx;
    __align__(16) bf16 g[64];
    for (int c = 0; c < 32; ++c) {
      const int sub = c & 15;
      const int yy = ly * 4 + sub / 4, x = lx * 4 + sub % 4;
      const size_t s = ((size_t)b * N + yy) * N + x;
      const float t = (c < 16 ? (U1[s] - U0[s]) : (V1[s] - V0[s])) / scale;
      const float d = y[lp * 64 + c] - t;
      if (interior) acc += d * d;
      g[c] = __float2bfloat16_rn(grad_scale * 2.0f * d);
    }
    for (int c = 32; c < 64; ++c) g[c] = __float2bfloat16_rn(0.0f);
    uint4 *dst = reinterpret_cast<uint4 *>(dy_pad + pidx(b, py, px, n) * 64);
    for (int k = 0; k < 8; ++k) dst[k] = reinterpret_cast<const uint4 *>(g)[k];
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(loss, sh[0]);
}

// db[c] += sum over interior pixels of dy[p][c]
__global__ void sur_bias_grad(const bf16 *__restrict__ dy_pad, float *db, int B, int n) {
  __shared__ float sh[4][64];
  const int c = threadIdx.x & 63, part = threadIdx.x >> 6;  // 256 threads = 4 x 64
  const long long total = (long long)B * n * n;
  float acc = 0.0f;
  for (long long p = (long long)blockIdx.x * 4 + part; p < total; p += (long long)gridDim.x * 4) {
    const int x = (int)(p % n), y = (int)((p / n) % n), b = (int)(p / ((long long)n * n));
    acc += __bfloat162float(dy_pad[pidx(b, y + 1, x + 1, n) * 64 + c]);
  }
  sh[part][c] = acc;
  __syncthreads();
  if (part == 0) atomicAdd(db + c, sh[0][c] + sh[1][c] + sh[2][c] + sh[3][c]);
}

// W'[ci][t][co] = W[co][8-t][ci]: the weights of the data gradient as a
// forward convolution (tap t' = -t).
__global__ void sur_flip(const bf16 *__restrict__ w, bf16 *wf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 64 * 9 * 64) return;
  const int co = i % 64, t = (i / 64) % 9, ci = i / (64 * 9);
  wf[i] = w[((size_t)co * 9 + (8 - t)) * 64 + ci];
}

// Adam on fp32 master weights [64][9][64] with gradient dWt[9][ci][co];
// `mask_co` >= 0 freezes output channels >= mask_co at zero.  Writes the bf16
// copy used by the convolutions.
__global__ void sur_adam_w(float *w, const float *__restrict__ gwt, float *m, float *v, bf16 *wb,
                           float lr, float b1, float b2, float eps, float c1, float c2,
                           int mask_co) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 64 * 9 * 64) return;
  const int ci = i % 64, t = (i / 64) % 9, co = i / (64 * 9);
  if (mask_co >= 0 && co >= mask_co) {
    w[i] = 0.0f;
    wb[i] = __float2bfloat16_rn(0.0f);
    return;
  }
  const float g = gwt[((size_t)t * 64 + ci) * 64 + co];
  const float mm = b1 * m[i] + (1.0f - b1) * g;
  const float vv = b2 * v[i] + (1.0f - b2) * g * g;
  m[i] = mm;
  v[i] = vv;
  const float nw = w[i] - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
  w[i] = nw;
  wb[i] = __float2bfloat16_rn(nw);
}

__global__ void sur_adam_b(float *bb, const float *__restrict__ g, float *m, float *v, float lr,
                           float b1, float b2, float eps, float c1, float c2, int mask_co) {
  const int i = threadIdx.x;
  if (i >= 64) return;
  if (mask_co >= 0 && i >= mask_co) {
    bb[i] = 0.0f;
    return;
  }
  const float mm = b1 * m[i] + (1.0f - b1) * g[i];
  const float vv = b2 * v[i] + (1.0f - b2) * g[i] * g[i];
  m[i] = mm;
  v[i] = vv;
  bb[i] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
}

__global__ void sur_gelu_bwd(long long count, const bf16 *__restrict__ dh,
                             const bf16 *__restrict__ z, bf16 *dz) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float x = __bfloat162float(z[i]);
  const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * __expf(-0.5f * x * x);
  dz[i] = __float2bfloat16_rn(__bfloat162float(dh[i]) * (cdf + x * pdf));
}

unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

extern "C" int fm_sur_pack(int B, int N, const float *U, const float *V, const float *F,
                           const float *K, void *xpad, void *stream) {
  FM_CHECK_ARG(U && V && F && K && xpad && B >= 1 && N >= 4 && N % 4 == 0,
               "fm_sur_pack: bad arguments (N must be a multiple of 4)");
  const int n = N / 4;
  const long long total = (long long)B * (n + 2) * (n + 2) * 4;
  sur_pack<<<blocks_for(total, 256), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      U, V, F, K, (bf16 *)xpad, B, N);
  FM_TRY_CUDA(cudaGetLastError());
  return FM_OK;
}

extern "C" int fm_sur_unpack(int B, int N, const float *y, float *U, float *V, float scale,
                             void *stream) {
  FM_CHECK_ARG(y && U && V && B >= 1 && N % 4 == 0, "fm_sur_unpack: bad arguments");
  sur_unpack<<<blocks_for((long long)B * N * N, 256), 256, 0,
               reinterpret_cast<cudaStream_t>(stream)>>>(y, U, V, B, N, scale);
  FM_TRY_CUDA(cudaGetLastError());
  return FM_OK;
}

extern "C" int fm_sur_loss_grad(int B, int N, const float *y, const float *U0, const float *V0,
                                const float *U1, const float *V1, void *dy_pad, float *loss,
                                float scale, float grad_scale, void *stream) {
  FM_CHECK_ARG(y && U0 && V0 && U1 && V1 && dy_pad && loss && N % 4 == 0,
               "fm_sur_loss_grad: bad arguments");
  const int n = N / 4;
  sur_loss_grad<<<blocks_for((long long)B * (n + 2) * (n + 2), 256), 256, 0,
                  reinterpret_cast<cudaStream_t>(stream)>>>(y, U0, V0, U1, V1, (bf16 *)dy_pad,
                                                            loss, B, N, scale, grad_scale);
  FM_TRY_CUDA(cudaGetLastError());
  return FM_OK;
}

extern "C" int fm_sur_bias_grad(int B, int n, const void *dy_pad, float *db, void *stream) {
  FM_CHECK_ARG(dy_pad && db && B >= 1 && n >= 1, "fm_sur_bias_grad: bad arguments");
  sur_bias_grad<<<512, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>((const bf16 *)dy_pad,
                                                                          db, B, n);
  FM_TRY_CUDA(cudaGetLastError());
  return FM_OK;
}

extern "C" int fm_sur_flip(const void *w, void *wf, void *stream) {
  FM_CHECK_ARG(w && wf, "fm_sur_flip: NULL");
  sur_flip<<<blocks_for(64 * 9 * 64, 256), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      (const bf16 *)w, (bf16 *)wf);
  FM_TRY_CUDA(cudaGetLastError());
  return FM_OK;
}

extern "C" int fm_sur_adam(float *w, const float *gwt, float *mw, float *vw, void *wb, float *b,
                           const float *gb, float *mb, float *vb, float lr, float b1, float b2,
                           float eps, int step, int mask_co, void *stream) {
  FM_CHECK_ARG(w && gwt && mw && vw && wb && b && gb && mb && vb && step >= 1,
               "fm_sur_adam: bad arguments");
  const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  sur_adam_w<<<blocks_for(64 * 9 * 64, 256), 256, 0, s>>>(w, gwt, mw, vw, (bf16 *)wb, lr, b1, b2,
                                                           eps, c1, c2, mask_co);
  sur_adam_b<<<1, 64, 0, s>>>(b, gb, mb, vb, lr, b1, b2, eps, c1, c2, mask_co);
  FM_TRY_CUDA(cudaGetLastError());
  return FM_OK;
}

extern "C" int fm_sur_gelu_bwd(long long count, const void *dh, const void *z, void *dz,
                               void *stream) {
  FM_CHECK_ARG(dh && z && dz && count >= 0, "fm_sur_gelu_bwd: bad arguments");
  if (count == 0) return FM_OK;
  sur_gelu_bwd<<<blocks_for(count, 256), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      count, (const bf16 *)dh, (const bf16 *)z, (bf16 *)dz);
  FM_TRY_CUDA(cudaGetLastError());
  return FM_OK;
}
