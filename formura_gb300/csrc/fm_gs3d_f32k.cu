// fm_gs3d_f32k.cu — 3D Gray-Scott (examples/pearson-3d.fmr form) in binary32
// with compensated (Kahan) time accumulation.
//
// Same per-cell DAG and operation order as the FP64 kernel, in float; the
// time update of each field is the Kahan sum
//     y = dt*dW - cW;  t = W + y;  cW' = (t - W) - y;  W' = t
// so that the O(1e-7) rounding of each increment does not pile up over
// thousands of steps.  State per cell: U, V, cU, cV (16 B).
//
// One step per launch, x-marching with register blocking along y and
// shuffles along z, like the FP64 kernel.  The temporally blocked kernel of
// the binary32 fast form is in fm_gs3d_f32k_tb.cu.
#include <algorithm>

#include "fm_common.cuh"

namespace {

using fm::div_const_f;

struct Gs32 {
  float F, Fk, Du, Dv, dt, dx, rdx;
};

// ---------------------------------------------------------------- tb = 1 --
constexpr int kWarps = 4;
constexpr int kRY = 2;
constexpr int kTY = kWarps * kRY;

__device__ __forceinline__ void kahan(float w, float dw, float cw, float dt, float &wn,
                                      float &cn) {
  const float y = dt * dw - cw;
  const float t = w + y;
  cn = (t - w) - y;
  wn = t;
}

__global__ void __launch_bounds__(kWarps * 32)
    gs3d_f32k_step(const float *__restrict__ U, const float *__restrict__ V,
                   const float *__restrict__ cU, const float *__restrict__ cV,
                   float *__restrict__ Un, float *__restrict__ Vn, float *__restrict__ cUn,
                   float *__restrict__ cVn, int nx, int ny, int nz, int xchunk,
                   int ntiles_yz, int ntiles, Gs32 c) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nzt = nz >> 5;
  const size_t sx = (size_t)ny * nz;
  const float dx = c.dx, rdx = c.rdx;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int tyz = t % ntiles_yz;
    const int tx = t / ntiles_yz;
    const int z = (tyz % nzt) * 32 + lane;
    const int y0 = (tyz / nzt) * kTY + warp * kRY;
    const int x0 = tx * xchunk;
    const int x1 = min(x0 + xchunk, nx);
    const int zm = fm::wrap_dn(z, nz), zp = fm::wrap_up(z, nz);
    int off[kRY];
#pragma unroll
    for (int j = 0; j < kRY; ++j) off[j] = (y0 + j) * nz + z;
    const int off_ym = fm::wrap_dn(y0, ny) * nz + z;
    const int off_yp = fm::wrap_up(y0 + kRY - 1, ny) * nz + z;
    float uc[kRY], vc[kRY], fxu[kRY], fxv[kRY];
    {
      const size_t pm = (size_t)fm::wrap_dn(x0, nx) * sx, pc = (size_t)x0 * sx;
#pragma unroll
      for (int j = 0; j < kRY; ++j) {
        const float um = __ldg(U + pm + off[j]), vm = __ldg(V + pm + off[j]);
        uc[j] = __ldg(U + pc + off[j]);
        vc[j] = __ldg(V + pc + off[j]);
        fxu[j] = div_const_f(uc[j] - um, dx, rdx);
        fxv[j] = div_const_f(vc[j] - vm, dx, rdx);
      }
    }
    for (int x = x0; x < x1; ++x) {
      const size_t pc = (size_t)x * sx;
      const size_t pp = (size_t)fm::wrap_up(x, nx) * sx;
      float up[kRY], vp[kRY];
#pragma unroll
      for (int j = 0; j < kRY; ++j) {
        up[j] = __ldg(U + pp + off[j]);
        vp[j] = __ldg(V + pp + off[j]);
      }
      float fyu[kRY + 1], fyv[kRY + 1];
      {
        const float um = __ldg(U + pc + off_ym), vm = __ldg(V + pc + off_ym);
        const float upp = __ldg(U + pc + off_yp), vpp = __ldg(V + pc + off_yp);
        fyu[0] = div_const_f(uc[0] - um, dx, rdx);
        fyv[0] = div_const_f(vc[0] - vm, dx, rdx);
#pragma unroll
        for (int j = 1; j < kRY; ++j) {
          fyu[j] = div_const_f(uc[j] - uc[j - 1], dx, rdx);
          fyv[j] = div_const_f(vc[j] - vc[j - 1], dx, rdx);
        }
        fyu[kRY] = div_const_f(upp - uc[kRY - 1], dx, rdx);
        fyv[kRY] = div_const_f(vpp - vc[kRY - 1], dx, rdx);
      }
#pragma unroll
      for (int j = 0; j < kRY; ++j) {
        const float u = uc[j], v = vc[j];
        float uzm = __shfl_up_sync(0xffffffffu, u, 1);
        float vzm = __shfl_up_sync(0xffffffffu, v, 1);
        if (lane == 0) {
          uzm = __ldg(U + pc + (size_t)(y0 + j) * nz + zm);
          vzm = __ldg(V + pc + (size_t)(y0 + j) * nz + zm);
        }
        const float fzu_m = div_const_f(u - uzm, dx, rdx);
        const float fzv_m = div_const_f(v - vzm, dx, rdx);
        float fzu_p = __shfl_down_sync(0xffffffffu, fzu_m, 1);
        float fzv_p = __shfl_down_sync(0xffffffffu, fzv_m, 1);
        if (lane == 31) {
          fzu_p = div_const_f(__ldg(U + pc + (size_t)(y0 + j) * nz + zp) - u, dx, rdx);
          fzv_p = div_const_f(__ldg(V + pc + (size_t)(y0 + j) * nz + zp) - v, dx, rdx);
        }
        const float fxu_p = div_const_f(up[j] - u, dx, rdx);
        const float fxv_p = div_const_f(vp[j] - v, dx, rdx);
        const float a_2 = (u * v) * v;
        const float a_7 = (-a_2) + c.F * (1.0f - u);
        const float lx = div_const_f(fxu_p - fxu[j], dx, rdx);
        const float ly = div_const_f(fyu[j + 1] - fyu[j], dx, rdx);
        const float lz = div_const_f(fzu_p - fzu_m, dx, rdx);
        const float dU = a_7 + c.Du * ((lx + ly) + lz);
        const float b_6 = a_2 - c.Fk * v;
        const float mx = div_const_f(fxv_p - fxv[j], dx, rdx);
        const float my = div_const_f(fyv[j + 1] - fyv[j], dx, rdx);
        const float mz = div_const_f(fzv_p - fzv_m, dx, rdx);
        const float dV = b_6 + c.Dv * ((mx + my) + mz);
        float un, cun, vn, cvn;
        kahan(u, dU, __ldg(cU + pc + off[j]), c.dt, un, cun);
        kahan(v, dV, __ldg(cV + pc + off[j]), c.dt, vn, cvn);
        Un[pc + off[j]] = un;
        cUn[pc + off[j]] = cun;
        Vn[pc + off[j]] = vn;
        cVn[pc + off[j]] = cvn;
        fxu[j] = fxu_p;
        fxv[j] = fxv_p;
        uc[j] = up[j];
        vc[j] = vp[j];
      }
    }
  }
}

int plan_step(int nx, int ny, int nz, int *xchunk, int *ntiles_yz, int *ntiles, int *grid) {
  int sms = 0;
  int st = fm::device_sm_count(&sms);
  if (st) return st;
  int per_sm = 0;
  FM_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gs3d_f32k_step,
                                                             kWarps * 32, 0));
  if (per_sm < 1) per_sm = 1;
  const int resident = sms * per_sm;
  const int nyz = (nz / 32) * (ny / kTY);
  double best = 1e300;
  int bx = 1;
  for (int xc : {1, 2, 4, 8, 16, 32}) {
    if (xc > nx) break;
    const long long nt = (long long)nyz * ((nx + xc - 1) / xc);
    const double cost = (double)((nt + resident - 1) / resident) * (xc + 0.5);
    if (cost < best - 1e-9) {
      best = cost;
      bx = xc;
    }
  }
  *xchunk = bx;
  *ntiles_yz = nyz;
  *ntiles = nyz * ((nx + bx - 1) / bx);
  *grid = std::min(*ntiles, resident);
  return FM_OK;
}

}  // namespace

extern "C" int fm_gs3d_f32k_forward(int nx, int ny, int nz, float *U, float *V, float *cU,
                                    float *cV, float *work, int steps, const fm_gs_params *p,
                                    void *stream) {
  FM_CHECK_ARG(p && U && V && cU && cV && work, "fm_gs3d_f32k_forward: NULL argument");
  FM_CHECK_ARG(nx >= 1 && nz >= 32 && nz % 32 == 0 && ny >= kTY && ny % kTY == 0,
               "fm_gs3d_f32k_forward: need nz %% 32 == 0 and ny %% %d == 0 (got %d,%d,%d)",
               kTY, nx, ny, nz);
  FM_CHECK_ARG((long long)ny * nz < (1ll << 31), "fm_gs3d_f32k_forward: plane too large");
  FM_CHECK_ARG(steps >= 0, "fm_gs3d_f32k_forward: steps < 0");
  const float dxf = (float)p->dx;
  FM_CHECK_ARG(dxf >= 0x1p-20f && dxf <= 0x1p20f,
               "fm_gs3d_f32k_forward: dx outside [2^-20, 2^20]");
  if (steps == 0) return FM_OK;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  Gs32 c;
  c.F = (float)p->F;
  c.Fk = c.F + (float)p->k;
  c.Du = (float)p->Du;
  c.Dv = (float)p->Dv;
  c.dt = (float)p->dt;
  c.dx = dxf;
  c.rdx = 1.0f / dxf;
  const size_t n = (size_t)nx * ny * nz;
  float *cur[4] = {U, V, cU, cV};
  float *nxt[4] = {work, work + n, work + 2 * n, work + 3 * n};
  int xchunk, nyz, nt, grid;
  int st = plan_step(nx, ny, nz, &xchunk, &nyz, &nt, &grid);
  if (st) return st;
  for (int i = 0; i < steps; ++i) {
    gs3d_f32k_step<<<grid, kWarps * 32, 0, s>>>(cur[0], cur[1], cur[2], cur[3], nxt[0],
                                                nxt[1], nxt[2], nxt[3], nx, ny, nz, xchunk,
                                                nyz, nt, c);
    for (int k = 0; k < 4; ++k) std::swap(cur[k], nxt[k]);
  }
  FM_TRY_CUDA(cudaGetLastError());
  if (cur[0] != U) {
    float *dst[4] = {U, V, cU, cV};
    for (int k = 0; k < 4; ++k)
      FM_TRY_CUDA(cudaMemcpyAsync(dst[k], cur[k], n * sizeof(float),
                                  cudaMemcpyDeviceToDevice, s));
  }
  return FM_OK;
}
