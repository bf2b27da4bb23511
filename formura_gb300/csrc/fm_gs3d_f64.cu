// fm_gs3d_f64.cu — 3D Gray-Scott (examples/pearson-3d.fmr form), FP64,
// bit-exact with the generated loop nest.
//
// The generated C evaluates, per cell, the whole U_next / V_next DAG with the
// half-point differences recomputed at every use (Manifestation inlines the
// delayed ddx node, src/Formura/OrthotopeMachine/Manifestation.hs:115-143).
// A recomputed IEEE expression has the same value, so these kernels compute
// each face flux (W[i+1]-W[i])/dx once and hand it to both cells that use it:
//   x (slowest axis): the CTA marches along x; the flux at x-1/2 is carried in
//                     registers from the previous plane.
//   y:                each thread owns RY consecutive y cells of one z column;
//                     RY+1 fluxes serve RY cells.
//   z (fastest axis): lanes of a warp are consecutive z; the flux at z+1/2 is
//                     the next lane's z-1/2 flux (warp shuffle).  Lane 31 takes
//                     it from the next warp through shared memory when the CTA
//                     spans the whole periodic z row (gs3d_f64_row), or
//                     computes it itself (gs3d_f64_tile, any nz).
//
// On GB300 the FP64 pipe (2 lanes/clk/SM), not HBM, bounds these kernels:
// the ~45 FP64 operations of one cell update take ~20x longer than moving its
// 32 bytes.  Divisions by dx are the bulk of it; four exact methods exist:
//   DIV = 0  fm::div_const   — Markstein: 1 DMUL + 2 DFMA
//   DIV = 1  fm::div_const_i — 1 DMUL, then the rounding decided with 128-bit
//                              integer products on the integer pipe (10.9
//                              GLUP/s at 256^3 against 6.2 for DIV = 0)
//   DIV = 2  fm::div_const_r — 1 DMUL + 1 DFMA (exact residual), rounding
//                              decided by integer compares of bit patterns.
//   DIV = 3  fm::soft::div_const_s — no FP64 instruction: the quotient
//                              significand from 32-bit partial products with
//                              a reciprocal prepared on the host, the rounding
//                              from the sign of an exact 64-bit remainder
//                              (default; 15.2 GLUP/s alone).
// With DIV = 3, MUL moves multiplications to the integer pipes as well
// (fm::soft::mul_const_s / mul_s): MUL = 1 the five multiplications by a
// constant (F, F+k, Du, Dv, dt) — the default, 18.0 GLUP/s — and MUL = 2
// also U*V and (U*V)*V (17.6: the general product costs more integer work
// than the FP64 time it frees).
// The integer parts read doubles only through __double2hiint/__double2loint:
// a 64-bit mask of a double's bit pattern is otherwise turned back into an
// FP64 abs by the compiler, which costs as much as the DFMA it replaced.
#include <algorithm>
#include <cstdlib>

#include "fm_common.cuh"
#include "fm_softfp.cuh"
#include "fm_tune.h"

// CTAs per SM the full-row kernel is compiled for at RY = 2: 3 (80 registers);
// 4 (64 registers, 56 bytes of spills) measured 18.7 against 19.5 GLUP/s
#ifndef FM_GS64_ROW_MINB
#define FM_GS64_ROW_MINB 3
#endif

namespace {

struct Gs64 {
  double F, Fk, Du, Dv, dt;
  fm::DivConst dx;
  fm::soft::DivConstS dxs;
  fm::soft::MulConstS Fs, Fks, Dus, Dvs, dts;
};

template <int DIV>
__device__ __forceinline__ double ddx(double x, const Gs64 &c) {
  if (DIV == 0) return fm::div_const(x, c.dx.d, c.dx.r);
  if (DIV == 2) return fm::div_const_r(x, c.dx.d, c.dx.r);
  if (DIV == 3) return fm::soft::div_const_s(x, c.dxs);
  return fm::div_const_i(x, c.dx);
}

// k*x for one of the constants (MUL >= 1: on the integer pipes)
template <int MUL>
__device__ __forceinline__ double kmul(double k, const fm::soft::MulConstS &ks, double x) {
  if (MUL >= 1) return fm::soft::mul_const_s(x, ks);
  return k * x;
}
// x*y of two state-dependent values (MUL == 2: on the integer pipes)
template <int MUL>
__device__ __forceinline__ double vmul(double x, double y) {
  if (MUL == 2) return fm::soft::mul_s(x, y);
  return x * y;
}

constexpr int kRY = 4;  // y cells per thread

// One cell's update from its fluxes (the U_next and V_next nodes).
template <int DIV, int MUL>
__device__ __forceinline__ void gs_cell(double u, double v, double fxu_m, double fxu_p,
                                        double fyu_m, double fyu_p, double fzu_m,
                                        double fzu_p, double fxv_m, double fxv_p,
                                        double fyv_m, double fyv_p, double fzv_m,
                                        double fzv_p, const Gs64 &c, double &un,
                                        double &vn) {
  // U_next: U + dt*(((-(U*V*V)) + F*(1-U)) + Du*((lx + ly) + lz))
  const double a_1 = vmul<MUL>(u, v);
  const double a_2 = vmul<MUL>(a_1, v);
  const double a_3 = -a_2;
  const double a_5 = 1.0 - u;
  const double a_6 = kmul<MUL>(c.F, c.Fs, a_5);
  const double a_7 = a_3 + a_6;
  const double lx = ddx<DIV>(fxu_p - fxu_m, c);
  const double ly = ddx<DIV>(fyu_p - fyu_m, c);
  const double lz = ddx<DIV>(fzu_p - fzu_m, c);
  const double a_l = (lx + ly) + lz;
  const double dU = a_7 + kmul<MUL>(c.Du, c.Dus, a_l);
  un = u + kmul<MUL>(c.dt, c.dts, dU);
  // V_next: V + dt*(((U*V*V) - (F+k)*V) + Dv*((mx + my) + mz))
  const double b_6 = a_2 - kmul<MUL>(c.Fk, c.Fks, v);
  const double mx = ddx<DIV>(fxv_p - fxv_m, c);
  const double my = ddx<DIV>(fyv_p - fyv_m, c);
  const double mz = ddx<DIV>(fzv_p - fzv_m, c);
  const double b_l = (mx + my) + mz;
  const double dV = b_6 + kmul<MUL>(c.Dv, c.Dvs, b_l);
  vn = v + kmul<MUL>(c.dt, c.dts, dV);
}

// ---------------------------------------------------------------------------
// gs3d_f64_row: CTA = nz threads (nz/32 warps along z, nz <= 256), each thread
// RY y cells (4: 128 registers, 2 CTAs per SM; 2: 80 registers, 3 CTAs — the
// default with DIV = 3, 19.3 GLUP/s at 256^3 against 18.1 for RY = 4); the CTA covers a full periodic z row, so no flux is computed
// twice along z.  Tiles: (ny/RY) y blocks x ceil(nx/xchunk) x chunks.
template <int DIV, int MUL, int RY>
__global__ void __launch_bounds__(256, RY >= 4 ? 2 : FM_GS64_ROW_MINB)
    gs3d_f64_row(const double *__restrict__ U, const double *__restrict__ V,
                 double *__restrict__ Un, double *__restrict__ Vn, int nx, int ny, int nz,
                 int xchunk, int ntiles, Gs64 c) {
  // [buffer][field][j][warp] lane-0 z fluxes, double-buffered by plane parity
  __shared__ double s_fz[2][2][RY][8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int wz = blockDim.x >> 5;
  const int wn = (w + 1 == wz) ? 0 : w + 1;
  const int z = threadIdx.x;
  const int zm = fm::wrap_dn(z, nz);
  const int nyt = ny / RY;
  const size_t sx = (size_t)ny * nz;
  int buf = 0;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int y0 = (t % nyt) * RY;
    const int x0 = (t / nyt) * xchunk;
    const int x1 = min(x0 + xchunk, nx);
    int off[RY];
#pragma unroll
    for (int j = 0; j < RY; ++j) off[j] = (y0 + j) * nz + z;
    const int off_ym = fm::wrap_dn(y0, ny) * nz + z;
    const int off_yp = fm::wrap_up(y0 + RY - 1, ny) * nz + z;
    double uc[RY], vc[RY], fxu[RY], fxv[RY];
    {
      const size_t pm = (size_t)fm::wrap_dn(x0, nx) * sx, pc = (size_t)x0 * sx;
#pragma unroll
      for (int j = 0; j < RY; ++j) {
        const double um = __ldg(U + pm + off[j]), vm = __ldg(V + pm + off[j]);
        uc[j] = __ldg(U + pc + off[j]);
        vc[j] = __ldg(V + pc + off[j]);
        fxu[j] = ddx<DIV>(uc[j] - um, c);
        fxv[j] = ddx<DIV>(vc[j] - vm, c);
      }
    }
    for (int x = x0; x < x1; ++x) {
      const size_t pc = (size_t)x * sx;
      const size_t pp = (size_t)fm::wrap_up(x, nx) * sx;
      double up[RY], vp[RY];
#pragma unroll
      for (int j = 0; j < RY; ++j) {
        up[j] = __ldg(U + pp + off[j]);
        vp[j] = __ldg(V + pp + off[j]);
      }
      // z fluxes at z-1/2
      double fzu[RY], fzv[RY];
#pragma unroll
      for (int j = 0; j < RY; ++j) {
        double uzm = __shfl_up_sync(0xffffffffu, uc[j], 1);
        double vzm = __shfl_up_sync(0xffffffffu, vc[j], 1);
        if (lane == 0) {
          uzm = __ldg(U + pc + (size_t)(y0 + j) * nz + zm);
          vzm = __ldg(V + pc + (size_t)(y0 + j) * nz + zm);
        }
        fzu[j] = ddx<DIV>(uc[j] - uzm, c);
        fzv[j] = ddx<DIV>(vc[j] - vzm, c);
        if (lane == 0) {
          s_fz[buf][0][j][w] = fzu[j];
          s_fz[buf][1][j][w] = fzv[j];
        }
      }
      // y fluxes: fy[j] at y0+j-1/2, j = 0..RY
      double fyu[RY + 1], fyv[RY + 1];
      {
        const double um = __ldg(U + pc + off_ym), vm = __ldg(V + pc + off_ym);
        const double upp = __ldg(U + pc + off_yp), vpp = __ldg(V + pc + off_yp);
        fyu[0] = ddx<DIV>(uc[0] - um, c);
        fyv[0] = ddx<DIV>(vc[0] - vm, c);
#pragma unroll
        for (int j = 1; j < RY; ++j) {
          fyu[j] = ddx<DIV>(uc[j] - uc[j - 1], c);
          fyv[j] = ddx<DIV>(vc[j] - vc[j - 1], c);
        }
        fyu[RY] = ddx<DIV>(upp - uc[RY - 1], c);
        fyv[RY] = ddx<DIV>(vpp - vc[RY - 1], c);
      }
      __syncthreads();
#pragma unroll
      for (int j = 0; j < RY; ++j) {
        double fzu_p = __shfl_down_sync(0xffffffffu, fzu[j], 1);
        double fzv_p = __shfl_down_sync(0xffffffffu, fzv[j], 1);
        if (lane == 31) {
          fzu_p = s_fz[buf][0][j][wn];
          fzv_p = s_fz[buf][1][j][wn];
        }
        const double fxu_p = ddx<DIV>(up[j] - uc[j], c);
        const double fxv_p = ddx<DIV>(vp[j] - vc[j], c);
        double un, vn;
        gs_cell<DIV, MUL>(uc[j], vc[j], fxu[j], fxu_p, fyu[j], fyu[j + 1], fzu[j], fzu_p, fxv[j],
                     fxv_p, fyv[j], fyv[j + 1], fzv[j], fzv_p, c, un, vn);
        Un[pc + off[j]] = un;
        Vn[pc + off[j]] = vn;
        fxu[j] = fxu_p;
        fxv[j] = fxv_p;
        uc[j] = up[j];
        vc[j] = vp[j];
      }
      buf ^= 1;
    }
  }
}

// ---------------------------------------------------------------------------
// gs3d_f64_tile: any nz % 32 == 0.  CTA = 4 warps stacked along y, lanes along
// z; lane 31 computes its own z+1/2 flux.
constexpr int kTileWarps = 4;
constexpr int kTY = kTileWarps * kRY;

template <int DIV, int MUL>
__global__ void __launch_bounds__(kTileWarps * 32)
    gs3d_f64_tile(const double *__restrict__ U, const double *__restrict__ V,
                  double *__restrict__ Un, double *__restrict__ Vn, int nx, int ny, int nz,
                  int xchunk, int ntiles_yz, int ntiles, Gs64 c) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nzt = nz >> 5;
  const size_t sx = (size_t)ny * nz;
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
    double uc[kRY], vc[kRY], fxu[kRY], fxv[kRY];
    {
      const size_t pm = (size_t)fm::wrap_dn(x0, nx) * sx, pc = (size_t)x0 * sx;
#pragma unroll
      for (int j = 0; j < kRY; ++j) {
        const double um = __ldg(U + pm + off[j]), vm = __ldg(V + pm + off[j]);
        uc[j] = __ldg(U + pc + off[j]);
        vc[j] = __ldg(V + pc + off[j]);
        fxu[j] = ddx<DIV>(uc[j] - um, c);
        fxv[j] = ddx<DIV>(vc[j] - vm, c);
      }
    }
    for (int x = x0; x < x1; ++x) {
      const size_t pc = (size_t)x * sx;
      const size_t pp = (size_t)fm::wrap_up(x, nx) * sx;
      double up[kRY], vp[kRY];
#pragma unroll
      for (int j = 0; j < kRY; ++j) {
        up[j] = __ldg(U + pp + off[j]);
        vp[j] = __ldg(V + pp + off[j]);
      }
      double fyu[kRY + 1], fyv[kRY + 1];
      {
        const double um = __ldg(U + pc + off_ym), vm = __ldg(V + pc + off_ym);
        const double upp = __ldg(U + pc + off_yp), vpp = __ldg(V + pc + off_yp);
        fyu[0] = ddx<DIV>(uc[0] - um, c);
        fyv[0] = ddx<DIV>(vc[0] - vm, c);
#pragma unroll
        for (int j = 1; j < kRY; ++j) {
          fyu[j] = ddx<DIV>(uc[j] - uc[j - 1], c);
          fyv[j] = ddx<DIV>(vc[j] - vc[j - 1], c);
        }
        fyu[kRY] = ddx<DIV>(upp - uc[kRY - 1], c);
        fyv[kRY] = ddx<DIV>(vpp - vc[kRY - 1], c);
      }
#pragma unroll
      for (int j = 0; j < kRY; ++j) {
        const double u = uc[j], v = vc[j];
        double uzm = __shfl_up_sync(0xffffffffu, u, 1);
        double vzm = __shfl_up_sync(0xffffffffu, v, 1);
        if (lane == 0) {
          uzm = __ldg(U + pc + (size_t)(y0 + j) * nz + zm);
          vzm = __ldg(V + pc + (size_t)(y0 + j) * nz + zm);
        }
        const double fzu_m = ddx<DIV>(u - uzm, c);
        const double fzv_m = ddx<DIV>(v - vzm, c);
        double fzu_p = __shfl_down_sync(0xffffffffu, fzu_m, 1);
        double fzv_p = __shfl_down_sync(0xffffffffu, fzv_m, 1);
        if (lane == 31) {
          fzu_p = ddx<DIV>(__ldg(U + pc + (size_t)(y0 + j) * nz + zp) - u, c);
          fzv_p = ddx<DIV>(__ldg(V + pc + (size_t)(y0 + j) * nz + zp) - v, c);
        }
        const double fxu_p = ddx<DIV>(up[j] - u, c);
        const double fxv_p = ddx<DIV>(vp[j] - v, c);
        double un, vn;
        gs_cell<DIV, MUL>(u, v, fxu[j], fxu_p, fyu[j], fyu[j + 1], fzu_m, fzu_p, fxv[j], fxv_p,
                     fyv[j], fyv[j + 1], fzv_m, fzv_p, c, un, vn);
        Un[pc + off[j]] = un;
        Vn[pc + off[j]] = vn;
        fxu[j] = fxu_p;
        fxv[j] = fxv_p;
        uc[j] = up[j];
        vc[j] = vp[j];
      }
    }
  }
}

struct LaunchPlan {
  bool row;
  int div, mul, ry, threads, xchunk, ntiles_yz, ntiles, grid;
};

template <typename K>
int resident_blocks(K kernel, int threads, int *out) {
  int sms = 0;
  int st = fm::device_sm_count(&sms);
  if (st) return st;
  int per_sm = 0;
  FM_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0));
  *out = sms * std::max(per_sm, 1);
  return FM_OK;
}

// Smallest (waves x (chunk + warm-up cost)) over candidate x chunks.
int pick_xchunk(int nx, long long tiles_per_chunk_row, int resident, int forced) {
  if (forced > 0) return std::min(forced, nx);
  double best = 1e300;
  int best_xc = 1;
  for (int xc : {1, 2, 3, 4, 6, 8, 12, 16, 24, 32, 48, 64}) {
    if (xc > nx) break;
    const long long nt = tiles_per_chunk_row * ((nx + xc - 1) / xc);
    const long long waves = (nt + resident - 1) / resident;
    const double cost = (double)waves * (xc + 0.35);
    if (cost < best - 1e-9) {
      best = cost;
      best_xc = xc;
    }
  }
  return best_xc;
}

// The instantiated (DIV, MUL, RY) variants: DIV 0..2 with (0, 4); DIV 3 with
// MUL 0..2 and RY 2 or 4.
template <int DIV, int MUL, int RY>
struct Variant {
  static int resident(bool row, int threads, int *out) {
    return row ? resident_blocks(gs3d_f64_row<DIV, MUL, RY>, threads, out)
               : resident_blocks(gs3d_f64_tile<DIV, MUL>, threads, out);
  }
  static void launch(const LaunchPlan &lp, cudaStream_t s, const double *u, const double *v,
                     double *un, double *vn, int nx, int ny, int nz, const Gs64 &c) {
    if (lp.row)
      gs3d_f64_row<DIV, MUL, RY><<<lp.grid, lp.threads, 0, s>>>(u, v, un, vn, nx, ny, nz,
                                                                lp.xchunk, lp.ntiles, c);
    else
      gs3d_f64_tile<DIV, MUL><<<lp.grid, lp.threads, 0, s>>>(
          u, v, un, vn, nx, ny, nz, lp.xchunk, lp.ntiles_yz, lp.ntiles, c);
  }
};

template <typename F>
auto dispatch(const LaunchPlan &lp, F &&f) {
  if (lp.div == 3 && lp.ry == 2) {
    if (lp.mul == 2) return f(Variant<3, 2, 2>());
    if (lp.mul == 1) return f(Variant<3, 1, 2>());
    return f(Variant<3, 0, 2>());
  }
  if (lp.div == 3 && lp.mul == 2) return f(Variant<3, 2, 4>());
  if (lp.div == 3 && lp.mul == 1) return f(Variant<3, 1, 4>());
  if (lp.div == 3) return f(Variant<3, 0, 4>());
  if (lp.div == 2) return f(Variant<2, 0, 4>());
  if (lp.div == 1) return f(Variant<1, 0, 4>());
  return f(Variant<0, 0, 4>());
}

bool soft_mul_ok(double k) {  // nonzero, normal, finite
  const double a = k < 0 ? -k : k;
  return a >= 0x1p-1022 && a <= 0x1.fffffffffffffp1023;
}

int plan_launch(int nx, int ny, int nz, const fm_gs_params *p, LaunchPlan *lp) {
  const int kind = fm::tune_get("gs3d_f64.kernel", 0);  // 0 auto, 1 tile, 2 row
  lp->div = fm::tune_get("gs3d_f64.div", 3);
  if (lp->div < 0 || lp->div > 3) lp->div = 3;
  if (lp->div == 2 && !(p->dx >= 0x1p-20 && p->dx <= 0x1p20)) lp->div = 0;
  lp->mul = lp->div == 3 ? fm::tune_get("gs3d_f64.mul", 1) : 0;
  if (lp->mul < 0 || lp->mul > 2) lp->mul = 0;
  if (lp->mul && !(soft_mul_ok(p->F) && soft_mul_ok(p->F + p->k) && soft_mul_ok(p->Du) &&
                   soft_mul_ok(p->Dv) && soft_mul_ok(p->dt)))
    lp->mul = 0;  // a zero or non-normal constant: hardware multiplications
  lp->ry = lp->div == 3 ? fm::tune_get("gs3d_f64.ry", 2) : 4;
  if (lp->ry != 4) lp->ry = 2;
  if (lp->div != 3) lp->ry = 4;  // the only row-kernel shape instantiated for them
  const bool row_ok = nz <= 256 && ny % lp->ry == 0;
  lp->row = (kind == 2 || kind == 0) && row_ok;
  if (kind == 1 || ny % kTY != 0) lp->row = false;
  if (!lp->row && ny % kTY != 0) {
    fm::set_error("fm_gs3d_f64_forward: ny must be a multiple of %d for nz > 256", kTY);
    return FM_ERR_UNSUPPORTED;
  }
  int resident = 0;
  const int forced = fm::tune_get("gs3d_f64.xchunk", 0);
  lp->threads = lp->row ? nz : kTileWarps * 32;
  const bool row = lp->row;
  const int threads = lp->threads;
  const int st =
      dispatch(*lp, [&](auto v) { return decltype(v)::resident(row, threads, &resident); });
  if (st) return st;
  lp->ntiles_yz = lp->row ? ny / lp->ry : (nz / 32) * (ny / kTY);
  lp->xchunk = pick_xchunk(nx, lp->ntiles_yz, resident, forced);
  lp->ntiles = lp->ntiles_yz * ((nx + lp->xchunk - 1) / lp->xchunk);
  lp->grid = std::min(lp->ntiles, resident);
  return FM_OK;
}

void launch(const LaunchPlan &lp, cudaStream_t s, const double *u, const double *v, double *un,
            double *vn, int nx, int ny, int nz, const Gs64 &c) {
  dispatch(lp, [&](auto var) {
    decltype(var)::launch(lp, s, u, v, un, vn, nx, ny, nz, c);
    return 0;
  });
}

}  // namespace

extern "C" int fm_gs3d_f64_forward(int nx, int ny, int nz, double *U, double *V,
                                   double *work_U, double *work_V,
                                   const fm_gs_params *p, int steps,
                                   void *stream) {
  FM_CHECK_ARG(p && U && V && work_U && work_V, "fm_gs3d_f64_forward: NULL argument");
  FM_CHECK_ARG(nx >= 1 && ny >= kTY && nz >= 32 && nz % 32 == 0 && ny % kTY == 0,
               "fm_gs3d_f64_forward: need nz %% 32 == 0 and ny %% %d == 0 (got %d,%d,%d)",
               kTY, nx, ny, nz);
  FM_CHECK_ARG((long long)ny * nz < (1ll << 31), "fm_gs3d_f64_forward: plane too large");
  FM_CHECK_ARG(steps >= 0, "fm_gs3d_f64_forward: steps < 0");
  FM_CHECK_ARG(p->dx >= 0x1p-40 && p->dx <= 0x1p40,
               "fm_gs3d_f64_forward: dx outside [2^-40, 2^40]");
  if (steps == 0) return FM_OK;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  LaunchPlan lp;
  int st = plan_launch(nx, ny, nz, p, &lp);
  if (st) return st;
  Gs64 c;
  c.F = p->F;
  c.Fk = p->F + p->k;  // node (F+k) of the V_next DAG
  c.Du = p->Du;
  c.Dv = p->Dv;
  c.dt = p->dt;
  c.dx = fm::make_div_const(p->dx);
  c.dxs = fm::soft::make_div_const_s(p->dx);
  if (lp.mul) {
    c.Fs = fm::soft::make_mul_const_s(c.F);
    c.Fks = fm::soft::make_mul_const_s(c.Fk);
    c.Dus = fm::soft::make_mul_const_s(c.Du);
    c.Dvs = fm::soft::make_mul_const_s(c.Dv);
    c.dts = fm::soft::make_mul_const_s(c.dt);
  } else {
    c.Fs = c.Fks = c.Dus = c.Dvs = c.dts = fm::soft::MulConstS();
  }
  double *cu = U, *cv = V, *nu = work_U, *nv = work_V;
  for (int i = 0; i < steps; ++i) {
    launch(lp, s, cu, cv, nu, nv, nx, ny, nz, c);
    std::swap(cu, nu);
    std::swap(cv, nv);
  }
  FM_TRY_CUDA(cudaGetLastError());
  if (cu != U) {
    const size_t bytes = (size_t)nx * ny * nz * sizeof(double);
    FM_TRY_CUDA(cudaMemcpyAsync(U, cu, bytes, cudaMemcpyDeviceToDevice, s));
    FM_TRY_CUDA(cudaMemcpyAsync(V, cv, bytes, cudaMemcpyDeviceToDevice, s));
  }
  return FM_OK;
}
