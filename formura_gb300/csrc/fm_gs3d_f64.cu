// fm_gs3d_f64.cu — 3D Gray-Scott (examples/pearson-3d.fmr form), FP64,
// bit-exact with the generated loop nest.
//
// The generated C evaluates, per cell, the whole U_next / V_next DAG with the
// half-point differences recomputed at every use (Manifestation inlines the
// delayed ddx node, src/Formura/OrthotopeMachine/Manifestation.hs:115-143).
// A recomputed IEEE expression has the same value, so this kernel computes
// each face flux (W[i+1]-W[i])/dx once and hands it to both cells that use it:
//   x (slowest axis): the CTA marches along x; the flux at x-1/2 is carried in
//                     registers from the previous plane.
//   y:                each thread owns RY consecutive y cells of one z column;
//                     RY+1 fluxes serve RY cells.
//   z (fastest axis): lanes of a warp are consecutive z; the flux at z+1/2 is
//                     the next lane's z-1/2 flux (warp shuffle), lane 31
//                     computes its own.
// Divisions by dx use fm::div_const (correctly rounded, 1 DMUL + 2 DFMA).
// On GB300 the FP64 pipe, not HBM, bounds this kernel (~70 FP64 instructions
// per cell update against 32 B of compulsory traffic).
#include <algorithm>

#include "fm_common.cuh"

namespace {

using fm::div_const;

struct Gs64 {
  double F, Fk, Du, Dv, dt, dx, rdx;
};

constexpr int kWarps = 4;  // warps per CTA, stacked along y
constexpr int kRY = 4;     // y cells per thread
constexpr int kTY = kWarps * kRY;

__global__ void __launch_bounds__(kWarps * 32)
    gs3d_f64_step(const double *__restrict__ U, const double *__restrict__ V,
                  double *__restrict__ Un, double *__restrict__ Vn, int nx,
                  int ny, int nz, int xchunk, int ntiles_yz, int ntiles,
                  Gs64 c) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nzt = nz >> 5;
  const size_t sx = (size_t)ny * nz;
  const double dx = c.dx, rdx = c.rdx;

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
        fxu[j] = div_const(uc[j] - um, dx, rdx);
        fxv[j] = div_const(vc[j] - vm, dx, rdx);
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
      // y fluxes: fy[j] is the flux at y0+j-1/2, j = 0..RY.
      double fyu[kRY + 1], fyv[kRY + 1];
      {
        const double um = __ldg(U + pc + off_ym), vm = __ldg(V + pc + off_ym);
        const double upp = __ldg(U + pc + off_yp), vpp = __ldg(V + pc + off_yp);
        fyu[0] = div_const(uc[0] - um, dx, rdx);
        fyv[0] = div_const(vc[0] - vm, dx, rdx);
#pragma unroll
        for (int j = 1; j < kRY; ++j) {
          fyu[j] = div_const(uc[j] - uc[j - 1], dx, rdx);
          fyv[j] = div_const(vc[j] - vc[j - 1], dx, rdx);
        }
        fyu[kRY] = div_const(upp - uc[kRY - 1], dx, rdx);
        fyv[kRY] = div_const(vpp - vc[kRY - 1], dx, rdx);
      }
#pragma unroll
      for (int j = 0; j < kRY; ++j) {
        const double u = uc[j], v = vc[j];
        // z fluxes at z-1/2 (this lane) and z+1/2 (next lane, or own for lane 31)
        double uzm = __shfl_up_sync(0xffffffffu, u, 1);
        double vzm = __shfl_up_sync(0xffffffffu, v, 1);
        if (lane == 0) {
          uzm = __ldg(U + pc + (size_t)(y0 + j) * nz + zm);
          vzm = __ldg(V + pc + (size_t)(y0 + j) * nz + zm);
        }
        const double fzu_m = div_const(u - uzm, dx, rdx);
        const double fzv_m = div_const(v - vzm, dx, rdx);
        double fzu_p = __shfl_down_sync(0xffffffffu, fzu_m, 1);
        double fzv_p = __shfl_down_sync(0xffffffffu, fzv_m, 1);
        if (lane == 31) {
          const double uzp = __ldg(U + pc + (size_t)(y0 + j) * nz + zp);
          const double vzp = __ldg(V + pc + (size_t)(y0 + j) * nz + zp);
          fzu_p = div_const(uzp - u, dx, rdx);
          fzv_p = div_const(vzp - v, dx, rdx);
        }
        const double fxu_p = div_const(up[j] - u, dx, rdx);
        const double fxv_p = div_const(vp[j] - v, dx, rdx);

        // U_next: U + dt*(((-(U*V*V)) + F*(1-U)) + Du*((lx + ly) + lz))
        const double a_1 = u * v;
        const double a_2 = a_1 * v;
        const double a_3 = -a_2;
        const double a_5 = 1.0 - u;
        const double a_6 = c.F * a_5;
        const double a_7 = a_3 + a_6;
        const double lx = div_const(fxu_p - fxu[j], dx, rdx);
        const double ly = div_const(fyu[j + 1] - fyu[j], dx, rdx);
        const double lz = div_const(fzu_p - fzu_m, dx, rdx);
        const double a_l = (lx + ly) + lz;
        const double dU = a_7 + c.Du * a_l;
        Un[pc + off[j]] = u + c.dt * dU;

        // V_next: V + dt*(((U*V*V) - (F+k)*V) + Dv*((mx + my) + mz))
        const double b_6 = a_2 - c.Fk * v;
        const double mx = div_const(fxv_p - fxv[j], dx, rdx);
        const double my = div_const(fyv[j + 1] - fyv[j], dx, rdx);
        const double mz = div_const(fzv_p - fzv_m, dx, rdx);
        const double b_l = (mx + my) + mz;
        const double dV = b_6 + c.Dv * b_l;
        Vn[pc + off[j]] = v + c.dt * dV;

        fxu[j] = fxu_p;
        fxv[j] = fxv_p;
        uc[j] = up[j];
        vc[j] = vp[j];
      }
    }
  }
}

struct LaunchPlan {
  int xchunk, ntiles_yz, ntiles, grid;
};

int plan_launch(int nx, int ny, int nz, LaunchPlan *lp) {
  int sms = 0;
  int st = fm::device_sm_count(&sms);
  if (st) return st;
  int per_sm = 0;
  FM_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gs3d_f64_step,
                                                             kWarps * 32, 0));
  if (per_sm < 1) per_sm = 1;
  const int resident = sms * per_sm;
  const int ntiles_yz = (nz / 32) * (ny / kTY);
  // Pick the x chunk that minimises waves x (chunk + warm-up plane cost).
  double best = 1e300;
  int best_xc = 1;
  for (int xc : {1, 2, 3, 4, 6, 8, 12, 16, 24, 32}) {
    if (xc > nx) break;
    const long long nt = (long long)ntiles_yz * ((nx + xc - 1) / xc);
    const long long waves = (nt + resident - 1) / resident;
    const double cost = (double)waves * (xc + 0.35);
    if (cost < best - 1e-9) {
      best = cost;
      best_xc = xc;
    }
  }
  lp->xchunk = best_xc;
  lp->ntiles_yz = ntiles_yz;
  lp->ntiles = ntiles_yz * ((nx + best_xc - 1) / best_xc);
  lp->grid = std::min(lp->ntiles, resident);
  return FM_OK;
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
  int st = plan_launch(nx, ny, nz, &lp);
  if (st) return st;
  Gs64 c;
  c.F = p->F;
  c.Fk = p->F + p->k;  // node (F+k) of the V_next DAG
  c.Du = p->Du;
  c.Dv = p->Dv;
  c.dt = p->dt;
  c.dx = p->dx;
  c.rdx = 1.0 / p->dx;
  double *cu = U, *cv = V, *nu = work_U, *nv = work_V;
  for (int i = 0; i < steps; ++i) {
    gs3d_f64_step<<<lp.grid, kWarps * 32, 0, s>>>(cu, cv, nu, nv, nx, ny, nz, lp.xchunk,
                                                 lp.ntiles_yz, lp.ntiles, c);
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
