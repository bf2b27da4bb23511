// fm_gs2d.cu — 2D Gray-Scott in the examples/pearson-2d.fmr form, binary32:
// one instance per launch (fm_gs2d_f32_forward) and uneven ensembles of
// instances with different F, k in one persistent launch
// (fm_gs2d_ensemble_*).
//
// Per cell, the pearson-2d DAG (examples/pearson-2d.fmr:21-25, the order of
// examples-generated/pearson.c:138-208) in float without FMA contraction:
//   dU = ((-(U*V*V)) + F*(1-U)) + (Du/(dx*dx)) * ((U[x+1]-U) - (U-U[x-1]) + (U[y+1]-U) - (U-U[y-1]))
//   dV = ((U*V*V) - (F+k)*V)   + (Dv/(dx*dx)) * (...)
//   U' = U + dt*dU,  V' = V + dt*dV
// Bit-exact with the binary32 restatement of that DAG.
//
// Ensemble kernel: all instances' U (and V) live back to back in one buffer.
// The work is a flat list of square output tiles over all instances.  For a
// time block of T steps, a CTA loads a tile plus a T-cell periodic halo (the
// instance wraps onto itself) into shared memory, advances it T steps there
// (the valid region shrinks by one cell per step), and writes the tile's
// interior back: ~(1 + 4T/tile) x 8 B read and 8 B written per T lattice
// updates.  Blocks meet at a grid barrier between time blocks (bounded
// waits; FM_ERR_TIMEOUT instead of a hang), so the whole run is ONE
// cooperative launch, which fm_gs2d_ensemble_forward replays from a captured
// CUDA graph.
#include <algorithm>
#include <mutex>
#include <vector>

#include "fm_common.cuh"
#include "fm_tune.h"

#ifndef FM_ENS_PF
#define FM_ENS_PF 2  // planes prefetched ahead by the wavefront kernel (3: 392, 4: 391 vs 397 GLUP/s)
#endif

namespace {

struct GridSync {
  unsigned int arrive;
  unsigned int gen;
  int err;
  int pad;
};

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ bool grid_barrier(GridSync *gs, unsigned nblocks, unsigned &gen_local,
                             long long limit) {
  __shared__ int s_fail;
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    int fail = 0;
    const unsigned target = gen_local + 1;
    __threadfence();
    if (atomicAdd(&gs->arrive, 1u) == nblocks - 1) {
      atomicExch(&gs->arrive, 0u);
      __threadfence();
      atomicExch(&gs->gen, target);
    } else {
      long long spins = 0;
      while (ld_acquire_u32(&gs->gen) != target) {
        if (++spins > limit || *((volatile int *)&gs->err) != 0) {
          atomicExch(&gs->err, 1);
          fail = 1;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    s_fail = fail;
  }
  __syncthreads();
  gen_local += 1;
  return s_fail == 0;
}

struct Gs2Const {
  float F, Fk, cu, cv, dt;
};

// Float pearson-2d DAG for one cell given its four neighbours.
__device__ __forceinline__ void gs2_cell(float a, float a0, float uxp, float uxm, float uyp,
                                         float uym, float vxp, float vxm, float vyp, float vym,
                                         const Gs2Const &c, float &un, float &vn) {
  const float a_1 = a * a0;
  const float a_2 = a_1 * a0;
  const float a_3 = -a_2;
  const float a_6 = 1.0f - a;
  const float a_7 = c.F * a_6;
  const float a_8 = a_3 + a_7;
  const float a_14 = uxp - a;
  const float a_16 = a - uxm;
  const float a_17 = a_14 - a_16;
  const float a_19 = uyp - a;
  const float a_21 = a - uym;
  const float a_22 = a_19 - a_21;
  const float a_23 = a_17 + a_22;
  const float a_24 = c.cu * a_23;
  const float dU = a_8 + a_24;
  const float b_6 = c.Fk * a0;
  const float b_7 = a_2 - b_6;
  const float b_13 = vxp - a0;
  const float b_15 = a0 - vxm;
  const float b_16 = b_13 - b_15;
  const float b_18 = vyp - a0;
  const float b_20 = a0 - vym;
  const float b_21 = b_18 - b_20;
  const float b_22 = b_16 + b_21;
  const float b_23 = c.cv * b_22;
  const float dV = b_7 + b_23;
  un = a + c.dt * dU;
  vn = a0 + c.dt * dV;
}

// ---------------------------------------------------------------- one instance
__global__ void __launch_bounds__(256)
    gs2d_step(const float *__restrict__ U, const float *__restrict__ V, float *__restrict__ Un,
              float *__restrict__ Vn, int nx, int ny, Gs2Const c) {
  const int y = blockIdx.x * 32 + (threadIdx.x & 31);
  const int x = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (x >= nx || y >= ny) return;
  const size_t r = (size_t)x * ny, rp = (size_t)fm::wrap_up(x, nx) * ny,
               rm = (size_t)fm::wrap_dn(x, nx) * ny;
  const int yp = fm::wrap_up(y, ny), ym = fm::wrap_dn(y, ny);
  float un, vn;
  gs2_cell(U[r + y], V[r + y], U[rp + y], U[rm + y], U[r + yp], U[r + ym], V[rp + y], V[rm + y],
           V[r + yp], V[r + ym], c, un, vn);
  Un[r + y] = un;
  Vn[r + y] = vn;
}

// ---------------------------------------------------------------- ensemble
struct EnsInst {
  long long off;  // first cell of the instance in the flat buffers
  int n;          // n x n, periodic
  int pad;
  Gs2Const c;
};

struct EnsTile {
  int inst;
  int x0, y0;  // first output cell (row x0, column y0) of the tile
};

// Tile of TSxTS outputs; T = maximum time steps per block (template), the
// block's actual count tb_run <= T.  Shared memory: 2 fields x 2 buffers x
// (TS+2T)^2 floats.
template <int TS, int T>
__global__ void __launch_bounds__(256)
    gs2d_ensemble(const EnsInst *__restrict__ insts, const EnsTile *__restrict__ tiles,
                  int ntiles, float *U0, float *V0, float *U1, float *V1, int steps, int tb,
                  GridSync *gs, long long limit) {
  constexpr int R = TS + 2 * T;  // region edge
  extern __shared__ float sm[];
  // buffer b of field f at sm + (2*f + b) * R*R
  const int lx = threadIdx.x;  // 0..31 along the fast axis (y)
  const int ly = threadIdx.y;  // 0..7 along x
  unsigned gen = 0;
  int blk = 0;
  for (int done = 0; done < steps; done += tb, ++blk) {
    const int tr = min(tb, steps - done);
    const int h = tr;  // halo this block needs
    const float *Us = (blk & 1) ? U1 : U0;
    const float *Vs = (blk & 1) ? V1 : V0;
    float *Ud = (blk & 1) ? U0 : U1;
    float *Vd = (blk & 1) ? V0 : V1;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const EnsTile tl = tiles[t];
      const EnsInst in = insts[tl.inst];
      const int n = in.n;
      const float *Ui = Us + in.off;
      const float *Vi = Vs + in.off;
      // load the (TS+2h)^2 region with periodic wrap into buffer 0
      const int re = TS + 2 * h;
      for (int r = ly; r < re; r += 8) {
        int gx = (tl.x0 - h + r) % n;
        if (gx < 0) gx += n;
        const float *urow = Ui + (size_t)gx * n;
        const float *vrow = Vi + (size_t)gx * n;
        for (int q = lx; q < re; q += 32) {
          int gy = (tl.y0 - h + q) % n;
          if (gy < 0) gy += n;
          sm[r * R + q] = __ldcg(urow + gy);
          sm[2 * R * R + r * R + q] = __ldcg(vrow + gy);
        }
      }
      __syncthreads();
      const Gs2Const c = in.c;
      for (int s = 1; s <= tr; ++s) {
        const float *au = sm + ((s - 1) & 1) * R * R, *av = au + 2 * R * R;
        float *bu = sm + (s & 1) * R * R, *bv = bu + 2 * R * R;
        for (int r = s + ly; r < re - s; r += 8) {
          for (int q = s + lx; q < re - s; q += 32) {
            const int i = r * R + q;
            float un, vn;
            gs2_cell(au[i], av[i], au[i + R], au[i - R], au[i + 1], au[i - 1], av[i + R],
                     av[i - R], av[i + 1], av[i - 1], c, un, vn);
            bu[i] = un;
            bv[i] = vn;
          }
        }
        __syncthreads();
      }
      // write the tile interior (rows/cols [h, h+TS) of the region)
      const float *ru = sm + (tr & 1) * R * R, *rv = ru + 2 * R * R;
      float *Uo = Ud + in.off, *Vo = Vd + in.off;
      const int rows = min(TS, n - tl.x0), cols = min(TS, n - tl.y0);
      for (int r = ly; r < rows; r += 8) {
        float *uo = Uo + (size_t)(tl.x0 + r) * n + tl.y0;
        float *vo = Vo + (size_t)(tl.x0 + r) * n + tl.y0;
        for (int q = lx; q < cols; q += 32) {
          __stcg(uo + q, ru[(r + h) * R + q + h]);
          __stcg(vo + q, rv[(r + h) * R + q + h]);
        }
      }
      __syncthreads();
    }
    if (!grid_barrier(gs, gridDim.x, gen, limit)) return;
  }
}

// ---------------------------------------------------------------- wavefront form
// gs2d_ens_wf<T>: one WARP owns a strip of 64 consecutive y cells of one
// instance (two cells per lane; periodic wrap inside the instance) and streams
// it along x over a chunk of planes, advancing up to T time levels in a
// pipeline: at iteration i it loads plane i (level 0) and level s = 1..T
// advances plane i-s from level s-1's planes i-s-1, i-s, i-s+1, held in a
// 3-plane register window per level; the y neighbours are the lane's other
// cell or the next/previous lane's (warp shuffles).  No shared memory and no
// block barrier: warps run independently.  Level s is valid on strip cells
// [s, 64-s), so a strip writes its middle 64-2T cells (its output strip) and
// the planes [x0, x1) of its chunk.  Blocks of T steps meet at the grid
// barrier, as in gs2d_ensemble.  Same gs2_cell arithmetic: bit-identical.
struct WfTile {
  int inst;
  int ys;      // first output y of the strip
  int x0, x1;  // output planes [x0, x1)
};
constexpr int kWfWidth = 64;

template <int T>
__global__ void __launch_bounds__(128)
    gs2d_ens_wf(const EnsInst *__restrict__ insts, const WfTile *__restrict__ tiles, int ntiles,
                float *U0, float *V0, float *U1, float *V1, int steps, int tb, GridSync *gs,
                long long limit) {
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * 4 + (threadIdx.x >> 5);
  const int nw = gridDim.x * 4;
  const int jA = 2 * lane, jB = jA + 1;
  unsigned gen = 0;
  int blk = 0;
  for (int done = 0; done < steps; done += tb, ++blk) {
    const int tr = min(tb, steps - done);  // levels of this block, <= T
    const float *Us = (blk & 1) ? U1 : U0;
    const float *Vs = (blk & 1) ? V1 : V0;
    float *Ud = (blk & 1) ? U0 : U1;
    float *Vd = (blk & 1) ? V0 : V1;
    for (int t = gw; t < ntiles; t += nw) {
      const WfTile tl = tiles[t];
      const EnsInst in = insts[tl.inst];
      const int n = in.n;
      const Gs2Const c = in.c;
      const float *Ui = Us + in.off, *Vi = Vs + in.off;
      float *Uo = Ud + in.off, *Vo = Vd + in.off;
      int yA = (tl.ys - T + jA) % n;
      yA = yA < 0 ? yA + n : yA;
      int yB = (tl.ys - T + jB) % n;
      yB = yB < 0 ? yB + n : yB;
      const bool oA = jA >= T && jA < kWfWidth - T && tl.ys + jA - T < n;
      const bool oB = jB >= T && jB < kWfWidth - T && tl.ys + jB - T < n;
      float wu[T][3][2], wv[T][3][2];
#pragma unroll
      for (int s = 0; s < T; ++s)
#pragma unroll
        for (int p = 0; p < 3; ++p) wu[s][p][0] = wu[s][p][1] = wv[s][p][0] = wv[s][p][1] = 0.0f;
      constexpr int kPF = FM_ENS_PF;
      float pu[kPF][2], pv[kPF][2];
#pragma unroll
      for (int k = 0; k < kPF; ++k) {
        int x = (tl.x0 - tr + k) % n;
        x = x < 0 ? x + n : x;
        const size_t r = (size_t)x * n;
        pu[k][0] = __ldcg(Ui + r + yA);
        pu[k][1] = __ldcg(Ui + r + yB);
        pv[k][0] = __ldcg(Vi + r + yA);
        pv[k][1] = __ldcg(Vi + r + yB);
      }
      const int iend = tl.x1 + tr;
      for (int i = tl.x0 - tr; i < iend; ++i) {
        // level 0: plane i
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          wu[0][0][q] = wu[0][1][q];
          wu[0][1][q] = wu[0][2][q];
          wu[0][2][q] = pu[0][q];
          wv[0][0][q] = wv[0][1][q];
          wv[0][1][q] = wv[0][2][q];
          wv[0][2][q] = pv[0][q];
        }
#pragma unroll
        for (int k = 0; k + 1 < kPF; ++k)
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            pu[k][q] = pu[k + 1][q];
            pv[k][q] = pv[k + 1][q];
          }
        if (i + kPF < iend) {
          // i + kPF lies in [x0 - T + kPF, x1 + T + kPF): one conditional wrap
          // for n >= 16 (T <= 8), the integer remainder only for smaller instances
          int x = i + kPF;
          if (n >= 16) {
            x = x < 0 ? x + n : (x >= n ? x - n : x);
          } else {
            x %= n;
            x = x < 0 ? x + n : x;
          }
          const size_t r = (size_t)x * n;
          pu[kPF - 1][0] = __ldcg(Ui + r + yA);
          pu[kPF - 1][1] = __ldcg(Ui + r + yB);
          pv[kPF - 1][0] = __ldcg(Vi + r + yA);
          pv[kPF - 1][1] = __ldcg(Vi + r + yB);
        }
        // levels 1..tr: level s advances plane i-s
#pragma unroll
        for (int s = 1; s <= T; ++s) {
          if (s > tr) break;
          const float uA = wu[s - 1][1][0], uB = wu[s - 1][1][1];
          const float vA = wv[s - 1][1][0], vB = wv[s - 1][1][1];
          const float uAl = __shfl_up_sync(0xffffffffu, uB, 1);    // cell jA - 1
          const float uBr = __shfl_down_sync(0xffffffffu, uA, 1);  // cell jB + 1
          const float vAl = __shfl_up_sync(0xffffffffu, vB, 1);
          const float vBr = __shfl_down_sync(0xffffffffu, vA, 1);
          float unA, vnA, unB, vnB;
          gs2_cell(uA, vA, wu[s - 1][2][0], wu[s - 1][0][0], uB, uAl, wv[s - 1][2][0],
                   wv[s - 1][0][0], vB, vAl, c, unA, vnA);
          gs2_cell(uB, vB, wu[s - 1][2][1], wu[s - 1][0][1], uBr, uA, wv[s - 1][2][1],
                   wv[s - 1][0][1], vBr, vA, c, unB, vnB);
          if (s < tr) {
            wu[s][0][0] = wu[s][1][0];
            wu[s][1][0] = wu[s][2][0];
            wu[s][2][0] = unA;
            wu[s][0][1] = wu[s][1][1];
            wu[s][1][1] = wu[s][2][1];
            wu[s][2][1] = unB;
            wv[s][0][0] = wv[s][1][0];
            wv[s][1][0] = wv[s][2][0];
            wv[s][2][0] = vnA;
            wv[s][0][1] = wv[s][1][1];
            wv[s][1][1] = wv[s][2][1];
            wv[s][2][1] = vnB;
          } else {
            const int pp = i - tr;
            if (pp >= tl.x0) {
              const size_t r = (size_t)pp * n;
              if (oA) {
                __stcg(Uo + r + yA, unA);
                __stcg(Vo + r + yA, vnA);
              }
              if (oB) {
                __stcg(Uo + r + yB, unB);
                __stcg(Vo + r + yB, vnB);
              }
            }
          }
        }
      }
    }
    if (!grid_barrier(gs, gridDim.x, gen, limit)) return;
  }
}

}  // namespace

// ============================================================== C ABI
struct fm_ensemble {
  int n_inst;
  int ts, tb;
  long long total;
  std::vector<long long> offsets;
  std::vector<int> sizes;
  EnsInst *d_inst = nullptr;
  EnsTile *d_tiles = nullptr;
  int ntiles = 0;
  int kind = 0;  // 0 shared-memory tiles, 1 wavefront strips
  int xchunk = 0;
  GridSync *d_sync = nullptr;
  // captured graph of the last forward call
  cudaGraphExec_t gexec = nullptr;
  const void *g_key[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  int g_steps = -1;
  long long g_limit = -1;
  cudaStream_t g_stream = nullptr;
};

namespace {

template <int TS, int T>
const void *ens_kernel() {
  return (const void *)gs2d_ensemble<TS, T>;
}

const void *pick_kernel(int ts, int tb) {
#define FM_ENS_CASE(TS_, T_) \
  if (ts == TS_ && tb <= T_) return ens_kernel<TS_, T_>();
  FM_ENS_CASE(32, 1) FM_ENS_CASE(32, 2) FM_ENS_CASE(32, 4) FM_ENS_CASE(32, 8)
  FM_ENS_CASE(64, 1) FM_ENS_CASE(64, 2) FM_ENS_CASE(64, 4) FM_ENS_CASE(64, 8)
#undef FM_ENS_CASE
  return nullptr;
}

const void *pick_wf(int tb) {
  if (tb <= 2) return (const void *)gs2d_ens_wf<2>;
  if (tb <= 4) return (const void *)gs2d_ens_wf<4>;
  if (tb <= 6) return (const void *)gs2d_ens_wf<6>;
  if (tb <= 8) return (const void *)gs2d_ens_wf<8>;
  return nullptr;
}

int wf_tmax(int tb) { return tb <= 2 ? 2 : tb <= 4 ? 4 : tb <= 6 ? 6 : 8; }

int kernel_tmax(int ts, int tb) {
  for (int t : {1, 2, 4, 8})
    if (tb <= t && pick_kernel(ts, t) == pick_kernel(ts, tb)) return t;
  return tb;
}

size_t ens_smem(int ts, int tmax) {
  const size_t r = (size_t)ts + 2 * tmax;
  return 4 * r * r * sizeof(float);
}

}  // namespace

extern "C" int fm_gs2d_f32_forward(int nx, int ny, float *U, float *V, float *work_U,
                                   float *work_V, const fm_gs_params *p, int steps,
                                   void *stream) {
  FM_CHECK_ARG(p && U && V && work_U && work_V, "fm_gs2d_f32_forward: NULL argument");
  FM_CHECK_ARG(nx >= 1 && ny >= 1, "fm_gs2d_f32_forward: empty grid");
  FM_CHECK_ARG(steps >= 0, "fm_gs2d_f32_forward: steps < 0");
  if (steps == 0) return FM_OK;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  Gs2Const c;
  c.F = (float)p->F;
  c.Fk = c.F + (float)p->k;
  const float dxf = (float)p->dx;
  const float dx2 = dxf * dxf;
  c.cu = (float)p->Du / dx2;
  c.cv = (float)p->Dv / dx2;
  c.dt = (float)p->dt;
  float *cu = U, *cv = V, *nu = work_U, *nv = work_V;
  const dim3 grid((ny + 31) / 32, (nx + 7) / 8);
  for (int i = 0; i < steps; ++i) {
    gs2d_step<<<grid, 256, 0, s>>>(cu, cv, nu, nv, nx, ny, c);
    std::swap(cu, nu);
    std::swap(cv, nv);
  }
  FM_TRY_CUDA(cudaGetLastError());
  if (cu != U) {
    const size_t bytes = (size_t)nx * ny * sizeof(float);
    FM_TRY_CUDA(cudaMemcpyAsync(U, cu, bytes, cudaMemcpyDeviceToDevice, s));
    FM_TRY_CUDA(cudaMemcpyAsync(V, cv, bytes, cudaMemcpyDeviceToDevice, s));
  }
  return FM_OK;
}

extern "C" int fm_gs2d_ensemble_create(fm_ensemble **out, int n_inst, const int *sizes,
                                       const double *F, const double *k, double Du, double Dv,
                                       double dt, double dx, int tile, int tb) {
  FM_CHECK_ARG(out && sizes && F && k && n_inst >= 1, "fm_gs2d_ensemble_create: bad arguments");
  *out = nullptr;
  if (tile == 0) tile = fm::tune_get("gs2d_ens.tile", 1);
  const int kind = tile == 1 ? 1 : 0;
  if (tb == 0) tb = fm::tune_get("gs2d_ens.tb", kind == 1 ? 2 : 4);
  FM_CHECK_ARG(kind == 1 ? (tb >= 1 && tb <= 8) : pick_kernel(tile, tb) != nullptr,
               "fm_gs2d_ensemble_create: unsupported tile %d / tb %d (tile 32 or 64, or 1 for "
               "wavefront strips; tb 1..8)", tile, tb);
  if (kind == 0) {
    int dev = 0, optin = 0;
    FM_TRY_CUDA(cudaGetDevice(&dev));
    FM_TRY_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const size_t need = ens_smem(tile, kernel_tmax(tile, tb));
    if (need > (size_t)optin) {
      fm::set_error("fm_gs2d_ensemble_create: tile %d / tb %d needs %zu B of shared memory, "
                    "device allows %d", tile, tb, need, optin);
      return FM_ERR_UNSUPPORTED;
    }
  }
  fm_ensemble *e = new fm_ensemble();
  e->n_inst = n_inst;
  e->ts = tile;
  e->tb = tb;
  e->kind = kind;
  e->xchunk = std::max(1, fm::tune_get("gs2d_ens.xchunk", 64));
  const int wf_out = kWfWidth - 2 * wf_tmax(tb);  // output y per strip
  std::vector<EnsInst> hi(n_inst);
  std::vector<EnsTile> ht;
  std::vector<WfTile> hw;
  long long off = 0;
  for (int i = 0; i < n_inst; ++i) {
    if (sizes[i] < 1) {
      delete e;
      fm::set_error("fm_gs2d_ensemble_create: instance %d has size %d", i, sizes[i]);
      return FM_ERR_ARG;
    }
    const int n = sizes[i];
    hi[i].off = off;
    hi[i].n = n;
    hi[i].pad = 0;
    // constants in float, in DAG order (pearson-2d.fmr:16-22)
    hi[i].c.F = (float)F[i];
    hi[i].c.Fk = (float)F[i] + (float)k[i];
    const float dxf = (float)dx, dx2 = dxf * dxf;
    hi[i].c.cu = (float)Du / dx2;
    hi[i].c.cv = (float)Dv / dx2;
    hi[i].c.dt = (float)dt;
    e->offsets.push_back(off);
    e->sizes.push_back(n);
    if (kind == 0) {
      for (int x0 = 0; x0 < n; x0 += tile)
        for (int y0 = 0; y0 < n; y0 += tile) ht.push_back(EnsTile{i, x0, y0});
    } else {
      for (int x0 = 0; x0 < n; x0 += e->xchunk)
        for (int ys = 0; ys < n; ys += wf_out)
          hw.push_back(WfTile{i, ys, x0, std::min(x0 + e->xchunk, n)});
    }
    off += (long long)n * n;
  }
  e->total = off;
  e->ntiles = kind == 0 ? (int)ht.size() : (int)hw.size();
  const size_t tile_bytes = kind == 0 ? sizeof(EnsTile) * ht.size() : sizeof(WfTile) * hw.size();
  const void *tile_src = kind == 0 ? (const void *)ht.data() : (const void *)hw.data();
  cudaError_t err;
  if ((err = cudaMalloc(&e->d_inst, sizeof(EnsInst) * n_inst)) != cudaSuccess ||
      (err = cudaMalloc((void **)&e->d_tiles, tile_bytes)) != cudaSuccess ||
      (err = cudaMalloc(&e->d_sync, sizeof(GridSync))) != cudaSuccess ||
      (err = cudaMemcpy(e->d_inst, hi.data(), sizeof(EnsInst) * n_inst,
                        cudaMemcpyHostToDevice)) != cudaSuccess ||
      (err = cudaMemcpy(e->d_tiles, tile_src, tile_bytes, cudaMemcpyHostToDevice)) !=
          cudaSuccess) {
    cudaFree(e->d_inst);
    cudaFree(e->d_tiles);
    cudaFree(e->d_sync);
    delete e;
    return fm::cuda_status(err, "fm_gs2d_ensemble_create");
  }
  *out = e;
  return FM_OK;
}

extern "C" int fm_gs2d_ensemble_layout(const fm_ensemble *e, int64_t *total_cells,
                                       int64_t *offsets, int *ntiles) {
  FM_CHECK_ARG(e, "fm_gs2d_ensemble_layout: NULL ensemble");
  if (total_cells) *total_cells = e->total;
  if (offsets)
    for (int i = 0; i < e->n_inst; ++i) offsets[i] = e->offsets[i];
  if (ntiles) *ntiles = e->ntiles;
  return FM_OK;
}

namespace {

struct EnsLaunch {
  const void *kern;
  size_t smem;
  int grid;
};

// Kernel choice, shared-memory opt-in and grid size; no stream work, so it
// runs before a graph capture begins.
int ens_prepare(fm_ensemble *e, EnsLaunch *L) {
  if (e->kind == 1) {
    L->kern = pick_wf(e->tb);
    L->smem = 0;
    int sms = 0;
    int st = fm::device_sm_count(&sms);
    if (st) return st;
    int per_sm = 0;
    FM_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, L->kern, 128, 0));
    if (per_sm < 1) {
      fm::set_error("fm_gs2d_ensemble_forward: wavefront kernel does not fit on an SM");
      return FM_ERR_UNSUPPORTED;
    }
    L->grid = std::max(1, std::min((e->ntiles + 3) / 4, sms * per_sm));
    return FM_OK;
  }
  const int tmax = kernel_tmax(e->ts, e->tb);
  L->kern = pick_kernel(e->ts, e->tb);
  L->smem = ens_smem(e->ts, tmax);
  FM_TRY_CUDA(
      cudaFuncSetAttribute(L->kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L->smem));
  int sms = 0;
  int st = fm::device_sm_count(&sms);
  if (st) return st;
  int per_sm = 0;
  FM_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, L->kern, 256, L->smem));
  if (per_sm < 1) {
    fm::set_error("fm_gs2d_ensemble_forward: tile does not fit on an SM");
    return FM_ERR_UNSUPPORTED;
  }
  L->grid = std::max(1, std::min(e->ntiles, sms * per_sm));
  return FM_OK;
}

int ens_launch(fm_ensemble *e, const EnsLaunch &L, float *U, float *V, float *wU, float *wV,
               int steps, long long limit, cudaStream_t s) {
  const void *kern = L.kern;
  const size_t smem = L.smem;
  const int grid = L.grid;
  FM_TRY_CUDA(cudaMemsetAsync(e->d_sync, 0, sizeof(GridSync), s));
  const EnsInst *di = e->d_inst;
  const EnsTile *dt = e->d_tiles;
  int nt = e->ntiles, stp = steps, tb = e->tb;
  GridSync *gs = e->d_sync;
  void *args[] = {&di, &dt, &nt, &U, &V, &wU, &wV, &stp, &tb, &gs, &limit};
  FM_TRY_CUDA(cudaLaunchCooperativeKernel(kern, dim3(grid), e->kind == 1 ? dim3(128) : dim3(32, 8),
                                          args, smem, s));
  return FM_OK;
}

}  // namespace

extern "C" int fm_gs2d_ensemble_forward(fm_ensemble *e, float *U, float *V, float *work_U,
                                        float *work_V, int steps, int use_graph,
                                        void *stream) {
  FM_CHECK_ARG(e && U && V && work_U && work_V, "fm_gs2d_ensemble_forward: NULL argument");
  FM_CHECK_ARG(steps >= 0, "fm_gs2d_ensemble_forward: steps < 0");
  if (steps == 0) return FM_OK;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  EnsLaunch L;
  int pst = ens_prepare(e, &L);
  if (pst) return pst;
  const long long limit = fm::spin_limit();
  if (use_graph) {
    const void *key[5] = {U, V, work_U, work_V, s};
    bool same = e->gexec && e->g_steps == steps && e->g_limit == limit;
    for (int i = 0; i < 5 && same; ++i) same = e->g_key[i] == key[i];
    if (!same) {
      if (e->gexec) {
        cudaGraphExecDestroy(e->gexec);
        e->gexec = nullptr;
      }
      cudaStream_t cap;
      FM_TRY_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
      cudaGraph_t g = nullptr;
      cudaError_t ce = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
      int st = FM_OK;
      if (ce == cudaSuccess) st = ens_launch(e, L, U, V, work_U, work_V, steps, limit, cap);
      cudaError_t ee = cudaStreamEndCapture(cap, &g);
      cudaStreamDestroy(cap);
      if (ce != cudaSuccess) return fm::cuda_status(ce, "cudaStreamBeginCapture");
      if (st) {
        if (g) cudaGraphDestroy(g);
        return st;
      }
      if (ee != cudaSuccess) return fm::cuda_status(ee, "cudaStreamEndCapture");
      ce = cudaGraphInstantiate(&e->gexec, g, 0);
      cudaGraphDestroy(g);
      if (ce != cudaSuccess) {
        e->gexec = nullptr;
        return fm::cuda_status(ce, "cudaGraphInstantiate");
      }
      for (int i = 0; i < 5; ++i) e->g_key[i] = key[i];
      e->g_steps = steps;
      e->g_limit = limit;
    }
    FM_TRY_CUDA(cudaGraphLaunch(e->gexec, s));
  } else {
    int st = ens_launch(e, L, U, V, work_U, work_V, steps, limit, s);
    if (st) return st;
  }
  // Result lands in work_* after an odd number of time blocks: copy back.
  const int blocks = (steps + e->tb - 1) / e->tb;
  if (blocks & 1) {
    const size_t bytes = (size_t)e->total * sizeof(float);
    FM_TRY_CUDA(cudaMemcpyAsync(U, work_U, bytes, cudaMemcpyDeviceToDevice, s));
    FM_TRY_CUDA(cudaMemcpyAsync(V, work_V, bytes, cudaMemcpyDeviceToDevice, s));
  }
  return FM_OK;
}

extern "C" int fm_gs2d_ensemble_status(fm_ensemble *e, void *stream) {
  FM_CHECK_ARG(e, "fm_gs2d_ensemble_status: NULL ensemble");
  GridSync h;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  FM_TRY_CUDA(cudaMemcpyAsync(&h, e->d_sync, sizeof(GridSync), cudaMemcpyDeviceToHost, s));
  FM_TRY_CUDA(cudaStreamSynchronize(s));
  if (h.err) {
    fm::set_error("fm_gs2d_ensemble: grid barrier wait gave up");
    return FM_ERR_TIMEOUT;
  }
  return FM_OK;
}

extern "C" int fm_gs2d_ensemble_destroy(fm_ensemble *e) {
  if (!e) return FM_OK;
  if (e->gexec) cudaGraphExecDestroy(e->gexec);
  cudaFree(e->d_inst);
  cudaFree(e->d_tiles);
  cudaFree(e->d_sync);
  delete e;
  return FM_OK;
}
