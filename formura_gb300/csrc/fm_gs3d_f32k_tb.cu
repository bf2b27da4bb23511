// fm_gs3d_f32k_tb.cu — 3D Gray-Scott, binary32 + Kahan time accumulation,
// temporally blocked: T time steps per HBM round trip.
//
// Formura's temporal blocking unrolls the step graph T times
// (src/Formura/OrthotopeMachine/TemporalBlocking.hs:49-134) and runs it over
// skewed space-time regions whose walls move with the stencil reach
// (src/Formura/MPICxx/Cut.hs:240-281) so that a region's intermediate time
// levels stay in cache.  Here the same idea is an overlapped tile streamed
// along x:
//
//  * A CTA of 32x32 threads owns an input column tile of 32 (y) x 32 (z)
//    cells (periodic wrap) whose inner (32-2T)^2 cells are written back.
//  * It marches along x.  At iteration i it loads plane i (level 0) and each
//    level s = 1..T advances plane i-s by one step, from level s-1's planes
//    i-s-1, i-s, i-s+1.  The x neighbours come from a 3-plane register
//    window per level, the z neighbours from the neighbouring lanes
//    (shuffles; a warp is one y row), the y neighbours from a shared-memory
//    copy of level s-1's plane i-s written by the rows above and below in the
//    previous iteration (double-buffered by parity: ONE __syncthreads per
//    plane for all T levels).  Level s is valid on rows/lanes [s, 32-s); the
//    rows outside skip the level.
//  * The Kahan compensation of each level lives in registers of the thread
//    that owns the cell (a cell's compensation is never read by a neighbour).
//
// HBM traffic per cell and pass: U,V,cU,cV in (16 B, plus the halo re-read
// when it misses L2) and out (16 B), i.e. ~32/T B per lattice update.
//
// Arithmetic: the binary32 fast form of the Gray-Scott step (oracle
// fo_gs3d_run_f32k_fast) — per axis the difference of the two face
// differences, explicit FMAs — so every T gives bit-identical results.
#include <algorithm>

#include "fm_common.cuh"
#include "fm_tune.h"

namespace {

constexpr int kE = 32;  // tile edge (threads per row = rows per CTA)

struct Gs32f {
  float F, Fk, cu, cv, dt;
};

// -x by flipping the sign bit (exact for every x, zeros and NaNs included)
__device__ __forceinline__ float neg(float x) { return __int_as_float(__float_as_int(x) ^ 0x80000000); }

__device__ __forceinline__ int wrap_any(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

// One fast-form step of a cell.
__device__ __forceinline__ void cell_step(float u, float v, float lu, float lv, float cu_in,
                                          float cv_in, const Gs32f &c, float &un, float &vn,
                                          float &cun, float &cvn) {
  const float uvv = (u * v) * v;
  const float dU = fmaf(c.cu, lu, fmaf(c.F, 1.0f - u, -uvv));
  const float dV = fmaf(c.cv, lv, fmaf(-c.Fk, v, uvv));
  const float yu = fmaf(c.dt, dU, -cu_in);
  const float tu = u + yu;
  cun = (tu - u) - yu;
  un = tu;
  const float yv = fmaf(c.dt, dV, -cv_in);
  const float tv = v + yv;
  cvn = (tv - v) - yv;
  vn = tv;
}

// The x-march work of a CTA, as pieces (column c of the (y,z) tile grid, planes
// [x0, x1)).  xchunk > 0: tiles of xchunk planes dealt round-robin to the CTAs.
// xchunk <= 0: the nyz * nx column-planes split into gridDim.x contiguous runs
// of (nearly) equal length, each run cut where it crosses into the next column,
// so a CTA refills its pipeline once or twice per launch instead of once per
// chunk.
// (The host uses runs only when nyz * nx < 2^31.)
struct Pieces {
  int q, qend;  // runs: next column-plane, end; chunks: next tile, -1
  __device__ Pieces(int nyz, int nx, int xchunk) {
    if (xchunk > 0) {
      q = blockIdx.x;
      qend = -1;
    } else {
      const long long total = (long long)nyz * nx;
      q = (int)(total * blockIdx.x / gridDim.x);
      qend = (int)(total * (blockIdx.x + 1) / gridDim.x);
    }
  }
  __device__ bool next(int nyz, int nx, int xchunk, int ntiles, int &c, int &x0, int &x1) {
    if (qend < 0) {
      if (q >= ntiles) return false;
      c = q % nyz;
      x0 = (q / nyz) * xchunk;
      x1 = min(x0 + xchunk, nx);
      q += gridDim.x;
      return true;
    }
    if (q >= qend) return false;
    c = q / nx;
    x0 = q - c * nx;
    x1 = min(nx, x0 + (qend - q));
    q += x1 - x0;
    return true;
  }
};

// x planes per tile: the "gs3d_f32k.xchunk" knob (> 0); 0 (default): the chunk
// that minimises waves x (chunk + 2T pipeline fill) over `resident` CTAs; -1:
// balanced contiguous runs (Pieces).  Runs refill the pipeline less often but
// measured slower (256^3, tb 3: 183 against 240 GLUP/s): the CTAs then march
// through different x ranges at once, and the halo rows that neighbouring
// tiles share no longer meet in L2.
int pick_xchunk(int nx, long long nyz, int resident, int T) {
  int xc = fm::tune_get("gs3d_f32k.xchunk", 0);
  if (xc == -1 && nyz * nx < (1ll << 31)) return 0;
  if (xc <= 0) {
    xc = 0;
    double best = 1e300;
    for (int cand = 4; cand <= nx; cand += 4) {
      const long long tiles = nyz * ((nx + cand - 1) / cand);
      const double cost = (double)((tiles + resident - 1) / resident) * (cand + 2 * T);
      if (cost < best - 1e-9) {
        best = cost;
        xc = cand;
      }
    }
    if (xc <= 0) xc = nx;
  }
  return std::min(xc, nx);
}

template <int T>
__global__ void __launch_bounds__(kE *kE, 1)
    gs3d_f32k_tb(const float *__restrict__ U, const float *__restrict__ V,
                 const float *__restrict__ cU, const float *__restrict__ cV,
                 float *__restrict__ Un, float *__restrict__ Vn, float *__restrict__ cUn,
                 float *__restrict__ cVn, int nx, int ny, int nz, int xchunk, int nty,
                 int ntz, int ntiles, Gs32f c) {
  constexpr int O = kE - 2 * T;  // output tile edge
  // s_u[level][parity][row][lane], same for s_v; levels 0..T-1 feed levels 1..T
  extern __shared__ float smem[];
  float *s_u = smem;
  float *s_v = smem + T * 2 * kE * kE;
  const int lane = threadIdx.x & 31;
  const int row = threadIdx.x >> 5;
  const size_t sx = (size_t)ny * nz;
  Pieces pcs(nty * ntz, nx, xchunk);
  int pc, x0, x1;
  while (pcs.next(nty * ntz, nx, xchunk, ntiles, pc, x0, x1)) {
    const int tz = pc % ntz;
    const int ty = pc / ntz;
    const int gy_out = ty * O + row - T;  // global y of this thread's column
    const int gz_out = tz * O + lane - T;
    const size_t col = (size_t)wrap_any(gy_out, ny) * nz + wrap_any(gz_out, nz);
    const bool writer = row >= T && row < T + O && lane >= T && lane < T + O &&
                        gy_out < ny && gz_out < nz;
    float wu[T][3], wv[T][3];  // level s window: planes (newest-2, newest-1, newest)
    float clu[T], clv[T];      // level s compensation at its newest plane
#pragma unroll
    for (int s = 0; s < T; ++s) {
      wu[s][0] = wu[s][1] = wu[s][2] = 0.0f;
      wv[s][0] = wv[s][1] = wv[s][2] = 0.0f;
      clu[s] = clv[s] = 0.0f;
    }
    // Input planes are prefetched kPF iterations ahead so that their load
    // latency overlaps the T levels of work of the planes before them.
    constexpr int kPF = 2;
    float pu[kPF], pv[kPF], pcu[kPF], pcv[kPF];
#pragma unroll
    for (int k = 0; k < kPF; ++k) {
      const int ip = x0 - T + k;
      const size_t g = (size_t)wrap_any(ip, nx) * sx + col;
      pu[k] = __ldg(U + g);
      pv[k] = __ldg(V + g);
      pcu[k] = __ldg(cU + g);
      pcv[k] = __ldg(cV + g);
    }
    // unrolled by 6 = lcm(3-plane windows, 2 shared-memory parities): the window
    // rotation becomes register renaming instead of moves (210 -> 228 GLUP/s at T = 3)
#pragma unroll 6
    for (int i = x0 - T; i < x1 + T; ++i) {
      const int par = i & 1;
      // ---- level 0: plane i from the prefetch queue; queue plane i+kPF
      const float in_u = pu[0], in_v = pv[0], in_cu = pcu[0], in_cv = pcv[0];
#pragma unroll
      for (int k = 0; k + 1 < kPF; ++k) {
        pu[k] = pu[k + 1];
        pv[k] = pv[k + 1];
        pcu[k] = pcu[k + 1];
        pcv[k] = pcv[k + 1];
      }
      if (i + kPF < x1 + T) {
        // i + kPF lies in [x0 - T + kPF, x1 + T + kPF): one conditional wrap when
        // nx >= 8 (T <= 4), the integer remainder only for smaller grids
        int ip = i + kPF;
        if (nx >= 8)
          ip = ip < 0 ? ip + nx : (ip >= nx ? ip - nx : ip);
        else
          ip = wrap_any(ip, nx);
        const size_t g = (size_t)ip * sx + col;
        pu[kPF - 1] = __ldg(U + g);
        pv[kPF - 1] = __ldg(V + g);
        pcu[kPF - 1] = __ldg(cU + g);
        pcv[kPF - 1] = __ldg(cV + g);
      }
      {
        wu[0][0] = wu[0][1];
        wu[0][1] = wu[0][2];
        wu[0][2] = in_u;
        wv[0][0] = wv[0][1];
        wv[0][1] = wv[0][2];
        wv[0][2] = in_v;
        s_u[((0 * 2 + par) * kE + row) * kE + lane] = in_u;
        s_v[((0 * 2 + par) * kE + row) * kE + lane] = in_v;
      }
      float carry_u = clu[0], carry_v = clv[0];  // level 0's c at plane i-1
      clu[0] = in_cu;
      clv[0] = in_cv;
      // ---- levels 1..T: level s advances plane i-s
#pragma unroll
      for (int s = 1; s <= T; ++s) {
        const float u = wu[s - 1][1], v = wv[s - 1][1];
        // z neighbours from lanes +-1 (lanes 0/31 are never valid at s >= 1)
        const float uzm = __shfl_up_sync(0xffffffffu, u, 1);
        const float uzp = __shfl_down_sync(0xffffffffu, u, 1);
        const float vzm = __shfl_up_sync(0xffffffffu, v, 1);
        const float vzp = __shfl_down_sync(0xffffffffu, v, 1);
        const float cin_u = carry_u, cin_v = carry_v;
        if (row >= s && row < kE - s) {  // warp-uniform
          const int base = ((s - 1) * 2 + (par ^ 1)) * kE;
          const float uym = s_u[(base + row - 1) * kE + lane];
          const float uyp = s_u[(base + row + 1) * kE + lane];
          const float vym = s_v[(base + row - 1) * kE + lane];
          const float vyp = s_v[(base + row + 1) * kE + lane];
          const float lu = (((wu[s - 1][2] - u) - (u - wu[s - 1][0])) + ((uyp - u) - (u - uym))) +
                           ((uzp - u) - (u - uzm));
          const float lv = (((wv[s - 1][2] - v) - (v - wv[s - 1][0])) + ((vyp - v) - (v - vym))) +
                           ((vzp - v) - (v - vzm));
          float un, vn, cun, cvn;
          cell_step(u, v, lu, lv, cin_u, cin_v, c, un, vn, cun, cvn);
          if (s < T) {
            carry_u = clu[s];
            carry_v = clv[s];
            clu[s] = cun;
            clv[s] = cvn;
            wu[s][0] = wu[s][1];
            wu[s][1] = wu[s][2];
            wu[s][2] = un;
            wv[s][0] = wv[s][1];
            wv[s][1] = wv[s][2];
            wv[s][2] = vn;
            s_u[((s * 2 + par) * kE + row) * kE + lane] = un;
            s_v[((s * 2 + par) * kE + row) * kE + lane] = vn;
          } else {
            const int p = i - T;
            if (writer && p >= x0) {
              const size_t g = (size_t)p * sx + col;
              Un[g] = un;
              Vn[g] = vn;
              cUn[g] = cun;
              cVn[g] = cvn;
            }
          }
        }
      }
      __syncthreads();
    }
  }
}

// gs3d_f32k_tbp<T>: the 32x32-thread pipeline of gs3d_f32k_tb with U and V of
// a cell held as one binary32 pair and advanced by packed FADD2/FFMA2
// instructions (the fast form applies the same operation sequence to both
// fields), so each packed instruction does the work of two scalar ones; the
// shared-memory planes interleave (u, v) so that a y neighbour is one 64-bit
// load, and (T <= 3) so is a z neighbour, read from the row's own plane.
// Per cell and level: 10 packed operations for the two Laplacians (the x face
// below a cell is the one above the previous plane's cell, carried in a
// register), 2 packed and 3 scalar for the reaction and 4 packed for the Kahan
// update, against 37 scalar operations.
//
// Each half performs exactly the scalar form's operations: the Laplacian and
// the Kahan update elementwise, the reaction as fma((F, -Fk), (1 - u, v),
// (-uvv, uvv)) with 1 - u and u*v*v scalar and the negations (of uvv and of the
// incoming compensation) by sign-bit flips, so the results (compensations and
// signs of zeros included) equal gs3d_f32k_tb's and the oracle's bit for bit.
template <int T>
__global__ void __launch_bounds__(kE *kE, 1)
    gs3d_f32k_tbp(const float *__restrict__ U, const float *__restrict__ V,
                  const float *__restrict__ cU, const float *__restrict__ cV,
                  float *__restrict__ Un, float *__restrict__ Vn, float *__restrict__ cUn,
                  float *__restrict__ cVn, int nx, int ny, int nz, int xchunk, int nty,
                  int ntz, int ntiles, Gs32f c) {
  constexpr int O = kE - 2 * T;
  // s_w[level][parity][row][lane] = (u, v); levels 0..T-1 feed levels 1..T
  extern __shared__ float2 s_w[];
  const int lane = threadIdx.x & 31;
  const int row = threadIdx.x >> 5;
  // z neighbours: for T <= 3 from the row's own copy of the level's plane in
  // shared memory (two 64-bit loads instead of four shuffles: 260 against 247
  // GLUP/s at T = 3); at T = 4 the extra registers spill, so shuffles
  constexpr bool ZS = T <= 3;
  const int lane_m = lane > 0 ? lane - 1 : 0, lane_p = lane < 31 ? lane + 1 : 31;
  const size_t sx = (size_t)ny * nz;
  const float2 kF = make_float2(c.F, -c.Fk), kD = make_float2(c.cu, c.cv);
  const float2 kDt = make_float2(c.dt, c.dt);
  Pieces pcs(nty * ntz, nx, xchunk);
  int pc, x0, x1;
  while (pcs.next(nty * ntz, nx, xchunk, ntiles, pc, x0, x1)) {
    const int tz = pc % ntz;
    const int ty = pc / ntz;
    const int gy_out = ty * O + row - T;
    const int gz_out = tz * O + lane - T;
    const size_t col = (size_t)wrap_any(gy_out, ny) * nz + wrap_any(gz_out, nz);
    const bool writer = row >= T && row < T + O && lane >= T && lane < T + O &&
                        gy_out < ny && gz_out < nz;
    // level s window of (u, v): planes (newest-1, newest), and the x face
    // difference between newest-1 and the plane before it (computed once, by
    // level s+1 in the previous iteration: the same operands, the same value)
    float2 w[T][2], fx[T];
    float2 cc[T];    // level s compensation at its newest plane
#pragma unroll
    for (int s = 0; s < T; ++s) {
      w[s][0] = w[s][1] = fx[s] = make_float2(0.0f, 0.0f);
      cc[s] = make_float2(0.0f, 0.0f);
    }
    constexpr int kPF = 2;
    float pu[kPF], pv[kPF], pcu[kPF], pcv[kPF];
#pragma unroll
    for (int k = 0; k < kPF; ++k) {
      const int ip = x0 - T + k;
      const size_t g = (size_t)wrap_any(ip, nx) * sx + col;
      pu[k] = __ldg(U + g);
      pv[k] = __ldg(V + g);
      pcu[k] = __ldg(cU + g);
      pcv[k] = __ldg(cV + g);
    }
    // unrolled by 4: a multiple of the 2-plane window and of the 2 shared-memory
    // parities (2: 262, 4: 280, 6: 279 GLUP/s at T = 3)
#pragma unroll 4
    for (int i = x0 - T; i < x1 + T; ++i) {
      const int par = i & 1;
      const float2 in = make_float2(pu[0], pv[0]);
      const float2 in_c = make_float2(pcu[0], pcv[0]);
#pragma unroll
      for (int k = 0; k + 1 < kPF; ++k) {
        pu[k] = pu[k + 1];
        pv[k] = pv[k + 1];
        pcu[k] = pcu[k + 1];
        pcv[k] = pcv[k + 1];
      }
      if (i + kPF < x1 + T) {
        int ip = i + kPF;
        if (nx >= 8)
          ip = ip < 0 ? ip + nx : (ip >= nx ? ip - nx : ip);
        else
          ip = wrap_any(ip, nx);
        const size_t g = (size_t)ip * sx + col;
        pu[kPF - 1] = __ldg(U + g);
        pv[kPF - 1] = __ldg(V + g);
        pcu[kPF - 1] = __ldg(cU + g);
        pcv[kPF - 1] = __ldg(cV + g);
      }
      w[0][0] = w[0][1];
      w[0][1] = in;
      s_w[((0 * 2 + par) * kE + row) * kE + lane] = in;
      float2 carry = cc[0];  // level 0's compensation at plane i-1
      cc[0] = in_c;
#pragma unroll
      for (int s = 1; s <= T; ++s) {
        const float2 m = w[s - 1][0];
        float2 zm, zp;
        if constexpr (!ZS) {
          zm.x = __shfl_up_sync(0xffffffffu, m.x, 1);
          zm.y = __shfl_up_sync(0xffffffffu, m.y, 1);
          zp.x = __shfl_down_sync(0xffffffffu, m.x, 1);
          zp.y = __shfl_down_sync(0xffffffffu, m.y, 1);
        }
        const float2 cin = carry;
        if (row >= s && row < kE - s) {  // warp-uniform
          const int base = ((s - 1) * 2 + (par ^ 1)) * kE;
          const float2 ym = s_w[(base + row - 1) * kE + lane];
          const float2 yp = s_w[(base + row + 1) * kE + lane];
          if constexpr (ZS) {
            // the row's own copy of the plane in shared memory (written by this
            // warp one iteration earlier); lanes 0 and 31 read a clamped index
            // (they are outside every level s >= 1)
            zm = s_w[(base + row) * kE + lane_m];
            zp = s_w[(base + row) * kE + lane_p];
          }
          using fm::f2add;
          using fm::f2sub;
          const float2 fp = f2sub(w[s - 1][1], m);  // x face above; the one below is fx
          const float2 lx = f2sub(fp, fx[s - 1]);
          fx[s - 1] = fp;
          const float2 ly = f2sub(f2sub(yp, m), f2sub(m, ym));
          const float2 lz = f2sub(f2sub(zp, m), f2sub(m, zm));
          const float2 lap = f2add(f2add(lx, ly), lz);
          // the reaction and the Kahan addend as the scalar form writes them; the
          // sign flips are integer operations, off the FMA pipe that the pair
          // operations keep busy
          const float uvv = (m.x * m.y) * m.y;
          const float2 nuvv = make_float2(neg(uvv), uvv);         // (-uvv, uvv)
          const float2 wv = make_float2(1.0f - m.x, m.y);         // (1 - u, v)
          const float2 d = fm::f2fma(kD, lap, fm::f2fma(kF, wv, nuvv));
          const float2 y = fm::f2fma(kDt, d, make_float2(neg(cin.x), neg(cin.y)));
          const float2 t = f2add(m, y);
          const float2 cn = f2sub(f2sub(t, m), y);
          if (s < T) {
            carry = cc[s];
            cc[s] = cn;
            w[s][0] = w[s][1];
            w[s][1] = t;
            s_w[((s * 2 + par) * kE + row) * kE + lane] = t;
          } else {
            const int p = i - T;
            if (writer && p >= x0) {
              const size_t g = (size_t)p * sx + col;
              Un[g] = t.x;
              Vn[g] = t.y;
              cUn[g] = cn.x;
              cVn[g] = cn.y;
            }
          }
        }
      }
      __syncthreads();
    }
  }
}

// gs3d_f32k_tbr<T, RY, W>: the same pipeline with register blocking along y
// and each face difference computed once.
//
//  * A CTA of W warps owns a tile of 32 (z, one cell per lane) x RY*W (y)
//    columns; each thread owns RY consecutive rows of one z column, for every
//    time level.  The inner (RY*W - 2T) x (32 - 2T) columns are written back.
//  * Per level l the thread keeps, for each of its cells and field, P = the
//    value at the plane level l+1 advances next, N = the plane after it, and
//    D = the face difference below P (P - previous plane).  Level l+1 forms
//    the x term as (N - P) - D and keeps N - P as the next D.
//  * y neighbours of the inner rows are the thread's own registers; its first
//    and last rows exchange values with the warps above and below through
//    shared memory (double-buffered by plane parity, one __syncthreads per
//    plane), so shared memory carries 2 of the RY rows.  The y term of row j
//    is f[j+1] - f[j] over the thread's RY+1 face differences.
//  * z: one shuffle brings the value of z+1, the face difference z+1/2 is
//    computed once, and a second shuffle brings the face below from lane - 1.
//  * Every level runs on every row; cells outside a level's valid region
//    (rows and lanes within s of the tile's edge at level s) hold values that
//    no valid cell reads.
// The operations per cell are the fast form's, in its order, so the results
// equal the 32x32-thread kernel's and the oracle's bit for bit.
template <int T, int RY, int W, int PF>
__global__ void __launch_bounds__(32 * W, 1)
    gs3d_f32k_tbr(const float *__restrict__ U, const float *__restrict__ V,
                  const float *__restrict__ cU, const float *__restrict__ cV,
                  float *__restrict__ Un, float *__restrict__ Vn, float *__restrict__ cUn,
                  float *__restrict__ cVn, int nx, int ny, int nz, int xchunk, int nty,
                  int ntz, int ntiles, Gs32f c) {
  constexpr int OY = RY * W - 2 * T, OZ = 32 - 2 * T;  // output tile
  // halo rows hs[level][parity][slot][edge][field][lane]: warp w writes slot w+1
  // (edge 0: its first row, edge 1: its last row); slots 0 and W+1 stay unwritten
  constexpr int kSlot = 2 * 2 * 32, kPar = (W + 2) * kSlot, kLev = 2 * kPar;
  extern __shared__ float hs[];
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const size_t sx = (size_t)ny * nz;
  Pieces pcs(nty * ntz, nx, xchunk);
  int pc, x0, x1;
  while (pcs.next(nty * ntz, nx, xchunk, ntiles, pc, x0, x1)) {
    const int tz = pc % ntz;
    const int ty = pc / ntz;
    const int gz = tz * OZ + lane - T;
    const int zc = wrap_any(gz, nz);
    const bool zw = lane >= T && lane < T + OZ && gz < nz;
    int col[RY];
    bool writer[RY];
#pragma unroll
    for (int j = 0; j < RY; ++j) {
      const int r = w * RY + j;
      const int gy = ty * OY + r - T;
      col[j] = wrap_any(gy, ny) * nz + zc;
      writer[j] = zw && r >= T && r < T + OY && gy < ny;
    }
    float P[T][2][RY], N[T][2][RY], D[T][2][RY], C[T][2][RY];
#pragma unroll
    for (int l = 0; l < T; ++l)
#pragma unroll
      for (int f = 0; f < 2; ++f)
#pragma unroll
        for (int j = 0; j < RY; ++j) P[l][f][j] = N[l][f][j] = D[l][f][j] = C[l][f][j] = 0.0f;
    constexpr int kPF = PF;  // planes prefetched ahead
    float pf[kPF][4][RY];
#pragma unroll
    for (int k = 0; k < kPF; ++k) {
      const size_t g = (size_t)wrap_any(x0 - T + k, nx) * sx;
#pragma unroll
      for (int j = 0; j < RY; ++j) {
        pf[k][0][j] = __ldg(U + g + col[j]);
        pf[k][1][j] = __ldg(V + g + col[j]);
        pf[k][2][j] = __ldg(cU + g + col[j]);
        pf[k][3][j] = __ldg(cV + g + col[j]);
      }
    }
    // unrolled by 2: the P/N roles, the prefetch queue and the parity rotate by renaming
#pragma unroll 2
    for (int i = x0 - T; i < x1 + T; ++i) {
      const int par = i & 1;
      float in[4][RY];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int j = 0; j < RY; ++j) {
          in[a][j] = pf[0][a][j];
#pragma unroll
          for (int k = 0; k + 1 < kPF; ++k) pf[k][a][j] = pf[k + 1][a][j];
        }
      if (i + kPF < x1 + T) {
        int ip = i + kPF;
        if (nx >= 8)
          ip = ip < 0 ? ip + nx : (ip >= nx ? ip - nx : ip);
        else
          ip = wrap_any(ip, nx);
        const size_t g = (size_t)ip * sx;
#pragma unroll
        for (int j = 0; j < RY; ++j) {
          pf[kPF - 1][0][j] = __ldg(U + g + col[j]);
          pf[kPF - 1][1][j] = __ldg(V + g + col[j]);
          pf[kPF - 1][2][j] = __ldg(cU + g + col[j]);
          pf[kPF - 1][3][j] = __ldg(cV + g + col[j]);
        }
      }
      // ---- level 0: plane i
      float carry[2][RY];
#pragma unroll
      for (int f = 0; f < 2; ++f) {
#pragma unroll
        for (int j = 0; j < RY; ++j) {
          P[0][f][j] = N[0][f][j];
          N[0][f][j] = in[f][j];
          carry[f][j] = C[0][f][j];  // level 0's compensation at plane i-1
          C[0][f][j] = in[2 + f][j];
        }
        float *h = hs + par * kPar + (w + 1) * kSlot + f * 32 + lane;
        h[0] = N[0][f][0];
        h[2 * 32] = N[0][f][RY - 1];
      }
      // ---- levels 1..T: level s advances plane i-s from level s-1
#pragma unroll
      for (int s = 1; s <= T; ++s) {
        const int l = s - 1;
        float lap[2][RY];
#pragma unroll
        for (int f = 0; f < 2; ++f) {
          const float *hr = hs + l * kLev + (par ^ 1) * kPar + f * 32 + lane;
          const float top = hr[w * kSlot + 2 * 32];   // last row of warp w-1
          const float bot = hr[(w + 2) * kSlot];      // first row of warp w+1
          float fy_prev = P[l][f][0] - top;           // face below row 0
#pragma unroll
          for (int j = 0; j < RY; ++j) {
            const float p = P[l][f][j];
            const float dn = N[l][f][j] - p;          // x face above
            const float lx = dn - D[l][f][j];
            D[l][f][j] = dn;
            const float fy = (j + 1 < RY ? P[l][f][j + 1] : bot) - p;
            const float ly = fy - fy_prev;
            fy_prev = fy;
            const float zp = __shfl_down_sync(0xffffffffu, p, 1);
            const float fz = zp - p;                  // z face above
            const float fzm = __shfl_up_sync(0xffffffffu, fz, 1);
            const float lz = fz - fzm;
            lap[f][j] = (lx + ly) + lz;
          }
        }
#pragma unroll
        for (int j = 0; j < RY; ++j) {
          float un, vn, cun, cvn;
          cell_step(P[l][0][j], P[l][1][j], lap[0][j], lap[1][j], carry[0][j], carry[1][j], c,
                    un, vn, cun, cvn);
          if (s < T) {
            carry[0][j] = C[s][0][j];
            carry[1][j] = C[s][1][j];
            C[s][0][j] = cun;
            C[s][1][j] = cvn;
            P[s][0][j] = N[s][0][j];
            N[s][0][j] = un;
            P[s][1][j] = N[s][1][j];
            N[s][1][j] = vn;
          } else {
            const int p = i - T;
            if (writer[j] && p >= x0) {
              const size_t g = (size_t)p * sx + col[j];
              Un[g] = un;
              Vn[g] = vn;
              cUn[g] = cun;
              cVn[g] = cvn;
            }
          }
        }
        if (s < T) {
#pragma unroll
          for (int f = 0; f < 2; ++f) {
            float *h = hs + s * kLev + par * kPar + (w + 1) * kSlot + f * 32 + lane;
            h[0] = N[s][f][0];
            h[2 * 32] = N[s][f][RY - 1];
          }
        }
      }
      __syncthreads();
    }
  }
}

template <int T, int RY, int W, int PF>
int launch_tbr(int nx, int ny, int nz, const float *u, const float *v, const float *cu,
               const float *cv, float *un, float *vn, float *cun, float *cvn, const Gs32f &c,
               cudaStream_t s) {
  constexpr int OY = RY * W - 2 * T, OZ = 32 - 2 * T;
  const size_t smem = (size_t)T * 2 * (W + 2) * 2 * 2 * 32 * sizeof(float);
  static bool attr_set[64] = {false};
  int dev = 0;
  FM_TRY_CUDA(cudaGetDevice(&dev));
  if (dev < 64 && !attr_set[dev]) {
    FM_TRY_CUDA(cudaFuncSetAttribute(gs3d_f32k_tbr<T, RY, W, PF>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set[dev] = true;
  }
  int sms = 0;
  int st = fm::device_sm_count(&sms);
  if (st) return st;
  int per_sm = 0;
  FM_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gs3d_f32k_tbr<T, RY, W, PF>,
                                                             32 * W, smem));
  if (per_sm < 1) {
    fm::set_error("fm_gs3d_f32k_tb_forward: register-blocked kernel does not fit on an SM");
    return FM_ERR_UNSUPPORTED;
  }
  const int resident = sms * per_sm;
  const int nty = (ny + OY - 1) / OY, ntz = (nz + OZ - 1) / OZ;
  const long long nyz = (long long)nty * ntz;
  const int xc = pick_xchunk(nx, nyz, resident, T);
  const long long ntiles = xc > 0 ? nyz * ((nx + xc - 1) / xc) : nyz * nx;
  if (ntiles > (1ll << 30)) {
    fm::set_error("fm_gs3d_f32k_tb_forward: grid too large");
    return FM_ERR_UNSUPPORTED;
  }
  const int grid = (int)std::min<long long>(ntiles, resident);
  gs3d_f32k_tbr<T, RY, W, PF><<<grid, 32 * W, smem, s>>>(u, v, cu, cv, un, vn, cun, cvn, nx, ny, nz,
                                                      xc, nty, ntz, (int)ntiles, c);
  FM_TRY_CUDA(cudaGetLastError());
  return FM_OK;
}

template <int T>
int launch_tb(int nx, int ny, int nz, const float *u, const float *v, const float *cu,
              const float *cv, float *un, float *vn, float *cun, float *cvn, const Gs32f &c,
              bool packed, cudaStream_t s) {
  auto kern = packed ? gs3d_f32k_tbp<T> : gs3d_f32k_tb<T>;
  constexpr int O = kE - 2 * T;
  const size_t smem = (size_t)2 * T * 2 * kE * kE * sizeof(float);
  static bool attr_set[2][64] = {};  // per kernel (scalar, packed) and device
  bool *set = attr_set[packed ? 1 : 0];
  int dev = 0;
  FM_TRY_CUDA(cudaGetDevice(&dev));
  if (dev < 64 && !set[dev]) {
    FM_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
    set[dev] = true;
  }
  int sms = 0;
  int st = fm::device_sm_count(&sms);
  if (st) return st;
  int per_sm = 0;
  FM_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kE * kE, smem));
  const int resident = sms * std::max(per_sm, 1);
  const int nty = (ny + O - 1) / O, ntz = (nz + O - 1) / O;
  const long long nyz = (long long)nty * ntz;
  const int xc = pick_xchunk(nx, nyz, resident, T);
  const long long ntiles = xc > 0 ? nyz * ((nx + xc - 1) / xc) : nyz * nx;
  if (ntiles > (1ll << 30)) {
    fm::set_error("fm_gs3d_f32k_tb_forward: grid too large");
    return FM_ERR_UNSUPPORTED;
  }
  const int grid = (int)std::min<long long>(ntiles, resident);
  kern<<<grid, kE * kE, smem, s>>>(u, v, cu, cv, un, vn, cun, cvn, nx, ny, nz, xc, nty, ntz,
                                   (int)ntiles, c);
  FM_TRY_CUDA(cudaGetLastError());
  return FM_OK;
}

}  // namespace

extern "C" int fm_gs3d_f32k_tb_forward(int nx, int ny, int nz, float *U, float *V, float *cU,
                                       float *cV, float *work, int steps, int tb,
                                       const fm_gs_params *p, void *stream) {
  FM_CHECK_ARG(p && U && V && cU && cV && work, "fm_gs3d_f32k_tb_forward: NULL argument");
  FM_CHECK_ARG(nx >= 1 && ny >= 1 && nz >= 1, "fm_gs3d_f32k_tb_forward: empty grid");
  FM_CHECK_ARG((long long)ny * nz < (1ll << 31), "fm_gs3d_f32k_tb_forward: plane too large");
  FM_CHECK_ARG(steps >= 0 && tb >= 0 && tb <= 4,
               "fm_gs3d_f32k_tb_forward: need steps >= 0 and 0 <= tb <= 4 (got %d, %d)", steps,
               tb);
  if (steps == 0) return FM_OK;
  if (tb == 0) tb = fm::tune_get("gs3d_f32k.tb", 3);  // 3: fastest at 256^3 on GB300
  tb = std::max(1, std::min(tb, 4));
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  Gs32f c;
  c.F = (float)p->F;
  c.Fk = (float)(p->F + p->k);
  c.cu = (float)(p->Du / (p->dx * p->dx));
  c.cv = (float)(p->Dv / (p->dx * p->dx));
  c.dt = (float)p->dt;
  const size_t n = (size_t)nx * ny * nz;
  float *cur[4] = {U, V, cU, cV};
  float *nxt[4] = {work, work + n, work + 2 * n, work + 3 * n};
  // 0: one row per warp (32x32 threads); 1: the
  // register-blocked kernel, 4 rows per thread, 8 warps; 2: 2 rows per thread, 16 warps;
  // 3: one row per warp with (u, v) advanced as packed binary32 pairs (the default: fastest
  // measured, 276 against 238 GLUP/s at 256^3, tb 3)
  const int kern = fm::tune_get("gs3d_f32k.kernel", 3);
  int done = 0;
  while (done < steps) {
    const int t = std::min(tb, steps - done);
    int st;
    if (kern == 1 || kern == 2) {
      float *a[8] = {cur[0], cur[1], cur[2], cur[3], nxt[0], nxt[1], nxt[2], nxt[3]};
#define FM_TBR(TT, RR, WW, PP) \
  launch_tbr<TT, RR, WW, PP>(nx, ny, nz, a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], c, s)
#define FM_TBR_T(RR, WW, PP)                                                         \
  (t == 1 ? FM_TBR(1, RR, WW, PP) : t == 2 ? FM_TBR(2, RR, WW, PP)                  \
          : t == 3 ? FM_TBR(3, RR, WW, PP) : FM_TBR(4, RR, WW, PP))
      st = kern == 1 ? FM_TBR_T(4, 8, 2) : FM_TBR_T(2, 16, 2);
#undef FM_TBR_T
#undef FM_TBR
      if (st) return st;
      for (int k = 0; k < 4; ++k) std::swap(cur[k], nxt[k]);
      done += t;
      continue;
    }
#define FM_TB(TT)                                                                          \
  launch_tb<TT>(nx, ny, nz, cur[0], cur[1], cur[2], cur[3], nxt[0], nxt[1], nxt[2], nxt[3], c, \
                kern == 3, s)
    st = t == 1 ? FM_TB(1) : t == 2 ? FM_TB(2) : t == 3 ? FM_TB(3) : FM_TB(4);
#undef FM_TB
    if (st) return st;
    for (int k = 0; k < 4; ++k) std::swap(cur[k], nxt[k]);
    done += t;
  }
  if (cur[0] != U) {
    float *dst[4] = {U, V, cU, cV};
    for (int k = 0; k < 4; ++k)
      FM_TRY_CUDA(cudaMemcpyAsync(dst[k], cur[k], n * sizeof(float), cudaMemcpyDeviceToDevice, s));
  }
  return FM_OK;
}
