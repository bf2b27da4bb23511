// fm_diff2d.cu — 2D diffusion (examples/diffusion.fmr form in 2D), FP64,
// bit-exact with the generated loop nest.
//
// 256^2 FP64 is 512 KB: the whole state lives in L2, and one step is ~1 us of
// FP64 work spread over every SM.  Launch overhead would dominate, so all
// steps run in ONE cooperative persistent launch; blocks meet at a grid
// barrier between steps.  Every wait in that barrier is bounded: past
// fm::spin_limit() polls the block sets an error word and all blocks return,
// and the entry point reports FM_ERR_TIMEOUT.
//
// Per cell (diffusion.fmr:5-7,20):  lap_a = ((d[+1]-d)/2 - (d-d[-1])/2)/2,
//   dens' = dens + coef*(lap_x + lap_y).  x/2 is evaluated as x*0.5 — the same
//   correctly rounded value for every double.  Lanes run along y (the fastest
//   axis); the y flux at +1/2 comes from the next lane by shuffle.
#include <algorithm>
#include <mutex>

#include "fm_common.cuh"
#include "fm_softfp.cuh"
#include "fm_tune.h"

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

// Grid-wide barrier for a cooperative launch; false if the wait gave up.
__device__ bool grid_barrier(GridSync *gs, unsigned nblocks, unsigned &gen_local,
                             long long limit) {
  __shared__ int s_fail;
  __syncthreads();
  if (threadIdx.x == 0) {
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

__device__ __forceinline__ double diff_cell(const double *__restrict__ src, int x, int y,
                                            int nx, int ny, int lane, double coef) {
  const size_t row = (size_t)x * ny;
  const double a = __ldcg(src + row + y);
  const double axp = __ldcg(src + (size_t)fm::wrap_up(x, nx) * ny + y);
  const double axm = __ldcg(src + (size_t)fm::wrap_dn(x, nx) * ny + y);
  double aym = __shfl_up_sync(0xffffffffu, a, 1);
  if (lane == 0) aym = __ldcg(src + row + fm::wrap_dn(y, ny));
  const double f_1 = (a - aym) * 0.5;  // (d - d[y-1])/2
  double f_0 = __shfl_down_sync(0xffffffffu, f_1, 1);
  if (lane == 31) f_0 = (__ldcg(src + row + fm::wrap_up(y, ny)) - a) * 0.5;
  const double e_0 = (axp - a) * 0.5;
  const double e_1 = (a - axm) * 0.5;
  const double e_2 = (e_0 - e_1) * 0.5;
  const double f_2 = (f_0 - f_1) * 0.5;
  const double g = e_2 + f_2;
  const double h = coef * g;
  return a + h;
}

__global__ void __launch_bounds__(256)
    diff2d_persistent(double *a, double *b, int nx, int ny, double coef, int steps,
                      GridSync *gs, long long limit) {
  const int lane = threadIdx.x & 31;
  const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int segs_per_row = ny >> 5;
  const int nseg = nx * segs_per_row;
  unsigned gen = 0;
  double *src = a, *dst = b;
  for (int s = 0; s < steps; ++s) {
    for (int sg = gwarp; sg < nseg; sg += nwarps) {
      const int x = sg / segs_per_row;
      const int y = (sg % segs_per_row) * 32 + lane;
      __stcg(dst + (size_t)x * ny + y, diff_cell(src, x, y, nx, ny, lane, coef));
    }
    if (!grid_barrier(gs, gridDim.x, gen, limit)) return;
    double *t = src;
    src = dst;
    dst = t;
  }
}

__global__ void __launch_bounds__(256)
    diff2d_step(const double *src, double *dst, int nx, int ny, double coef) {
  const int lane = threadIdx.x & 31;
  const int segs_per_row = ny >> 5;
  const int nseg = nx * segs_per_row;
  const int sg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (sg >= nseg) return;
  const int x = sg / segs_per_row;
  const int y = (sg % segs_per_row) * 32 + lane;
  dst[(size_t)x * ny + y] = diff_cell(src, x, y, nx, ny, lane, coef);
}

// x * 0.5 for a double, exactly, on the integer pipe: for normal x with a
// biased exponent >= 2 the product is x with the exponent lowered by one;
// zero is unchanged.  A result that would be subnormal (exponent 1), a
// subnormal x, Inf and NaN take the FP64 multiplication out of line.
static __device__ __noinline__ double half_slow(double x) { return __dmul_rn(x, 0.5); }
__device__ __forceinline__ double half(double x) {
  const unsigned h = (unsigned)__double2hiint(x), l = (unsigned)__double2loint(x);
  const unsigned e = (h >> 20) & 0x7ffu;
  double r = __hiloint2double((int)(h - (1u << 20)), (int)l);
  if (((h << 1) | l) == 0u) r = x;
  else if (e - 2u >= 2045u) r = half_slow(x);
  return r;
}

// diff2d_tb: K steps per grid barrier.  A CTA owns a TX x TY tile; per block of
// k <= K steps it stages the tile and a k-cell periodic halo into shared
// memory, advances k steps there (step s updates the cells within k - s of
// the tile), and writes the tile back.  Per cell, the expressions of
// diff_cell, with x * 0.5 by half() and coef * g by fm::soft::mul_const_s
// (when coef is normal and nonzero): the same values, bit for bit, with half
// of the FP64 instructions.
constexpr int kDX = 16, kDY = 32;
template <int K>
__global__ void __launch_bounds__(256)
    diff2d_tb(double *a, double *b, int nx, int ny, double coef, fm::soft::MulConstS cs,
              int soft_coef, int steps, int ntx, int nty, GridSync *gs, long long limit) {
  constexpr int RX = kDX + 2 * K, RY = kDY + 2 * K;
  __shared__ double buf[2][RX][RY];
  unsigned gen = 0;
  double *src = a, *dst = b;
  const int ntiles = ntx * nty;
  for (int done = 0; done < steps; done += K) {
    const int k = min(K, steps - done);
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const int x0 = (t / nty) * kDX, y0 = (t % nty) * kDY;
      const int rx = kDX + 2 * k, ry = kDY + 2 * k;
      // the staged region spans [x0 - k, x0 + kDX + k): one conditional wrap per
      // coordinate when the grid is at least that wide, the remainder otherwise
      const bool near = nx >= kDX + 2 * K && ny >= kDY + 2 * K;
      {
        // (i, j) of q = threadIdx.x + 256 m, advanced without a division per cell
        int i = threadIdx.x / ry, j = threadIdx.x - i * ry;
        const int di = 256 / ry, dj = 256 - di * ry;
        for (int q = threadIdx.x; q < rx * ry; q += 256) {
          int gx = x0 - k + i, gy = y0 - k + j;
          if (near) {
            gx = gx < 0 ? gx + nx : (gx >= nx ? gx - nx : gx);
            gy = gy < 0 ? gy + ny : (gy >= ny ? gy - ny : gy);
          } else {
            gx %= nx;
            gx = gx < 0 ? gx + nx : gx;
            gy %= ny;
            gy = gy < 0 ? gy + ny : gy;
          }
          buf[0][i][j] = __ldcg(src + (size_t)gx * ny + gy);
          i += di;
          j += dj;
          if (j >= ry) {
            j -= ry;
            ++i;
          }
        }
      }
      __syncthreads();
      for (int st = 1; st <= k; ++st) {
        const int lo = st, hx = rx - st, hy = ry - st;  // update [lo, hx) x [lo, hy)
        const int w = hy - lo;
        const double(*in)[RY] = buf[(st - 1) & 1];
        double(*out)[RY] = buf[st & 1];
        const int di = 256 / w, dj = 256 - di * w;
        int qi = threadIdx.x / w, qj = threadIdx.x - qi * w;
        for (int q = threadIdx.x; q < (hx - lo) * w; q += 256) {
          const int i = lo + qi, j = lo + qj;
          qi += di;
          qj += dj;
          if (qj >= w) {
            qj -= w;
            ++qi;
          }
          const double av = in[i][j];
          const double f_1 = half(av - in[i][j - 1]);
          const double f_0 = half(in[i][j + 1] - av);
          const double e_0 = half(in[i + 1][j] - av);
          const double e_1 = half(av - in[i - 1][j]);
          const double e_2 = half(e_0 - e_1);
          const double f_2 = half(f_0 - f_1);
          const double g = e_2 + f_2;
          const double h = soft_coef ? fm::soft::mul_const_s(g, cs) : coef * g;
          out[i][j] = av + h;
        }
        __syncthreads();
      }
      const double(*res)[RY] = buf[k & 1];
      const int rows = min(kDX, nx - x0), cols = min(kDY, ny - y0);
      {
        int i = threadIdx.x / cols, j = threadIdx.x - i * cols;
        const int di = 256 / cols, dj = 256 - di * cols;
        for (int q = threadIdx.x; q < rows * cols; q += 256) {
          __stcg(dst + (size_t)(x0 + i) * ny + (y0 + j), res[i + k][j + k]);
          i += di;
          j += dj;
          if (j >= cols) {
            j -= cols;
            ++i;
          }
        }
      }
      __syncthreads();
    }
    if (!grid_barrier(gs, gridDim.x, gen, limit)) return;
    double *tmp = src;
    src = dst;
    dst = tmp;
  }
}

std::mutex g_mu;
GridSync *g_sync[64] = {nullptr};

int get_sync(GridSync **out) {
  int dev = 0;
  FM_TRY_CUDA(cudaGetDevice(&dev));
  if (dev >= 64) return FM_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_sync[dev]) FM_TRY_CUDA(cudaMalloc(&g_sync[dev], sizeof(GridSync)));
  *out = g_sync[dev];
  return FM_OK;
}

}  // namespace

extern "C" int fm_diff2d_f64_forward(int nx, int ny, double *dens, double *work,
                                     double coef, int steps, void *stream) {
  FM_CHECK_ARG(dens && work, "fm_diff2d_f64_forward: NULL argument");
  FM_CHECK_ARG(nx >= 1 && ny >= 32 && ny % 32 == 0,
               "fm_diff2d_f64_forward: need ny %% 32 == 0 (got %d x %d)", nx, ny);
  FM_CHECK_ARG(steps >= 0, "fm_diff2d_f64_forward: steps < 0");
  if (steps == 0) return FM_OK;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const size_t n = (size_t)nx * ny;
  int sms = 0;
  int st = fm::device_sm_count(&sms);
  if (st) return st;
  int per_sm = 0;
  FM_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, diff2d_persistent, 256, 0));
  const long long nseg = (long long)nx * (ny / 32);
  const int want = (int)std::min<long long>((nseg + 7) / 8, (long long)sms * std::min(per_sm, 2));
  int coop = 0, dev = 0;
  FM_TRY_CUDA(cudaGetDevice(&dev));
  FM_TRY_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  const int tb = fm::tune_get("diff2d.tb", 4);  // steps per grid barrier; 0: one step per barrier
  if (coop && (tb == 2 || tb == 4 || tb == 8)) {
    const int ntx = (nx + kDX - 1) / kDX, nty = (ny + kDY - 1) / kDY;
    const void *fn = tb == 2 ? (const void *)diff2d_tb<2>
                     : tb == 4 ? (const void *)diff2d_tb<4> : (const void *)diff2d_tb<8>;
    int per = 0;
    FM_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, 256, 0));
    const int grid = (int)std::min<long long>((long long)ntx * nty, (long long)sms * std::max(per, 1));
    if (per >= 1) {
      GridSync *gs = nullptr;
      st = get_sync(&gs);
      if (st) return st;
      FM_TRY_CUDA(cudaMemsetAsync(gs, 0, sizeof(GridSync), s));
      const double ac = coef < 0 ? -coef : coef;
      int soft = ac >= 0x1p-1022 && ac <= 0x1.fffffffffffffp1023;
      fm::soft::MulConstS cs = soft ? fm::soft::make_mul_const_s(coef) : fm::soft::MulConstS();
      double *a = dens, *b = work;
      int nxv = nx, nyv = ny, stv = steps, ntxv = ntx, ntyv = nty;
      double cf = coef;
      long long lim = fm::spin_limit();
      void *args[] = {&a, &b, &nxv, &nyv, &cf, &cs, &soft, &stv, &ntxv, &ntyv, &gs, &lim};
      FM_TRY_CUDA(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(256), args, 0, s));
      GridSync host;
      FM_TRY_CUDA(cudaMemcpyAsync(&host, gs, sizeof(GridSync), cudaMemcpyDeviceToHost, s));
      FM_TRY_CUDA(cudaStreamSynchronize(s));
      if (host.err) {
        fm::set_error("fm_diff2d_f64_forward: grid barrier wait gave up");
        return FM_ERR_TIMEOUT;
      }
      const int blocks = (steps + tb - 1) / tb;
      if (blocks & 1) FM_TRY_CUDA(cudaMemcpyAsync(dens, work, n * sizeof(double),
                                                  cudaMemcpyDeviceToDevice, s));
      return FM_OK;
    }
  }
  if (coop && per_sm >= 1 && want >= 1) {
    GridSync *gs = nullptr;
    st = get_sync(&gs);
    if (st) return st;
    FM_TRY_CUDA(cudaMemsetAsync(gs, 0, sizeof(GridSync), s));
    double *a = dens, *b = work;
    int nxv = nx, nyv = ny, stv = steps;
    double cf = coef;
    long long lim = fm::spin_limit();
    void *args[] = {&a, &b, &nxv, &nyv, &cf, &stv, &gs, &lim};
    FM_TRY_CUDA(cudaLaunchCooperativeKernel((const void *)diff2d_persistent, dim3(want),
                                            dim3(256), args, 0, s));
    GridSync host;
    FM_TRY_CUDA(cudaMemcpyAsync(&host, gs, sizeof(GridSync), cudaMemcpyDeviceToHost, s));
    FM_TRY_CUDA(cudaStreamSynchronize(s));
    if (host.err) {
      fm::set_error("fm_diff2d_f64_forward: grid barrier wait gave up");
      return FM_ERR_TIMEOUT;
    }
    if (steps & 1) FM_TRY_CUDA(cudaMemcpyAsync(dens, work, n * sizeof(double),
                                               cudaMemcpyDeviceToDevice, s));
    return FM_OK;
  }
  // Fallback on devices without cooperative launch: one launch per step.
  double *src = dens, *dst = work;
  const int blocks = (int)((nseg * 32 + 255) / 256);
  for (int i = 0; i < steps; ++i) {
    diff2d_step<<<blocks, 256, 0, s>>>(src, dst, nx, ny, coef);
    std::swap(src, dst);
  }
  FM_TRY_CUDA(cudaGetLastError());
  if (src != dens)
    FM_TRY_CUDA(cudaMemcpyAsync(dens, src, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  return FM_OK;
}

// ---------------------------------------------------------------------------
// No-allocation variant.
//
// Some callers cannot call cudaMalloc: a host application that reserved its
// whole device-memory budget up front and hands the library only its own
// arrays, or a latency-critical loop that must not hit cudaMalloc's implicit
// device-wide synchronization.  For them fm_diff2d_f64_forward_noalloc takes
// only the state array; its ping-pong buffer and grid-barrier word live in
// the file-scope device arrays below (8 MB + 256 B, held by every GPU that
// loads this library until the process exits).
namespace {

constexpr size_t kNoAllocMaxCells = (size_t)FM_DIFF2D_NOALLOC_MAX_CELLS;
static __device__ __align__(256) double g_noalloc_work[kNoAllocMaxCells];
static __device__ __align__(256) GridSync g_noalloc_sync[1];

struct NoAllocScratch {
  double *work;
  GridSync *sync;
};

std::mutex g_noalloc_mu;
bool g_noalloc_ready[64] = {false};
NoAllocScratch g_noalloc[64];

// Device addresses of the scratch arrays for the current device.  In host
// code g_noalloc_work names a host-side stand-in, not device memory, so the
// address a kernel may use is looked up once per device (first call on that
// device) with cudaGetSymbolAddress and cached.
int noalloc_scratch(NoAllocScratch *out) {
  int dev = 0;
  FM_TRY_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    fm::set_error("fm_diff2d_f64_forward_noalloc: device index %d not supported", dev);
    return FM_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ready[dev]) {
    NoAllocScratch s;
    FM_TRY_CUDA(cudaGetSymbolAddress((void **)&s.work, g_noalloc_work));
    FM_TRY_CUDA(cudaGetSymbolAddress((void **)&s.sync, g_noalloc_sync));
    g_noalloc[dev] = s;
    g_noalloc_ready[dev] = true;
  }
  *out = g_noalloc[dev];
  return FM_OK;
}

}  // namespace

extern "C" int fm_diff2d_f64_forward_noalloc(int nx, int ny, double *dens, double coef,
                                             int steps, void *stream) {
  FM_CHECK_ARG(dens, "fm_diff2d_f64_forward_noalloc: dens is NULL");
  FM_CHECK_ARG(nx >= 1 && ny >= 32 && ny % 32 == 0,
               "fm_diff2d_f64_forward_noalloc: need ny %% 32 == 0 (got %d x %d)", nx, ny);
  FM_CHECK_ARG((size_t)nx * (size_t)ny <= kNoAllocMaxCells,
               "fm_diff2d_f64_forward_noalloc: %d x %d = %zu cells exceeds the %zu-cell "
               "static scratch (FM_DIFF2D_NOALLOC_MAX_CELLS); use fm_diff2d_f64_forward",
               nx, ny, (size_t)nx * (size_t)ny, kNoAllocMaxCells);
  FM_CHECK_ARG(steps >= 0, "fm_diff2d_f64_forward_noalloc: steps < 0");
  if (steps == 0) return FM_OK;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  NoAllocScratch sc;
  int st = noalloc_scratch(&sc);
  if (st) return st;
  int dev = 0, coop = 0, sms = 0;
  FM_TRY_CUDA(cudaGetDevice(&dev));
  FM_TRY_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  if (!coop) {
    fm::set_error("fm_diff2d_f64_forward_noalloc: device has no cooperative launch");
    return FM_ERR_UNSUPPORTED;
  }
  st = fm::device_sm_count(&sms);
  if (st) return st;
  // The kernel of fm_diff2d_f64_forward: diff2d_tb<K> with K steps per grid
  // barrier ("diff2d.tb", default 4), or one step per barrier for tb 0.
  const int tb = fm::tune_get("diff2d.tb", 4);
  const bool tiled = tb == 2 || tb == 4 || tb == 8;
  const void *fn = !tiled    ? (const void *)diff2d_persistent
                   : tb == 2 ? (const void *)diff2d_tb<2>
                   : tb == 4 ? (const void *)diff2d_tb<4>
                             : (const void *)diff2d_tb<8>;
  int per_sm = 0;
  FM_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, 0));
  if (per_sm < 1) {
    fm::set_error("fm_diff2d_f64_forward_noalloc: kernel does not fit on an SM");
    return FM_ERR_UNSUPPORTED;
  }
  // The barrier word keeps the previous call's contents: it must start at zero.
  FM_TRY_CUDA(cudaMemsetAsync(sc.sync, 0, sizeof(GridSync), s));
  double *a = dens, *b = sc.work;
  int nxv = nx, nyv = ny, stv = steps;
  double cf = coef;
  GridSync *gs = sc.sync;
  long long lim = fm::spin_limit();
  bool odd;
  if (tiled) {
    const int ntx = (nx + kDX - 1) / kDX, nty = (ny + kDY - 1) / kDY;
    const int grid = (int)std::min<long long>((long long)ntx * nty, (long long)sms * per_sm);
    const double ac = coef < 0 ? -coef : coef;
    int soft = ac >= 0x1p-1022 && ac <= 0x1.fffffffffffffp1023;
    fm::soft::MulConstS cs = soft ? fm::soft::make_mul_const_s(coef) : fm::soft::MulConstS();
    int ntxv = ntx, ntyv = nty;
    void *args[] = {&a, &b, &nxv, &nyv, &cf, &cs, &soft, &stv, &ntxv, &ntyv, &gs, &lim};
    FM_TRY_CUDA(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(256), args, 0, s));
    odd = ((steps + tb - 1) / tb) & 1;
  } else {
    const long long nseg = (long long)nx * (ny / 32);
    const int grid = (int)std::max<long long>(
        1, std::min<long long>((nseg + 7) / 8, (long long)sms * std::min(per_sm, 2)));
    void *args[] = {&a, &b, &nxv, &nyv, &cf, &stv, &gs, &lim};
    FM_TRY_CUDA(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(256), args, 0, s));
    odd = steps & 1;
  }
  GridSync host;
  FM_TRY_CUDA(cudaMemcpyAsync(&host, sc.sync, sizeof(GridSync), cudaMemcpyDeviceToHost, s));
  // After an odd number of passes the result is in the static scratch: the
  // copy back into dens is queued before the synchronization below, so that
  // dens is final (and the scratch free for the next call) when this returns.
  if (odd)
    FM_TRY_CUDA(cudaMemcpyAsync(dens, sc.work, (size_t)nx * ny * sizeof(double),
                                cudaMemcpyDeviceToDevice, s));
  FM_TRY_CUDA(cudaStreamSynchronize(s));
  if (host.err) {
    fm::set_error("fm_diff2d_f64_forward_noalloc: grid barrier wait gave up");
    return FM_ERR_TIMEOUT;
  }
  return FM_OK;
}
