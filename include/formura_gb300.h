/*
 * formura_gb300.h — thin C ABI of the GB300 stencil engine (libformura_gb300.so).
 *
 * Formura's generated C runs its time-step loop inside Formura_Forward
 * (src/Formura/MPICxx/Translate.hs:1106-1131): M = monitor_interval steps of
 * region loop nests (genComputation, Translate.hs:671-737), ridge copies
 * (genStagingCode, :742-796) and MPI facet exchanges (:798-836).  This library
 * replaces that body.  The per-program host code that the back end
 * (formura_gb300/backend.py) emits — the header with `struct Formura_Navigator`,
 * the global state arrays, Formura_Init and Formura_Forward — calls the entry
 * points below with plain device pointers.
 *
 * Conventions
 *  - Arrays are dense, row-major, last axis fastest (U[x][y][z]), exactly the
 *    index order of the generated code; periodic boundaries are applied by index
 *    wrap inside the kernels (the one-GPU form of the self-send halo exchange,
 *    Translate.hs:1062-1068).
 *  - Every entry point returns an fm_status (0 = FM_OK).  On error,
 *    fm_last_error() returns a message for the calling thread.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *    Entry points enqueue work and return; they do not synchronize unless the
 *    comment says so.
 *  - Device arrays must be 256-byte aligned (cudaMalloc guarantees it).
 *  - There is no CPU fallback: without a CUDA device every compute entry point
 *    returns FM_ERR_CUDA.
 */
#ifndef FORMURA_GB300_H
#define FORMURA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Exported even when the library is compiled with -fvisibility=hidden. */
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

typedef enum {
  FM_OK = 0,
  FM_ERR_ARG = 1,         /* bad size, pointer or parameter */
  FM_ERR_CUDA = 2,        /* a CUDA runtime call failed (no device, launch error, ...) */
  FM_ERR_TIMEOUT = 3,     /* a bounded device-side wait gave up (see fm_*_status words) */
  FM_ERR_NONFINITE = 4,   /* a conserved-total check found NaN or Inf */
  FM_ERR_UNSUPPORTED = 5, /* shape or option this build does not handle */
  FM_ERR_NOMEM = 6        /* device allocation failed */
} fm_status;

/* ---- runtime helpers used by the emitted host code ----------------------- */

/* Message for the last failing call on this thread ("" if none). */
const char *fm_last_error(void);
/* Static name of a status code. */
const char *fm_status_name(int status);
/* Library version string, e.g. "formura-gb300 0.1 sm_103a". */
const char *fm_version(void);
/* Number of visible CUDA devices (0 when there is none; never fails). */
int fm_device_count(void);

int fm_malloc(void **ptr, size_t bytes);
int fm_free(void *ptr);
int fm_memset(void *ptr, int value, size_t bytes, void *stream);
int fm_memcpy_h2d(void *dst, const void *src, size_t bytes, void *stream);
int fm_memcpy_d2h(void *dst, const void *src, size_t bytes, void *stream);
int fm_memcpy_d2d(void *dst, const void *src, size_t bytes, void *stream);
int fm_stream_sync(void *stream);
/* Page-locks an existing host range (the generated globals) so that the
 * copies above run at full link speed; fm_host_unregister undoes it. */
int fm_host_register(void *ptr, size_t bytes);
int fm_host_unregister(void *ptr);

/* ---- Gray-Scott reaction-diffusion ---------------------------------------- */

/* Constants of the Gray-Scott .fmr forms (examples/pearson-2d.fmr:16-17,
 * examples/pearson-3d.fmr:3-4 in the F,k parameterisation). */
typedef struct {
  double F, k, Du, Dv, dt, dx;
} fm_gs_params;

/*
 * 3D Gray-Scott in the examples/pearson-3d.fmr form, FP64, bit-exact with the
 * generated loop nest (Translate.hs:671-737 over the DAG of pearson-3d.fmr:13-24
 * with the F,k reaction of pearson-2d.fmr:21-22):
 *   lap_a(W) = ((W[+1]-W)/dx - (W-W[-1])/dx)/dx,  lap = (lap_x + lap_y) + lap_z
 *   U' = U + dt*(((-(U*V*V)) + F*(1-U)) + Du*lap(U))
 *   V' = V + dt*(((U*V*V) - (F+k)*V) + Dv*lap(V))
 * Advances U,V ([nx][ny][nz] device arrays) by `steps` in place.  work_U,
 * work_V are device arrays of the same size used as the other half of the
 * ping-pong pair (contents on return unspecified).
 * Replaces the Computation loop nests of Formura_Forward
 * (Translate.hs:1121-1131, genComputation :671-737).
 * Requires nz % 32 == 0, ny % 16 == 0, nx >= 1, and 2^-40 <= dx <= 2^40.
 */
int fm_gs3d_f64_forward(int nx, int ny, int nz, double *U, double *V,
                        double *work_U, double *work_V, const fm_gs_params *p,
                        int steps, void *stream);

/*
 * 3D Gray-Scott, the same generated DAG evaluated in binary32 (the .fmr
 * program with `float` state), with compensated (Kahan) time accumulation:
 * per field y = dt*dW - cW; t = W + y; cW = (t - W) - y; W = t.
 * U,V,cU,cV are [nx][ny][nz] float device arrays (cU,cV = running
 * compensation, zero them before the first call); work must hold 4*nx*ny*nz
 * floats.  One step per launch.  Bit-exact with the binary32 restatement of
 * the DAG without FMA contraction.
 * Requires nz % 32 == 0, ny % 8 == 0, 2^-20 <= (float)dx <= 2^20.
 */
int fm_gs3d_f32k_forward(int nx, int ny, int nz, float *U, float *V, float *cU,
                         float *cV, float *work, int steps,
                         const fm_gs_params *p, void *stream);

/*
 * 3D Gray-Scott in binary32 with Kahan time accumulation, temporally blocked:
 * `tb` steps (1..4; 0 = tuned default) run per HBM round trip, streaming
 * overlapped 32x32 (y,z) tiles along x (Formura's temporal blocking,
 * src/Formura/OrthotopeMachine/TemporalBlocking.hs:49-134 and the skewed
 * regions of src/Formura/MPICxx/Cut.hs:240-281, as on-chip pipelines).
 * Arithmetic is the binary32 "fast form" (per axis the difference of the
 * two face differences, (W[+1]-W) - (W-W[-1]),
 * explicit FMAs, constants Du/dx^2, Dv/dx^2, F+k rounded once to float):
 * results are bit-identical for every tb and are scored by their error against
 * the FP64 run.  Same arrays as fm_gs3d_f32k_forward; any nx, ny, nz >= 1.
 */
int fm_gs3d_f32k_tb_forward(int nx, int ny, int nz, float *U, float *V,
                            float *cU, float *cV, float *work, int steps,
                            int tb, const fm_gs_params *p, void *stream);

/* ---- 2D Gray-Scott and uneven ensembles ------------------------------------- */

/*
 * 2D Gray-Scott in the examples/pearson-2d.fmr form, binary32, one instance:
 * the float evaluation of the DAG of examples-generated/pearson.c:138-208
 * (no FMA contraction; Du/(dx*dx), Dv/(dx*dx), F+k evaluated in float in DAG
 * order).  U,V are [nx][ny]; work_U, work_V the ping-pong pair.  One launch
 * per step (the "sequential per-instance launches" baseline of ensembles).
 */
int fm_gs2d_f32_forward(int nx, int ny, float *U, float *V, float *work_U,
                        float *work_V, const fm_gs_params *p, int steps,
                        void *stream);

/*
 * An ensemble of independent periodic 2D Gray-Scott instances of uneven sizes
 * (n_i x n_i) and their own F_i, k_i, sharing Du, Dv, dt, dx — the batched
 * form of the pearson-2d program.  All instances' U (and V) are stored back to
 * back in one float buffer; fm_gs2d_ensemble_layout gives each instance's
 * first cell.  Per cell the arithmetic is that of fm_gs2d_f32_forward
 * (bit-identical results).
 *
 * fm_gs2d_ensemble_create builds the plan (device instance and tile tables):
 * `tile` = output tile edge of the shared-memory kernel (32 or 64), or 1 for
 * the wavefront kernel (one warp streams a 64-cell y strip along x, time
 * levels pipelined in registers); 0 = tuned default; `tb` = time steps per
 * pass over the state (1..8; 0 = tuned default).
 * fm_gs2d_ensemble_forward advances every instance `steps` steps in ONE
 * cooperative persistent launch (grid barrier between passes, bounded
 * waits); with use_graph != 0 the launch is captured once into a CUDA graph
 * (re-captured when the buffers, stream, step count or "sync.spin_limit"
 * change) and replayed.
 * work_U, work_V: ping-pong buffers of total_cells floats.
 * fm_gs2d_ensemble_status synchronizes `stream` and returns FM_ERR_TIMEOUT if
 * the last run's grid barrier gave up.
 */
typedef struct fm_ensemble fm_ensemble;
int fm_gs2d_ensemble_create(fm_ensemble **out, int n_inst, const int *sizes,
                            const double *F, const double *k, double Du,
                            double Dv, double dt, double dx, int tile, int tb);
int fm_gs2d_ensemble_layout(const fm_ensemble *e, int64_t *total_cells,
                            int64_t *offsets, int *ntiles);
int fm_gs2d_ensemble_forward(fm_ensemble *e, float *U, float *V, float *work_U,
                             float *work_V, int steps, int use_graph,
                             void *stream);
int fm_gs2d_ensemble_status(fm_ensemble *e, void *stream);
int fm_gs2d_ensemble_destroy(fm_ensemble *e);

/* ---- 3D MHD ----------------------------------------------------------------- */

/*
 * Time steps of the reference program examples/3d-mhd-rk4.fmr: 9 fields
 * (dens = perturbation of dens0 = 1, vx, vy, vz, Bx, By, Bz, s, Psi), each
 * an [n][n][n] device array, periodic, dx = 1/n, dt = 0.1/n as the program
 * defines them.  Per step: four manifested low-storage Runge-Kutta stages
 * (q4 = S + dt/4 f(S), q3 = S + dt/3 f(q4), q2 = S + dt/2 f(q3),
 * next = S + dt f(q2); f = ddt_sys with 4th-order central differences,
 * 3d-mhd-rk4.fmr:83-110), then the artificial-viscosity fluxes of `next`
 * along x, y, z applied in turn, dens floored at -0.9, and
 * s += numerical_heat (3d-mhd-rk4.fmr:112-145).  `work` holds 18*n^3
 * elements.  Replaces the Computation loop nests of that program's
 * Formura_Forward (src/Formura/MPICxx/Translate.hs:671-737).
 *
 * fm_mhd_forward_f64: all-FP64, bit-exact with the generated DAG.
 * fm_mhd_forward_f32: the bulk in binary32; the numerical-heat (energy)
 * update of s in FP64.  Requires n >= 5.
 */
int fm_mhd_forward_f64(int n, double *const fields[9], double *work, int steps,
                       void *stream);
int fm_mhd_forward_f32(int n, float *const fields[9], float *work, int steps,
                       void *stream);
/*
 * FP64 conserved totals of an MHD state into out_device[0..3]: sum of dens,
 * sum of (1/2 (1+dens)|v|^2 + |B|^2/(8 pi)), sum of s, sum of (1+dens) vx.
 * fp64 != 0: fields are double, else float.  `partials` holds
 * fm_mhd_totals_scratch_elems(n) doubles.  Deterministic for a given n.
 */
size_t fm_mhd_totals_scratch_elems(int n);
int fm_mhd_totals(int n, int fp64, void *const fields[9], double *partials,
                  double *out_device, void *stream);

/* ---- tensor-core building block ---------------------------------------------- */

/*
 * C[M x N] (fp32, row-major) = A[M x K] * B[N x K]^T with A, B row-major
 * bf16 (16-byte aligned), on the tcgen05 tensor cores with FP32 accumulation
 * in tensor memory.  No counterpart in the reference (it has no GPU code);
 * the building block of the learned surrogate's convolutions.
 * M % 128 == 0, N % 64 == 0, K % 64 == 0.  *err_device (an int the caller
 * zeroes) becomes 1 if a bounded wait on the tensor core gave up.
 */
int fm_tc_gemm_bf16(int M, int N, int K, const void *A, const void *B, float *C,
                    int *err_device, void *stream);

/* ---- learned 16-step surrogate (BF16 tcgen05 convolutions) ------------------- */

/*
 * No counterpart in the reference (a new form: a convolutional neural operator
 * that jumps 16 steps of the pearson-2d Gray-Scott program, with the plain
 * stencil as its fallback and as the reference for its error).
 *
 * Latent tensors are NHWC bf16 with a one-pixel periodic halo,
 * [B][H+2][W+2][64]; weights [cout][9][64] bf16 (tap t = (dy+1)*3 + dx+1).
 *
 * fm_conv3x3_fwd_bf16: y = act(conv3x3(x, w) (+ bias) (* gelu'(gate)) (+ resid))
 * on the tcgen05 tensor cores (implicit GEMM, FP32 accumulation in tensor
 * memory).  cout 32 or 64; H, W >= 2 (cout 32: B*H*W % 128 == 0); act 0 =
 * none, 1 = GELU (erf).  cout 64 runs the weight-resident persistent kernel.
 * Outputs (any subset): z_pad_out = value before act (bf16, padded),
 * y_pad_out (bf16, padded, halo written), y_f32_out ([B][H][W][cout] fp32).
 * fm_conv3x3_wgrad_bf16: dwt[t][ci][co] += sum_p dy[p][co] * x[p+t][ci]
 * (split-K over pixels, fp32 atomics; zero dwt first).
 * *err_device becomes 1 if a bounded tensor-core wait gave up.
 */
int fm_conv3x3_fwd_bf16(int B, int H, int W, int cout, const void *x_pad,
                        const void *w, const float *bias, const void *gate_pad,
                        const void *resid_pad, int act, void *z_pad_out,
                        void *y_pad_out, float *y_f32_out, int *err_device,
                        void *stream);
int fm_conv3x3_wgrad_bf16(int B, int H, int W, int cout, const void *x_pad,
                          const void *dy_pad, float *dwt, int *err_device,
                          void *stream);

/* Latent packing: (U, V, F, k) of B periodic N x N fields -> [B][N/4+2][N/4+2][64]
 * (4x4 space-to-depth, channel q*16 + sy*4 + sx, q = U, V, (F-0.04)*50,
 * (k-0.06)*100; halo filled).  Unpacking: U += scale*y[..][sub],
 * V += scale*y[..][16+sub] from an fp32 latent [B][N/4][N/4][64]. */
int fm_sur_pack(int B, int N, const float *U, const float *V, const float *F,
                const float *K, void *xpad, void *stream);
int fm_sur_unpack(int B, int N, const float *y, float *U, float *V, float scale,
                  void *stream);
/* Training: MSE of the latent prediction y against (S1 - S0)/scale; writes
 * grad_scale * dL/dy as a padded bf16 latent and adds the loss to *loss. */
int fm_sur_loss_grad(int B, int N, const float *y, const float *U0,
                     const float *V0, const float *U1, const float *V1,
                     void *dy_pad, float *loss, float scale, float grad_scale,
                     void *stream);
/* db[c] += sum over interior pixels of dy_pad[..][c] (n = latent edge). */
int fm_sur_bias_grad(int B, int n, const void *dy_pad, float *db, void *stream);
/* wf[ci][t][co] = w[co][8-t][ci]: data-gradient weights as a forward conv. */
int fm_sur_flip(const void *w, void *wf, void *stream);
/* One Adam step on fp32 master weights w [64][9][64] (gradient dwt[9][ci][co])
 * and bias b [64]; writes the bf16 copy wb.  mask_co >= 0 pins output
 * channels >= mask_co to zero.  step counts from 1. */
int fm_sur_adam(float *w, const float *gwt, float *mw, float *vw, void *wb,
                float *b, const float *gb, float *mb, float *vb, float lr,
                float b1, float b2, float eps, int step, int mask_co,
                void *stream);
/* dz = dh * gelu'(z) over padded bf16 latents of `count` elements. */
int fm_sur_gelu_bwd(long long count, const void *dh, const void *z, void *dz,
                    void *stream);

/* ---- 2D diffusion --------------------------------------------------------- */

/*
 * 2D diffusion in the examples/diffusion.fmr form reduced to 2D, FP64, bit-exact:
 *   dens' = dens + (Dt / pow(Dx,2)) * (lap_x + lap_y),
 *   lap_a = ((d[+1]-d)/2 - (d-d[-1])/2)/2.
 * `coef` is the node Dt / Dx**2, evaluated by the caller in double with the
 * host libm pow exactly as the generated code does (diffusion.fmr:20,
 * Translate.hs:594).  dens is [nx][ny]; work is another nx*ny doubles.
 * Runs all `steps` in one persistent launch when the grid fits the device
 * (grid barriers with bounded waits); else one launch per step.
 * Requires ny % 32 == 0.
 */
int fm_diff2d_f64_forward(int nx, int ny, double *dens, double *work,
                          double coef, int steps, void *stream);

/*
 * fm_diff2d_f64_forward without any device allocation.  No counterpart in the
 * reference (its generated C allocates nothing on a GPU).
 *
 * For callers that cannot call cudaMalloc: a host application that reserved
 * its device-memory budget up front and passes only its own arrays, or a
 * latency-critical loop that must not trigger cudaMalloc's implicit
 * device-wide synchronization.  The caller passes only the state array; the
 * ping-pong buffer and the grid-barrier word are a static device array of
 * FM_DIFF2D_NOALLOC_MAX_CELLS doubles (8 MB) plus 256 bytes inside the
 * library, which every GPU that loads the library holds until the process
 * exits.  nx*ny above FM_DIFF2D_NOALLOC_MAX_CELLS returns FM_ERR_ARG.
 *
 * Runs the kernel of fm_diff2d_f64_forward (the same "diff2d.tb" choice) on
 * the static scratch: same results, bit for bit.  The first call on a
 * device looks up the scratch's device address (cudaGetSymbolAddress), which
 * may load the library's device code on that device; make that first call
 * before any stream capture.  Every call shares the one scratch area, so
 * calls whose work overlaps on the GPU (different streams, or different host
 * threads, without ordering between them) race; the barrier word is cleared
 * at the start of each call.  Synchronizes `stream` before returning, after
 * every copy of the call (including the copy of the result out of the
 * scratch), so on return dens is final for any stream and the scratch is
 * free for the next call.
 */
#define FM_DIFF2D_NOALLOC_MAX_CELLS (1 << 20)
int fm_diff2d_f64_forward_noalloc(int nx, int ny, double *dens, double coef,
                                  int steps, void *stream);

/* ---- conserved totals ------------------------------------------------------ */

/*
 * Sum of n doubles (mass/energy totals) into *out_device (one double in device
 * memory).  Deterministic: a fixed two-level tree whose shape depends only on
 * n.  `partials` is caller-provided scratch of fm_sum_f64_scratch_elems(n)
 * doubles.  A NaN or Inf anywhere in the input propagates to the total; the
 * emitted host code reads it back and returns FM_ERR_NONFINITE.
 */
size_t fm_sum_f64_scratch_elems(int64_t n);
int fm_sum_f64(int64_t n, const double *a, double *partials, double *out_device,
               void *stream);
/* Same tree over binary32 input, accumulated in double (FP32 state totals). */
int fm_sum_f32_as_f64(int64_t n, const float *a, double *partials,
                      double *out_device, void *stream);

/* ---- plane snapshots (monitor output) --------------------------------------- */

/*
 * No counterpart in the reference: its drivers read mid-planes of the host
 * globals for their monitor files (examples/pearson-3d-main.cpp:116-157).
 * With the state resident on the GPU, fm_snapshot_begin gathers the plane
 * (axis, index) of a row-major device array with `shape` into device staging
 * on `stream` (ordered before every later kernel on that stream, so the array
 * may be overwritten right after) and copies it to pinned host staging on an
 * internal stream; fm_snapshot_wait blocks until that copy is done and
 * writes the plane (row-major over the remaining axes) to host_out, which
 * must hold fm_snapshot_plane_elems(s, axis) elements.  One snapshot may be
 * in flight per object.  elem_size: 1, 2, 4 or 8 bytes; 1 <= ndim <= 8.
 */
typedef struct fm_snapshot fm_snapshot;
int fm_snapshot_create(fm_snapshot **out, int ndim, const int *shape, int elem_size);
long long fm_snapshot_plane_elems(const fm_snapshot *s, int axis);
int fm_snapshot_begin(fm_snapshot *s, const void *array, int axis, int index, void *stream);
int fm_snapshot_wait(fm_snapshot *s, void *host_out);
void fm_snapshot_destroy(fm_snapshot *s);

/* ---- TMA tensor maps -------------------------------------------------------------- */

/*
 * No counterpart in the reference (it has no GPU code): encodes into `map` (a
 * 128-byte, 64-byte-aligned CUtensorMap) a tiled TMA description of a dense
 * row-major [n0][n1][n2] array of 4- or 8-byte elements at `base`, with a box
 * of box0 x box1 x box2 elements (each 1..256).  The generated temporally
 * blocked kernels of .fmr programs stage the planes of their tiles with it.
 * Requires base 16-byte aligned and n2, box2 rows of a multiple of 16 bytes;
 * FM_ERR_UNSUPPORTED when the driver offers no encoder.
 */
int fm_tensor_map_3d(void *map, const void *base, int elem_bytes, int n0, int n1, int n2,
                     int box0, int box1, int box2);

/* ---- tuning ------------------------------------------------------------------ */

/*
 * Process-wide tuning knobs.  Every knob has an automatic default; a set value
 * overrides it for later calls.  No knob changes results (all variants of a
 * stencil kernel are bit-exact with each other).  Known keys:
 *   "gs3d_f64.kernel"  0 auto, 1 tile kernel (any nz), 2 full-z-row kernel (nz <= 256)
 *   "gs3d_f64.div"     0 Markstein division (3 FP64 ops), 1 integer-corrected (1 FP64 op +
 *                      128-bit integer products), 2 residual + integer compare
 *                      (2 FP64 ops), 3 no FP64 op (significand from 32-bit partial
 *                      products, rounding from an exact 64-bit remainder; default)
 *   "gs3d_f64.mul"     with div 3: 0 hardware multiplications, 1 multiplications by the
 *                      constants F, F+k, Du, Dv, dt on the integer pipes (default), 2 all
 *                      of them
 *   "gs3d_f64.ry"      with div 3, y cells per thread of the full-z-row kernel: 2 (3 CTAs
 *                      per SM; default) or 4 (2 CTAs per SM)
 *   "gs3d_f64.xchunk"  x planes per CTA tile (0 = automatic)
 *   "gs3d_f32k.tb"     default temporal-blocking depth of fm_gs3d_f32k_tb_forward (1..4)
 *   "gs3d_f32k.kernel" form of fm_gs3d_f32k_tb_forward: 0 one row per warp, 1 and 2
 *                      register-blocked (4 or 2 rows per thread), 3 one row per warp with
 *                      (u, v) advanced as packed binary32 pairs (default)
 *   "gs3d_f32k.xchunk" x planes per tile of the temporally blocked kernel (0 = automatic)
 *   "gs2d_ens.tile"    default ensemble kernel: 1 wavefront strips (default), 32 or 64
 *                      shared-memory tiles of that edge
 *   "gs2d_ens.xchunk"  x planes per wavefront strip (default 64)
 *   "gs2d_ens.tb"      default steps per shared-memory pass of ensembles
 *   "diff2d.tb"        steps per grid barrier of fm_diff2d_f64_forward on shared-memory
 *                      tiles with a halo: 2, 4 (default) or 8; 0 = one step per barrier
 *   "mhd.stage"        Runge-Kutta stage kernel of fm_mhd_forward_*: 2 x-marching kernel with
 *                      the x composites in a register ring (default for f64), 1 shared-memory
 *                      tile kernel (default for f32), 0 per-point kernel
 *   "mhd.soft"         exact binary64 operations of fm_mhd_forward_f64 on the integer pipes:
 *                      1 (default) scalings, products with constants, divisions, fmax/fmin;
 *                      0 FP64 instructions only.  Both give identical bits
 *   "mhd.stage_xchunk" x planes per tile of the x-marching stage kernel (default 16)
 *   "mhd.finish"       artificial-viscosity kernel of fm_mhd_forward_*: 2 x-marching kernel
 *                      computing each slope and face flux once, all fields per plane
 *                      (default for f64), 0 per-point kernel (default for f32)
 *   "mhd.xchunk"       x planes per tile of the x-marching kernel (0 = automatic)
 *   "sync.spin_limit"  polls before a grid-barrier wait of the persistent kernels
 *                      (fm_diff2d_f64_forward[_noalloc], fm_gs2d_ensemble_forward) gives
 *                      up, sets the error word and returns FM_ERR_TIMEOUT (>= 1; default
 *                      20,000,000, seconds of waiting).  A small value makes the waits run
 *                      out on purpose, to test the timeout path; it does not change results
 *                      of runs that finish
 *   "conv.kernel"      fm_conv3x3_fwd_bf16 with 64 output channels: 1 weight-resident
 *                      persistent kernel (default; falls back to 0 when its staged region
 *                      does not fit in shared memory), 2 the same with its regions and
 *                      residual rows staged by TMA and its steps chained by mbarriers
 *                      (falls back to 1), 0 per-tap gather kernel (B*H*W % 128 == 0).
 * fm_tune_clear() restores every default.
 */
int fm_tune_set(const char *key, int value);
int fm_tune_get(const char *key, int fallback);
int fm_tune_clear(void);

/* ---- measurement ------------------------------------------------------------ */

/*
 * FMA-pipe probe used to measure the arithmetic roofline of this GPU:
 * blocks x threads threads each run `iters` rounds of 8 independent FMA
 * chains (fp64 != 0: double, else float), i.e. 16*iters flops per thread.
 * `sink` is a device buffer of `blocks` elements of that type (never written
 * in practice).  The caller times the launch on `stream`.
 */
int fm_probe_fma(int fp64, int blocks, int threads, int iters, void *sink,
                 void *stream);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif
#endif /* FORMURA_GB300_H */
