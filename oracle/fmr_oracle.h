/*
 * fmr_oracle.h — CPU restatement of the per-cell arithmetic that Formura's
 * generated C performs for the stencil programs this repository runs on the GPU.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code; only the tests, the smoke check and the CPU-baseline leg of
 * the benchmark do, as the checker and the timed CPU baseline.
 *
 * Every update follows the expression order that Formura's C back end emits
 * (src/Formura/MPICxx/Translate.hs:481-629: one SSA temporary per DAG node,
 * `**` -> pow, immediates -> double literals) for the named .fmr form, with
 * periodic boundaries (the self-exchange of src/Formura/MPICxx/Translate.hs:1062-1068
 * when mpi_grid_shape is all ones).  Built with -ffp-contract=off, each
 * function is bit-for-bit the generated loop nest; the 2D Gray-Scott step is
 * pinned against the reference's own examples-generated/pearson.c.
 *
 * Layout: row-major, last axis fastest (U[x][y][z]), no margin.
 */
#ifndef FMR_ORACLE_H
#define FMR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Gray-Scott constants as the .fmr files name them. */
typedef struct {
  double F, k, Du, Dv, dt, dx;
} fo_gs_params;

/* 2D Gray-Scott, pearson-2d.fmr / examples-generated/pearson.fmr form
 * (dU_dt and dV_dt manifested, then U_next = U + dt*dU_dt).  U,V are [nx][ny];
 * advanced in place by `steps`.  Follows examples-generated/pearson.c:138-208. */
void fo_gs2d_run_f64(int nx, int ny, double *U, double *V, int steps,
                     const fo_gs_params *p);

/* Same form in binary32 arithmetic (constants rounded to float, derived
 * constants computed in float in DAG order): the oracle of the FP32 ensemble. */
void fo_gs2d_run_f32(int nx, int ny, float *U, float *V, int steps,
                     float F, float k, float Du, float Dv, float dt, float dx);

/* 2D diffusion, examples/diffusion.fmr form reduced to 2D:
 *   dens_next = dens + Dt / Dx**2 * sum_i ddx_i(ddx_i dens),
 *   ddx a = (a[i+1/2] - a[i-1/2]) / 2.                       */
void fo_diff2d_run_f64(int nx, int ny, double *dens, int steps, double Dt,
                       double Dx);

/* 3D Gray-Scott, examples/pearson-3d.fmr form (ddx a = (a[i+1/2]-a[i-1/2])/dx,
 * reaction of pearson-2d.fmr:21-22, no manifest annotations).  [nx][ny][nz]. */
void fo_gs3d_run_f64(int nx, int ny, int nz, double *U, double *V, int steps,
                     const fo_gs_params *p);

/* Same form in binary32 with compensated (Kahan) time accumulation:
 *   y = dt*dU - cU;  t = U + y;  cU = (t - U) - y;  U = t.
 * cU, cV carry the compensation between steps (start them at zero). */
void fo_gs3d_run_f32_kahan(int nx, int ny, int nz, float *U, float *V,
                           float *cU, float *cV, int steps, float F, float k,
                           float Du, float Dv, float dt, float dx);

/* The binary32 "fast form" of the same 3D Gray-Scott step that the
 * temporally blocked GPU kernel evaluates (FMAs explicit, no divisions):
 *   s_a = (W[a+1]-W) - (W-W[a-1]);  lap = (s_x + s_y) + s_z
 * (the difference of the two face differences, the generated DAG's order
 * without its divisions; a face difference is the same IEEE value for both
 * cells it separates, so a kernel may compute it once) 
 *   uvv = (U*V)*V
 *   dU = fmaf(cu, lapU, fmaf(F, 1-U, -uvv))     cu = (float)(Du/(dx*dx))
 *   dV = fmaf(cv, lapV, fmaf(-Fk, V, uvv))      cv = (float)(Dv/(dx*dx)), Fk = (float)(F+k)
 *   Kahan per field: y = fmaf(dt, dW, -cW); t = W + y; cW = (t - W) - y; W = t
 * It is not the generated DAG (that is fo_gs3d_run_f32_kahan); its accuracy is
 * measured against fo_gs3d_run_f64. */
void fo_gs3d_run_f32k_fast(int nx, int ny, int nz, float *U, float *V,
                           float *cU, float *cV, int steps, double F, double k,
                           double Du, double Dv, double dt, double dx);

/* One-or-more time steps of examples/3d-mhd-rk4.fmr in double (fmr_mhd.c).
 * fields[0..8] = dens, vx, vy, vz, Bx, By, Bz, s, Psi, each [nx][ny][nz],
 * advanced in place.  dx = 1/nx and dt = 0.1/max(n) as the program defines
 * them (a cubic grid, nx = ny = nz, is assumed for dx = dy = dz). */
void fo_mhd_run_f64(int nx, int ny, int nz, double *const fields[9], int steps);

/* Plain left-to-right double sum (conserved-total check). */
double fo_sum_f64(int64_t n, const double *a);

/* Number of OpenMP threads the oracle uses (1 without OpenMP). */
int fo_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
