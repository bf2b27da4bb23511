/*
 * fmr_oracle.c — CPU restatement of Formura-generated loop nests.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline); the
 * product library never links or calls it.  Build with -ffp-contract=off for
 * parity: every statement below is one node of the generated SSA chain, in the
 * order src/Formura/MPICxx/Translate.hs:481-629 emits them, so IEEE results
 * equal the generated code's.  OpenMP follows the generated code's
 * `#pragma omp parallel for` over the outer loop (Translate.hs:647-650).
 */
#include "fmr_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int fo_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static inline int wrap_up(int i, int n) { return (i + 1 == n) ? 0 : i + 1; }
static inline int wrap_dn(int i, int n) { return (i == 0) ? n - 1 : i - 1; }

/* ------------------------------------------------------------------------ */
/* 2D Gray-Scott, pearson form.  One step of examples-generated/pearson.c:
 *   dU_dt (node 29 of examples-generated/pearson.log, pearson.c:138-161)
 *   dV_dt (node 49, pearson.c:166-193), U_next/V_next (nodes 51,53,
 *   pearson.c:194-208: a_2 = dt*dU_dt; a_3 = U + a_2).                       */
static void gs2d_step_f64(int nx, int ny, const double *restrict U,
                          const double *restrict V, double *restrict Un,
                          double *restrict Vn, const fo_gs_params *p) {
  const double F = p->F, k = p->k, Du = p->Du, Dv = p->Dv, dt = p->dt,
               dx = p->dx;
#pragma omp parallel for schedule(static)
  for (int x = 0; x < nx; ++x) {
    const int xp = wrap_up(x, nx), xm = wrap_dn(x, nx);
    for (int y = 0; y < ny; ++y) {
      const int yp = wrap_up(y, ny), ym = wrap_dn(y, ny);
      const double a = U[(size_t)x * ny + y];
      const double a_0 = V[(size_t)x * ny + y];
      /* dU_dt = -U*V*V + F*(1-U) + Du/(dx*dx) * sum_i (d_i . d_i) U */
      double a_1 = a * a_0;
      double a_2 = a_1 * a_0;
      double a_3 = -a_2;
      double a_6 = 1.0 - a;
      double a_7 = F * a_6;
      double a_8 = a_3 + a_7;
      double a_11 = dx * dx;
      double a_12 = Du / a_11;
      double a_14 = U[(size_t)xp * ny + y] - a;
      double a_16 = a - U[(size_t)xm * ny + y];
      double a_17 = a_14 - a_16;
      double a_19 = U[(size_t)x * ny + yp] - a;
      double a_21 = a - U[(size_t)x * ny + ym];
      double a_22 = a_19 - a_21;
      double a_23 = a_17 + a_22;
      double a_24 = a_12 * a_23;
      const double dU = a_8 + a_24;
      /* dV_dt = U*V*V - (F+k)*V + Dv/(dx*dx) * sum_i (d_i . d_i) V */
      double b_1 = a * a_0;
      double b_2 = b_1 * a_0;
      double b_5 = F + k;
      double b_6 = b_5 * a_0;
      double b_7 = b_2 - b_6;
      double b_10 = dx * dx;
      double b_11 = Dv / b_10;
      double b_13 = V[(size_t)xp * ny + y] - a_0;
      double b_15 = a_0 - V[(size_t)xm * ny + y];
      double b_16 = b_13 - b_15;
      double b_18 = V[(size_t)x * ny + yp] - a_0;
      double b_20 = a_0 - V[(size_t)x * ny + ym];
      double b_21 = b_18 - b_20;
      double b_22 = b_16 + b_21;
      double b_23 = b_11 * b_22;
      const double dV = b_7 + b_23;
      /* U_next = U + dt * dU_dt ; V_next = V + dt * dV_dt */
      double c_2 = dt * dU;
      Un[(size_t)x * ny + y] = a + c_2;
      double d_2 = dt * dV;
      Vn[(size_t)x * ny + y] = a_0 + d_2;
    }
  }
}

void fo_gs2d_run_f64(int nx, int ny, double *U, double *V, int steps,
                     const fo_gs_params *p) {
  const size_t n = (size_t)nx * ny;
  double *Un = (double *)malloc(n * sizeof(double));
  double *Vn = (double *)malloc(n * sizeof(double));
  double *cu = U, *cv = V, *nu = Un, *nv = Vn;
  for (int s = 0; s < steps; ++s) {
    gs2d_step_f64(nx, ny, cu, cv, nu, nv, p);
    double *t = cu; cu = nu; nu = t;
    t = cv; cv = nv; nv = t;
  }
  if (cu != U) {
    memcpy(U, cu, n * sizeof(double));
    memcpy(V, cv, n * sizeof(double));
  }
  free(Un);
  free(Vn);
}

/* Binary32 version of the same chain. */
static void gs2d_step_f32(int nx, int ny, const float *restrict U,
                          const float *restrict V, float *restrict Un,
                          float *restrict Vn, float F, float k, float Du,
                          float Dv, float dt, float dx) {
#pragma omp parallel for schedule(static)
  for (int x = 0; x < nx; ++x) {
    const int xp = wrap_up(x, nx), xm = wrap_dn(x, nx);
    for (int y = 0; y < ny; ++y) {
      const int yp = wrap_up(y, ny), ym = wrap_dn(y, ny);
      const float a = U[(size_t)x * ny + y];
      const float a_0 = V[(size_t)x * ny + y];
      float a_1 = a * a_0;
      float a_2 = a_1 * a_0;
      float a_3 = -a_2;
      float a_6 = 1.0f - a;
      float a_7 = F * a_6;
      float a_8 = a_3 + a_7;
      float a_11 = dx * dx;
      float a_12 = Du / a_11;
      float a_14 = U[(size_t)xp * ny + y] - a;
      float a_16 = a - U[(size_t)xm * ny + y];
      float a_17 = a_14 - a_16;
      float a_19 = U[(size_t)x * ny + yp] - a;
      float a_21 = a - U[(size_t)x * ny + ym];
      float a_22 = a_19 - a_21;
      float a_23 = a_17 + a_22;
      float a_24 = a_12 * a_23;
      const float dU = a_8 + a_24;
      float b_5 = F + k;
      float b_6 = b_5 * a_0;
      float b_7 = a_2 - b_6;
      float b_11 = Dv / a_11;
      float b_13 = V[(size_t)xp * ny + y] - a_0;
      float b_15 = a_0 - V[(size_t)xm * ny + y];
      float b_16 = b_13 - b_15;
      float b_18 = V[(size_t)x * ny + yp] - a_0;
      float b_20 = a_0 - V[(size_t)x * ny + ym];
      float b_21 = b_18 - b_20;
      float b_22 = b_16 + b_21;
      float b_23 = b_11 * b_22;
      const float dV = b_7 + b_23;
      float c_2 = dt * dU;
      Un[(size_t)x * ny + y] = a + c_2;
      float d_2 = dt * dV;
      Vn[(size_t)x * ny + y] = a_0 + d_2;
    }
  }
}

void fo_gs2d_run_f32(int nx, int ny, float *U, float *V, int steps, float F,
                     float k, float Du, float Dv, float dt, float dx) {
  const size_t n = (size_t)nx * ny;
  float *Un = (float *)malloc(n * sizeof(float));
  float *Vn = (float *)malloc(n * sizeof(float));
  float *cu = U, *cv = V, *nu = Un, *nv = Vn;
  for (int s = 0; s < steps; ++s) {
    gs2d_step_f32(nx, ny, cu, cv, nu, nv, F, k, Du, Dv, dt, dx);
    float *t = cu; cu = nu; nu = t;
    t = cv; cv = nv; nv = t;
  }
  if (cu != U) {
    memcpy(U, cu, n * sizeof(float));
    memcpy(V, cv, n * sizeof(float));
  }
  free(Un);
  free(Vn);
}

/* ------------------------------------------------------------------------ */
/* 2D diffusion in the examples/diffusion.fmr form (diffusion.fmr:5-21 with the
 * z axis dropped):  dens + Dt / Dx**2 * ((lap_x) + (lap_y)),
 *   lap_x = ((d[x+1]-d)/2 - (d-d[x-1])/2)/2.
 * `Dt / Dx**2` is the node pair pow(Dx,2) then Dt/that (Translate.hs:594).   */
void fo_diff2d_run_f64(int nx, int ny, double *dens, int steps, double Dt,
                       double Dx) {
  const size_t n = (size_t)nx * ny;
  double *tmp = (double *)malloc(n * sizeof(double));
  double *cur = dens, *nxt = tmp;
  const double a_2 = pow(Dx, 2.0);
  const double a_3 = Dt / a_2;
  for (int s = 0; s < steps; ++s) {
#pragma omp parallel for schedule(static)
    for (int x = 0; x < nx; ++x) {
      const int xp = wrap_up(x, nx), xm = wrap_dn(x, nx);
      for (int y = 0; y < ny; ++y) {
        const int yp = wrap_up(y, ny), ym = wrap_dn(y, ny);
        const double a = cur[(size_t)x * ny + y];
        double e_0 = (cur[(size_t)xp * ny + y] - a) / 2.0;
        double e_1 = (a - cur[(size_t)xm * ny + y]) / 2.0;
        double e_2 = (e_0 - e_1) / 2.0;
        double f_0 = (cur[(size_t)x * ny + yp] - a) / 2.0;
        double f_1 = (a - cur[(size_t)x * ny + ym]) / 2.0;
        double f_2 = (f_0 - f_1) / 2.0;
        double g = e_2 + f_2;
        double h = a_3 * g;
        nxt[(size_t)x * ny + y] = a + h;
      }
    }
    double *t = cur; cur = nxt; nxt = t;
  }
  if (cur != dens) memcpy(dens, cur, n * sizeof(double));
  free(tmp);
}

/* ------------------------------------------------------------------------ */
/* 3D Gray-Scott, pearson-3d form.  Per axis a (with `/dx` inside ddx as in
 * examples/pearson-3d.fmr:6-8):
 *   lap_a = ((W[+1]-W)/dx - (W-W[-1])/dx)/dx,  lap = (lap_x + lap_y) + lap_z
 *   dU = ((-(U*V*V)) + F*(1-U)) + Du*lap_U ;  dV = ((U*V*V) - (F+k)*V) + Dv*lap_V
 *   U_next = U + dt*dU ;  V_next = V + dt*dV                                  */
#define IDX3(x, y, z) (((size_t)(x) * ny + (y)) * nz + (z))

static void gs3d_step_f64(int nx, int ny, int nz, const double *restrict U,
                          const double *restrict V, double *restrict Un,
                          double *restrict Vn, const fo_gs_params *p) {
  const double F = p->F, k = p->k, Du = p->Du, Dv = p->Dv, dt = p->dt,
               dx = p->dx;
#pragma omp parallel for collapse(2) schedule(static)
  for (int x = 0; x < nx; ++x) {
    for (int y = 0; y < ny; ++y) {
      const int xp = wrap_up(x, nx), xm = wrap_dn(x, nx);
      const int yp = wrap_up(y, ny), ym = wrap_dn(y, ny);
      for (int z = 0; z < nz; ++z) {
        const int zp = wrap_up(z, nz), zm = wrap_dn(z, nz);
        const double u = U[IDX3(x, y, z)];
        const double v = V[IDX3(x, y, z)];
        /* U_next node */
        double a_1 = u * v;
        double a_2 = a_1 * v;
        double a_3 = -a_2;
        double a_5 = 1.0 - u;
        double a_6 = F * a_5;
        double a_7 = a_3 + a_6;
        double lx = ((U[IDX3(xp, y, z)] - u) / dx - (u - U[IDX3(xm, y, z)]) / dx) / dx;
        double ly = ((U[IDX3(x, yp, z)] - u) / dx - (u - U[IDX3(x, ym, z)]) / dx) / dx;
        double lz = ((U[IDX3(x, y, zp)] - u) / dx - (u - U[IDX3(x, y, zm)]) / dx) / dx;
        double a_s = lx + ly;
        double a_l = a_s + lz;
        double a_d = Du * a_l;
        double dU = a_7 + a_d;
        double a_t = dt * dU;
        Un[IDX3(x, y, z)] = u + a_t;
        /* V_next node */
        double b_1 = u * v;
        double b_2 = b_1 * v;
        double b_4 = F + k;
        double b_5 = b_4 * v;
        double b_6 = b_2 - b_5;
        double mx = ((V[IDX3(xp, y, z)] - v) / dx - (v - V[IDX3(xm, y, z)]) / dx) / dx;
        double my = ((V[IDX3(x, yp, z)] - v) / dx - (v - V[IDX3(x, ym, z)]) / dx) / dx;
        double mz = ((V[IDX3(x, y, zp)] - v) / dx - (v - V[IDX3(x, y, zm)]) / dx) / dx;
        double b_s = mx + my;
        double b_l = b_s + mz;
        double b_d = Dv * b_l;
        double dV = b_6 + b_d;
        double b_t = dt * dV;
        Vn[IDX3(x, y, z)] = v + b_t;
      }
    }
  }
}

void fo_gs3d_run_f64(int nx, int ny, int nz, double *U, double *V, int steps,
                     const fo_gs_params *p) {
  const size_t n = (size_t)nx * ny * nz;
  double *Un = (double *)malloc(n * sizeof(double));
  double *Vn = (double *)malloc(n * sizeof(double));
  double *cu = U, *cv = V, *nu = Un, *nv = Vn;
  for (int s = 0; s < steps; ++s) {
    gs3d_step_f64(nx, ny, nz, cu, cv, nu, nv, p);
    double *t = cu; cu = nu; nu = t;
    t = cv; cv = nv; nv = t;
  }
  if (cu != U) {
    memcpy(U, cu, n * sizeof(double));
    memcpy(V, cv, n * sizeof(double));
  }
  free(Un);
  free(Vn);
}

/* Binary32 + Kahan time accumulation. */
static void gs3d_step_f32k(int nx, int ny, int nz, const float *restrict U,
                           const float *restrict V, const float *restrict cU,
                           const float *restrict cV, float *restrict Un,
                           float *restrict Vn, float *restrict cUn,
                           float *restrict cVn, float F, float k, float Du,
                           float Dv, float dt, float dx) {
#pragma omp parallel for collapse(2) schedule(static)
  for (int x = 0; x < nx; ++x) {
    for (int y = 0; y < ny; ++y) {
      const int xp = wrap_up(x, nx), xm = wrap_dn(x, nx);
      const int yp = wrap_up(y, ny), ym = wrap_dn(y, ny);
      for (int z = 0; z < nz; ++z) {
        const int zp = wrap_up(z, nz), zm = wrap_dn(z, nz);
        const float u = U[IDX3(x, y, z)];
        const float v = V[IDX3(x, y, z)];
        float a_1 = u * v;
        float a_2 = a_1 * v;
        float a_3 = -a_2;
        float a_5 = 1.0f - u;
        float a_6 = F * a_5;
        float a_7 = a_3 + a_6;
        float lx = ((U[IDX3(xp, y, z)] - u) / dx - (u - U[IDX3(xm, y, z)]) / dx) / dx;
        float ly = ((U[IDX3(x, yp, z)] - u) / dx - (u - U[IDX3(x, ym, z)]) / dx) / dx;
        float lz = ((U[IDX3(x, y, zp)] - u) / dx - (u - U[IDX3(x, y, zm)]) / dx) / dx;
        float a_s = lx + ly;
        float a_l = a_s + lz;
        float a_d = Du * a_l;
        float dU = a_7 + a_d;
        float b_4 = F + k;
        float b_5 = b_4 * v;
        float b_6 = a_2 - b_5;
        float mx = ((V[IDX3(xp, y, z)] - v) / dx - (v - V[IDX3(xm, y, z)]) / dx) / dx;
        float my = ((V[IDX3(x, yp, z)] - v) / dx - (v - V[IDX3(x, ym, z)]) / dx) / dx;
        float mz = ((V[IDX3(x, y, zp)] - v) / dx - (v - V[IDX3(x, y, zm)]) / dx) / dx;
        float b_s = mx + my;
        float b_l = b_s + mz;
        float b_d = Dv * b_l;
        float dV = b_6 + b_d;
        /* compensated accumulation of U += dt*dU */
        float yu = dt * dU - cU[IDX3(x, y, z)];
        float tu = u + yu;
        cUn[IDX3(x, y, z)] = (tu - u) - yu;
        Un[IDX3(x, y, z)] = tu;
        float yv = dt * dV - cV[IDX3(x, y, z)];
        float tv = v + yv;
        cVn[IDX3(x, y, z)] = (tv - v) - yv;
        Vn[IDX3(x, y, z)] = tv;
      }
    }
  }
}

void fo_gs3d_run_f32_kahan(int nx, int ny, int nz, float *U, float *V,
                           float *cU, float *cV, int steps, float F, float k,
                           float Du, float Dv, float dt, float dx) {
  const size_t n = (size_t)nx * ny * nz;
  float *buf = (float *)malloc(4 * n * sizeof(float));
  float *cu = U, *cv = V, *ccu = cU, *ccv = cV;
  float *nu = buf, *nv = buf + n, *ncu = buf + 2 * n, *ncv = buf + 3 * n;
  for (int s = 0; s < steps; ++s) {
    gs3d_step_f32k(nx, ny, nz, cu, cv, ccu, ccv, nu, nv, ncu, ncv, F, k, Du, Dv,
                   dt, dx);
    float *t;
    t = cu; cu = nu; nu = t;
    t = cv; cv = nv; nv = t;
    t = ccu; ccu = ncu; ncu = t;
    t = ccv; ccv = ncv; ncv = t;
  }
  if (cu != U) {
    memcpy(U, cu, n * sizeof(float));
    memcpy(V, cv, n * sizeof(float));
    memcpy(cU, ccu, n * sizeof(float));
    memcpy(cV, ccv, n * sizeof(float));
  }
  free(buf);
}

/* Fast binary32 form (see fmr_oracle.h). */
static void gs3d_step_f32k_fast(int nx, int ny, int nz, const float *restrict U,
                                const float *restrict V, const float *restrict cU,
                                const float *restrict cV, float *restrict Un,
                                float *restrict Vn, float *restrict cUn,
                                float *restrict cVn, float F, float Fk, float cu,
                                float cv, float dt) {
#pragma omp parallel for collapse(2) schedule(static)
  for (int x = 0; x < nx; ++x) {
    for (int y = 0; y < ny; ++y) {
      const int xp = wrap_up(x, nx), xm = wrap_dn(x, nx);
      const int yp = wrap_up(y, ny), ym = wrap_dn(y, ny);
      for (int z = 0; z < nz; ++z) {
        const int zp = wrap_up(z, nz), zm = wrap_dn(z, nz);
        const size_t i = IDX3(x, y, z);
        const float u = U[i], v = V[i];
        const float sxu = (U[IDX3(xp, y, z)] - u) - (u - U[IDX3(xm, y, z)]);
        const float syu = (U[IDX3(x, yp, z)] - u) - (u - U[IDX3(x, ym, z)]);
        const float szu = (U[IDX3(x, y, zp)] - u) - (u - U[IDX3(x, y, zm)]);
        const float lu = (sxu + syu) + szu;
        const float sxv = (V[IDX3(xp, y, z)] - v) - (v - V[IDX3(xm, y, z)]);
        const float syv = (V[IDX3(x, yp, z)] - v) - (v - V[IDX3(x, ym, z)]);
        const float szv = (V[IDX3(x, y, zp)] - v) - (v - V[IDX3(x, y, zm)]);
        const float lv = (sxv + syv) + szv;
        const float uvv = (u * v) * v;
        const float dU = fmaf(cu, lu, fmaf(F, 1.0f - u, -uvv));
        const float dV = fmaf(cv, lv, fmaf(-Fk, v, uvv));
        const float yu = fmaf(dt, dU, -cU[i]);
        const float tu = u + yu;
        cUn[i] = (tu - u) - yu;
        Un[i] = tu;
        const float yv = fmaf(dt, dV, -cV[i]);
        const float tv = v + yv;
        cVn[i] = (tv - v) - yv;
        Vn[i] = tv;
      }
    }
  }
}

void fo_gs3d_run_f32k_fast(int nx, int ny, int nz, float *U, float *V,
                           float *cU, float *cV, int steps, double F, double k,
                           double Du, double Dv, double dt, double dx) {
  const size_t n = (size_t)nx * ny * nz;
  const float Ff = (float)F, Fk = (float)(F + k), cu = (float)(Du / (dx * dx)),
              cv = (float)(Dv / (dx * dx)), dtf = (float)dt;
  float *buf = (float *)malloc(4 * n * sizeof(float));
  float *cu_ = U, *cv_ = V, *ccu = cU, *ccv = cV;
  float *nu = buf, *nv = buf + n, *ncu = buf + 2 * n, *ncv = buf + 3 * n;
  for (int s = 0; s < steps; ++s) {
    gs3d_step_f32k_fast(nx, ny, nz, cu_, cv_, ccu, ccv, nu, nv, ncu, ncv, Ff, Fk, cu, cv, dtf);
    float *t;
    t = cu_; cu_ = nu; nu = t;
    t = cv_; cv_ = nv; nv = t;
    t = ccu; ccu = ncu; ncu = t;
    t = ccv; ccv = ncv; ncv = t;
  }
  if (cu_ != U) {
    memcpy(U, cu_, n * sizeof(float));
    memcpy(V, cv_, n * sizeof(float));
    memcpy(cU, ccu, n * sizeof(float));
    memcpy(cV, ccv, n * sizeof(float));
  }
  free(buf);
}

double fo_sum_f64(int64_t n, const double *a) {
  double s = 0.0;
  for (int64_t i = 0; i < n; ++i) s += a[i];
  return s;
}
