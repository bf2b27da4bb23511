/*
 * fmr_mhd.c — CPU restatement of one time step of the reference program
 * examples/3d-mhd-rk4.fmr (9 fields: dens, vx, vy, vz, Bx, By, Bz, s, Psi),
 * in double.  TEST INFRASTRUCTURE ONLY (the checker of the GPU MHD kernels).
 *
 * Expression trees follow the .fmr source with Formura's parser rules
 * (src/Formura/Parser.hs:198-216: `*` `/` left-assoc above unary minus above
 * `+` `-`; min/max/minmod chains flatten into one n-ary node) and emission
 * rules (src/Formura/MPICxx/Translate.hs:585-620: immediates are double
 * literals, `>?`/`<?` fold right into fmax/fmin, `<%` of xs is
 * fmin(0,fmax-chain(xs)) + fmax(0,fmin-chain(xs)), `if` is ?:).  Composite
 * sub-expressions that the generated code recomputes at every shifted use
 * (e.g. dens*v_i at x-2..x+2) are computed once per cell here: a recomputed
 * IEEE expression has the same value.
 *
 * Constants (3d-mhd-rk4.fmr:4-11), with NX = NY = NZ = N:
 *   dt = 0.1/(NX >? NY >? NZ), dx = 1/NX, c_h = dx/dt, ch2_cp2 = c_h/0.18,
 *   dp_ddens = 1, dp_ds = 2/5, dens0 = 1, pi = 3.141592653589793.
 * Step (3d-mhd-rk4.fmr:104-145): the four manifested stages
 *   q4 = S + dt/4 f(S); q3 = S + dt/3 f(q4); q2 = S + dt/2 f(q3); nx = S + dt f(q2)
 * then artificial-viscosity fluxes of nx along x, y, z applied in turn, the
 * density floor fmax(dens, -0.9) and the numerical-heat update of s.
 */
#include "fmr_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NF 9
enum { F_DENS = 0, F_VX = 1, F_BX = 4, F_S = 7, F_PSI = 8 };

typedef struct {
  int n[3];
  size_t st[3];  /* element strides of x, y, z */
  size_t cells;
} grid3;

static inline size_t shift(const grid3 *g, size_t idx, const int c[3], int axis, int d) {
  int q[3] = {c[0], c[1], c[2]};
  q[axis] = ((q[axis] + d) % g->n[axis] + g->n[axis]) % g->n[axis];
  (void)idx;
  return (size_t)q[0] * g->st[0] + (size_t)q[1] * g->st[1] + (size_t)q[2] * g->st[2];
}

/* ddx of 3d-mhd-rk4.fmr:13-15: (a[i-2] + 8*a[i+1] - 8*a[i-1] - a[i+2])/(12*dx) */
static inline double d4(const grid3 *g, const double *a, const int c[3], int axis, double h12) {
  const double am2 = a[shift(g, 0, c, axis, -2)], ap1 = a[shift(g, 0, c, axis, 1)];
  const double am1 = a[shift(g, 0, c, axis, -1)], ap2 = a[shift(g, 0, c, axis, 2)];
  const double t1 = 8.0 * ap1;
  const double t2 = am2 + t1;
  const double t3 = 8.0 * am1;
  const double t4 = t2 - t3;
  const double t5 = t4 - ap2;
  return t5 / h12;
}

typedef struct {
  double dt, dx, h12, c_h, ch2_cp2, c8, c4, dp_ddens, dp_ds, dens0;
} mhd_consts;

static mhd_consts consts(int nx, int ny, int nz) {
  mhd_consts k;
  const double NX = nx, NY = ny, NZ = nz;
  const double pi = 3.141592653589793;
  k.dt = 0.1 / fmax(NX, fmax(NY, NZ));
  k.dx = 1.0 / NX;  /* dx = dy = dz for a cubic grid; the form uses dx, dy, dz per axis */
  k.h12 = 12.0 * k.dx;
  k.c_h = k.dx / k.dt;
  k.ch2_cp2 = k.c_h / 0.18;
  k.c8 = 1.0 / (8.0 * pi);
  k.c4 = 1.0 / (4.0 * pi);
  k.dp_ddens = 1.0;
  k.dp_ds = 2.0 / 5.0;
  k.dens0 = 1.0;
  return k;
}

/* out[f] = S[f] + coef * ddt_sys(Q)[f]  (3d-mhd-rk4.fmr:83-110) */
static void stage(const grid3 *g, const mhd_consts *k, double *const Q[NF],
                  double *const S[NF], double *const out[NF], double coef, double *tmp) {
  const size_t n = g->cells;
  /* composites: dens, m_i = dens*v_i, P, BB[j][i] = B_j*B_i, E[i][j] */
  double *dens = tmp, *m[3], *P, *BB[3][3], *E[3][3];
  for (int i = 0; i < 3; ++i) m[i] = tmp + (size_t)(1 + i) * n;
  P = tmp + 4 * n;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) BB[j][i] = tmp + (size_t)(5 + 3 * j + i) * n;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) E[i][j] = tmp + (size_t)(14 + 3 * i + j) * n;
  const double *v[3] = {Q[1], Q[2], Q[3]}, *B[3] = {Q[4], Q[5], Q[6]};
  const double *s = Q[7], *Psi = Q[8];
#pragma omp parallel for schedule(static)
  for (size_t p = 0; p < n; ++p) {
    const double d = k->dens0 + Q[0][p];
    dens[p] = d;
    for (int i = 0; i < 3; ++i) m[i][p] = d * v[i][p];
    /* dp_ddens*dens + dp_ds*s + 1/(8*pi) * sum_j B_j*B_j */
    const double b2 = ((B[0][p] * B[0][p]) + (B[1][p] * B[1][p])) + (B[2][p] * B[2][p]);
    P[p] = ((k->dp_ddens * d) + (k->dp_ds * s[p])) + (k->c8 * b2);
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) BB[j][i][p] = B[j][p] * B[i][p];
    /* -0*(del i j) * Psi + v i * B j - v j * B i */
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        const double z = 0.0 * (i == j ? 1.0 : 0.0);
        const double t = -(z * Psi[p]);
        E[i][j][p] = (t + (v[i][p] * B[j][p])) - (v[j][p] * B[i][p]);
      }
  }
#pragma omp parallel for collapse(2) schedule(static)
  for (int x = 0; x < g->n[0]; ++x)
    for (int y = 0; y < g->n[1]; ++y)
      for (int z = 0; z < g->n[2]; ++z) {
        const int c[3] = {x, y, z};
        const size_t p = (size_t)x * g->st[0] + (size_t)y * g->st[1] + z;
        const double h = k->h12;
        double f[NF];
        /* ddt_dens = - sum_i d_i(dens * v_i) */
        f[0] = -(((d4(g, m[0], c, 0, h)) + (d4(g, m[1], c, 1, h))) + (d4(g, m[2], c, 2, h)));
        /* ddt_v_i = (-(sum_j v_j * d_i(v_i))) - d_i(P)/dens + 1/(4pi) * (sum_j d_j(B_j B_i))/dens */
        for (int i = 0; i < 3; ++i) {
          const double dvi = d4(g, v[i], c, i, h);
          const double A = ((v[0][p] * dvi) + (v[1][p] * dvi)) + (v[2][p] * dvi);
          const double dP = d4(g, P, c, i, h);
          const double Y = ((d4(g, BB[0][i], c, 0, h)) + (d4(g, BB[1][i], c, 1, h))) +
                           (d4(g, BB[2][i], c, 2, h));
          f[1 + i] = ((-A) - (dP / dens[p])) + ((k->c4 * Y) / dens[p]);
        }
        /* ddt_B_i = sum_j d_j(E_ij) */
        for (int i = 0; i < 3; ++i)
          f[4 + i] = ((d4(g, E[i][0], c, 0, h)) + (d4(g, E[i][1], c, 1, h))) +
                     (d4(g, E[i][2], c, 2, h));
        /* ddt_s = sum_j v_j * d_j(s) */
        f[7] = ((v[0][p] * d4(g, s, c, 0, h)) + (v[1][p] * d4(g, s, c, 1, h))) +
               (v[2][p] * d4(g, s, c, 2, h));
        /* ddt_Psi = - c_h*c_h * (sum_i d_i(B_i)) - ch2_cp2 * Psi */
        const double divB = ((d4(g, B[0], c, 0, h)) + (d4(g, B[1], c, 1, h))) +
                            (d4(g, B[2], c, 2, h));
        f[8] = (-((k->c_h * k->c_h) * divB)) - (k->ch2_cp2 * Psi[p]);
        for (int q = 0; q < NF; ++q) out[q][p] = S[q][p] + (coef * f[q]);
      }
}

/* minmod of three (`<%` chain, Translate.hs:608-609) */
static inline double minmod3(double a, double b, double c) {
  return fmin(0.0, fmax(a, fmax(b, c))) + fmax(0.0, fmin(a, fmin(b, c)));
}

/* av_flux of 3d-mhd-rk4.fmr:43-47 */
static inline double av_flux(double num, double den) {
  const double nd = num * den;
  const double r = num / den;
  const double t = 0.75 * (r - 1.0);
  const double phi1 = fmin(1.0, fmax(0.0, 1.0 + t));
  const double Phi = (nd <= 0.0) ? 0.0 : phi1;
  return -((0.15 * Phi) * num);
}

/* slope delta_u at cell c along `axis` (3d-mhd-rk4.fmr:52) */
static inline double delta(const grid3 *g, const double *u, const int c[3], int axis) {
  const double u0 = u[shift(g, 0, c, axis, 0)];
  const double up = u[shift(g, 0, c, axis, 1)], um = u[shift(g, 0, c, axis, -1)];
  return minmod3((up - um) / 2.0, 1.4 * (up - u0), 1.4 * (u0 - um));
}

/* flux at the face between c and c+1 along `axis` (3d-mhd-rk4.fmr:49-58) */
static inline double face_flux(const grid3 *g, const double *u, const int c[3], int axis) {
  int c1[3] = {c[0], c[1], c[2]};
  c1[axis] = (c1[axis] + 1) % g->n[axis];
  const double ui = u[shift(g, 0, c, axis, 0)], ui1 = u[shift(g, 0, c, axis, 1)];
  const double u_l = ui + (0.5 * delta(g, u, c, axis));
  const double u_r = ui1 - (0.5 * delta(g, u, c1, axis));
  const double num = u_r - u_l;
  const double den = ui1 - ui;
  return av_flux(num, den);
}

void fo_mhd_run_f64(int nx, int ny, int nz, double *const fields[9], int steps) {
  grid3 g;
  g.n[0] = nx; g.n[1] = ny; g.n[2] = nz;
  g.st[2] = 1; g.st[1] = (size_t)nz; g.st[0] = (size_t)ny * nz;
  g.cells = (size_t)nx * ny * nz;
  const size_t n = g.cells;
  const mhd_consts k = consts(nx, ny, nz);
  double *buf = (double *)malloc((size_t)(2 * NF + 23) * n * sizeof(double));
  double *A[NF], *Bq[NF], *S[NF];
  for (int f = 0; f < NF; ++f) {
    A[f] = buf + (size_t)f * n;
    Bq[f] = buf + (size_t)(NF + f) * n;
    S[f] = fields[f];
  }
  double *tmp = buf + (size_t)2 * NF * n;
  for (int st = 0; st < steps; ++st) {
    stage(&g, &k, S, S, A, k.dt / 4.0, tmp);   /* sys_q4   */
    stage(&g, &k, A, S, Bq, k.dt / 3.0, tmp);  /* sys_q3   */
    stage(&g, &k, Bq, S, A, k.dt / 2.0, tmp);  /* sys_q2   */
    stage(&g, &k, A, S, Bq, k.dt, tmp);        /* sys_next */
    /* artificial viscosity from sys_next, then floor and heat; written into S */
#pragma omp parallel for collapse(2) schedule(static)
    for (int x = 0; x < nx; ++x)
      for (int y = 0; y < ny; ++y)
        for (int z = 0; z < nz; ++z) {
          const int c[3] = {x, y, z};
          const size_t p = (size_t)x * g.st[0] + (size_t)y * g.st[1] + z;
          double nv[NF];
          for (int f = 0; f < NF; ++f) {
            double w = Bq[f][p];
            for (int ax = 0; ax < 3; ++ax) {
              int cm[3] = {x, y, z};
              cm[ax] = (cm[ax] - 1 + g.n[ax]) % g.n[ax];
              const double fm = face_flux(&g, Bq[f], cm, ax);  /* avf[i-1/2] */
              const double fp = face_flux(&g, Bq[f], c, ax);   /* avf[i+1/2] */
              w = (w + fm) - fp;
            }
            nv[f] = w;
          }
          /* numerical_heat (3d-mhd-rk4.fmr:141-143) with dens = the step's input */
          const double svr = ((Bq[1][p] * Bq[1][p]) + (Bq[2][p] * Bq[2][p])) + (Bq[3][p] * Bq[3][p]);
          const double svn = ((nv[1] * nv[1]) + (nv[2] * nv[2])) + (nv[3] * nv[3]);
          const double sbr = ((Bq[4][p] * Bq[4][p]) + (Bq[5][p] * Bq[5][p])) + (Bq[6][p] * Bq[6][p]);
          const double sbn = ((nv[4] * nv[4]) + (nv[5] * nv[5])) + (nv[6] * nv[6]);
          const double pi = 3.141592653589793;
          const double den8 = (8.0 * pi) * (k.dens0 + S[0][p]);
          const double heat = ((1.0 / 2.0) * (svr - svn)) + ((1.0 / den8) * (sbr - sbn));
          S[0][p] = fmax(nv[0], -0.9);
          for (int f = 1; f < NF; ++f) S[f][p] = nv[f];
          S[7][p] = nv[7] + heat;
        }
  }
  free(buf);
}
