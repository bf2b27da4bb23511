// fm_mhd_impl.cuh — 3D ideal MHD with Dedner divergence cleaning and
// artificial viscosity: the time step of the reference program
// examples/3d-mhd-rk4.fmr.  Kernels and host templates; instantiated by
// fm_mhd.cu (binary32 bulk, totals) and fm_mhd_f64.cu (all binary64), two
// translation units so that they compile in parallel.
//
// Fields (SoA, [n][n][n] each): dens (perturbation of dens0 = 1), vx, vy, vz,
// Bx, By, Bz, s, Psi.  One step (3d-mhd-rk4.fmr:104-145):
//   q4 = S + dt/4 f(S);  q3 = S + dt/3 f(q4);  q2 = S + dt/2 f(q3);
//   nx = S + dt f(q2)                                  (mhd_stage, 4 launches)
//   then, per field, the artificial-viscosity fluxes of nx along x, y, z
//   applied in turn, dens floored at -0.9, and s += numerical heat
//                                                      (mhd_finish, 1 launch)
// f = ddt_sys (3d-mhd-rk4.fmr:83-101) uses the 4th-order difference
// (a[i-2] + 8a[i+1] - 8a[i-1] - a[i+2])/(12 dx) of 33 quantities per cell;
// composite arguments (dens*v_i, pressure, B_j*B_i, v_i*B_j - v_j*B_i) are
// re-evaluated at each of the four neighbours, as the generated code does.
//
// Precision: template parameter R is the bulk type.  R = double reproduces
// the all-FP64 program bit for bit (IEEE divisions: fm::div_const_i for the
// constant 12*dx, __ddiv_rn for /dens and num/den).  R = float is the
// production path: the bulk in binary32, the numerical-heat (energy) update
// of s in FP64 — the difference of kinetic and magnetic energies before and
// after the viscosity step is a cancellation-prone small difference — and the
// conserved totals in FP64 (fm_mhd_totals).
#pragma once

#include <algorithm>
#include <type_traits>

#include "fm_common.cuh"
#include "fm_softfp.cuh"
#include "fm_tune.h"

namespace {

constexpr int NF = 9;

struct Fields {
  void *p[NF];
};

template <typename R>
struct MhdC {
  R dt_c;  // stage coefficient (dt/4, dt/3, dt/2, dt)
  R h12;   // 12*dx
  R c_h2;  // c_h*c_h
  R ch2_cp2, c8, c4, dp_ddens, dp_ds, dens0;
  fm::DivConst h12d;  // for the double path's exact division
  float h12f, rh12f;  // for the float path's exact division
  // the same constants for the double path's integer-pipe forms (S = 1)
  fm::soft::DivConstS h12s;
  fm::soft::MulConstS dts, c_h2s, ch2_cp2s, c8s, c4s, dp_ddens_s, dp_ds_s;
  fm::soft::MulConstS c1_4s, c0_75s, c0_15s;  // the viscosity limiter's factors
  fm::soft::MulConstS c8pi_s;                 // 8*pi of the numerical heat
};

template <typename R>
__device__ __forceinline__ R div_h(R x, const MhdC<R> &k);
template <>
__device__ __forceinline__ double div_h<double>(double x, const MhdC<double> &k) {
  return fm::div_const_i(x, k.h12d);
}
template <>
__device__ __forceinline__ float div_h<float>(float x, const MhdC<float> &k) {
  return fm::div_const_f(x, k.h12f, k.rh12f);
}

__device__ __forceinline__ double vdiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float vdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double vmax(double a, double b) { return fmax(a, b); }
__device__ __forceinline__ float vmax(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ double vmin(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ float vmin(float a, float b) { return fminf(a, b); }

template <typename R>
__device__ __forceinline__ R ld(const void *f, size_t i) {
  return __ldg(reinterpret_cast<const R *>(f) + i);
}

// The arithmetic forms of the operations that have an exact integer-pipe
// equivalent.  SF = 0: the FP64/FP32 instructions.  SF >= 1 (double only):
// the same IEEE results from fm_softfp.cuh — the FP64 pipe (2 lanes per clock
// per SM on this part, against 64 + 64 integer lanes) is what bounds the
// double path, so every FP64 instruction that becomes a short integer
// sequence raises the cell rate.  SF = 1: scalings by powers of two, products
// with constants, divisions, fmax/fmin and the sign test (the products of two
// fields stay on the FP64 pipe: moving them too measured slower).  Bit-identical.
template <typename R>
struct ArHw {
  static __device__ __forceinline__ R x8(R x) { return R(8) * x; }
  static __device__ __forceinline__ R half(R x) { return R(0.5) * x; }
  static __device__ __forceinline__ R mul(R x, R y) { return x * y; }
  static __device__ __forceinline__ R cmul(R c, const fm::soft::MulConstS &, R x) { return c * x; }
  static __device__ __forceinline__ R divh(R x, const MhdC<R> &k) { return div_h<R>(x, k); }
  // division by a run-time value, prepared once for several quotients
  using Den = R;
  static __device__ __forceinline__ Den prep(R d) { return d; }
  static __device__ __forceinline__ R div(R x, Den d) { return vdiv(x, d); }
  // x / d where the quotient is used only if !unused
  static __device__ __forceinline__ R div_unless(R x, R d, bool) { return vdiv(x, d); }
  static __device__ __forceinline__ R max(R x, R y) { return vmax(x, y); }
  static __device__ __forceinline__ R min(R x, R y) { return vmin(x, y); }
  static __device__ __forceinline__ bool le0(R x) { return x <= R(0); }
  // -(0 * Psi) + x  (the Kronecker-delta term of E_ij, 3d-mhd-rk4.fmr:70)
  static __device__ __forceinline__ R zp_add(R Psi, R x) { return (-(R(0) * Psi)) + x; }
};

__device__ __noinline__ double zp_add_slow(double Psi, double x) { return (-(0.0 * Psi)) + x; }

template <int SF>
struct ArSoft {
  static __device__ __forceinline__ double x8(double x) { return fm::soft::scale_pow2(x, 3); }
  static __device__ __forceinline__ double half(double x) { return fm::soft::scale_pow2(x, -1); }
  static __device__ __forceinline__ double mul(double x, double y) { return x * y; }
  static __device__ __forceinline__ double cmul(double, const fm::soft::MulConstS &c, double x) {
    return fm::soft::mul_const_s(x, c);
  }
  static __device__ __forceinline__ double divh(double x, const MhdC<double> &k) {
    return fm::soft::div_const_s(x, k.h12s);
  }
  using Den = fm::soft::DivVarS;
  static __device__ __forceinline__ Den prep(double d) { return fm::soft::prep_div_s(d); }
  static __device__ __forceinline__ double div(double x, const Den &d) {
    return fm::soft::div_var_s(x, d);
  }
  // dividing by 1 where the quotient is not used keeps zero divisors (flat
  // fields) out of the division's slow path
  static __device__ __forceinline__ double div_unless(double x, double d, bool unused) {
    return fm::soft::div_s(x, unused ? 1.0 : d);
  }
  static __device__ __forceinline__ double max(double x, double y) { return fm::soft::max_s(x, y); }
  static __device__ __forceinline__ double min(double x, double y) { return fm::soft::min_s(x, y); }
  static __device__ __forceinline__ bool le0(double x) { return fm::soft::le_zero_s(x); }
  // For a finite Psi, -(0 * Psi) is a zero of the sign opposite to Psi's;
  // adding it returns x unless x is a zero too, and a sum of two zeros is -0
  // only when both are -0.  Infinite or NaN operands take the FP64 form.
  static __device__ __forceinline__ double zp_add(double Psi, double x) {
    const uint32_t ph = fm::soft::hi_word(Psi), xh = fm::soft::hi_word(x),
                   xl = fm::soft::lo_word(x);
    double r = x;
    if (((xh << 1) | xl) == 0u) r = ((ph >> 31) == 0u && (xh >> 31) != 0u) ? -0.0 : 0.0;
    if ((ph & 0x7ff00000u) == 0x7ff00000u || (xh & 0x7ff00000u) == 0x7ff00000u)
      r = zp_add_slow(Psi, x);
    return r;
  }
};

template <typename R, int SF>
using Ar = typename std::conditional<(SF > 0 && sizeof(R) == 8), ArSoft<SF>, ArHw<R>>::type;

// (((a[-2] + 8*a[+1]) - 8*a[-1]) - a[+2]) / (12*dx)
template <typename R, int SF>
__device__ __forceinline__ R d4(R am2, R am1, R ap1, R ap2, const MhdC<R> &k) {
  using AR = Ar<R, SF>;
  const R t1 = AR::x8(ap1);
  const R t2 = am2 + t1;
  const R t3 = AR::x8(am1);
  const R t4 = t2 - t3;
  const R t5 = t4 - ap2;
  return AR::divh(t5, k);
}

// The quantities whose derivative along axis a is needed, at one point.
template <typename R>
struct AxisQ {
  R m, v, P, BB[3], E[3], s, B;
};

// the 11 quantities in a fixed order: m, v, P, BB[0..2], E[0..2], s, B
template <typename R>
__device__ __forceinline__ void axis_arr(const AxisQ<R> &a, R (&q)[11]) {
  q[0] = a.m;
  q[1] = a.v;
  q[2] = a.P;
  q[3] = a.BB[0];
  q[4] = a.BB[1];
  q[5] = a.BB[2];
  q[6] = a.E[0];
  q[7] = a.E[1];
  q[8] = a.E[2];
  q[9] = a.s;
  q[10] = a.B;
}

template <typename R, int SF>
__device__ __forceinline__ AxisQ<R> axis_q(const Fields &Q, size_t i, int a, const MhdC<R> &k) {
  using AR = Ar<R, SF>;
  const R dn = ld<R>(Q.p[0], i);
  const R v0 = ld<R>(Q.p[1], i), v1 = ld<R>(Q.p[2], i), v2 = ld<R>(Q.p[3], i);
  const R B0 = ld<R>(Q.p[4], i), B1 = ld<R>(Q.p[5], i), B2 = ld<R>(Q.p[6], i);
  const R s = ld<R>(Q.p[7], i), Psi = ld<R>(Q.p[8], i);
  const R v[3] = {v0, v1, v2}, B[3] = {B0, B1, B2};
  AxisQ<R> q;
  const R d = k.dens0 + dn;
  q.m = AR::mul(d, v[a]);
  q.v = v[a];
  const R b2 = (AR::mul(B0, B0) + AR::mul(B1, B1)) + AR::mul(B2, B2);
  q.P = (AR::cmul(k.dp_ddens, k.dp_ddens_s, d) + AR::cmul(k.dp_ds, k.dp_ds_s, s)) + AR::cmul(k.c8, k.c8s, b2);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    q.BB[c] = AR::mul(B[a], B[c]);  // B_j * B_i with j = a
    // E_ij = -(0*del_ij*Psi) + v_i*B_j - v_j*B_i with j = a, i = c (0*del_ij is
    // +0 for either value of the delta)
    q.E[c] = AR::zp_add(Psi, AR::mul(v[c], B[a])) - AR::mul(v[a], B[c]);
  }
  q.s = s;
  q.B = B[a];
  return q;
}

// the tile of the staged stage kernels: 32 (z) x 8 (y) cells and a 2-cell halo
constexpr int kTZ = 32, kTY = 8, kH = 2, kRZ = kTZ + 2 * kH, kRY = kTY + 2 * kH;
constexpr int kNP = kRZ * kRY;  // 432 points
constexpr int kNV = 20;

// One point of the staged region of the tiled stage kernels: the 20 y/z-derivative
// quantities (d v_y, d v_z, v_y, v_z, P, B_y B_c, B_z B_c, E_cy, E_cz, s, B_y, B_z)
// of point i, stored at index pt of each quantity's plane in shared memory.
template <typename R, int SF>
__device__ __forceinline__ void stage_point(const Fields &Q, size_t i, const MhdC<R> &k, R *sv,
                                            int pt) {
  using AR = Ar<R, SF>;
  const R dn = ld<R>(Q.p[0], i);
  const R v[3] = {ld<R>(Q.p[1], i), ld<R>(Q.p[2], i), ld<R>(Q.p[3], i)};
  const R B[3] = {ld<R>(Q.p[4], i), ld<R>(Q.p[5], i), ld<R>(Q.p[6], i)};
  const R s = ld<R>(Q.p[7], i), Psi = ld<R>(Q.p[8], i);
  const R d = k.dens0 + dn;
  const R b2 = (AR::mul(B[0], B[0]) + AR::mul(B[1], B[1])) + AR::mul(B[2], B[2]);
  sv[0 * kNP + pt] = AR::mul(d, v[1]);
  sv[1 * kNP + pt] = AR::mul(d, v[2]);
  sv[2 * kNP + pt] = v[1];
  sv[3 * kNP + pt] = v[2];
  sv[4 * kNP + pt] = (AR::cmul(k.dp_ddens, k.dp_ddens_s, d) + AR::cmul(k.dp_ds, k.dp_ds_s, s)) + AR::cmul(k.c8, k.c8s, b2);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    sv[(5 + c) * kNP + pt] = AR::mul(B[1], B[c]);
    sv[(8 + c) * kNP + pt] = AR::mul(B[2], B[c]);
    sv[(11 + c) * kNP + pt] = AR::zp_add(Psi, AR::mul(v[c], B[1])) - AR::mul(v[1], B[c]);
    sv[(14 + c) * kNP + pt] = AR::zp_add(Psi, AR::mul(v[c], B[2])) - AR::mul(v[2], B[c]);
  }
  sv[17 * kNP + pt] = s;
  sv[18 * kNP + pt] = B[1];
  sv[19 * kNP + pt] = B[2];
}

// f = ddt_sys (3d-mhd-rk4.fmr:83-101) from the 33 derivatives, the velocity, Psi
// and the prepared divisor dens (the expressions and order of the generated code).
template <typename R, int SF>
__device__ __forceinline__ void assemble_f(const R (&dm)[3], const R (&dv)[3], const R (&dP)[3],
                                           const R (&dBB)[3][3], const R (&dE)[3][3],
                                           const R (&ds)[3], const R (&dB)[3], const R (&v)[3],
                                           R Psi, const typename Ar<R, SF>::Den &dd,
                                           const MhdC<R> &k, R (&f)[NF]) {
  using AR = Ar<R, SF>;
  f[0] = -(((dm[0]) + (dm[1])) + (dm[2]));
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const R A = (AR::mul(v[0], dv[i]) + AR::mul(v[1], dv[i])) + AR::mul(v[2], dv[i]);
    const R Y = ((dBB[0][i]) + (dBB[1][i])) + (dBB[2][i]);
    f[1 + i] = ((-A) - AR::div(dP[i], dd)) + AR::div(AR::cmul(k.c4, k.c4s, Y), dd);
    f[4 + i] = ((dE[i][0]) + (dE[i][1])) + (dE[i][2]);
  }
  f[7] = (AR::mul(v[0], ds[0]) + AR::mul(v[1], ds[1])) + AR::mul(v[2], ds[2]);
  const R divB = ((dB[0]) + (dB[1])) + (dB[2]);
  f[8] = (-AR::cmul(k.c_h2, k.c_h2s, divB)) - AR::cmul(k.ch2_cp2, k.ch2_cp2s, Psi);
}

template <typename R, int SF>
__global__ void __launch_bounds__(128)
    mhd_stage(Fields Q, Fields S, Fields O, int n, MhdC<R> k) {
  using AR = Ar<R, SF>;
  const int z = blockIdx.x * 32 + (threadIdx.x & 31);
  const int y = blockIdx.y * 4 + (threadIdx.x >> 5);
  const int x = blockIdx.z;
  if (z >= n || y >= n) return;
  const size_t sx = (size_t)n * n, sy = (size_t)n;
  const size_t c = (size_t)x * sx + (size_t)y * sy + z;
  const int co[3] = {x, y, z};
  const size_t st[3] = {sx, sy, 1};
  // derivative results
  R dm[3], dv[3], dP[3], dBB[3][3], dE[3][3], ds[3], dB[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const size_t base = c - (size_t)co[a] * st[a];
    const int im2 = co[a] - 2 < 0 ? co[a] - 2 + n : co[a] - 2;
    const int im1 = co[a] - 1 < 0 ? co[a] - 1 + n : co[a] - 1;
    const int ip1 = co[a] + 1 >= n ? co[a] + 1 - n : co[a] + 1;
    const int ip2 = co[a] + 2 >= n ? co[a] + 2 - n : co[a] + 2;
    const AxisQ<R> qm2 = axis_q<R, SF>(Q, base + (size_t)im2 * st[a], a, k);
    const AxisQ<R> qm1 = axis_q<R, SF>(Q, base + (size_t)im1 * st[a], a, k);
    const AxisQ<R> qp1 = axis_q<R, SF>(Q, base + (size_t)ip1 * st[a], a, k);
    const AxisQ<R> qp2 = axis_q<R, SF>(Q, base + (size_t)ip2 * st[a], a, k);
    dm[a] = d4<R, SF>(qm2.m, qm1.m, qp1.m, qp2.m, k);
    dv[a] = d4<R, SF>(qm2.v, qm1.v, qp1.v, qp2.v, k);
    dP[a] = d4<R, SF>(qm2.P, qm1.P, qp1.P, qp2.P, k);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      dBB[a][i] = d4<R, SF>(qm2.BB[i], qm1.BB[i], qp1.BB[i], qp2.BB[i], k);
      dE[i][a] = d4<R, SF>(qm2.E[i], qm1.E[i], qp1.E[i], qp2.E[i], k);
    }
    ds[a] = d4<R, SF>(qm2.s, qm1.s, qp1.s, qp2.s, k);
    dB[a] = d4<R, SF>(qm2.B, qm1.B, qp1.B, qp2.B, k);
  }
  const R dn = ld<R>(Q.p[0], c);
  const R v[3] = {ld<R>(Q.p[1], c), ld<R>(Q.p[2], c), ld<R>(Q.p[3], c)};
  const R Psi = ld<R>(Q.p[8], c);
  const R dens = k.dens0 + dn;
  const typename AR::Den dd = AR::prep(dens);
  R f[NF];
  assemble_f<R, SF>(dm, dv, dP, dBB, dE, ds, dB, v, Psi, dd, k, f);
#pragma unroll
  for (int q = 0; q < NF; ++q)
    reinterpret_cast<R *>(O.p[q])[c] = ld<R>(S.p[q], c) + AR::cmul(k.dt_c, k.dts, f[q]);
}

// mhd_stage_tile: the same stage, with the composite quantities of the y and z
// derivatives computed ONCE per point.  A CTA owns a 32 (z) x 8 (y) tile of
// one x plane; it first evaluates, for every point of the tile and a 2-point
// periodic halo in y and z (36 x 12 points), the 20 values the y and z
// derivatives read (d*v_a, v_a, P, B_a*B_c, E_ca, s, B_a for a = y, z) into
// shared memory ([value][point], conflict-free along z); the y and z
// derivatives then read their four neighbours there.  The x derivatives
// evaluate the composites at x-2 .. x+2 as mhd_stage does.  Every value is
// the same IEEE expression as in axis_q, so results are bit-identical with
// mhd_stage (and, for R = double, with the all-FP64 program).

// binary32: 5 CTAs per SM (48 registers, 24 bytes spilled) measured 3.51 against 3.43
// GLUP/s at 4 (64 registers)
template <typename R, int SF>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 5 : 1)
    mhd_stage_tile(Fields Q, Fields S, Fields O, int n, MhdC<R> k) {
  using AR = Ar<R, SF>;
  extern __shared__ __align__(16) unsigned char mhd_smem[];
  R *sv = reinterpret_cast<R *>(mhd_smem);  // [kNV][kNP]
  const int tz = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int z0 = blockIdx.x * kTZ, y0 = blockIdx.y * kTY, x = blockIdx.z;
  const size_t sx = (size_t)n * n, sy = (size_t)n;
  const bool big = n >= kRZ;  // one conditional add/subtract wraps every region coordinate
  for (int pt = threadIdx.x; pt < kNP; pt += 256) {
    const int ry = pt / kRZ, rz = pt - ry * kRZ;
    int gy = y0 - kH + ry, gz = z0 - kH + rz;
    if (big) {
      gy = gy < 0 ? gy + n : (gy >= n ? gy - n : gy);
      gz = gz < 0 ? gz + n : (gz >= n ? gz - n : gz);
    } else {
      gy %= n;
      gy = gy < 0 ? gy + n : gy;
      gz %= n;
      gz = gz < 0 ? gz + n : gz;
    }
    const size_t i = (size_t)x * sx + (size_t)gy * sy + gz;
    stage_point<R, SF>(Q, i, k, sv, pt);
  }
  __syncthreads();
  const int y = y0 + ty, z = z0 + tz;
  if (y >= n || z >= n) return;
  const size_t c = (size_t)x * sx + (size_t)y * sy + z;
  const int p0 = (ty + kH) * kRZ + (tz + kH);
  auto dy = [&](int v) {
    const R *b = sv + v * kNP + p0;
    return d4<R, SF>(b[-2 * kRZ], b[-kRZ], b[kRZ], b[2 * kRZ], k);
  };
  auto dz = [&](int v) {
    const R *b = sv + v * kNP + p0;
    return d4<R, SF>(b[-2], b[-1], b[1], b[2], k);
  };
  if constexpr (sizeof(R) == 8) {
    // FP64: 70 instead of 114 registers (3 CTAs per SM instead of 2), +2 %.
    // x derivatives of the 11 x composites, accumulated in d4's order of
    // operations (((a[-2] + 8a[+1]) - 8a[-1]) - a[+2]) / (12 dx) so that one
    // neighbour's composites are live at a time
    R gx[11];
    {
      const int im2 = x - 2 < 0 ? x - 2 + n : x - 2;
      const int im1 = x - 1 < 0 ? x - 1 + n : x - 1;
      const int ip1 = x + 1 >= n ? x + 1 - n : x + 1;
      const int ip2 = x + 2 >= n ? x + 2 - n : x + 2;
      const size_t base = c - (size_t)x * sx;
      R q[11];
      axis_arr<R>(axis_q<R, SF>(Q, base + (size_t)im2 * sx, 0, k), q);
#pragma unroll
      for (int j = 0; j < 11; ++j) gx[j] = q[j];
      axis_arr<R>(axis_q<R, SF>(Q, base + (size_t)ip1 * sx, 0, k), q);
#pragma unroll
      for (int j = 0; j < 11; ++j) gx[j] = gx[j] + AR::x8(q[j]);
      axis_arr<R>(axis_q<R, SF>(Q, base + (size_t)im1 * sx, 0, k), q);
#pragma unroll
      for (int j = 0; j < 11; ++j) gx[j] = gx[j] - AR::x8(q[j]);
      axis_arr<R>(axis_q<R, SF>(Q, base + (size_t)ip2 * sx, 0, k), q);
#pragma unroll
      for (int j = 0; j < 11; ++j) gx[j] = AR::divh(gx[j] - q[j], k);
    }
    // f = ddt_sys, each component assembled as its y and z derivatives are
    // taken from shared memory, and written out at once
    const R dn = ld<R>(Q.p[0], c);
    const R v[3] = {ld<R>(Q.p[1], c), sv[2 * kNP + p0], sv[3 * kNP + p0]};
    const R Psi = ld<R>(Q.p[8], c);
    const R dens = k.dens0 + dn;
    const typename AR::Den dd = AR::prep(dens);
    auto out = [&](int q, R fq) {
      reinterpret_cast<R *>(O.p[q])[c] = ld<R>(S.p[q], c) + AR::cmul(k.dt_c, k.dts, fq);
    };
    out(0, -((gx[0] + dy(0)) + dz(1)));
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const R dvi = i == 0 ? gx[1] : (i == 1 ? dy(2) : dz(3));
      const R A = (AR::mul(v[0], dvi) + AR::mul(v[1], dvi)) + AR::mul(v[2], dvi);
      const R Y = (gx[3 + i] + dy(5 + i)) + dz(8 + i);
      const R dPi = i == 0 ? gx[2] : (i == 1 ? dy(4) : dz(4));
      out(1 + i, ((-A) - AR::div(dPi, dd)) + AR::div(AR::cmul(k.c4, k.c4s, Y), dd));
      out(4 + i, (gx[6 + i] + dy(11 + i)) + dz(14 + i));
    }
    out(7, (AR::mul(v[0], gx[9]) + AR::mul(v[1], dy(17))) + AR::mul(v[2], dz(17)));
    const R divB = (gx[10] + dy(18)) + dz(19);
    out(8, (-AR::cmul(k.c_h2, k.c_h2s, divB)) - AR::cmul(k.ch2_cp2, k.ch2_cp2s, Psi));
  } else {
    // binary32 (issue-bound): all 33 derivatives first measured 6 % faster
    R dm[3], dv[3], dP[3], dBB[3][3], dE[3][3], ds[3], dB[3];
    {
      const int im2 = x - 2 < 0 ? x - 2 + n : x - 2;
      const int im1 = x - 1 < 0 ? x - 1 + n : x - 1;
      const int ip1 = x + 1 >= n ? x + 1 - n : x + 1;
      const int ip2 = x + 2 >= n ? x + 2 - n : x + 2;
      const size_t base = c - (size_t)x * sx;
      const AxisQ<R> qm2 = axis_q<R, SF>(Q, base + (size_t)im2 * sx, 0, k);
      const AxisQ<R> qm1 = axis_q<R, SF>(Q, base + (size_t)im1 * sx, 0, k);
      const AxisQ<R> qp1 = axis_q<R, SF>(Q, base + (size_t)ip1 * sx, 0, k);
      const AxisQ<R> qp2 = axis_q<R, SF>(Q, base + (size_t)ip2 * sx, 0, k);
      dm[0] = d4<R, SF>(qm2.m, qm1.m, qp1.m, qp2.m, k);
      dv[0] = d4<R, SF>(qm2.v, qm1.v, qp1.v, qp2.v, k);
      dP[0] = d4<R, SF>(qm2.P, qm1.P, qp1.P, qp2.P, k);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        dBB[0][i] = d4<R, SF>(qm2.BB[i], qm1.BB[i], qp1.BB[i], qp2.BB[i], k);
        dE[i][0] = d4<R, SF>(qm2.E[i], qm1.E[i], qp1.E[i], qp2.E[i], k);
      }
      ds[0] = d4<R, SF>(qm2.s, qm1.s, qp1.s, qp2.s, k);
      dB[0] = d4<R, SF>(qm2.B, qm1.B, qp1.B, qp2.B, k);
    }
    dm[1] = dy(0);
    dm[2] = dz(1);
    dv[1] = dy(2);
    dv[2] = dz(3);
    dP[1] = dy(4);
    dP[2] = dz(4);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      dBB[1][i] = dy(5 + i);
      dBB[2][i] = dz(8 + i);
      dE[i][1] = dy(11 + i);
      dE[i][2] = dz(14 + i);
    }
    ds[1] = dy(17);
    ds[2] = dz(17);
    dB[1] = dy(18);
    dB[2] = dz(19);
    const R dn = ld<R>(Q.p[0], c);
    const R v[3] = {ld<R>(Q.p[1], c), sv[2 * kNP + p0], sv[3 * kNP + p0]};
    const R Psi = ld<R>(Q.p[8], c);
    const R dens = k.dens0 + dn;
    const typename AR::Den dd = AR::prep(dens);
    R f[NF];
    assemble_f<R, SF>(dm, dv, dP, dBB, dE, ds, dB, v, Psi, dd, k, f);
#pragma unroll
    for (int q = 0; q < NF; ++q)
      reinterpret_cast<R *>(O.p[q])[c] = ld<R>(S.p[q], c) + AR::cmul(k.dt_c, k.dts, f[q]);
  }
}

// Exact binary64 values of binary32 quantities for the FP64 numerical heat of
// the float path, built on the integer pipes (the FP64 pipe is the scarce one):
// a float widens to double exactly (rebias the exponent, shift the fraction),
// and the square of a float is exact in double (a 24-bit significand squared
// has at most 48 bits).  Zero is handled inline; subnormal, infinite and NaN
// inputs take the FP64 instructions.  For R = double both are the plain
// operations.
__device__ __forceinline__ double widen(float a) {
  const unsigned b = __float_as_uint(a);
  const unsigned e = (b >> 23) & 0xffu;
  if (e - 1u < 254u) {
    const unsigned m = b & 0x7fffffu;
    return __hiloint2double((int)((b & 0x80000000u) | ((e + 896u) << 20) | (m >> 3)),
                            (int)(m << 29));
  }
  if ((b << 1) == 0u) return __hiloint2double((int)(b & 0x80000000u), 0);
  return (double)a;
}
__device__ __forceinline__ double widen(double a) { return a; }

__device__ __forceinline__ double exact_sq(float a) {
  const unsigned b = __float_as_uint(a);
  const unsigned e = (b >> 23) & 0xffu;
  if (e - 1u < 254u) {
    const unsigned M = (b & 0x7fffffu) | 0x800000u;
    const unsigned long long P = (unsigned long long)M * M;  // in [2^46, 2^48)
    const unsigned top = (unsigned)(P >> 47);                // 1 if P >= 2^47
    const unsigned long long F = (P << (5 + (top ^ 1u))) & 0x000fffffffffffffull;
    const unsigned E = 2u * e + 769u + top;                  // biased exponent
    return __hiloint2double((int)((E << 20) | (unsigned)(F >> 32)), (int)(unsigned)F);
  }
  if ((b << 1) == 0u) return 0.0;
  const double d = (double)a;
  return d * d;
}
__device__ __forceinline__ double exact_sq(double a) { return a * a; }

// numerical_heat (3d-mhd-rk4.fmr:141-143) in FP64: r, b the velocity and field
// of the stage output, nn, nm after the viscosity step, dens the step's input
// density perturbation.
template <typename R, int SF>
__device__ __forceinline__ double numerical_heat(const R r[3], const R b[3], const R nn[3],
                                                 const R nm[3], R dens, const MhdC<R> &k) {
  using AD = Ar<double, sizeof(R) == 8 ? SF : 0>;
  const double svr = (exact_sq(r[0]) + exact_sq(r[1])) + exact_sq(r[2]);
  const double svn = (exact_sq(nn[0]) + exact_sq(nn[1])) + exact_sq(nn[2]);
  const double sbr = (exact_sq(b[0]) + exact_sq(b[1])) + exact_sq(b[2]);
  const double sbn = (exact_sq(nm[0]) + exact_sq(nm[1])) + exact_sq(nm[2]);
  const double den8 = AD::cmul(8.0 * 3.141592653589793, k.c8pi_s, 1.0 + widen(dens));
  return AD::half(svr - svn) + AD::mul(AD::div(1.0, AD::prep(den8)), sbr - sbn);
}

// mhd_stage_march: mhd_stage_tile marching along x over a chunk of planes,
// with the 11 composite quantities of the x derivatives (axis_q along x) of
// planes x-2 .. x+2 kept in a register ring per thread: each plane's
// composites are evaluated once instead of at four x neighbours.  Same
// expressions: bit-identical with mhd_stage and mhd_stage_tile.
template <typename R, int SF>
__device__ __forceinline__ void x_comp(const Fields &Q, size_t i, const MhdC<R> &k, R (&q)[11]) {
  axis_arr<R>(axis_q<R, SF>(Q, i, 0, k), q);
}

template <typename R, int SF>
__global__ void __launch_bounds__(256, 2)
    mhd_stage_march(Fields Q, Fields S, Fields O, int n, int xchunk, int ntiles_yz, int ntiles,
                    MhdC<R> k) {
  using AR = Ar<R, SF>;
  extern __shared__ __align__(16) unsigned char mhd_smem[];
  R *sv = reinterpret_cast<R *>(mhd_smem);  // [kNV][kNP]
  const int tz = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const size_t sx = (size_t)n * n, sy = (size_t)n;
  const int ntz = (n + kTZ - 1) / kTZ;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int tyz = t % ntiles_yz;
    const int z0 = (tyz % ntz) * kTZ, y0 = (tyz / ntz) * kTY;
    const int x0 = (t / ntiles_yz) * xchunk;
    const int x1 = min(x0 + xchunk, n);
    const int y = y0 + ty, z = z0 + tz;
    const bool own = y < n && z < n;
    const size_t yz = own ? (size_t)y * sy + z : 0;
    // region points this thread stages (in-plane offsets)
    size_t soff[2];
    int spt[2];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int pt = threadIdx.x + 256 * j;
      spt[j] = pt < kNP ? pt : -1;
      const int ptc = pt < kNP ? pt : 0;
      const int ry = ptc / kRZ, rz = ptc - ry * kRZ;
      int gy = (y0 - kH + ry) % n;
      gy = gy < 0 ? gy + n : gy;
      int gz = (z0 - kH + rz) % n;
      gz = gz < 0 ? gz + n : gz;
      soff[j] = (size_t)gy * sy + gz;
    }
    R ring[5][11];  // x composites of planes x-2 .. x+2
    if (own) {
#pragma unroll
      for (int d = 0; d < 4; ++d) {
        int q = (x0 - 2 + d) % n;
        q = q < 0 ? q + n : q;
        x_comp<R, SF>(Q, (size_t)q * sx + yz, k, ring[d + 1]);
      }
    }
    for (int x = x0; x < x1; ++x) {
      const size_t px = (size_t)x * sx;
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        if (spt[j] < 0) continue;
        const int pt = spt[j];
        const size_t i = px + soff[j];
        stage_point<R, SF>(Q, i, k, sv, pt);
      }
      __syncthreads();
      if (own) {
        // ring: planes x-2 .. x+2 after shifting in plane x+2
#pragma unroll
        for (int d = 0; d < 4; ++d)
#pragma unroll
          for (int v = 0; v < 11; ++v) ring[d][v] = ring[d + 1][v];
        x_comp<R, SF>(Q, (size_t)((x + 2) % n) * sx + yz, k, ring[4]);
        const size_t c = px + yz;
        const int p0 = (ty + kH) * kRZ + (tz + kH);
        auto dy = [&](int v) {
          const R *b = sv + v * kNP + p0;
          return d4<R, SF>(b[-2 * kRZ], b[-kRZ], b[kRZ], b[2 * kRZ], k);
        };
        auto dz = [&](int v) {
          const R *b = sv + v * kNP + p0;
          return d4<R, SF>(b[-2], b[-1], b[1], b[2], k);
        };
        auto dx = [&](int v) { return d4<R, SF>(ring[0][v], ring[1][v], ring[3][v], ring[4][v], k); };
        R dm[3], dv[3], dP[3], dBB[3][3], dE[3][3], ds[3], dB[3];
        dm[0] = dx(0);
        dv[0] = dx(1);
        dP[0] = dx(2);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          dBB[0][i] = dx(3 + i);
          dE[i][0] = dx(6 + i);
        }
        ds[0] = dx(9);
        dB[0] = dx(10);
        dm[1] = dy(0);
        dm[2] = dz(1);
        dv[1] = dy(2);
        dv[2] = dz(3);
        dP[1] = dy(4);
        dP[2] = dz(4);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          dBB[1][i] = dy(5 + i);
          dBB[2][i] = dz(8 + i);
          dE[i][1] = dy(11 + i);
          dE[i][2] = dz(14 + i);
        }
        ds[1] = dy(17);
        ds[2] = dz(17);
        dB[1] = dy(18);
        dB[2] = dz(19);
        const R dn = ld<R>(Q.p[0], c);
        const R v[3] = {ring[2][1], sv[2 * kNP + p0], sv[3 * kNP + p0]};
        const R Psi = ld<R>(Q.p[8], c);
        const R dens = k.dens0 + dn;
        const typename AR::Den dd = AR::prep(dens);
        R f[NF];
        assemble_f<R, SF>(dm, dv, dP, dBB, dE, ds, dB, v, Psi, dd, k, f);
#pragma unroll
        for (int q = 0; q < NF; ++q)
          reinterpret_cast<R *>(O.p[q])[c] = ld<R>(S.p[q], c) + AR::cmul(k.dt_c, k.dts, f[q]);
      }
      __syncthreads();
    }
  }
}

// `<%` of three: fmin(0, fmax(a, fmax(b, c))) + fmax(0, fmin(a, fmin(b, c)))
template <typename R, int SF>
__device__ __forceinline__ R minmod3(R a, R b, R c) {
  using AR = Ar<R, SF>;
  return AR::min(R(0), AR::max(a, AR::max(b, c))) + AR::max(R(0), AR::min(a, AR::min(b, c)));
}

// (up - um)/2 is x*0.5 exactly; the limiter's factors 1.4, 0.75, 0.15 and
// the products go through Ar.
template <typename R, int SF>
__device__ __forceinline__ R slope(R um, R u0, R up, const MhdC<R> &k) {
  using AR = Ar<R, SF>;
  return minmod3<R, SF>(AR::half(up - um), AR::cmul(R(1.4), k.c1_4s, up - u0),
                    AR::cmul(R(1.4), k.c1_4s, u0 - um));
}

template <typename R, int SF>
__device__ __forceinline__ R av_flux(R num, R den, const MhdC<R> &k) {
  using AR = Ar<R, SF>;
  const R nd = AR::mul(num, den);
  const bool cut = AR::le0(nd);
  const R r = AR::div_unless(num, den, cut);
  const R t = AR::cmul(R(0.75), k.c0_75s, r - R(1));
  const R phi1 = AR::min(R(1), AR::max(R(0), R(1) + t));
  const R Phi = cut ? R(0) : phi1;
  return -AR::mul(AR::cmul(R(0.15), k.c0_15s, Phi), num);
}

// flux at the face between u0 and u1, given u[-1], u0, u1, u[+2]
template <typename R, int SF>
__device__ __forceinline__ R face(R um, R u0, R u1, R u2, const MhdC<R> &k) {
  using AR = Ar<R, SF>;
  const R ul = u0 + AR::half(slope<R, SF>(um, u0, u1, k));
  const R ur = u1 - AR::half(slope<R, SF>(u0, u1, u2, k));
  return av_flux<R, SF>(ur - ul, u1 - u0, k);
}

// binary32: 8 CTAs per SM (64 registers) measured 3.54 against 3.51 GLUP/s at 7
template <typename R, int SF>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? 8 : 1)
    mhd_finish(Fields N, Fields S, int n, MhdC<R> k) {
  const int z = blockIdx.x * 32 + (threadIdx.x & 31);
  const int y = blockIdx.y * 4 + (threadIdx.x >> 5);
  const int x = blockIdx.z;
  if (z >= n || y >= n) return;
  const size_t sx = (size_t)n * n, sy = (size_t)n;
  const size_t c = (size_t)x * sx + (size_t)y * sy + z;
  const int co[3] = {x, y, z};
  const size_t st[3] = {sx, sy, 1};
  size_t off[3][5];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const size_t base = c - (size_t)co[a] * st[a];
#pragma unroll
    for (int d = -2; d <= 2; ++d) {
      int q = co[a] + d;
      q = q < 0 ? q + n : (q >= n ? q - n : q);
      off[a][d + 2] = base + (size_t)q * st[a];
    }
  }
  R nv[NF];
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    const R uc = ld<R>(N.p[f], c);  // off[a][2] == c on every axis
    R w = uc;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const R u[5] = {ld<R>(N.p[f], off[a][0]), ld<R>(N.p[f], off[a][1]), uc,
                      ld<R>(N.p[f], off[a][3]), ld<R>(N.p[f], off[a][4])};
      const R fm = face<R, SF>(u[0], u[1], u[2], u[3], k);  // avf[i-1/2]
      const R fp = face<R, SF>(u[1], u[2], u[3], u[4], k);  // avf[i+1/2]
      w = (w + fm) - fp;
    }
    nv[f] = w;
  }
  // numerical_heat (3d-mhd-rk4.fmr:141-143), always in FP64; dens = the
  // step's input density perturbation.  S is written below, so it is read
  // through the coherent path (not __ldg).
  const R r[3] = {ld<R>(N.p[1], c), ld<R>(N.p[2], c), ld<R>(N.p[3], c)};
  const R b[3] = {ld<R>(N.p[4], c), ld<R>(N.p[5], c), ld<R>(N.p[6], c)};
  const R nn[3] = {nv[1], nv[2], nv[3]}, nm[3] = {nv[4], nv[5], nv[6]};
  const double heat =
      numerical_heat<R, SF>(r, b, nn, nm, reinterpret_cast<const R *>(S.p[0])[c], k);
  reinterpret_cast<R *>(S.p[0])[c] = Ar<R, SF>::max(nv[0], R(-0.9));
#pragma unroll
  for (int f = 1; f < NF; ++f)
    if (f != 7) reinterpret_cast<R *>(S.p[f])[c] = nv[f];
  reinterpret_cast<R *>(S.p[7])[c] = (R)(widen(nv[7]) + heat);
}

// The flux at the face between ua and ub from the slopes at both cells: the
// expression of face() with slope(um, ua, ub) = sla and slope(ua, ub, u2) = slb.
template <typename R, int SF>
__device__ __forceinline__ R face_from_slopes(R ua, R ub, R sla, R slb, const MhdC<R> &k) {
  using AR = Ar<R, SF>;
  const R ul = ua + AR::half(sla);
  const R ur = ub - AR::half(slb);
  return av_flux<R, SF>(ur - ul, ub - ua, k);
}

// mhd_finish_v2: the finishing step with every slope computed once per cell
// and axis (a slope is shared by the two faces of its cell) and every face
// flux once per face (shared by the two cells of the face), all 9 fields per
// plane.  CTA = a 32 (z) x 8 (y) tile marching along x over a chunk of
// planes.  Per plane: the 9 fields over the tile and a 2-point periodic halo
// are staged into shared memory; y slopes (10 rows) and z slopes (34 columns)
// go to shared memory, then the 9 y faces and 33 z faces of the tile; x
// slopes and faces are carried in registers along the march.  Same
// expressions and the same accumulation order as mhd_finish: bit-identical.
constexpr int kFY = kTY + 1, kFZ = kTZ + 1;      // faces per column / row
constexpr int kSY = kTY + 2, kSZ = kTZ + 2;      // slopes per column / row
template <typename R>
struct FinishSmem {
  R u[NF][kRY][kRZ];
  R sly[NF][kSY][kTZ];
  R slz[NF][kTY][kSZ];
  R fy[NF][kFY][kTZ];
  R fz[NF][kTY][kFZ];
};

template <typename R, int SF>
__global__ void __launch_bounds__(256, 2)
    mhd_finish_v2(Fields N, Fields S, int n, int xchunk, int ntiles_yz, int ntiles, MhdC<R> k) {
  extern __shared__ __align__(16) unsigned char fin_smem[];
  FinishSmem<R> &sm = *reinterpret_cast<FinishSmem<R> *>(fin_smem);
  const int tz = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const size_t sx = (size_t)n * n, sy = (size_t)n;
  const int ntz = (n + kTZ - 1) / kTZ;
  const R *uf[NF];
#pragma unroll
  for (int f = 0; f < NF; ++f) uf[f] = reinterpret_cast<const R *>(N.p[f]);
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int tyz = t % ntiles_yz;
    const int z0 = (tyz % ntz) * kTZ, y0 = (tyz / ntz) * kTY;
    const int x0 = (t / ntiles_yz) * xchunk;
    const int x1 = min(x0 + xchunk, n);
    const int y = y0 + ty, z = z0 + tz;
    const bool own = y < n && z < n;
    const size_t yz = own ? (size_t)y * sy + z : 0;
    // in-plane offsets of the (up to two) region points this thread stages
    size_t soff[2];
    int spt[2];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int pt = threadIdx.x + 256 * j;
      spt[j] = pt < kNP ? pt : -1;
      const int ptc = pt < kNP ? pt : 0;
      const int ry = ptc / kRZ, rz = ptc - ry * kRZ;
      int gy = (y0 - kH + ry) % n;
      gy = gy < 0 ? gy + n : gy;
      int gz = (z0 - kH + rz) % n;
      gz = gz < 0 ? gz + n : gz;
      soff[j] = (size_t)gy * sy + gz;
    }
    // x carry per field: u[x], u[x+1], slope at x, flux at x-1/2
    R cu1[NF], cu2[NF], csl[NF], cfm[NF];
    if (own) {
      int q[4];
#pragma unroll
      for (int d = 0; d < 4; ++d) {
        q[d] = (x0 - 2 + d) % n;
        q[d] = q[d] < 0 ? q[d] + n : q[d];
      }
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        const R a = __ldg(uf[f] + (size_t)q[0] * sx + yz), b = __ldg(uf[f] + (size_t)q[1] * sx + yz);
        const R c = __ldg(uf[f] + (size_t)q[2] * sx + yz), d = __ldg(uf[f] + (size_t)q[3] * sx + yz);
        const R slm = slope<R, SF>(a, b, c, k);  // at x0-1
        const R sl0 = slope<R, SF>(b, c, d, k);  // at x0
        cfm[f] = face_from_slopes<R, SF>(b, c, slm, sl0, k);
        cu1[f] = c;
        cu2[f] = d;
        csl[f] = sl0;
      }
    }
    for (int x = x0; x < x1; ++x) {
      const size_t px = (size_t)x * sx;
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        if (spt[j] >= 0) {
          const int ry = spt[j] / kRZ, rz = spt[j] - ry * kRZ;
#pragma unroll
          for (int f = 0; f < NF; ++f) sm.u[f][ry][rz] = __ldg(uf[f] + px + soff[j]);
        }
      }
      __syncthreads();
      // slopes: y at region rows 1..10 over the tile columns; z at region
      // columns 1..34 over the tile rows
      for (int q = threadIdx.x; q < NF * kSY * kTZ; q += 256) {
        const int f = q / (kSY * kTZ), rem = q - f * (kSY * kTZ);
        const int r = rem / kTZ, c = rem - r * kTZ;
        const int ry = r + 1, rz = c + kH;
        sm.sly[f][r][c] = slope<R, SF>(sm.u[f][ry - 1][rz], sm.u[f][ry][rz], sm.u[f][ry + 1][rz], k);
      }
      for (int q = threadIdx.x; q < NF * kTY * kSZ; q += 256) {
        const int f = q / (kTY * kSZ), rem = q - f * (kTY * kSZ);
        const int r = rem / kSZ, c = rem - r * kSZ;
        const int ry = r + kH, rz = c + 1;
        sm.slz[f][r][c] = slope<R, SF>(sm.u[f][ry][rz - 1], sm.u[f][ry][rz], sm.u[f][ry][rz + 1], k);
      }
      __syncthreads();
      // faces: y face i lies between region rows i+1 and i+2 (slope rows i, i+1);
      // z face j between region columns j+1 and j+2 (slope columns j, j+1)
      for (int q = threadIdx.x; q < NF * kFY * kTZ; q += 256) {
        const int f = q / (kFY * kTZ), rem = q - f * (kFY * kTZ);
        const int i = rem / kTZ, c = rem - i * kTZ;
        sm.fy[f][i][c] = face_from_slopes<R, SF>(sm.u[f][i + 1][c + kH], sm.u[f][i + 2][c + kH],
                                             sm.sly[f][i][c], sm.sly[f][i + 1][c], k);
      }
      for (int q = threadIdx.x; q < NF * kTY * kFZ; q += 256) {
        const int f = q / (kTY * kFZ), rem = q - f * (kTY * kFZ);
        const int r = rem / kFZ, j = rem - r * kFZ;
        sm.fz[f][r][j] = face_from_slopes<R, SF>(sm.u[f][r + kH][j + 1], sm.u[f][r + kH][j + 2],
                                             sm.slz[f][r][j], sm.slz[f][r][j + 1], k);
      }
      __syncthreads();
      if (own) {
        const int q2 = (x + 2) % n;
        const size_t c = px + yz;
        R nv[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) {
          const R u2 = __ldg(uf[f] + (size_t)q2 * sx + yz);
          const R sl1 = slope<R, SF>(cu1[f], cu2[f], u2, k);  // at x+1
          const R fxp = face_from_slopes<R, SF>(cu1[f], cu2[f], csl[f], sl1, k);
          R w = sm.u[f][ty + kH][tz + kH];
          w = (w + cfm[f]) - fxp;
          w = (w + sm.fy[f][ty][tz]) - sm.fy[f][ty + 1][tz];
          w = (w + sm.fz[f][ty][tz]) - sm.fz[f][ty][tz + 1];
          nv[f] = w;
          cfm[f] = fxp;
          cu1[f] = cu2[f];
          cu2[f] = u2;
          csl[f] = sl1;
        }
        // numerical_heat (3d-mhd-rk4.fmr:141-143), always in FP64
        const int cy = ty + kH, cz = tz + kH;
        const R r[3] = {sm.u[1][cy][cz], sm.u[2][cy][cz], sm.u[3][cy][cz]};
        const R b[3] = {sm.u[4][cy][cz], sm.u[5][cy][cz], sm.u[6][cy][cz]};
        const R nn[3] = {nv[1], nv[2], nv[3]}, nm[3] = {nv[4], nv[5], nv[6]};
        const double heat =
            numerical_heat<R, SF>(r, b, nn, nm, reinterpret_cast<const R *>(S.p[0])[c], k);
        reinterpret_cast<R *>(S.p[0])[c] = Ar<R, SF>::max(nv[0], R(-0.9));
#pragma unroll
        for (int f = 1; f < NF; ++f)
          if (f != 7) reinterpret_cast<R *>(S.p[f])[c] = nv[f];
        reinterpret_cast<R *>(S.p[7])[c] = (R)(widen(nv[7]) + heat);
      }
      __syncthreads();
    }
  }
}

// Conserved totals in FP64: mass perturbation, kinetic + magnetic energy,
// s, and the x-momentum; fixed tree as in fm_reduce.cu.
template <typename R>
__global__ void __launch_bounds__(256)
    mhd_totals_stage1(Fields S, long long ncell, long long chunk, double *partials) {
  __shared__ double sh[4][256];
  const long long lo = (long long)blockIdx.x * chunk;
  const long long hi = min(lo + chunk, ncell);
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const double c8 = 1.0 / (8.0 * 3.141592653589793);
  for (long long i = lo + threadIdx.x; i < hi; i += 256) {
    const double d = 1.0 + (double)ld<R>(S.p[0], i);
    const double v0 = ld<R>(S.p[1], i), v1 = ld<R>(S.p[2], i), v2 = ld<R>(S.p[3], i);
    const double B0 = ld<R>(S.p[4], i), B1 = ld<R>(S.p[5], i), B2 = ld<R>(S.p[6], i);
    acc[0] = acc[0] + (double)ld<R>(S.p[0], i);
    acc[1] = acc[1] + (0.5 * d * (v0 * v0 + v1 * v1 + v2 * v2) + c8 * (B0 * B0 + B1 * B1 + B2 * B2));
    acc[2] = acc[2] + (double)ld<R>(S.p[7], i);
    acc[3] = acc[3] + d * v0;
  }
  for (int q = 0; q < 4; ++q) sh[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int q = 0; q < 4; ++q) sh[q][threadIdx.x] = sh[q][threadIdx.x] + sh[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 4) partials[(size_t)blockIdx.x * 4 + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void __launch_bounds__(256) mhd_totals_stage2(int g, const double *partials, double *out) {
  __shared__ double sh[4][256];
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < g; i += 256)
    for (int q = 0; q < 4; ++q) acc[q] = acc[q] + partials[(size_t)i * 4 + q];
  for (int q = 0; q < 4; ++q) sh[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int q = 0; q < 4; ++q) sh[q][threadIdx.x] = sh[q][threadIdx.x] + sh[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 4) out[threadIdx.x] = sh[threadIdx.x][0];
}

template <typename R>
MhdC<R> make_consts(int n, double coef) {
  // 3d-mhd-rk4.fmr:4-11 evaluated in double as the generated code does
  const double NX = n;
  const double pi = 3.141592653589793;
  const double dt = 0.1 / fmax(NX, fmax(NX, NX));
  const double dx = 1.0 / NX;
  const double c_h = dx / dt;
  MhdC<R> k;
  k.dt_c = (R)coef;
  k.h12 = (R)(12.0 * dx);
  k.c_h2 = (R)(c_h * c_h);
  k.ch2_cp2 = (R)(c_h / 0.18);
  k.c8 = (R)(1.0 / (8.0 * pi));
  k.c4 = (R)(1.0 / (4.0 * pi));
  k.dp_ddens = (R)1.0;
  k.dp_ds = (R)(2.0 / 5.0);
  k.dens0 = (R)1.0;
  k.h12d = fm::make_div_const(12.0 * dx);
  k.h12f = (float)(12.0 * dx);
  k.rh12f = 1.0f / k.h12f;
  k.h12s = fm::soft::make_div_const_s(12.0 * dx);
  k.dts = fm::soft::make_mul_const_s((double)k.dt_c);
  k.c_h2s = fm::soft::make_mul_const_s((double)k.c_h2);
  k.ch2_cp2s = fm::soft::make_mul_const_s((double)k.ch2_cp2);
  k.c8s = fm::soft::make_mul_const_s((double)k.c8);
  k.c4s = fm::soft::make_mul_const_s((double)k.c4);
  k.dp_ddens_s = fm::soft::make_mul_const_s((double)k.dp_ddens);
  k.dp_ds_s = fm::soft::make_mul_const_s((double)k.dp_ds);
  k.c1_4s = fm::soft::make_mul_const_s(1.4);
  k.c0_75s = fm::soft::make_mul_const_s(0.75);
  k.c0_15s = fm::soft::make_mul_const_s(0.15);
  k.c8pi_s = fm::soft::make_mul_const_s(8.0 * 3.141592653589793);
  return k;
}

// `steps` steps with arithmetic form SF (Ar<R, SF>): stage and finishing kernels as
// selected by the mhd.stage / mhd.finish knobs.
template <typename R, int SF>
int mhd_run(int n, R *const *fields, R *work, int steps, cudaStream_t s) {
  const size_t cells = (size_t)n * n * n;
  Fields S, A, B;
  for (int f = 0; f < NF; ++f) {
    S.p[f] = fields[f];
    A.p[f] = work + (size_t)f * cells;
    B.p[f] = work + (size_t)(NF + f) * cells;
  }
  const double NX = n;
  const double dt = 0.1 / fmax(NX, fmax(NX, NX));
  const MhdC<R> k4 = make_consts<R>(n, dt / 4.0), k3 = make_consts<R>(n, dt / 3.0),
                k2 = make_consts<R>(n, dt / 2.0), k1 = make_consts<R>(n, dt);
  const dim3 grid((n + 31) / 32, (n + 3) / 4, n);
  // 2 x-marching with a register ring of x composites, 1 tiled, 0 per-point.  Whole
  // step at 256^3 (GLUP/s, 2 / 1 / 0): float 2.65 / 3.40 / 2.9; double with FP64
  // instructions 0.184 / 0.171 / 0.13; double with the integer-pipe arithmetic
  // (mhd.soft = 1) 0.316 / 0.301 — the march kernel bounded to 2 CTAs per SM (128
  // registers, spilling the ring) keeps the composites it saves and enough warps
  // (0.285 at 1 CTA per SM).
  const int stage_kernel = fm::tune_get("mhd.stage", sizeof(R) == 8 ? 2 : 1);
  const dim3 tgrid((n + kTZ - 1) / kTZ, (n + kTY - 1) / kTY, n);
  const size_t tsmem = (size_t)kNV * kNP * sizeof(R);
  if (stage_kernel == 1)
    FM_TRY_CUDA(cudaFuncSetAttribute(mhd_stage_tile<R, SF>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsmem));
  if (stage_kernel == 2)
    FM_TRY_CUDA(cudaFuncSetAttribute(mhd_stage_march<R, SF>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsmem));
  int msms = 0;
  {
    const int st0 = fm::device_sm_count(&msms);
    if (st0) return st0;
  }
  const int m_ntiles_yz = ((n + kTZ - 1) / kTZ) * ((n + kTY - 1) / kTY);
  int m_xchunk = fm::tune_get("mhd.stage_xchunk", 16);
  m_xchunk = std::max(1, std::min(m_xchunk, n));
  const int m_ntiles = m_ntiles_yz * ((n + m_xchunk - 1) / m_xchunk);
  const int m_grid = std::min(m_ntiles, 8 * msms);
  auto stage = [&](const Fields &in, Fields &out, const MhdC<R> &kk) {
    if (stage_kernel == 2)
      mhd_stage_march<R, SF><<<m_grid, 256, tsmem, s>>>(in, S, out, n, m_xchunk, m_ntiles_yz,
                                                        m_ntiles, kk);
    else if (stage_kernel == 1)
      mhd_stage_tile<R, SF><<<tgrid, 256, tsmem, s>>>(in, S, out, n, kk);
    else
      mhd_stage<R, SF><<<grid, 128, 0, s>>>(in, S, out, n, kk);
  };
  // 2 shared slopes and faces, all fields per plane; 0 per-point.  Measured at
  // 256^3 (GLUP/s of the whole step, 0/2): float 3.13/2.49, double 0.129/0.171
  // — the shared-memory form pays for its staging and barriers at 2 CTAs per
  // SM unless the arithmetic is FP64.  (A form marching one field at a time,
  // 2.75/0.155, was slower than both.)
  const int finish_kernel = fm::tune_get("mhd.finish", sizeof(R) == 8 ? 2 : 0);
  const size_t fsmem = sizeof(FinishSmem<R>);
  if (finish_kernel == 2)
    FM_TRY_CUDA(cudaFuncSetAttribute(mhd_finish_v2<R, SF>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsmem));
  int sms = 0;
  int st = fm::device_sm_count(&sms);
  if (st) return st;
  const int ntiles_yz = ((n + kTZ - 1) / kTZ) * ((n + kTY - 1) / kTY);
  int xchunk = fm::tune_get("mhd.xchunk", 0);
  if (xchunk <= 0) {  // >= 16 tiles per SM (load balance), chunks of at most 32 planes
    // (FP64 at 256^3: chunks of 16 planes 0.318 GLUP/s, 32: 0.315, 64: 0.312, 8: 0.313)
    xchunk = 32;
    while (xchunk > 4 && (long long)ntiles_yz * ((n + xchunk - 1) / xchunk) < 16ll * sms)
      xchunk /= 2;
  }
  xchunk = std::min(xchunk, n);
  const int ntiles = ntiles_yz * ((n + xchunk - 1) / xchunk);
  const int fgrid = std::min(ntiles, 8 * sms);
  for (int i = 0; i < steps; ++i) {
    stage(S, A, k4);
    stage(A, B, k3);
    stage(B, A, k2);
    stage(A, B, k1);
    if (finish_kernel == 2)
      mhd_finish_v2<R, SF><<<fgrid, 256, fsmem, s>>>(B, S, n, xchunk, ntiles_yz, ntiles, k1);
    else
      mhd_finish<R, SF><<<grid, 128, 0, s>>>(B, S, n, k1);
  }
  FM_TRY_CUDA(cudaGetLastError());
  return FM_OK;
}

template <typename R>
int mhd_totals(int n, R *const *fields, double *partials, double *out, cudaStream_t s) {
  Fields S;
  for (int f = 0; f < NF; ++f) S.p[f] = fields[f];
  const long long cells = (long long)n * n * n;
  const int g = (int)std::max<long long>(1, std::min<long long>((cells + 4095) / 4096, 1024));
  const long long chunk = (cells + g - 1) / g;
  mhd_totals_stage1<R><<<g, 256, 0, s>>>(S, cells, chunk, partials);
  mhd_totals_stage2<<<1, 256, 0, s>>>(g, partials, out);
  FM_TRY_CUDA(cudaGetLastError());
  return FM_OK;
}

}  // namespace
