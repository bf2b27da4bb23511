// fm_common.cuh — shared device helpers of the GB300 stencil engine.
//
// Every translation unit of the library is compiled with --fmad=false, so a
// written `a*b + c` stays two IEEE operations, as in the generated C built
// with -ffp-contract=off.  Kernels that want a fused multiply-add call
// fma()/fmaf() explicitly.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "../../include/formura_gb300.h"

namespace fm {

// Records a printf-style message for fm_last_error() on this host thread.
void set_error(const char *fmt, ...);
void clear_error();

// Returns FM_ERR_CUDA with a message when `e` is not cudaSuccess.
int cuda_status(cudaError_t e, const char *what);

#define FM_TRY_CUDA(expr)                                   \
  do {                                                      \
    cudaError_t fm_e_ = (expr);                             \
    if (fm_e_ != cudaSuccess) return fm::cuda_status(fm_e_, #expr); \
  } while (0)

#define FM_CHECK_ARG(cond, ...)              \
  do {                                       \
    if (!(cond)) {                           \
      fm::set_error(__VA_ARGS__);            \
      return FM_ERR_ARG;                     \
    }                                        \
  } while (0)

// Number of SMs and max cooperative grid helpers (cached per device).
int device_sm_count(int *sms);

// Bounded spin limit for the grid barriers of the persistent kernels: a wait
// that exceeds it records an error word and returns instead of hanging the
// GPU.  The default (~ seconds with __nanosleep) can be lowered per process
// with the tuning knob "sync.spin_limit" (polls, >= 1), which the failure
// tests use to make a wait run out; spin_limit() reads it on the host and the
// kernels receive the value as an argument.
constexpr long long kSpinLimitDefault = 20000000;
long long spin_limit();

__device__ __forceinline__ int wrap_dn(int i, int n) { return i == 0 ? n - 1 : i - 1; }
__device__ __forceinline__ int wrap_up(int i, int n) { return i + 1 == n ? 0 : i + 1; }

// IEEE division for the rare operands outside a fast path's range.  Kept out
// of line so that the compiler branches around it instead of if-converting
// it: a predicated-off division sequence would still occupy the FP64 pipe.
static __device__ __noinline__ double ddiv_slow(double x, double d) { return __ddiv_rn(x, d); }
static __device__ __noinline__ float fdiv_slow(float x, float d) { return __fdiv_rn(x, d); }

// Correctly rounded x/d for a constant d > 0, given r = RN(1/d).
//
// Markstein's correction (P. W. Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1),
// 1990): when q0 = RN(x*r) is within one ulp of x/d and r within half an ulp
// of 1/d, the residual e = x - q0*d is exact in one fma and RN(q0 + e*r) is
// the correctly rounded quotient.  The argument needs x*r and q0*d to stay in
// the normal range, so |x| outside [2^-958, 2^960) (and NaN/Inf) takes the
// IEEE division instead; zero is exact on the fast path up to the sign, which
// copysign restores.  Costs one DMUL and two DFMA on the fast path instead of
// the reciprocal-iteration sequence of a general division.
__device__ __forceinline__ double div_const(double x, double d, double r) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const unsigned ex = (unsigned)(bits >> 52) & 0x7ffu;
  const bool zero = (bits << 1) == 0ull;
  const bool normal = (ex - 65u) <= (1982u - 65u);
  double q;
  if (normal || zero) {
    const double q0 = x * r;
    const double e = fma(-q0, d, x);
    q = copysign(fma(e, r, q0), x);
  } else {
    q = __ddiv_rn(x, d);
  }
  return q;
}

// Constant divisor prepared for div_const_i: d, r = RN(1/d), d's integer
// significand (implicit bit set) and biased exponent.
struct DivConst {
  double d, r;
  unsigned long long md;
  int ed;
};

inline DivConst make_div_const(double d) {
  DivConst c;
  c.d = d;
  c.r = 1.0 / d;
  unsigned long long b;
  memcpy(&b, &d, sizeof b);
  c.md = (b & 0x000fffffffffffffull) | 0x0010000000000000ull;
  c.ed = (int)((b >> 52) & 0x7ff);
  return c;
}

// Correctly rounded x/d with one FP64 instruction: q0 = RN(x*r) is within
// one ulp of x/d (the premise of Markstein's correction above), so RN(x/d)
// is q0 or one of its neighbours.  Which one is decided exactly on the
// integer pipe: with x = mx*2^(EX-52), d = md*2^(ED-52), q0 = mq*2^(EQ-52),
// x/d lies above the midpoint q0 + ulp/2 iff mx*2^s > md*(2*mq+1) with
// s = EX-ED-EQ+53 (52..55), and below q0 - ulp/2 iff mx*2^s < md*(2*mq-1)
// (md*(4*mq-1) against mx*2^(s+1) when q0 is a power of two, whose lower
// neighbour is half an ulp away).  Both sides are < 2^108, compared as
// 128-bit integers.  A quotient of two binary64 numbers is never exactly a
// midpoint, so no tie case exists.  Same range rule as div_const.
__device__ __forceinline__ double div_const_i(double x, const DivConst &c) {
  // Word-level extraction (see div_const_r) keeps every step off the FP64 pipe.
  const unsigned xh = (unsigned)__double2hiint(x), xl = (unsigned)__double2loint(x);
  const unsigned ex = (xh >> 20) & 0x7ffu;
  const bool zero = ((xh << 1) | xl) == 0u;
  const bool normal = (ex - 65u) <= (1982u - 65u);
  const double q0 = x * c.r;
  const unsigned qh = (unsigned)__double2hiint(q0), ql = (unsigned)__double2loint(q0);
  const unsigned eq = (qh >> 20) & 0x7ffu;
  const unsigned long long mx =
      ((unsigned long long)((xh & 0x000fffffu) | 0x00100000u) << 32) | xl;
  const unsigned long long mq =
      ((unsigned long long)((qh & 0x000fffffu) | 0x00100000u) << 32) | ql;
  // s is 52..55 for every x on the fast path; the mask only keeps the shifts
  // defined for the zero/non-normal lanes whose result is replaced below.
  const int s = ((int)ex - c.ed - (int)eq + 1076) & 63;
  unsigned long long a_hi = (mx >> 1) >> (63 - s), a_lo = mx << s;
  const unsigned long long t = 2ull * mq + 1ull;
  const unsigned long long p_lo = c.md * t, p_hi = __umul64hi(c.md, t);
  const bool up = (a_hi > p_hi) || (a_hi == p_hi && a_lo > p_lo);
  unsigned long long l_hi, l_lo;
  const bool pow2 = mq == 0x0010000000000000ull;
  if (!pow2) {
    const unsigned long long two = 2ull * c.md;
    l_lo = p_lo - two;
    l_hi = p_hi - (p_lo < two ? 1ull : 0ull);
  } else {
    const unsigned long long t4 = 4ull * mq - 1ull;
    l_lo = c.md * t4;
    l_hi = __umul64hi(c.md, t4);
    a_hi = (a_hi << 1) | (a_lo >> 63);
    a_lo <<= 1;
  }
  const bool dn = (a_hi < l_hi) || (a_hi == l_hi && a_lo < l_lo);
  // q0's magnitude bits +-1, sign kept (q0 has x's sign since r > 0)
  unsigned rl = ql, rh = qh;
  if (up) {
    rl = ql + 1u;
    rh = qh + (rl == 0u ? 1u : 0u);
  }
  if (dn) {
    rl = ql - 1u;
    rh = qh - (ql == 0u ? 1u : 0u);
  }
  if (zero) {
    rl = xl;
    rh = xh;
  }
  double q = __hiloint2double((int)rh, (int)rl);
  if (__builtin_expect(!(normal || zero), 0)) q = ddiv_slow(x, c.d);
  return q;
}

// Correctly rounded x/d with two FP64 instructions: q0 = RN(x*r), then the
// exact residual e = x - q0*d (one fma — exact because q0 is within one ulp of
// x/d, Markstein's premise).  x/d - q0 = e/d, so RN(x/d) moves q0 one ulp
// away from zero iff e has q0's sign and |e| > d*ulp(q0)/2, and one ulp
// toward zero iff e has the other sign and |e| exceeds that bound (a quarter
// ulp when q0 is a power of two, whose lower neighbour is half an ulp away).
// d*ulp(q0)/2 = d*2^(EQ-53) is d's bit pattern with q0's exponent added, and
// positive doubles order like their bit patterns, so the test is two integer
// compares; no tie is possible (a binary64 quotient is never a midpoint).
// Fast path for x = 0 and 2^-900 <= |x| < 2^900 with 2^-20 <= d <= 2^20 (all
// quantities stay normal); IEEE division otherwise.
__device__ __forceinline__ double div_const_r(double x, double d, double r) {
  // Everything after the two FP64 operations works on 32-bit words of the
  // bit patterns (__double2hiint/__double2loint), so that no step can be
  // re-expressed by the compiler as another FP64 instruction (an abs, a
  // compare or a select of doubles would run on the FP64 pipe).
  const unsigned xh = (unsigned)__double2hiint(x), xl = (unsigned)__double2loint(x);
  const unsigned ex = (xh >> 20) & 0x7ffu;
  const bool zero = ((xh << 1) | xl) == 0u;
  const bool fast = (ex - 123u) < (1923u - 123u);
  const double q0 = x * r;
  const double e = fma(-q0, d, x);
  const unsigned qh = (unsigned)__double2hiint(q0), ql = (unsigned)__double2loint(q0);
  const unsigned eh = (unsigned)__double2hiint(e), el = (unsigned)__double2loint(e);
  const unsigned qah = qh & 0x7fffffffu, eah = eh & 0x7fffffffu;
  // T = d * 2^(EQ-53): d's high word plus q0's exponent field, low word = d's
  const unsigned th = (unsigned)__double2hiint(d) + (qah & 0x7ff00000u) - (1076u << 20);
  const unsigned tl = (unsigned)__double2loint(d);
  const bool same = ((qh ^ eh) >> 31) == 0u;
  const bool pow2 = ((qah & 0x000fffffu) | ql) == 0u;
  const unsigned tdh = pow2 ? th - (1u << 20) : th;
  const bool gt_t = (eah > th) || (eah == th && el > tl);
  const bool gt_td = (eah > tdh) || (eah == tdh && el > tl);
  const bool inc = same && gt_t;
  const bool dec = !same && gt_td;
  // q0's bit pattern +-1 (the neighbour away from / toward zero)
  unsigned rl = ql, rh = qh;
  if (inc) {
    rl = ql + 1u;
    rh = qh + (rl == 0u ? 1u : 0u);
  }
  if (dec) {
    rl = ql - 1u;
    rh = qh - (ql == 0u ? 1u : 0u);
  }
  if (zero) {
    rl = ql;
    rh = qh;
  }
  double q = __hiloint2double((int)rh, (int)rl);
  if (__builtin_expect(!(fast || zero), 0)) q = ddiv_slow(x, d);
  return q;
}

// binary32 counterpart: Markstein's step with r = RN(1/d) in float, for a
// positive d.  For |x| in [2^-94, 2^93] no intermediate leaves the normal
// range and the step gives x/d correctly rounded (with the sign of x); zero
// returns x; anything else (subnormal, huge, Inf, NaN) takes the IEEE
// division.  The range test is two float compares on |x|.
__device__ __forceinline__ float div_const_f(float x, float d, float r) {
  const float ax = fabsf(x);
  float q;
  if (ax >= 0x1p-94f && ax <= 0x1p93f) {
    const float q0 = x * r;
    const float e = fmaf(-q0, d, x);
    q = fmaf(e, r, q0);
  } else if (ax == 0.0f) {
    q = x;
  } else {
    q = __fdiv_rn(x, d);
  }
  return q;
}

// Packed binary32 pairs (sm_100 and later: one FADD2/FMUL2/FFMA2 instruction
// does the IEEE operation, round to nearest even, on both halves).  A kernel
// that applies the same operation sequence to two fields of a cell (U and V of
// Gray-Scott) evaluates both in one instruction stream with results identical
// to the scalar operations, at half the issue slots.
//
// Rule for exact kernels: never feed a pair product (f2mul) into a pair add
// or subtract.  Measured on sm_103a (65536 random operands, CUDA 13.0): the
// sequence mul.rn.f32x2 -> add.rn.f32x2 came out rounded once, equal to
// fma.rn.f32x2 in every case, whether written as PTX with the .rn modifier or
// through __fmul2_rn/__fadd2_rn, and with --fmad=false given to nvcc and to
// ptxas; the scalar sequence rounds twice.  Products whose rounding the
// program observes stay scalar (or the arithmetic is an explicit fma).  Each
// operation alone matches its scalar counterpart bit for bit, subnormals
// included.
#define FM_F2_OP2(name, op)                                                        \
  __device__ __forceinline__ float2 name(float2 a, float2 b) {                     \
    float2 r;                                                                      \
    asm("{\n\t.reg .b64 pa, pb, pd;\n\t"                                          \
        "mov.b64 pa, {%2, %3};\n\t"                                                \
        "mov.b64 pb, {%4, %5};\n\t" op " pd, pa, pb;\n\t"                          \
        "mov.b64 {%0, %1}, pd;\n\t}"                                               \
        : "=f"(r.x), "=f"(r.y)                                                     \
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));                                 \
    return r;                                                                      \
  }
FM_F2_OP2(f2add, "add.rn.f32x2")
FM_F2_OP2(f2sub, "sub.rn.f32x2")
FM_F2_OP2(f2mul, "mul.rn.f32x2")
#undef FM_F2_OP2
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) {
  float2 r;
  asm("{\n\t.reg .b64 pa, pb, pc, pd;\n\t"
      "mov.b64 pa, {%2, %3};\n\t"
      "mov.b64 pb, {%4, %5};\n\t"
      "mov.b64 pc, {%6, %7};\n\t"
      "fma.rn.f32x2 pd, pa, pb, pc;\n\t"
      "mov.b64 {%0, %1}, pd;\n\t}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return r;
}

}  // namespace fm
