// fm_softfp.cuh — correctly rounded binary64 division (by a constant, or by a
// run-time divisor), multiplication and scaling by powers of two computed on
// the INTEGER pipes, with no FP64 instruction on the fast path.
//
// Why: a GB300 SM retires 2 FP64 lanes per clock against 64 integer-ALU and
// 64 IMAD lanes, and the FP64 stencils of this library are FP64-pipe-bound
// with most integer issue slots idle.  Moving whole IEEE operations to the
// integer pipes trades ~30-40 cheap instructions for one scarce one.
//
// Both operations follow the textbook construction of an IEEE operation from
// an integer significand product (e.g. J.-M. Muller et al., "Handbook of
// Floating-Point Arithmetic", 2nd ed., ch. 7-8):
//   1. an approximate significand Q (53 bits + a few guard bits) from three
//      32x32-bit partial products — its error is far below half an ulp;
//   2. the rounding decided EXACTLY by the sign of (true value - midpoint
//      Q + 1/2), evaluated as the low 64 bits of an integer expression whose
//      true magnitude is known to be < 2^63;
//   3. the exponent and sign packed by integer addition, which also carries a
//      significand that rounded up to 2^53 into the next binade (and to
//      infinity from the largest binade, the correct round-to-nearest result).
// Operands or results outside the normal range (zero excepted, handled
// inline) take the IEEE hardware operation in an out-of-line slow path.
//
// The header compiles as plain C++ too (host build of the same code), so
// the bit-exactness checks run on the CPU against the host's IEEE arithmetic.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define FM_SOFT_HD __host__ __device__ __forceinline__
#else
#define FM_SOFT_HD inline
#endif

namespace fm {
namespace soft {

FM_SOFT_HD uint32_t hi_word(double x) {
#if defined(__CUDA_ARCH__)
  return (uint32_t)__double2hiint(x);
#else
  uint64_t b;
  memcpy(&b, &x, 8);
  return (uint32_t)(b >> 32);
#endif
}
FM_SOFT_HD uint32_t lo_word(double x) {
#if defined(__CUDA_ARCH__)
  return (uint32_t)__double2loint(x);
#else
  uint64_t b;
  memcpy(&b, &x, 8);
  return (uint32_t)b;
#endif
}
FM_SOFT_HD double from_words(uint32_t h, uint32_t l) {
#if defined(__CUDA_ARCH__)
  return __hiloint2double((int)h, (int)l);
#else
  const uint64_t b = ((uint64_t)h << 32) | l;
  double x;
  memcpy(&x, &b, 8);
  return x;
#endif
}
FM_SOFT_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

#if defined(__CUDA_ARCH__)
static __device__ __noinline__ double div_slow(double x, double d) { return __ddiv_rn(x, d); }
static __device__ __noinline__ double mul_slow(double x, double y) { return __dmul_rn(x, y); }
#elif defined(FM_SOFT_SLOW_SENTINEL)
// Host checks of the fast path alone: the slow path returns a marked NaN.
inline double sentinel() {
  double s;
  const uint64_t b = 0x7ff8dead0000beefull;
  memcpy(&s, &b, 8);
  return s;
}
inline double div_slow(double, double) { return sentinel(); }
inline double mul_slow(double, double) { return sentinel(); }
#else
inline double div_slow(double x, double d) { return x / d; }
inline double mul_slow(double x, double y) { return x * y; }
#endif

// ---------------------------------------------------------------------------
// Division by a constant d (positive, normal).
//
// With x = mx*2^(ex-1075), d = md*2^(ed-1075) (53-bit significands mx, md):
// R = ceil(2^115/md) is prepared once; P = (mx*2^11)*R / 2^64, taken from
// three partial products, satisfies (mx/md)*2^62 - 3 < P < (mx/md)*2^62 + 1.
// A = P >> 62 is 1 iff mx >= md (the one exception, mx == md giving A = 0, is
// repaired by the exact step: Q rounds up to 2^53 and the pack carries it).
// Q = P >> (10 - ... ) : Q = P >> 10 if A else P >> 9 is the truncated
// quotient significand; the true one, Qx = mx*2^(52+1-A)/md, lies in
// (Q - 2^-9, Q + 1 + 2^-7).  RN(Qx) = Q + 1 iff Qx > Q + 1/2, i.e. iff
// mx*2^(54-A) - md*(2Q+1) > 0; that difference is below 2^56 in magnitude,
// so its low 64 bits, read as signed, give its sign.  No tie exists: a
// quotient of two binary64 numbers is never a midpoint.
struct DivConstS {
  uint32_t r_hi, r_lo;    // R = ceil(2^115 / md)
  uint32_t md_hi, md_lo;  // md
  int ed;                 // biased exponent of d
  double d;
};

// Host-side preparation; d must be positive and normal.
inline DivConstS make_div_const_s(double d) {
  DivConstS c;
  uint64_t b;
  memcpy(&b, &d, 8);
  const uint64_t md = (b & 0x000fffffffffffffull) | 0x0010000000000000ull;
  // ceil(2^115 / md) by long division on 64-bit words: 2^115 = 2^63 * 2^52
  const uint64_t num_hi = 1ull << 51;  // 2^115 = num_hi * 2^64
  uint64_t q = 0, rem = 0;
  // schoolbook binary long division of num_hi:0 by md (116 bits, md < 2^53)
  for (int i = 127; i >= 0; --i) {
    const uint64_t bit = i >= 64 ? (num_hi >> (i - 64)) & 1ull : 0ull;
    rem = (rem << 1) | bit;  // rem < 2*md < 2^54: no overflow
    q <<= 1;
    if (rem >= md) {
      rem -= md;
      q |= 1ull;
    }
  }
  if (rem) ++q;
  c.r_hi = (uint32_t)(q >> 32);
  c.r_lo = (uint32_t)q;
  c.md_hi = (uint32_t)(md >> 32);
  c.md_lo = (uint32_t)md;
  c.ed = (int)((b >> 52) & 0x7ff);
  c.d = d;
  return c;
}

// The quotient step for a prepared divisor c; the result's sign is x's XOR
// dsign, and dnormal says whether the divisor is a normal number (a zero,
// subnormal, infinite or NaN divisor takes the slow path with c.d).
FM_SOFT_HD double div_core(double x, const DivConstS &c, uint32_t dsign, bool dnormal) {
  const uint32_t xh = hi_word(x), xl = lo_word(x);
  const uint32_t ex = (xh >> 20) & 0x7ffu;
  const uint32_t mxh = (xh & 0x000fffffu) | 0x00100000u;
  // a = mx << 11
  const uint32_t a_hi = (mxh << 11) | (xl >> 21);
  const uint32_t a_lo = xl << 11;
  // P = a_hi*r_hi + hi(a_hi*r_lo) + hi(a_lo*r_hi)
  uint64_t P = (uint64_t)a_hi * c.r_hi;
  P += mulhi32(a_hi, c.r_lo);
  P += mulhi32(a_lo, c.r_hi);
  const uint32_t A = (uint32_t)(P >> 62);
  const uint64_t Q = P >> (9 + A);
  // low 64 bits of md*(2Q+1)
  const uint64_t M = 2ull * Q + 1ull;
  const uint64_t md = ((uint64_t)c.md_hi << 32) | c.md_lo;
  const uint64_t prod = md * M;
  // low 64 bits of mx << (54 - A): only xl survives, in the high word
  const uint64_t sx = (uint64_t)(xl << (22 - A)) << 32;
  const int64_t diff = (int64_t)(sx - prod);
  const uint64_t Qr = Q + (diff > 0 ? 1ull : 0ull);
  const int E = (int)ex - c.ed + 1022 + (int)A;
  // pack: (E-1) << 52 plus Q (implicit bit included), the quotient's sign
  const uint32_t sign = (xh ^ dsign) & 0x80000000u;
  const uint32_t rh = (((uint32_t)(E - 1) << 20) + (uint32_t)(Qr >> 32)) | sign;
  double q = from_words(rh, (uint32_t)Qr);
  const bool zero = ((xh << 1) | xl) == 0u;
  const bool ok = (ex - 1u) < 2046u && (uint32_t)(E - 1) < 2046u;
  if (zero) q = from_words(sign, 0u);
  if (!((ok || zero) && dnormal)) q = div_slow(x, c.d);
  return q;
}

FM_SOFT_HD double div_const_s(double x, const DivConstS &c) { return div_core(x, c, 0u, true); }

// ---------------------------------------------------------------------------
// Division by a divisor known only at run time: the same quotient step after
// computing R = ceil(2^115/md) on the integer pipes —
//   R0: 24 bits from a binary32 reciprocal of md's top 24 bits (relative
//       error < 2^-22.4: 2^-24 from the rounding, < 2^-23 from the truncation);
//   R1, R2: two Newton-Raphson steps R + R*(2^115 - md*R)/2^115 in fixed
//       point (errors 2^-44.7 relative, then below one unit plus the floors:
//       ceil(2^115/md) - R2 is 0 or 1);
//   exact correction: D = 2^115 - md*R2 (its magnitude < 2^55, so the low 64
//       bits of md*R2 give it) decides R2 + 1.
// Two upward and one downward correction steps are applied for margin.
FM_SOFT_HD void umul128(uint64_t a, uint64_t b, uint64_t &hi, uint64_t &lo) {
#if defined(__CUDA_ARCH__)
  lo = a * b;
  hi = __umul64hi(a, b);
#else
  const unsigned __int128 p = (unsigned __int128)a * b;
  lo = (uint64_t)p;
  hi = (uint64_t)(p >> 64);
#endif
}

// floor(a * b / 2^64) for a signed a and an unsigned b (the result fits)
FM_SOFT_HD int64_t smulhi(int64_t a, uint64_t b) {
  uint64_t hi, lo;
  umul128((uint64_t)a, b, hi, lo);
  return (int64_t)(hi - (a < 0 ? b : 0ull));
}

// (2^115 - (p_hi:p_lo)) >> k as a signed 64-bit value, for 2^115 - p of
// magnitude below 2^(63+k)
FM_SOFT_HD int64_t resid115(uint64_t p_hi, uint64_t p_lo, int k) {
  const uint64_t e_lo = 0ull - p_lo;
  const uint64_t e_hi = (1ull << 51) - p_hi - (p_lo != 0ull ? 1ull : 0ull);
  return (int64_t)((e_hi << (64 - k)) | (e_lo >> k));
}

FM_SOFT_HD uint64_t recip115(uint64_t md) {
  const uint32_t top = (uint32_t)(md >> 29);  // [2^23, 2^24)
  float f;
  {
    const uint32_t fb = 0x3f800000u | (top & 0x7fffffu);  // top * 2^-23, exactly
    memcpy(&f, &fb, 4);
  }
#if defined(__CUDA_ARCH__)
  const float rf = __frcp_rn(f);
#else
  const float rf = 1.0f / f;
#endif
  uint32_t rb;
  memcpy(&rb, &rf, 4);
  const uint32_t mr = (rb & 0x7fffffu) | 0x800000u;
  const int s = 40 + (int)(rb >> 23) - 127;  // rf in (0.5, 1]: 39, or 40 for rf == 1
  const uint64_t R0 = (uint64_t)mr << s;
  uint64_t h, l;
  umul128(md, mr, h, l);
  const int64_t e0 = resid115((h << s) | (l >> (64 - s)), l << s, 51);
  const uint64_t R1 = R0 + (uint64_t)smulhi(e0, R0);
  umul128(md, R1, h, l);
  const int64_t e1 = resid115(h, l, 20);
  uint64_t R = R1 + (uint64_t)(smulhi(e1, R1) >> 31);
  int64_t D = (int64_t)(0ull - md * R);
  if (D > 0) {
    ++R;
    D -= (int64_t)md;
  }
  if (D > 0) {
    ++R;
    D -= (int64_t)md;
  }
  if (D <= -(int64_t)md) --R;
  return R;
}

// A divisor prepared at run time (any value; non-normal ones take the slow
// path in div_var_s).  Several divisions by one value share the reciprocal.
struct DivVarS {
  DivConstS c;
  uint32_t sign;
  bool normal;
};

FM_SOFT_HD DivVarS prep_div_s(double d) {
  DivVarS v;
  const uint32_t dh = hi_word(d), dl = lo_word(d);
  const uint64_t md = ((uint64_t)((dh & 0x000fffffu) | 0x00100000u) << 32) | dl;
  const uint64_t R = recip115(md);
  v.c.r_hi = (uint32_t)(R >> 32);
  v.c.r_lo = (uint32_t)R;
  v.c.md_hi = (uint32_t)(md >> 32);
  v.c.md_lo = (uint32_t)md;
  v.c.ed = (int)((dh >> 20) & 0x7ffu);
  v.c.d = d;
  v.sign = dh & 0x80000000u;
  v.normal = ((uint32_t)v.c.ed - 1u) < 2046u;
  return v;
}

FM_SOFT_HD double div_var_s(double x, const DivVarS &v) {
  return div_core(x, v.c, v.sign, v.normal);
}

FM_SOFT_HD double div_s(double x, double y) { return div_var_s(x, prep_div_s(y)); }

// ---------------------------------------------------------------------------
// Multiplication.  With x = mx*2^(ex-1075), y = my*2^(ey-1075): the exact
// product mx*my lies in [2^104, 2^106).  P = (mx*2^11)*(my*2^11) / 2^64 from
// three partial products satisfies mx*my/2^42 - 3 < P <= mx*my/2^42;
// A = P >> 63 picks the binade (a product just below 2^105 read as A = 0 when
// it is just above rounds to 2^105 either way, through the carry), and
// Q = P >> (10 + A) is the truncated significand at scale 2^(52+A).  The
// rounding: with t = mx*my - (2Q+1)*2^(51+A) (true magnitude < 2^56, so its
// low 64 bits decide), RN goes up iff t > 0, or t == 0 (a tie) and Q is odd.
// E = ex + ey - 1023 + A.
struct MulConstS {  // a constant factor y, nonzero normal
  uint32_t b_hi, b_lo;    // my << 11
  uint32_t my_hi, my_lo;  // my
  uint32_t sign;          // y's sign bit (bit 31)
  int ey;
  double y;
};

inline MulConstS make_mul_const_s(double y) {
  MulConstS c;
  uint64_t b;
  memcpy(&b, &y, 8);
  const uint64_t my = (b & 0x000fffffffffffffull) | 0x0010000000000000ull;
  const uint64_t bb = my << 11;
  c.b_hi = (uint32_t)(bb >> 32);
  c.b_lo = (uint32_t)bb;
  c.my_hi = (uint32_t)(my >> 32);
  c.my_lo = (uint32_t)my;
  c.sign = (uint32_t)(b >> 32) & 0x80000000u;
  c.ey = (int)((b >> 52) & 0x7ff);
  c.y = y;
  return c;
}

// The shared core: significands (hi words with the implicit bit) and biased
// exponents of two normal operands -> packed product words.
FM_SOFT_HD void mul_core(uint32_t mxh, uint32_t xl, uint32_t b_hi, uint32_t b_lo,
                         uint32_t myh, uint32_t yl, int exy, uint32_t sign, uint32_t &rh,
                         uint32_t &rl, int &E) {
  const uint32_t a_hi = (mxh << 11) | (xl >> 21);
  const uint32_t a_lo = xl << 11;
  uint64_t P = (uint64_t)a_hi * b_hi;
  P += mulhi32(a_hi, b_lo);
  P += mulhi32(a_lo, b_hi);
  const uint32_t A = (uint32_t)(P >> 63);
  const uint64_t Q = P >> (10 + A);
  // low 64 bits of mx*my
  const uint64_t lo = (uint64_t)xl * yl;
  const uint32_t lo_hi = (uint32_t)(lo >> 32) + xl * myh + mxh * yl;
  // low 64 bits of (2Q+1) << (51+A): only the high word is nonzero
  const uint32_t mid_hi = (2u * (uint32_t)Q + 1u) << (19 + A);
  const uint32_t t_hi = lo_hi - mid_hi;
  const uint32_t t_lo = (uint32_t)lo;
  const bool pos = (int32_t)t_hi > 0 || (t_hi == 0u && t_lo != 0u);
  const bool tie = t_hi == 0u && t_lo == 0u;
  const uint64_t Qr = Q + ((pos || (tie && (Q & 1ull))) ? 1ull : 0ull);
  E = exy - 1023 + (int)A;
  rh = (((uint32_t)(E - 1) << 20) + (uint32_t)(Qr >> 32)) | sign;
  rl = (uint32_t)Qr;
}

FM_SOFT_HD double mul_const_s(double x, const MulConstS &c) {
  const uint32_t xh = hi_word(x), xl = lo_word(x);
  const uint32_t ex = (xh >> 20) & 0x7ffu;
  const uint32_t mxh = (xh & 0x000fffffu) | 0x00100000u;
  uint32_t rh, rl;
  int E;
  mul_core(mxh, xl, c.b_hi, c.b_lo, c.my_hi, c.my_lo, (int)ex + c.ey,
           (xh & 0x80000000u) ^ c.sign, rh, rl, E);
  double r = from_words(rh, rl);
  const bool zero = ((xh << 1) | xl) == 0u;
  const bool ok = (ex - 1u) < 2046u && (uint32_t)(E - 1) < 2046u;
  if (zero) r = from_words((xh ^ c.sign) & 0x80000000u, 0u);
  if (!(ok || zero)) r = mul_slow(x, c.y);
  return r;
}

FM_SOFT_HD double mul_s(double x, double y) {
  const uint32_t xh = hi_word(x), xl = lo_word(x);
  const uint32_t yh = hi_word(y), yl = lo_word(y);
  const uint32_t ex = (xh >> 20) & 0x7ffu, ey = (yh >> 20) & 0x7ffu;
  const uint32_t mxh = (xh & 0x000fffffu) | 0x00100000u;
  const uint32_t myh = (yh & 0x000fffffu) | 0x00100000u;
  const uint32_t b_hi = (myh << 11) | (yl >> 21);
  const uint32_t b_lo = yl << 11;
  uint32_t rh, rl;
  int E;
  const uint32_t sign = (xh ^ yh) & 0x80000000u;
  mul_core(mxh, xl, b_hi, b_lo, myh, yl, (int)(ex + ey), sign, rh, rl, E);
  double r = from_words(rh, rl);
  const bool zero = ((xh << 1) | xl) == 0u || ((yh << 1) | yl) == 0u;
  const bool ok = (ex - 1u) < 2046u && (ey - 1u) < 2046u && (uint32_t)(E - 1) < 2046u;
  // a zero times a finite number: signed zero (Inf/NaN operands go the slow way)
  const bool zfin = zero && ex != 2047u && ey != 2047u;
  if (zfin) r = from_words(sign, 0u);
  if (!(ok || zfin)) r = mul_slow(x, y);
  return r;
}

// ---------------------------------------------------------------------------
// x * 2^k, exactly, for a small |k|: a normal x whose scaled exponent stays in
// [1, 2046] only has its exponent field moved; zero is unchanged; results that
// would be subnormal or overflow, subnormal x, Inf and NaN take the FP64
// multiplication out of line.
#if defined(__CUDA_ARCH__)
static __device__ __noinline__ double scale_slow(double x, double f) { return __dmul_rn(x, f); }
#elif defined(FM_SOFT_SLOW_SENTINEL)
inline double scale_slow(double, double) { return sentinel(); }
#else
inline double scale_slow(double x, double f) { return x * f; }
#endif

FM_SOFT_HD double scale_pow2(double x, int k) {
  const uint32_t xh = hi_word(x), xl = lo_word(x);
  const int e = (int)((xh >> 20) & 0x7ffu);
  double r = from_words(xh + ((uint32_t)k << 20), xl);
  const bool zero = ((xh << 1) | xl) == 0u;
  if (zero) r = x;
  else if (e == 0 || e == 0x7ff || e + k < 1 || e + k > 2046)
    r = scale_slow(x, k >= 0 ? (double)(1ull << k) : 1.0 / (double)(1ull << -k));
  return r;
}

// ---------------------------------------------------------------------------
// fmax, fmin and x <= 0 on the integer pipes.  For operands that are not NaN,
// and not a +0/-0 pair (whose result the hardware instruction decides), the
// order of binary64 values is the order of their bit patterns read as signed
// 64-bit integers after the magnitude bits of negative values are inverted
// (-0 below +0).  NaN operands and +0/-0 pairs take fmax/fmin out of line.
#if defined(__CUDA_ARCH__)
static __device__ __noinline__ double max_slow(double a, double b) { return fmax(a, b); }
static __device__ __noinline__ double min_slow(double a, double b) { return fmin(a, b); }
#elif defined(FM_SOFT_SLOW_SENTINEL)
inline double max_slow(double, double) { return sentinel(); }
inline double min_slow(double, double) { return sentinel(); }
#else
inline double max_slow(double a, double b) { return fmax(a, b); }
inline double min_slow(double a, double b) { return fmin(a, b); }
#endif

FM_SOFT_HD uint64_t bits64(double x) { return ((uint64_t)hi_word(x) << 32) | lo_word(x); }
FM_SOFT_HD int64_t order_key(uint64_t b) {
  return (int64_t)(b ^ ((uint64_t)((int64_t)b >> 63) >> 1));
}
FM_SOFT_HD bool minmax_special(uint64_t a, uint64_t b) {
  const bool nan = (a << 1) > 0xffe0000000000000ull || (b << 1) > 0xffe0000000000000ull;
  const bool mixed_zeros = ((a | b) << 1) == 0ull && a != b;
  return nan || mixed_zeros;
}

FM_SOFT_HD double max_s(double x, double y) {
  const uint64_t a = bits64(x), b = bits64(y);
  double r = order_key(a) >= order_key(b) ? x : y;
  if (minmax_special(a, b)) r = max_slow(x, y);
  return r;
}

FM_SOFT_HD double min_s(double x, double y) {
  const uint64_t a = bits64(x), b = bits64(y);
  double r = order_key(a) <= order_key(b) ? x : y;
  if (minmax_special(a, b)) r = min_slow(x, y);
  return r;
}

// IEEE comparisons on the same keys: unordered (a NaN operand) is false for
// <, <=, == and true for !=; +0 and -0 compare equal.  No slow path.
FM_SOFT_HD bool unordered_s(uint64_t a, uint64_t b) {
  return (a << 1) > 0xffe0000000000000ull || (b << 1) > 0xffe0000000000000ull;
}
FM_SOFT_HD bool lt_s(double x, double y) {
  const uint64_t a = bits64(x), b = bits64(y);
  return !unordered_s(a, b) && ((a | b) << 1) != 0ull && order_key(a) < order_key(b);
}
FM_SOFT_HD bool le_s(double x, double y) {
  const uint64_t a = bits64(x), b = bits64(y);
  return !unordered_s(a, b) && (((a | b) << 1) == 0ull || order_key(a) <= order_key(b));
}
FM_SOFT_HD bool eq_s(double x, double y) {
  const uint64_t a = bits64(x), b = bits64(y);
  return !unordered_s(a, b) && (a == b || ((a | b) << 1) == 0ull);
}

// x <= 0 (false for NaN)
FM_SOFT_HD bool le_zero_s(double x) {
  const uint64_t a = bits64(x);
  return (a << 1) <= 0xffe0000000000000ull && ((a >> 63) != 0ull || (a << 1) == 0ull);
}

// ---- binary32 <-> binary64 conversions on the integer pipes ------------------
//
// A binary32 program divided or multiplied by a binary64 constant (C promotes
// the float operand, as Formura's generated code does for its double literals)
// runs as (float)op((double)x, c).  The widening is exact; the narrowing rounds
// to nearest even.  Both are assembled from the IEEE fields: normal inputs (and
// zeros) inline, everything else — subnormal, infinite, NaN, and narrowing
// results outside the binary32 normal range — by the hardware conversion out
// of line.
#if defined(__CUDA_ARCH__)
static __device__ __noinline__ double f2d_slow(float x) { return (double)x; }
static __device__ __noinline__ float d2f_slow(double x) { return __double2float_rn(x); }
#elif defined(FM_SOFT_SLOW_SENTINEL)
inline double f2d_slow(float) { return sentinel(); }
inline float d2f_slow(double) { return (float)sentinel(); }
#else
inline double f2d_slow(float x) { return (double)x; }
inline float d2f_slow(double x) { return (float)x; }
#endif

FM_SOFT_HD uint32_t f32_bits(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t b;
  memcpy(&b, &x, 4);
  return b;
#endif
}
FM_SOFT_HD float f32_from_bits(uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  float x;
  memcpy(&x, &b, 4);
  return x;
#endif
}

// (double)x, exactly: biased exponent + (1023 - 127), significand moved up 29 bits.
FM_SOFT_HD double f2d_s(float x) {
  const uint32_t b = f32_bits(x);
  const uint32_t e = (b >> 23) & 0xffu;
  if ((b << 1) == 0u) return from_words(b & 0x80000000u, 0u);  // +-0
  if (e - 1u >= 254u) return f2d_slow(x);
  return from_words((b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7fffffu) >> 3), b << 29);
}

// (float)x rounded to nearest even: the top 23 significand bits, rounded on the
// 29 dropped bits; the integer addition of the round-up carries a significand
// that overflows into the exponent (and from the largest binade to infinity,
// the correctly rounded result).
FM_SOFT_HD float d2f_s(double x) {
  const uint32_t h = hi_word(x), l = lo_word(x);
  const uint32_t e = (h >> 20) & 0x7ffu;
  if (((h << 1) | l) == 0u) return f32_from_bits(h & 0x80000000u);  // +-0
  if (e - 897u > 253u) return d2f_slow(x);  // binary32 subnormal or beyond its range
  uint32_t f = (h & 0x80000000u) | ((e - 896u) << 23) | ((h & 0xfffffu) << 3) | (l >> 29);
  const uint32_t rest = l & 0x1fffffffu;
  if (rest > 0x10000000u || (rest == 0x10000000u && (f & 1u))) f += 1u;
  return f32_from_bits(f);
}

}  // namespace soft
}  // namespace fm
