// fm_common.cuh — shared device helpers of the GB300 stencil engine.
//
// Every translation unit of the library is compiled with --fmad=false, so a
// written `a*b + c` stays two IEEE operations, as in the generated C built
// with -ffp-contract=off.  Kernels that want a fused multiply-add call
// fma()/fmaf() explicitly.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

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

// Bounded spin limit for device-side waits: a wait that exceeds it records an
// error word and returns instead of hanging the GPU.
constexpr long long kSpinLimit = 20000000;  // ~ seconds with __nanosleep

__device__ __forceinline__ int wrap_dn(int i, int n) { return i == 0 ? n - 1 : i - 1; }
__device__ __forceinline__ int wrap_up(int i, int n) { return i + 1 == n ? 0 : i + 1; }

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

// binary32 counterpart: Markstein's step with r = RN(1/d) in float.
__device__ __forceinline__ float div_const_f(float x, float d, float r) {
  const unsigned bits = (unsigned)__float_as_int(x);
  const unsigned ex = (bits >> 23) & 0xffu;
  const bool zero = (bits << 1) == 0u;
  const bool normal = (ex - 33u) <= (220u - 33u);
  float q;
  if (normal || zero) {
    const float q0 = x * r;
    const float e = fmaf(-q0, d, x);
    q = copysignf(fmaf(e, r, q0), x);
  } else {
    q = __fdiv_rn(x, d);
  }
  return q;
}

}  // namespace fm
