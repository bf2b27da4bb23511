// Host build of formura_gb300/csrc/fm_softfp.cuh for the CPU bit-exactness
// checks in tests/test_softfp.py (compiled there with g++ into a temporary
// shared library).  Each function applies one soft operation element-wise.
#include "../../formura_gb300/csrc/fm_softfp.cuh"

extern "C" {

void softfp_div_const(const double *x, long n, double d, double *out) {
  const fm::soft::DivConstS c = fm::soft::make_div_const_s(d);
  for (long i = 0; i < n; ++i) out[i] = fm::soft::div_const_s(x[i], c);
}

void softfp_mul_const(const double *x, long n, double y, double *out) {
  const fm::soft::MulConstS c = fm::soft::make_mul_const_s(y);
  for (long i = 0; i < n; ++i) out[i] = fm::soft::mul_const_s(x[i], c);
}

void softfp_mul(const double *x, const double *y, long n, double *out) {
  for (long i = 0; i < n; ++i) out[i] = fm::soft::mul_s(x[i], y[i]);
}

void softfp_scale_pow2(const double *x, long n, int k, double *out) {
  for (long i = 0; i < n; ++i) out[i] = fm::soft::scale_pow2(x[i], k);
}

void softfp_div(const double *x, const double *y, long n, double *out) {
  for (long i = 0; i < n; ++i) out[i] = fm::soft::div_s(x[i], y[i]);
}

void softfp_recip115(const unsigned long long *md, long n, unsigned long long *out) {
  for (long i = 0; i < n; ++i) out[i] = fm::soft::recip115(md[i]);
}

void softfp_max(const double *x, const double *y, long n, double *out) {
  for (long i = 0; i < n; ++i) out[i] = fm::soft::max_s(x[i], y[i]);
}

void softfp_min(const double *x, const double *y, long n, double *out) {
  for (long i = 0; i < n; ++i) out[i] = fm::soft::min_s(x[i], y[i]);
}

void softfp_le_zero(const double *x, long n, unsigned char *out) {
  for (long i = 0; i < n; ++i) out[i] = fm::soft::le_zero_s(x[i]) ? 1 : 0;
}

void softfp_cmp(const double *x, const double *y, long n, unsigned char *out) {
  // bit 0: <, bit 1: <=, bit 2: ==
  for (long i = 0; i < n; ++i)
    out[i] = (fm::soft::lt_s(x[i], y[i]) ? 1 : 0) | (fm::soft::le_s(x[i], y[i]) ? 2 : 0) |
             (fm::soft::eq_s(x[i], y[i]) ? 4 : 0);
}

void softfp_div_reciprocal_words(double d, unsigned *r_hi, unsigned *r_lo) {
  const fm::soft::DivConstS c = fm::soft::make_div_const_s(d);
  *r_hi = c.r_hi;
  *r_lo = c.r_lo;
}

void softfp_f2d(const float *x, long n, double *out) {
  for (long i = 0; i < n; ++i) out[i] = fm::soft::f2d_s(x[i]);
}

void softfp_d2f(const double *x, long n, float *out) {
  for (long i = 0; i < n; ++i) out[i] = fm::soft::d2f_s(x[i]);
}
}
