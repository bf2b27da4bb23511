// fm_mhd_f64.cu — 3D MHD: the all-binary64 time step (bit-exact with the
// generated C).  The default form runs the exactly replaceable binary64
// operations on the integer pipes (Ar<double, 1>); the form with FP64
// instructions only (mhd.soft = 0) is instantiated in fm_mhd_f64_fp64ops.cu.
// The kernels are in fm_mhd_impl.cuh; three translation units so that the
// library builds in parallel.
#include "fm_mhd_impl.cuh"

namespace fm {
int mhd_run_f64_fp64ops(int n, double *const *fields, double *work, int steps, cudaStream_t s);
}

extern "C" int fm_mhd_forward_f64(int n, double *const fields[9], double *work, int steps,
                                  void *stream) {
  FM_CHECK_ARG(fields && work && n >= 5 && steps >= 0,
               "fm_mhd_forward_f64: need n >= 5, fields, work, steps >= 0");
  for (int f = 0; f < NF; ++f) FM_CHECK_ARG(fields[f], "fm_mhd_forward_f64: field %d is NULL", f);
  if (steps == 0) return FM_OK;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  // 1 (default): scalings, products with constants, divisions, fmax/fmin on the integer
  // pipes; 0: FP64 instructions only (products of two fields on the integer pipes as
  // well measured slower: 0.203 / 0.268 GLUP/s with the march / tile kernel)
  if (fm::tune_get("mhd.soft", 1) == 0) return fm::mhd_run_f64_fp64ops(n, fields, work, steps, s);
  return mhd_run<double, 1>(n, fields, work, steps, s);
}
