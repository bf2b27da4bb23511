// fm_mhd_f64_fp64ops.cu — 3D MHD, all binary64, with FP64 instructions only
// (mhd.soft = 0): the reference form against which the integer-pipe form of
// fm_mhd_f64.cu is checked bit for bit.  The kernels are in fm_mhd_impl.cuh.
#include "fm_mhd_impl.cuh"

namespace fm {
int mhd_run_f64_fp64ops(int n, double *const *fields, double *work, int steps, cudaStream_t s) {
  return mhd_run<double, 0>(n, fields, work, steps, s);
}
}  // namespace fm
