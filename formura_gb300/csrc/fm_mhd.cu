// fm_mhd.cu — 3D MHD: the binary32-bulk time step (FP64 energy update) and the
// FP64 conserved totals; the kernels are in fm_mhd_impl.cuh, the all-binary64
// step in fm_mhd_f64.cu.
#include "fm_mhd_impl.cuh"

extern "C" int fm_mhd_forward_f32(int n, float *const fields[9], float *work, int steps,
                                  void *stream) {
  FM_CHECK_ARG(fields && work && n >= 5 && steps >= 0,
               "fm_mhd_forward_f32: need n >= 5, fields, work, steps >= 0");
  for (int f = 0; f < NF; ++f) FM_CHECK_ARG(fields[f], "fm_mhd_forward_f32: field %d is NULL", f);
  if (steps == 0) return FM_OK;
  return mhd_run<float, 0>(n, fields, work, steps, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" size_t fm_mhd_totals_scratch_elems(int n) {
  const long long cells = (long long)n * n * n;
  return 4 * (size_t)std::max<long long>(1, std::min<long long>((cells + 4095) / 4096, 1024));
}

extern "C" int fm_mhd_totals(int n, int fp64, void *const fields[9], double *partials,
                             double *out_device, void *stream) {
  FM_CHECK_ARG(fields && partials && out_device && n >= 1, "fm_mhd_totals: bad arguments");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (fp64) return mhd_totals<double>(n, reinterpret_cast<double *const *>(fields), partials, out_device, s);
  return mhd_totals<float>(n, reinterpret_cast<float *const *>(fields), partials, out_device, s);
}
