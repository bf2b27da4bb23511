// fm_tma.cu — tensor maps for the TMA-staged kernels that the .fmr front end
// generates (formura_gb300/fmr/emit_cuda.py, TBEmitter): cuTensorMapEncodeTiled
// reached through the runtime's driver entry point, so neither the library nor
// the generated programs link libcuda directly.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "fm_common.cuh"

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
  });
  return fn;
}

}  // namespace

extern "C" int fm_tensor_map_3d(void *map, const void *base, int elem_bytes, int n0, int n1,
                                int n2, int box0, int box1, int box2) {
  FM_CHECK_ARG(map && base, "fm_tensor_map_3d: NULL argument");
  FM_CHECK_ARG(elem_bytes == 4 || elem_bytes == 8, "fm_tensor_map_3d: elem_bytes must be 4 or 8");
  FM_CHECK_ARG(n0 >= 1 && n1 >= 1 && n2 >= 1, "fm_tensor_map_3d: empty array");
  FM_CHECK_ARG(box0 >= 1 && box0 <= 256 && box1 >= 1 && box1 <= 256 && box2 >= 1 && box2 <= 256,
               "fm_tensor_map_3d: box edges must be 1..256");
  FM_CHECK_ARG(((uintptr_t)base & 15u) == 0, "fm_tensor_map_3d: base not 16-byte aligned");
  FM_CHECK_ARG(((uintptr_t)map & 63u) == 0, "fm_tensor_map_3d: map not 64-byte aligned");
  FM_CHECK_ARG(((long long)n2 * elem_bytes) % 16 == 0 && ((long long)box2 * elem_bytes) % 16 == 0,
               "fm_tensor_map_3d: rows and box rows must be multiples of 16 bytes");
  auto enc = encoder();
  if (!enc) {
    fm::set_error("fm_tensor_map_3d: cuTensorMapEncodeTiled is not available");
    return FM_ERR_UNSUPPORTED;
  }
  // dimension 0 of the map is the array's fastest axis (n2)
  cuuint64_t dims[3] = {(cuuint64_t)n2, (cuuint64_t)n1, (cuuint64_t)n0};
  cuuint64_t strides[2] = {(cuuint64_t)n2 * elem_bytes, (cuuint64_t)n2 * n1 * elem_bytes};
  cuuint32_t box[3] = {(cuuint32_t)box2, (cuuint32_t)box1, (cuuint32_t)box0};
  cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = enc(reinterpret_cast<CUtensorMap *>(map),
                         elem_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                         : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                         3, const_cast<void *>(base), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    fm::set_error("fm_tensor_map_3d: cuTensorMapEncodeTiled failed (%d)", (int)r);
    return FM_ERR_ARG;
  }
  return FM_OK;
}
