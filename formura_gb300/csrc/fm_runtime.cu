// fm_runtime.cu — error reporting and the memory/stream helpers that the
// emitted per-program host code calls (it includes no CUDA header itself).
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "fm_common.cuh"

namespace fm {

static thread_local char g_err[512] = {0};

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

void clear_error() { g_err[0] = 0; }

int cuda_status(cudaError_t e, const char *what) {
  set_error("%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
  return (e == cudaErrorMemoryAllocation) ? FM_ERR_NOMEM : FM_ERR_CUDA;
}

int device_sm_count(int *sms) {
  static std::mutex mu;
  static int cached[64] = {0};
  int dev = 0;
  FM_TRY_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  if (dev < 64 && cached[dev] > 0) {
    *sms = cached[dev];
    return FM_OK;
  }
  int n = 0;
  FM_TRY_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
  if (dev < 64) cached[dev] = n;
  *sms = n;
  return FM_OK;
}

}  // namespace fm

static cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

extern "C" {

const char *fm_last_error(void) { return fm::g_err; }

const char *fm_status_name(int status) {
  switch (status) {
    case FM_OK: return "FM_OK";
    case FM_ERR_ARG: return "FM_ERR_ARG";
    case FM_ERR_CUDA: return "FM_ERR_CUDA";
    case FM_ERR_TIMEOUT: return "FM_ERR_TIMEOUT";
    case FM_ERR_NONFINITE: return "FM_ERR_NONFINITE";
    case FM_ERR_UNSUPPORTED: return "FM_ERR_UNSUPPORTED";
    case FM_ERR_NOMEM: return "FM_ERR_NOMEM";
    default: return "FM_ERR_UNKNOWN";
  }
}

const char *fm_version(void) { return "formura-gb300 0.1 sm_103a"; }

int fm_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int fm_malloc(void **ptr, size_t bytes) {
  FM_CHECK_ARG(ptr != nullptr, "fm_malloc: ptr is NULL");
  *ptr = nullptr;
  if (bytes == 0) return FM_OK;
  FM_TRY_CUDA(cudaMalloc(ptr, bytes));
  return FM_OK;
}

int fm_free(void *ptr) {
  if (ptr) FM_TRY_CUDA(cudaFree(ptr));
  return FM_OK;
}

int fm_memset(void *ptr, int value, size_t bytes, void *stream) {
  if (bytes == 0) return FM_OK;
  FM_CHECK_ARG(ptr != nullptr, "fm_memset: ptr is NULL");
  FM_TRY_CUDA(cudaMemsetAsync(ptr, value, bytes, as_stream(stream)));
  return FM_OK;
}

int fm_memcpy_h2d(void *dst, const void *src, size_t bytes, void *stream) {
  if (bytes == 0) return FM_OK;
  FM_CHECK_ARG(dst && src, "fm_memcpy_h2d: NULL pointer");
  FM_TRY_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, as_stream(stream)));
  return FM_OK;
}

int fm_memcpy_d2h(void *dst, const void *src, size_t bytes, void *stream) {
  if (bytes == 0) return FM_OK;
  FM_CHECK_ARG(dst && src, "fm_memcpy_d2h: NULL pointer");
  FM_TRY_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, as_stream(stream)));
  return FM_OK;
}

int fm_memcpy_d2d(void *dst, const void *src, size_t bytes, void *stream) {
  if (bytes == 0) return FM_OK;
  FM_CHECK_ARG(dst && src, "fm_memcpy_d2d: NULL pointer");
  FM_TRY_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, as_stream(stream)));
  return FM_OK;
}

int fm_stream_sync(void *stream) {
  FM_TRY_CUDA(cudaStreamSynchronize(as_stream(stream)));
  return FM_OK;
}

int fm_host_register(void *ptr, size_t bytes) {
  FM_CHECK_ARG(ptr && bytes, "fm_host_register: empty range");
  cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
  if (e == cudaErrorHostMemoryAlreadyRegistered) {
    cudaGetLastError();
    return FM_OK;
  }
  FM_TRY_CUDA(e);
  return FM_OK;
}

int fm_host_unregister(void *ptr) {
  cudaError_t e = cudaHostUnregister(ptr);
  if (e == cudaErrorHostMemoryNotRegistered) {
    cudaGetLastError();
    return FM_OK;
  }
  FM_TRY_CUDA(e);
  return FM_OK;
}

}  // extern "C"
