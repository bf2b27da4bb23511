// fm_snapshot.cu — asynchronous snapshots of one plane of a device array.
//
// The monitor of a Formura driver writes, every T_MONITOR steps, mid-planes
// of the state arrays (examples/pearson-3d-main.cpp:116-157).  With the
// state resident on the GPU, a plane is taken in two stages so that the
// time stepping need not wait for the host:
//   1. on the caller's (compute) stream: a strided device-to-device gather of
//      the plane into a device staging buffer — ordered before every later
//      kernel on that stream, so the state may be overwritten right after;
//   2. on the snapshot's own copy stream, after an event on the compute
//      stream: device staging -> pinned host staging.
// fm_snapshot_wait blocks on the copy's event and hands the plane out.
//
// A plane of a row-major array of shape (n_0, ..., n_{d-1}) at axis a, index
// i consists of outer = n_0 * ... * n_{a-1} blocks of inner = n_{a+1} * ...
// * n_{d-1} contiguous elements spaced n_a * inner elements apart: one 2D copy.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "fm_common.cuh"

struct fm_snapshot {
  int ndim = 0;
  long long shape[8] = {0};
  int elem_size = 0;
  size_t cap_bytes = 0;  // largest plane
  void *dev_stage = nullptr;
  void *host_stage = nullptr;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t gathered = nullptr, copied = nullptr;
  size_t pending_bytes = 0;
  bool pending = false;
};

namespace {

void plane_geometry(const fm_snapshot *s, int axis, long long *outer, long long *inner) {
  long long o = 1, in = 1;
  for (int k = 0; k < axis; ++k) o *= s->shape[k];
  for (int k = axis + 1; k < s->ndim; ++k) in *= s->shape[k];
  *outer = o;
  *inner = in;
}

void release(fm_snapshot *s) {
  if (!s) return;
  if (s->copy_stream) cudaStreamSynchronize(s->copy_stream);
  if (s->gathered) cudaEventDestroy(s->gathered);
  if (s->copied) cudaEventDestroy(s->copied);
  if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
  if (s->dev_stage) cudaFree(s->dev_stage);
  if (s->host_stage) cudaFreeHost(s->host_stage);
  delete s;
}

}  // namespace

extern "C" int fm_snapshot_create(fm_snapshot **out, int ndim, const int *shape, int elem_size) {
  FM_CHECK_ARG(out && shape, "fm_snapshot_create: NULL argument");
  FM_CHECK_ARG(ndim >= 1 && ndim <= 8, "fm_snapshot_create: ndim must be 1..8");
  FM_CHECK_ARG(elem_size == 1 || elem_size == 2 || elem_size == 4 || elem_size == 8,
               "fm_snapshot_create: elem_size must be 1, 2, 4 or 8");
  *out = nullptr;
  fm_snapshot *s = new fm_snapshot();
  s->ndim = ndim;
  s->elem_size = elem_size;
  long long total = 1;
  for (int k = 0; k < ndim; ++k) {
    if (shape[k] < 1) {
      delete s;
      fm::set_error("fm_snapshot_create: shape[%d] = %d", k, shape[k]);
      return FM_ERR_ARG;
    }
    s->shape[k] = shape[k];
    total *= shape[k];
  }
  long long cap = 0;
  for (int a = 0; a < ndim; ++a) cap = std::max(cap, total / s->shape[a]);
  s->cap_bytes = (size_t)cap * elem_size;
  cudaError_t e = cudaMalloc(&s->dev_stage, s->cap_bytes);
  if (e == cudaSuccess) e = cudaMallocHost(&s->host_stage, s->cap_bytes);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->gathered, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->copied, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    release(s);
    return fm::cuda_status(e, "fm_snapshot_create");
  }
  *out = s;
  return FM_OK;
}

extern "C" long long fm_snapshot_plane_elems(const fm_snapshot *s, int axis) {
  if (!s || axis < 0 || axis >= s->ndim) return -1;
  long long outer, inner;
  plane_geometry(s, axis, &outer, &inner);
  return outer * inner;
}

extern "C" int fm_snapshot_begin(fm_snapshot *s, const void *array, int axis, int index,
                                 void *stream) {
  FM_CHECK_ARG(s && array, "fm_snapshot_begin: NULL argument");
  FM_CHECK_ARG(axis >= 0 && axis < s->ndim, "fm_snapshot_begin: axis %d out of range", axis);
  FM_CHECK_ARG(index >= 0 && index < s->shape[axis], "fm_snapshot_begin: index %d out of range",
               index);
  FM_CHECK_ARG(!s->pending, "fm_snapshot_begin: the previous snapshot was not waited for");
  cudaStream_t cs = reinterpret_cast<cudaStream_t>(stream);
  long long outer, inner;
  plane_geometry(s, axis, &outer, &inner);
  const size_t es = (size_t)s->elem_size;
  const size_t row = (size_t)inner * es;
  const size_t pitch = (size_t)s->shape[axis] * row;
  const char *src = static_cast<const char *>(array) + (size_t)index * row;
  FM_TRY_CUDA(cudaMemcpy2DAsync(s->dev_stage, row, src, pitch, row, (size_t)outer,
                                cudaMemcpyDeviceToDevice, cs));
  FM_TRY_CUDA(cudaEventRecord(s->gathered, cs));
  FM_TRY_CUDA(cudaStreamWaitEvent(s->copy_stream, s->gathered, 0));
  s->pending_bytes = row * (size_t)outer;
  FM_TRY_CUDA(cudaMemcpyAsync(s->host_stage, s->dev_stage, s->pending_bytes,
                              cudaMemcpyDeviceToHost, s->copy_stream));
  FM_TRY_CUDA(cudaEventRecord(s->copied, s->copy_stream));
  s->pending = true;
  return FM_OK;
}

extern "C" int fm_snapshot_wait(fm_snapshot *s, void *host_out) {
  FM_CHECK_ARG(s && host_out, "fm_snapshot_wait: NULL argument");
  FM_CHECK_ARG(s->pending, "fm_snapshot_wait: no snapshot in flight");
  s->pending = false;
  FM_TRY_CUDA(cudaEventSynchronize(s->copied));
  std::memcpy(host_out, s->host_stage, s->pending_bytes);
  return FM_OK;
}

extern "C" void fm_snapshot_destroy(fm_snapshot *s) { release(s); }
