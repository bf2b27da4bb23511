"""The thin C ABI on torch device tensors.

PyTorch provides device memory and streams here; every computation is a call
into libformura_gb300.so.  Each function checks shapes, dtypes, devices and
contiguity before the call, and raises FormuraError on a non-zero status.
"""
from __future__ import annotations

import ctypes

import torch

from ._lib import GsParams, check, lib


def _stream_ptr(stream) -> int:
    if stream is None:
        stream = torch.cuda.current_stream()
    return int(stream.cuda_stream)


def _need(t: torch.Tensor, dtype, shape, name):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise ValueError("%s must be a CUDA tensor" % name)
    if t.dtype != dtype:
        raise ValueError("%s must be %s, got %s" % (name, dtype, t.dtype))
    if tuple(t.shape) != tuple(shape):
        raise ValueError("%s must have shape %s, got %s" % (name, tuple(shape), tuple(t.shape)))
    if not t.is_contiguous():
        raise ValueError("%s must be contiguous" % name)
    return ctypes.c_void_p(t.data_ptr())


def gs_params(F, k, Du, Dv, dt, dx) -> GsParams:
    return GsParams(float(F), float(k), float(Du), float(Dv), float(dt), float(dx))


def gs3d_f64_forward(U, V, work_U, work_V, params: GsParams, steps: int, stream=None):
    """Advance FP64 U,V ([nx,ny,nz] CUDA tensors) by `steps` in place."""
    shp = tuple(U.shape)
    if len(shp) != 3:
        raise ValueError("U must be 3D")
    args = [_need(t, torch.float64, shp, n) for t, n in
            ((U, "U"), (V, "V"), (work_U, "work_U"), (work_V, "work_V"))]
    st = lib().fm_gs3d_f64_forward(shp[0], shp[1], shp[2], *args, ctypes.byref(params),
                                   int(steps), ctypes.c_void_p(_stream_ptr(stream)))
    check(st, "fm_gs3d_f64_forward")


def _f32k_args(U, V, cU, cV, work):
    shp = tuple(U.shape)
    if len(shp) != 3:
        raise ValueError("U must be 3D")
    args = [_need(t, torch.float32, shp, n) for t, n in ((U, "U"), (V, "V"), (cU, "cU"), (cV, "cV"))]
    n = shp[0] * shp[1] * shp[2]
    return shp, args, _need(work, torch.float32, (4 * n,), "work")


def gs3d_f32k_forward(U, V, cU, cV, work, params: GsParams, steps: int, stream=None):
    """Advance FP32 U,V (generated DAG in float) with Kahan compensations cU,cV."""
    shp, args, w = _f32k_args(U, V, cU, cV, work)
    st = lib().fm_gs3d_f32k_forward(shp[0], shp[1], shp[2], *args, w, int(steps),
                                    ctypes.byref(params), ctypes.c_void_p(_stream_ptr(stream)))
    check(st, "fm_gs3d_f32k_forward")


def gs3d_f32k_tb_forward(U, V, cU, cV, work, params: GsParams, steps: int, tb: int = 0,
                         stream=None):
    """Advance FP32 U,V (fast form, Kahan) by `steps`, `tb` steps per HBM pass."""
    shp, args, w = _f32k_args(U, V, cU, cV, work)
    st = lib().fm_gs3d_f32k_tb_forward(shp[0], shp[1], shp[2], *args, w, int(steps), int(tb),
                                       ctypes.byref(params), ctypes.c_void_p(_stream_ptr(stream)))
    check(st, "fm_gs3d_f32k_tb_forward")


def diff2d_f64_forward(dens, work, coef: float, steps: int, stream=None):
    shp = tuple(dens.shape)
    if len(shp) != 2:
        raise ValueError("dens must be 2D")
    a = _need(dens, torch.float64, shp, "dens")
    w = _need(work, torch.float64, shp, "work")
    st = lib().fm_diff2d_f64_forward(shp[0], shp[1], a, w, float(coef), int(steps),
                                     ctypes.c_void_p(_stream_ptr(stream)))
    check(st, "fm_diff2d_f64_forward")


def sum_scratch_elems(n: int) -> int:
    return int(lib().fm_sum_f64_scratch_elems(int(n)))


def total(a: torch.Tensor, partials: torch.Tensor | None = None, stream=None) -> torch.Tensor:
    """Deterministic FP64 total of a float64 or float32 CUDA tensor (0-d tensor)."""
    if not a.is_cuda or not a.is_contiguous():
        raise ValueError("a must be a contiguous CUDA tensor")
    n = a.numel()
    if partials is None:
        partials = torch.empty(sum_scratch_elems(n), dtype=torch.float64, device=a.device)
    out = torch.empty((), dtype=torch.float64, device=a.device)
    s = ctypes.c_void_p(_stream_ptr(stream))
    if a.dtype == torch.float64:
        st = lib().fm_sum_f64(n, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(partials.data_ptr()),
                              ctypes.c_void_p(out.data_ptr()), s)
    elif a.dtype == torch.float32:
        st = lib().fm_sum_f32_as_f64(n, ctypes.c_void_p(a.data_ptr()),
                                     ctypes.c_void_p(partials.data_ptr()),
                                     ctypes.c_void_p(out.data_ptr()), s)
    else:
        raise ValueError("total: float64 or float32 only")
    check(st, "fm_sum")
    return out


def probe_fma(fp64: bool, blocks: int, threads: int, iters: int, sink: torch.Tensor, stream=None):
    st = lib().fm_probe_fma(1 if fp64 else 0, blocks, threads, iters,
                            ctypes.c_void_p(sink.data_ptr()), ctypes.c_void_p(_stream_ptr(stream)))
    check(st, "fm_probe_fma")
