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


def gs2d_f32_forward(U, V, work_U, work_V, params: GsParams, steps: int, stream=None):
    """One 2D Gray-Scott instance (pearson-2d form, float), one launch per step."""
    shp = tuple(U.shape)
    if len(shp) != 2:
        raise ValueError("U must be 2D")
    args = [_need(t, torch.float32, shp, n) for t, n in
            ((U, "U"), (V, "V"), (work_U, "work_U"), (work_V, "work_V"))]
    st = lib().fm_gs2d_f32_forward(shp[0], shp[1], *args, ctypes.byref(params), int(steps),
                                   ctypes.c_void_p(_stream_ptr(stream)))
    check(st, "fm_gs2d_f32_forward")


class Ensemble:
    """An uneven ensemble of periodic 2D Gray-Scott instances (fm_gs2d_ensemble_*).

    ``sizes[i]`` x ``sizes[i]`` cells with their own ``F[i]``, ``k[i]``; all
    instances' U (and V) back to back in one float32 CUDA buffer, instance i
    starting at ``offsets[i]``.
    """

    def __init__(self, sizes, F, k, Du=2e-5, Dv=1e-5, dt=1.0, dx=0.01, tile=0, tb=0):
        import numpy as np

        n = len(sizes)
        if not (len(F) == len(k) == n) or n == 0:
            raise ValueError("sizes, F, k must have the same nonzero length")
        self.sizes = [int(s) for s in sizes]
        sz = (ctypes.c_int * n)(*self.sizes)
        f = (ctypes.c_double * n)(*map(float, F))
        kk = (ctypes.c_double * n)(*map(float, k))
        h = ctypes.c_void_p()
        check(lib().fm_gs2d_ensemble_create(ctypes.byref(h), n, sz, f, kk, float(Du), float(Dv),
                                            float(dt), float(dx), int(tile), int(tb)),
              "fm_gs2d_ensemble_create")
        self._h = h
        total = ctypes.c_int64()
        offs = (ctypes.c_int64 * n)()
        nt = ctypes.c_int()
        check(lib().fm_gs2d_ensemble_layout(h, ctypes.byref(total), offs, ctypes.byref(nt)),
              "fm_gs2d_ensemble_layout")
        self.total_cells = int(total.value)
        self.offsets = np.array(offs[:], dtype=np.int64)
        self.ntiles = int(nt.value)

    def view(self, flat, i):
        o, s = int(self.offsets[i]), self.sizes[i]
        return flat[o:o + s * s].view(s, s)

    def forward(self, U, V, work_U, work_V, steps: int, use_graph: bool = True, stream=None):
        shp = (self.total_cells,)
        args = [_need(t, torch.float32, shp, n) for t, n in
                ((U, "U"), (V, "V"), (work_U, "work_U"), (work_V, "work_V"))]
        check(lib().fm_gs2d_ensemble_forward(self._h, *args, int(steps), 1 if use_graph else 0,
                                             ctypes.c_void_p(_stream_ptr(stream))),
              "fm_gs2d_ensemble_forward")

    def status(self, stream=None):
        check(lib().fm_gs2d_ensemble_status(self._h, ctypes.c_void_p(_stream_ptr(stream))),
              "fm_gs2d_ensemble_status")

    def close(self):
        if getattr(self, "_h", None):
            lib().fm_gs2d_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


MHD_NFIELDS = 9


def _mhd_ptrs(fields, dtype, n):
    if len(fields) != MHD_NFIELDS:
        raise ValueError("9 MHD fields expected (dens, vx, vy, vz, Bx, By, Bz, s, Psi)")
    return (ctypes.c_void_p * MHD_NFIELDS)(
        *[_need(f, dtype, (n, n, n), "field %d" % i).value for i, f in enumerate(fields)])


def mhd_forward(fields, work, steps: int, stream=None):
    """Advance the 9 MHD fields (float64: all-FP64 path; float32: binary32 bulk
    with the FP64 energy update) by `steps` time steps of 3d-mhd-rk4.fmr."""
    n = int(fields[0].shape[0])
    dtype = fields[0].dtype
    if dtype not in (torch.float64, torch.float32):
        raise ValueError("MHD fields must be float64 or float32")
    ptrs = _mhd_ptrs(fields, dtype, n)
    w = _need(work, dtype, (18 * n ** 3,), "work")
    fn = lib().fm_mhd_forward_f64 if dtype == torch.float64 else lib().fm_mhd_forward_f32
    check(fn(n, ptrs, w, int(steps), ctypes.c_void_p(_stream_ptr(stream))), "fm_mhd_forward")


def mhd_totals(fields, stream=None):
    """FP64 totals (mass, kinetic+magnetic energy, sum s, x-momentum) as a
    4-element float64 CUDA tensor."""
    n = int(fields[0].shape[0])
    dtype = fields[0].dtype
    ptrs = _mhd_ptrs(fields, dtype, n)
    part = torch.empty(int(lib().fm_mhd_totals_scratch_elems(n)), dtype=torch.float64,
                       device=fields[0].device)
    out = torch.empty(4, dtype=torch.float64, device=fields[0].device)
    check(lib().fm_mhd_totals(n, 1 if dtype == torch.float64 else 0, ptrs,
                              ctypes.c_void_p(part.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                              ctypes.c_void_p(_stream_ptr(stream))), "fm_mhd_totals")
    return out
