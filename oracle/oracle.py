"""ctypes front of the CPU oracle (fmr_oracle.c) and of the reference's own
generated C (examples-generated/pearson.c, built into oracle/_ref/).

TEST INFRASTRUCTURE ONLY: the checker of the GPU engine and the timed CPU
baseline.  The product never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF = HERE / "_ref"
DEFAULT_REFERENCE = Path(os.environ.get("FORMURA_REFERENCE", "/root/reference"))


class GsParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("F", "k", "Du", "Dv", "dt", "dx")]


def build(reference: bool = True) -> None:
    """make the oracle (parity + speed builds) and, when the reference tree is
    present, the reference's pearson.c."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    if reference and (DEFAULT_REFERENCE / "examples-generated" / "pearson.c").exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", "REF=%s" % DEFAULT_REFERENCE],
                       check=True)


_libs = {}


def _load(name: str) -> ctypes.CDLL:
    if name in _libs:
        return _libs[name]
    path = BUILD / name
    if not path.exists():
        build(reference=False)
    h = ctypes.CDLL(str(path))
    P = ctypes.c_void_p
    i, d, f = ctypes.c_int, ctypes.c_double, ctypes.c_float
    h.fo_gs2d_run_f64.argtypes = [i, i, P, P, i, ctypes.POINTER(GsParams)]
    h.fo_gs2d_run_f32.argtypes = [i, i, P, P, i, f, f, f, f, f, f]
    h.fo_diff2d_run_f64.argtypes = [i, i, P, i, d, d]
    h.fo_gs3d_run_f64.argtypes = [i, i, i, P, P, i, ctypes.POINTER(GsParams)]
    h.fo_gs3d_run_f32_kahan.argtypes = [i, i, i, P, P, P, P, i, f, f, f, f, f, f]
    h.fo_gs3d_run_f32k_fast.argtypes = [i, i, i, P, P, P, P, i, d, d, d, d, d, d]
    h.fo_mhd_run_f64.argtypes = [i, i, i, ctypes.POINTER(P), i]
    h.fo_sum_f64.argtypes = [ctypes.c_int64, P]
    h.fo_sum_f64.restype = d
    h.fo_num_threads.restype = i
    _libs[name] = h
    return h


def lib(fast: bool = False) -> ctypes.CDLL:
    return _load("libfmr_oracle_fast.so" if fast else "libfmr_oracle.so")


def _ptr(a: np.ndarray):
    assert a.flags.c_contiguous
    return ctypes.c_void_p(a.ctypes.data)


def gs2d_f64(U, V, steps, F, k, Du, Dv, dt, dx, fast=False):
    U = np.ascontiguousarray(U, dtype=np.float64).copy()
    V = np.ascontiguousarray(V, dtype=np.float64).copy()
    p = GsParams(F, k, Du, Dv, dt, dx)
    lib(fast).fo_gs2d_run_f64(U.shape[0], U.shape[1], _ptr(U), _ptr(V), int(steps), ctypes.byref(p))
    return U, V


def gs2d_f32(U, V, steps, F, k, Du, Dv, dt, dx, fast=False):
    U = np.ascontiguousarray(U, dtype=np.float32).copy()
    V = np.ascontiguousarray(V, dtype=np.float32).copy()
    lib(fast).fo_gs2d_run_f32(U.shape[0], U.shape[1], _ptr(U), _ptr(V), int(steps),
                              *[ctypes.c_float(x) for x in (F, k, Du, Dv, dt, dx)])
    return U, V


def diff2d_f64(dens, steps, Dt, Dx, fast=False):
    a = np.ascontiguousarray(dens, dtype=np.float64).copy()
    lib(fast).fo_diff2d_run_f64(a.shape[0], a.shape[1], _ptr(a), int(steps), float(Dt), float(Dx))
    return a


def gs3d_f64(U, V, steps, F, k, Du, Dv, dt, dx, fast=False):
    U = np.ascontiguousarray(U, dtype=np.float64).copy()
    V = np.ascontiguousarray(V, dtype=np.float64).copy()
    p = GsParams(F, k, Du, Dv, dt, dx)
    nx, ny, nz = U.shape
    lib(fast).fo_gs3d_run_f64(nx, ny, nz, _ptr(U), _ptr(V), int(steps), ctypes.byref(p))
    return U, V


def gs3d_f32_kahan(U, V, cU, cV, steps, F, k, Du, Dv, dt, dx, fast=False):
    arrs = [np.ascontiguousarray(a, dtype=np.float32).copy() for a in (U, V, cU, cV)]
    nx, ny, nz = arrs[0].shape
    lib(fast).fo_gs3d_run_f32_kahan(nx, ny, nz, *[_ptr(a) for a in arrs], int(steps),
                                    *[ctypes.c_float(x) for x in (F, k, Du, Dv, dt, dx)])
    return tuple(arrs)


def gs3d_f32k_fast(U, V, cU, cV, steps, F, k, Du, Dv, dt, dx, fast=False):
    """The binary32 fast form with Kahan accumulation (the TB kernel's math)."""
    arrs = [np.ascontiguousarray(a, dtype=np.float32).copy() for a in (U, V, cU, cV)]
    nx, ny, nz = arrs[0].shape
    lib(fast).fo_gs3d_run_f32k_fast(nx, ny, nz, *[_ptr(a) for a in arrs], int(steps),
                                    float(F), float(k), float(Du), float(Dv), float(dt), float(dx))
    return tuple(arrs)


def mhd_f64(fields, steps, fast=False):
    """examples/3d-mhd-rk4.fmr steps in double; fields = 9 arrays [n][n][n]
    (dens, vx, vy, vz, Bx, By, Bz, s, Psi).  Returns new arrays."""
    arrs = [np.ascontiguousarray(a, dtype=np.float64).copy() for a in fields]
    nx, ny, nz = arrs[0].shape
    ptrs = (ctypes.c_void_p * 9)(*[a.ctypes.data for a in arrs])
    lib(fast).fo_mhd_run_f64(nx, ny, nz, ptrs, int(steps))
    return arrs


def num_threads(fast: bool = False) -> int:
    return int(lib(fast).fo_num_threads())


# ---- the reference's own generated C ---------------------------------------

class PearsonNavigator(ctypes.Structure):
    """The navigator examples-generated/pearson.c writes (pearson.c:75-85)."""
    _fields_ = [(n, ctypes.c_int) for n in ("time_step", "lower_x", "upper_x", "offset_x",
                                              "lower_y", "upper_y", "offset_y")]


class ReferencePearson:
    """examples-generated/pearson.c: 2D Gray-Scott, 600x600 periodic, data at
    offset +2 in 604x604 arrays, 20 steps per Formura_Forward."""

    N = 600
    PAD = 604
    OFF = 2
    STEPS_PER_FORWARD = 20
    CONSTANTS = dict(F=0.015, k=0.05, Du=2e-5, Dv=1e-5, dt=1.0, dx=0.01)

    def __init__(self):
        path = REF / "libpearson_ref.so"
        if not path.exists():
            build(reference=True)
        if not path.exists():
            raise FileNotFoundError("reference pearson.c not built (reference tree absent)")
        self.lib = ctypes.CDLL(str(path))
        n = self.PAD * self.PAD
        self.U = np.frombuffer((ctypes.c_double * n).in_dll(self.lib, "U"),
                               dtype=np.float64).reshape(self.PAD, self.PAD)
        self.V = np.frombuffer((ctypes.c_double * n).in_dll(self.lib, "V"),
                               dtype=np.float64).reshape(self.PAD, self.PAD)
        self.navi = PearsonNavigator()

    def run(self, U0, V0, n_forward: int):
        o, n = self.OFF, self.N
        self.U[:] = 0.0
        self.V[:] = 0.0
        self.U[o:o + n, o:o + n] = U0
        self.V[o:o + n, o:o + n] = V0
        self.lib.Formura_Init(ctypes.byref(self.navi), 0)
        for _ in range(n_forward):
            self.lib.Formura_Forward(ctypes.byref(self.navi))
        return (self.U[o:o + n, o:o + n].copy(), self.V[o:o + n, o:o + n].copy(),
                int(self.navi.time_step))


def reference_available() -> bool:
    return (REF / "libpearson_ref.so").exists() or (
        DEFAULT_REFERENCE / "examples-generated" / "pearson.c").exists()
