"""Autotuner for the engine's tile shapes and blocking depths.

Formura tuned its CPU code by asynchronous simulated annealing over generated
variants (the "incubator", exe-src/c-incubator.hs:45-160: intra-node shape,
temporal-blocking depth, subroutine grouping, compiler flags).  On one GPU
the search space is small and every variant of a kernel is bit-exact with the
others, so the tuner here times each candidate directly on the caller's own
workload (a short sample of steps, CUDA events on the launching stream) and
keeps the fastest.  Results are cached per GPU model and workload signature
in a JSON file (``formura_gb300/_build/tune_cache.json`` unless
``FORMURA_TUNE_CACHE`` names another path).
"""
from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path
from typing import Dict, Iterable, List, Sequence, Tuple

import torch

from . import build as _build
from ._lib import lib
from . import kernels

ENSEMBLE_CANDIDATES: Tuple[Tuple[int, int], ...] = (
    (32, 2), (32, 4), (32, 8), (64, 1), (64, 2), (64, 4), (64, 8),
    (1, 2), (1, 4), (1, 6), (1, 8))  # tile 1: wavefront strips streamed along x


def _cache_path() -> Path:
    return Path(os.environ.get("FORMURA_TUNE_CACHE", str(_build.BUILD / "tune_cache.json")))


def _load_cache() -> Dict[str, dict]:
    p = _cache_path()
    try:
        return json.loads(p.read_text())
    except Exception:
        return {}


def _store(key: str, value: dict) -> None:
    p = _cache_path()
    cache = _load_cache()
    cache[key] = value
    p.parent.mkdir(parents=True, exist_ok=True)
    tmp = p.with_suffix(".tmp")
    tmp.write_text(json.dumps(cache, indent=1, sort_keys=True))
    os.replace(tmp, p)


def _gpu_name() -> str:
    return torch.cuda.get_device_name(torch.cuda.current_device())


def _time(fn, reps: int = 2) -> float:
    """Best-of-`reps` seconds of fn() measured with CUDA events."""
    fn()
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        b.synchronize()
        best = min(best, a.elapsed_time(b) / 1e3)
    return best


def ensemble_key(sizes: Sequence[int], F, k) -> str:
    h = hashlib.sha256(repr((list(sizes), [round(float(x), 12) for x in F],
                             [round(float(x), 12) for x in k])).encode()).hexdigest()[:16]
    return "gs2d_ens|%s|%s" % (_gpu_name(), h)


def tune_ensemble(sizes, F, k, Du=2e-5, Dv=1e-5, dt=1.0, dx=0.01, sample_steps: int = 64,
                  candidates: Iterable[Tuple[int, int]] = ENSEMBLE_CANDIDATES,
                  use_cache: bool = True) -> dict:
    """Pick (tile, tb) for an ensemble by timing each candidate on the real
    ensemble for `sample_steps` steps.  Returns {"tile", "tb", "timings"} and
    sets the "gs2d_ens.tile"/"gs2d_ens.tb" defaults to the winner."""
    key = ensemble_key(sizes, F, k)
    if use_cache:
        hit = _load_cache().get(key)
        if hit:
            _apply_ensemble(hit)
            return hit
    from . import inits

    U0, V0 = inits.gs2d_ensemble_state(sizes, seed=7)
    U = torch.from_numpy(U0).cuda()
    V = torch.from_numpy(V0).cuda()
    wU, wV = torch.empty_like(U), torch.empty_like(V)
    timings: List[Tuple[int, int, float]] = []
    for tile, tb in candidates:
        e = kernels.Ensemble(sizes, F, k, Du, Dv, dt, dx, tile=tile, tb=tb)
        try:
            t = _time(lambda: e.forward(U, V, wU, wV, sample_steps, use_graph=False))
            e.status()
        finally:
            e.close()
        timings.append((tile, tb, t))
    tile, tb, t = min(timings, key=lambda r: r[2])
    res = {"tile": tile, "tb": tb, "seconds_per_step": t / sample_steps,
           "timings": [[a, b, c / sample_steps] for a, b, c in timings]}
    _store(key, res)
    _apply_ensemble(res)
    return res


def _apply_ensemble(res: dict) -> None:
    lib().fm_tune_set(b"gs2d_ens.tile", int(res["tile"]))
    lib().fm_tune_set(b"gs2d_ens.tb", int(res["tb"]))


GS3D_F32K_CANDIDATES: Tuple[Tuple[int, int], ...] = tuple(
    (kern, tb) for kern in (0, 1, 2, 3) for tb in (1, 2, 3, 4))  # (gs3d_f32k.kernel, tb)


def tune_gs3d_f32k(n: Tuple[int, int, int] = (256, 256, 256), sample_steps: int = 24,
                   candidates: Iterable[Tuple[int, int]] = GS3D_F32K_CANDIDATES,
                   use_cache: bool = True) -> dict:
    """Pick the kernel form and the temporal-blocking depth of
    fm_gs3d_f32k_tb_forward on an n-sized problem; sets the "gs3d_f32k.kernel"
    and "gs3d_f32k.tb" defaults.  Returns {"kernel", "tb", "timings"}."""
    key = "gs3d_f32k|%s|%s" % (_gpu_name(), "x".join(map(str, n)))
    if use_cache:
        hit = _load_cache().get(key)
        if hit and "kernel" in hit:
            _apply_gs3d_f32k(hit)
            return hit
    from . import inits

    U0, V0 = inits.gray_scott_3d(*n, seed=1)
    U = torch.from_numpy(U0.astype("float32")).cuda()
    V = torch.from_numpy(V0.astype("float32")).cuda()
    cU, cV = torch.zeros_like(U), torch.zeros_like(V)
    w = torch.empty(4 * U.numel(), dtype=torch.float32, device="cuda")
    p = kernels.gs_params(0.04, 0.06, 2e-5, 1e-5, 0.5, 0.01)
    timings = []
    L = lib()
    prev = L.fm_tune_get(b"gs3d_f32k.kernel", -1)
    try:
        for kern, tb in candidates:
            L.fm_tune_set(b"gs3d_f32k.kernel", int(kern))
            t = _time(lambda: kernels.gs3d_f32k_tb_forward(U, V, cU, cV, w, p, sample_steps, tb))
            timings.append((kern, tb, t / sample_steps))
    finally:
        if prev >= 0:
            L.fm_tune_set(b"gs3d_f32k.kernel", prev)
    kern, tb, t = min(timings, key=lambda r: r[2])
    res = {"kernel": kern, "tb": tb, "seconds_per_step": t,
           "timings": [list(r) for r in timings]}
    _store(key, res)
    _apply_gs3d_f32k(res)
    return res


def _apply_gs3d_f32k(res: dict) -> None:
    lib().fm_tune_set(b"gs3d_f32k.kernel", int(res["kernel"]))
    lib().fm_tune_set(b"gs3d_f32k.tb", int(res["tb"]))
