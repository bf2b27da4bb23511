"""Benchmark of the GB300 engine on the 3D Gray-Scott workload.

Workload: 3D Gray-Scott (examples/gray-scott-3d.fmr, the pearson-3d.fmr form
with the F,k reaction), 256^3 FP64, periodic, Du=2e-5 Dv=1e-5 F=0.04 k=0.06
dx=0.01 dt=0.5; seeded start (8 cubes of side 16).  One bench step = one
Formura_Forward of the emitted program = 2000 time steps.

  value   GLUP/s with the state resident in HBM (Formura_Advance), CUDA events
          on the launching stream; 268 MB of state > 129 MB L2 (no flush needed).
  e2e     GLUP/s through Formura_Forward on the host globals: pinned H2D copy of
          U,V, 2000 steps, D2H copy, every step.
  roofline  the dominant kernel (gs3d_f64_row) against the FP64 FMA pipe
          measured in this run, and its HBM fraction.  Algorithmic work is the
          generated DAG's 46 FP64 operations per cell update; the kernel runs the
          divisions by dx and the multiplications by constants as exact integer
          sequences, so the FP64 pipe executes 26 FP64 instructions per update.
  cpu_baseline  the oracle's OpenMP speed build on all host cores, on a
          bounded sample of the same workload.
  parity  computed in the run: the state after one Formura_Forward (2000
          steps at 256^3) against the oracle's parity build from the same
          seeded start (bit-exact flag and max relative error), the same for
          2D diffusion 256^2 x 1000 and for FP64 MHD at the largest size the
          oracle finishes in about a minute (labelled).

--impl reference times that CPU implementation alone (the reference's path
is CPU code; its compiler cannot run here), with the same metric and config.
Multi-GPU: replicas only (one independent program per rank, weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = "gray_scott_3d"
# The one metric name both arms print (the engine and --impl reference).
METRIC = "GLUP/s (3D Gray-Scott 256^3 FP64)"
N = 256
GS = dict(F=0.04, k=0.06, Du=2e-5, Dv=1e-5, dt=0.5, dx=0.01)
# Algorithmic work per lattice-site update of the pearson-3d DAG (counted on the
# constant-folded OM graph, division = 1 flop): 46 flops, 32 B.
FLOPS_PER_LUP = 46
BYTES_PER_LUP = 32


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        return json.loads(p.read_text())
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                self.out = ""

    def summary(self):
        rows = []
        for line in (self.out or "").splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append(dict(sm=float(parts[1]), smax=float(parts[2]), reasons=parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        seen = sorted({names[i] for r in rows for i, v in enumerate(r["reasons"])
                       if v.lower().startswith("active")})
        return {"sm_mhz": statistics.median(r["sm"] for r in rows),
                "sm_max_mhz": max(r["smax"] for r in rows), "reasons": seen,
                "samples": len(rows)}


def measure_fma_peak(torch, kernels, fp64: bool, sms: int):
    blocks, threads = sms * 8, 256
    iters = 2048 if fp64 else 65536
    sink = torch.zeros(blocks, dtype=torch.float64 if fp64 else torch.float32, device="cuda")
    kernels.probe_fma(fp64, blocks, threads, 64, sink)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(3):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        kernels.probe_fma(fp64, blocks, threads, iters, sink)
        b.record()
        b.synchronize()
        best = min(best, a.elapsed_time(b) / 1e3)
    return blocks * threads * iters * 16 / best / 1e12  # TFLOP/s


def read_profile_traffic():
    """dram bytes per launch of gs3d_f64_row from the committed ncu summary."""
    p = ROOT / "profiles" / "gs3d_f64_row_256.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith("dram_bytes_per_launch"):
            try:
                return int(float(line.split("=")[1].split()[0]))
            except Exception:
                return None
    return None


def cpu_baseline(seconds: float = 18.0):
    """The oracle's speed build (OpenMP, all host cores) on 256^3 x S steps."""
    import numpy as np

    from formura_gb300 import inits
    from oracle import oracle

    U0, V0 = inits.gray_scott_3d(N, N, N, seed=1)
    oracle.gs3d_f64(U0, V0, 1, **GS, fast=True)  # warm (page-in, thread pool)
    t = time.perf_counter()
    oracle.gs3d_f64(U0, V0, 2, **GS, fast=True)
    per = (time.perf_counter() - t) / 2
    steps = max(2, min(2000, int(seconds / max(per, 1e-6))))  # ~`seconds` of CPU work
    t = time.perf_counter()
    oracle.gs3d_f64(U0, V0, steps, **GS, fast=True)
    dt = time.perf_counter() - t
    return dict(value=round(N ** 3 * steps / dt / 1e9, 4), unit="GLUP/s",
                cores=oracle.num_threads(fast=True), kind="port",
                sample="256^3 FP64 Gray-Scott x %d steps (of 2000), oracle -O3 OpenMP" % steps,
                seconds=round(dt, 3))


def _event_time(torch, fn):
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    fn()
    b.record()
    b.synchronize()
    return a.elapsed_time(b) / 1e3


def compare(got, want):
    """Bit-exactness and max relative error of a state against the oracle's
    (relative to |want| per cell, cells where want == 0 by absolute error)."""
    import numpy as np

    got = np.ascontiguousarray(got)
    want = np.ascontiguousarray(want, dtype=got.dtype)
    # bit patterns of the state itself: +0 and -0 differ
    ut = {4: np.uint32, 8: np.uint64}[got.dtype.itemsize]
    same = bool(np.array_equal(got.view(ut), want.view(ut)))
    got = got.astype(np.float64)
    want = want.astype(np.float64)
    diff = np.abs(got - want)
    den = np.abs(want)
    rel = np.where(den > 0, diff / np.where(den > 0, den, 1.0), diff)
    return {"bit_exact": same,
            "max_rel_err": float(rel.max()) if rel.size else 0.0,
            "max_abs_err": float(diff.max()) if diff.size else 0.0}


def run_parity(torch, U_final, V_final, U0, V0):
    """The engine's results against the oracle's parity build (-O2
    -ffp-contract=off, OpenMP), computed in this run from the same seeded
    inputs: the headline state after one Formura_Forward (256^3 x 2000 steps),
    2D diffusion 256^2 x 1000 steps, and FP64 MHD x 500 steps at the largest
    cube the oracle finishes in about a minute."""
    import numpy as np

    from formura_gb300 import inits, kernels
    from oracle import oracle

    out = {}
    t = time.perf_counter()
    Uo, Vo = oracle.gs3d_f64(U0, V0, 2000, **GS)
    cu, cv = compare(U_final, Uo), compare(V_final, Vo)
    out["gray_scott_3d_256_2000_steps"] = {
        "bit_exact": cu["bit_exact"] and cv["bit_exact"],
        "max_rel_err": max(cu["max_rel_err"], cv["max_rel_err"]),
        "max_abs_err": max(cu["max_abs_err"], cv["max_abs_err"]),
        "tolerance": 1e-12, "path": "Formura_Forward (host globals in and out)",
        "oracle_seconds": round(time.perf_counter() - t, 1)}
    del Uo, Vo
    # 2D diffusion through the emitted program (coefficient 0.4 = the
    # program's Dt/Dx**2: 0.1 on the 5-point difference)
    d0 = inits.diffusion_2d(256, 256, seed=1)
    d = torch.from_numpy(d0).cuda()
    kernels.diff2d_f64_forward(d, torch.empty_like(d), 0.4, 1000)
    c = compare(d.cpu().numpy(), oracle.diff2d_f64(d0, 1000, 0.4, 1.0))
    out["diffusion_2d_256_1000_steps"] = dict(c, tolerance=1e-12)
    # FP64 MHD: size from the oracle's measured rate (about a minute of CPU)
    f_probe = inits.mhd_3d(32, seed=1)
    oracle.mhd_f64(f_probe, 1)
    t = time.perf_counter()
    oracle.mhd_f64(f_probe, 2)
    per_lup = (time.perf_counter() - t) / (2 * 32 ** 3)
    n = 32
    for cand in (96, 80, 64, 48, 40):
        if cand ** 3 * 500 * per_lup <= 60.0:
            n = cand
            break
    f0 = inits.mhd_3d(n, seed=1)
    t64 = [torch.from_numpy(x).cuda() for x in f0]
    kernels.mhd_forward(t64, torch.empty(18 * n ** 3, dtype=torch.float64, device="cuda"), 500)
    t = time.perf_counter()
    fo = oracle.mhd_f64(f0, 500)
    worst = {"bit_exact": True, "max_rel_err": 0.0, "max_abs_err": 0.0}
    for x, y in zip(t64, fo):
        c = compare(x.cpu().numpy(), y)
        worst = {"bit_exact": worst["bit_exact"] and c["bit_exact"],
                 "max_rel_err": max(worst["max_rel_err"], c["max_rel_err"]),
                 "max_abs_err": max(worst["max_abs_err"], c["max_abs_err"])}
    out["mhd_3d_fp64_500_steps"] = dict(worst, grid=[n, n, n], tolerance=1e-12,
                                        fields=9, oracle_seconds=round(time.perf_counter() - t, 1))
    return out


def run_variants(torch, prog, U_fp64_final, U0, V0, peaks):
    """The other forms of the hot path, each timed on the device after a warm-up
    (CUDA events on the launching stream), at the sizes the workloads name."""
    import numpy as np

    from formura_gb300 import autotune, inits, kernels
    from oracle import oracle

    out = {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    # -- 3D Gray-Scott FP32 + Kahan, temporally blocked, scored against the FP64 run
    M = prog.steps_per_forward
    U = torch.from_numpy(U0.astype(np.float32)).cuda()
    V = torch.from_numpy(V0.astype(np.float32)).cuda()
    cU, cV = torch.zeros_like(U), torch.zeros_like(V)
    w = torch.empty(4 * U.numel(), dtype=torch.float32, device="cuda")
    prm = kernels.gs_params(**GS)
    tune = autotune.tune_gs3d_f32k((N, N, N))
    Uw, Vw = U.clone(), V.clone()
    kernels.gs3d_f32k_tb_forward(Uw, Vw, torch.zeros_like(U), torch.zeros_like(V), w, prm, 24)
    sec = _event_time(torch, lambda: kernels.gs3d_f32k_tb_forward(U, V, cU, cV, w, prm, M))
    Uf = U.double().cpu().numpy()
    err = float(np.linalg.norm(Uf - U_fp64_final) / np.linalg.norm(U_fp64_final))
    errmax = float(np.abs(Uf - U_fp64_final).max() / np.abs(U_fp64_final).max())
    g = N ** 3 * M / sec / 1e9
    out["gray_scott_3d_f32_kahan_tb"] = {
        "value": round(g, 2), "unit": "GLUP/s", "steps": M, "tb": tune["tb"],
        "rel_l2_error_vs_fp64": err, "max_rel_error_vs_fp64": errmax,
        "hbm_untiled_roofline_glups": round(hbm / 32.0, 1),
        "hbm_roofline_at_tb_glups": round(hbm / (32.0 / tune["tb"]), 1),
        "frac_of_hbm_roofline_at_tb": round(g / (hbm / (32.0 / tune["tb"])), 3),
        "kernel": ["gs3d_f32k_tb (one row per warp)", "gs3d_f32k_tbr<4 rows, 8 warps>",
                   "gs3d_f32k_tbr<2 rows, 16 warps>",
                   "gs3d_f32k_tbp (one row per warp, (u, v) as packed binary32 pairs)"
                   ][tune["kernel"]],
        "tuned": {"timings_s_per_step": tune["timings"]}}
    del U, V, cU, cV, w, Uw, Vw
    # -- uneven ensemble of 512 2D Gray-Scott instances, 5000 steps, one launch
    sizes, F, k = inits.gs2d_ensemble(512, seed=1)
    total = sum(n * n for n in sizes)
    res = autotune.tune_ensemble(sizes, F, k, sample_steps=40)
    e = kernels.Ensemble(sizes, F, k)
    Ue, Ve = inits.gs2d_ensemble_state(sizes, seed=1)
    Ue, Ve = torch.from_numpy(Ue).cuda(), torch.from_numpy(Ve).cuda()
    wU, wV = torch.empty_like(Ue), torch.empty_like(Ve)
    e.forward(Ue, Ve, wU, wV, 5000, use_graph=True)  # capture + warm
    sec = _event_time(torch, lambda: e.forward(Ue, Ve, wU, wV, 5000, use_graph=True))
    e.status()
    ens = total * 5000 / sec / 1e9
    sub = list(range(0, 512, 16))
    bufs = []
    for i in sub:
        u0, v0 = inits.gray_scott_2d_square(sizes[i], sizes[i], seed=i)
        u = torch.from_numpy(u0.astype(np.float32)).cuda()
        v = torch.from_numpy(v0.astype(np.float32)).cuda()
        bufs.append((u, v, torch.empty_like(u), torch.empty_like(v),
                     kernels.gs_params(F[i], k[i], 2e-5, 1e-5, 1.0, 0.01)))
    seq_cells = sum(sizes[i] ** 2 for i in sub)

    def seq():
        for u, v, wu, wv, prm_i in bufs:
            kernels.gs2d_f32_forward(u, v, wu, wv, prm_i, 100)

    seq()
    ssec = _event_time(torch, seq)
    out["gray_scott_2d_ensemble_512"] = {
        "value": round(ens, 2), "unit": "GLUP/s", "instances": 512, "steps": 5000,
        "total_cells": total, "tile": res["tile"], "tb": res["tb"],
        "graph_captured": True, "one_persistent_launch": True,
        "sequential_per_instance_launches_glups": round(seq_cells * 100 / ssec / 1e9, 2),
        "sequential_sample": "32 of 512 instances x 100 steps, one launch per step",
        "kernel": "gs2d_ens_wf (wavefront strips)" if res["tile"] == 1 else "gs2d_ensemble"}
    e.close()
    del Ue, Ve, wU, wV, bufs
    # -- 2D diffusion 256^2 FP64, 1000 steps in one persistent launch
    d0 = inits.diffusion_2d(256, 256, seed=1)
    d = torch.from_numpy(d0).cuda()
    wd = torch.empty_like(d)
    kernels.diff2d_f64_forward(d, wd, 0.4, 50)
    sec = _event_time(torch, lambda: kernels.diff2d_f64_forward(d, wd, 0.4, 1000))
    out["diffusion_2d_256_fp64"] = {"value": round(256 * 256 * 1000 / sec / 1e9, 2),
                                    "unit": "GLUP/s", "steps": 1000, "ms": round(sec * 1e3, 3),
                                    "parity": "see parity.diffusion_2d_256_1000_steps",
                                    "kernel": "diff2d_tb (4 steps per grid barrier)"}
    # -- 3D MHD 256^3, 500 steps: binary32 bulk with the FP64 energy update
    f0 = inits.mhd_3d(N, seed=1)
    t32 = [torch.from_numpy(x.astype(np.float32)).cuda() for x in f0]
    w32 = torch.empty(18 * N ** 3, dtype=torch.float32, device="cuda")
    kernels.mhd_forward([x.clone() for x in t32], w32, 1)
    sec = _event_time(torch, lambda: kernels.mhd_forward(t32, w32, 500))
    tot = kernels.mhd_totals(t32).cpu().numpy()
    del w32
    # the same 500 steps all in FP64 (bit-exact with the oracle): its speed, and the
    # FP32 run's error against it at the full 256^3
    t64 = [torch.from_numpy(x).cuda() for x in f0]
    w64 = torch.empty(18 * N ** 3, dtype=torch.float64, device="cuda")
    kernels.mhd_forward([x.clone() for x in t64], w64, 1)
    sec64 = _event_time(torch, lambda: kernels.mhd_forward(t64, w64, 500))
    del w64
    errs = {}
    for name, x, y in zip(inits.MHD_FIELDS, t32, t64):
        errs[name] = float((x.double() - y).abs().max() / y.abs().max().clamp_min(1e-300))
    del t32, t64
    out["gray_scott_3d_generated_from_fmr"] = run_generated_variant(torch, U0, V0)
    out["generated_temporal_blocking"] = run_generated_blocked_variant(torch, U0, V0, hbm)
    out["surrogate_gs2d_512"] = run_surrogate_variant(torch)
    out["mhd_3d_256_fp32_bulk_fp64_energy"] = {
        "value": round(N ** 3 * 500 / sec / 1e9, 3), "unit": "GLUP/s", "steps": 500,
        "seconds": round(sec, 3), "totals_fp64": [float(x) for x in tot],
        "max_rel_error_vs_fp64_256cube_500steps": errs, "kernel": "mhd_stage_tile x4 + mhd_finish"}
    out["mhd_3d_256_fp64"] = {
        "value": round(N ** 3 * 500 / sec64 / 1e9, 4), "unit": "GLUP/s", "steps": 500,
        "seconds": round(sec64, 3), "parity": "see parity.mhd_3d_fp64_500_steps",
        "kernel": "mhd_stage_march<double, 1> x4 + mhd_finish_v2<double, 1> "
                  "(exact binary64 scalings, constant products, divisions, fmax/fmin on the "
                  "integer pipes)"}
    return out


def run_generated_variant(torch, U0, V0):
    """examples/gray-scott-3d.fmr compiled by the front end (generated kernels,
    no hand tuning) at 256^3: Formura_Advance of 200 steps on the resident
    state, and bit-equality with the hand-written kernel after those steps."""
    import numpy as np

    from formura_gb300 import kernels
    from formura_gb300.fmr import load_program
    from formura_gb300.runtime import load_program as load_lib

    steps = 200
    p = load_program(ROOT / "examples" / "gray-scott-3d.fmr", intra_node_shape=[N, N, N],
                     monitor_interval=steps)
    prog = load_lib(p)
    prog.init()
    prog.state["U"][...] = U0
    prog.state["V"][...] = V0
    prog.upload()
    prog.advance(1)  # warm-up (and the first 200 steps of the comparison)
    sec = _event_time(torch, lambda: prog.advance(1))
    prog.upload()
    prog.advance(1)
    prog.download()
    U = torch.from_numpy(U0).cuda()
    V = torch.from_numpy(V0).cuda()
    kernels.gs3d_f64_forward(U, V, torch.empty_like(U), torch.empty_like(V),
                             kernels.gs_params(**GS), steps)
    same = bool(np.array_equal(prog.state["U"], U.cpu().numpy()) and
                np.array_equal(prog.state["V"], V.cpu().numpy()))
    prog.finalize()
    return {"value": round(N ** 3 * steps / sec / 1e9, 3), "unit": "GLUP/s", "steps": steps,
            "bit_equal_to_hand_kernel": same, "kernel": "fmr_level_0 (generated from .fmr)"}


def run_generated_blocked_variant(torch, U0, V0, hbm):
    """Temporal blocking of programs compiled by the front end, at 256^3 in
    binary32 with temporal_blocking_interval 4: the generated blocked kernel
    (4 steps per pass; tiles away from the periodic boundary staged by TMA)
    against the same program one step per launch, each timed over one
    Formura_Advance of 2000 steps on the resident state, and bit-equality of
    the two.  examples/heat-3d-float.fmr is memory-bound (every operation a
    float one); examples/gray-scott-3d-float.fmr divides by dx = 0.01, a
    double constant, as the reference's generated C does, so it stays bound
    by the FP64 pipe and blocking cannot pay there: by default (tb_kernel 0)
    only the light one is blocked."""
    import numpy as np

    from formura_gb300 import backend
    from formura_gb300.fmr import load_program
    from formura_gb300.runtime import load_program as load_lib

    out = {}
    for prog_name, bytes_per_cell, init in (
            ("heat-3d-float", 8, lambda: {"u": U0.astype(np.float32)}),
            ("gray-scott-3d-float", 16, lambda: {"U": U0.astype(np.float32),
                                                 "V": V0.astype(np.float32)})):
        res, finals = {}, []
        for tbk, label in ((1, "blocked"), (-1, "per_step")):
            p = load_program(ROOT / "examples" / (prog_name + ".fmr"), tb_kernel=tbk,
                             name="fmr_%s_%s" % (prog_name.replace("-", "_"), label))
            plan = backend.blocked_kernel(p)
            prog = load_lib(p)
            prog.init()
            for k, v in init().items():
                prog.state[k][...] = v
            prog.upload()
            prog.advance(1)  # warm-up
            prog.upload()
            sec = _event_time(torch, lambda: prog.advance(1))
            prog.download()
            finals.append([prog.state[k].copy() for k in sorted(prog.state)])
            res[label] = round(N ** 3 * p.steps_per_forward / sec / 1e9, 2)
            if plan is not None:
                pl = plan[1]
                res["tile"] = {"interior": pl.TI[1:], "region": pl.RG[1:], "planes_per_block": pl.XC,
                               "column_planes": pl.ntiles, "smem_bytes": pl.smem, "tma": pl.tma}
            prog.finalize()
        out[prog_name] = {
            "value": res["blocked"], "unit": "GLUP/s", "steps": 2000, "tb": 4,
            "per_step_glups": res["per_step"],
            "bit_equal_blocked_vs_per_step": all(np.array_equal(a, b)
                                                 for a, b in zip(finals[0], finals[1])),
            "hbm_roofline_per_step_glups": round(hbm / bytes_per_cell, 1),
            "hbm_roofline_at_tb_glups": round(hbm / (bytes_per_cell / 4), 1),
            "tile": res.get("tile"),
            # the kernel a program gets by default (tb_kernel 0): blocked only when light
            "default_kernel": ("blocked" if backend.blocked_kernel(
                load_program(ROOT / "examples" / (prog_name + ".fmr"))) is not None
                else "per_step"),
            "kernel": "fmr_level_tb (generated, 4 steps per pass) vs fmr_level_0"}
    return out


def run_surrogate_variant(torch):
    """The learned 16-step surrogate on 8 instances of 512^2 (trained weights in
    formura_gb300/weights): network-jump throughput against the plain FP32
    stencil on the same batch, and a 4096-step run with re-anchoring every 256
    steps and stencil fallback, scored against the FP64 oracle."""
    import numpy as np

    from formura_gb300 import inits
    from formura_gb300 import surrogate_run as sr
    from formura_gb300.surrogate import JUMP, Surrogate
    from oracle import oracle

    B, Nn = 8, 512
    net = Surrogate(seed=0)
    net.load_npz(ROOT / "formura_gb300" / "weights" / "gs2d_surrogate.npz")
    sizes, Fl, Kl = inits.gs2d_ensemble(B, seed=2024, sizes=(Nn,))
    U0, V0 = inits.gs2d_ensemble_state(sizes, seed=2024)
    Ft = torch.tensor(Fl, dtype=torch.float32, device="cuda")
    Kt = torch.tensor(Kl, dtype=torch.float32, device="cuda")

    def fresh():
        return (torch.from_numpy(U0).cuda().view(B, Nn, Nn).clone(),
                torch.from_numpy(V0).cuda().view(B, Nn, Nn).clone())

    U, V = fresh()
    net.predict(U, V, Ft, Kt)
    jump_s = _event_time(torch, lambda: [net.predict(U, V, Ft, Kt) for _ in range(16)]) / 16
    flops = 14 * 2 * 576 * 64 * B * (Nn // 4) ** 2
    U, V = fresh()
    sr.run_plain(U, V, Ft, Kt, JUMP)
    plain16_s = _event_time(torch, lambda: sr.run_plain(U, V, Ft, Kt, JUMP))
    Up, Vp = fresh()
    plain_s = _event_time(torch, lambda: sr.run_plain(Up, Vp, Ft, Kt, 4096))
    info = sr.run_with_surrogate(net, *fresh(), Ft, Kt, 4096, 256, 1e-2)  # warm-up
    Us, Vs = fresh()
    sur_s = _event_time(torch, lambda: sr.run_with_surrogate(net, Us, Vs, Ft, Kt, 4096, 256, 1e-2))
    errs = []
    for i in range(2):
        u0 = U0[i * Nn * Nn:(i + 1) * Nn * Nn].reshape(Nn, Nn).astype(np.float64)
        v0 = V0[i * Nn * Nn:(i + 1) * Nn * Nn].reshape(Nn, Nn).astype(np.float64)
        uo, vo = oracle.gs2d_f64(u0, v0, 4096, Fl[i], Kl[i], 2e-5, 1e-5, 1.0, 0.01, fast=True)
        us, vs = Us[i].double().cpu().numpy(), Vs[i].double().cpu().numpy()
        errs.append(float(np.sqrt((np.linalg.norm(us - uo) ** 2 + np.linalg.norm(vs - vo) ** 2) /
                                  (np.linalg.norm(uo) ** 2 + np.linalg.norm(vo) ** 2))))
    held = sr.jump_error(net, n_inst=16, N=128, seed=99)
    return {
        "network_jump_ms": round(jump_s * 1e3, 3),
        "conv_tflops": round(flops / jump_s / 1e12, 1),
        "network_steps_per_s": round(B * JUMP / jump_s, 1),
        "plain_stencil_16_steps_ms": round(plain16_s * 1e3, 3),
        "plain_stencil_steps_per_s": round(B * 4096 / plain_s, 1),
        "surrogate_run_steps_per_s": round(B * 4096 / sur_s, 1),
        "speedup_vs_plain": round(plain_s / sur_s, 4),
        "network_only_speed_ratio_vs_plain": round(plain16_s / jump_s, 4),
        "fallback_instances": int(sum(info["fallback"])), "instances": B,
        "rel_l2_vs_fp64_after_4096": errs,
        "heldout_jump_rel_l2": held["state_rel_l2"],
        "heldout_persistence_rel_l2": held["state_rel_l2_persistence"],
        "config": "8 x 512^2, F~U[0.02,0.06], k~U[0.05,0.07]; 4096 steps, re-anchor every 256, "
                  "fallback tolerance 1e-2",
        "kernel": "conv3x3_fwd_res (tcgen05)"}


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    import numpy as np

    from formura_gb300 import inits
    from oracle import oracle

    oracle.build(reference=False)
    U0, V0 = inits.gray_scott_3d(N, N, N, seed=1)
    sample_steps = 4
    for _ in range(args.warmup):
        oracle.gs3d_f64(U0, V0, sample_steps, **GS, fast=True)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        oracle.gs3d_f64(U0, V0, sample_steps, **GS, fast=True)
        times.append(time.perf_counter() - t)
    tot = sum(times)
    val = N ** 3 * sample_steps * len(times) / tot / 1e9
    cores = oracle.num_threads(fast=True)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(val, 4),
        "unit": "GLUP/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(tot / len(times) * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": "gray_scott_3d 256^3 FP64 (pearson-3d.fmr form)",
                   "step": "%d time steps of the CPU restatement per bench step" % sample_steps},
        "cpu_baseline": {"value": round(val, 4), "unit": "GLUP/s", "cores": cores, "kind": "port",
                         "sample": "256^3 x %d steps per bench step; oracle/fmr_oracle.c -O3 "
                                   "OpenMP (the reference compiler cannot run here)" % sample_steps},
        "e2e": {"value": round(val, 4), "unit": "GLUP/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def aggregate_replicas(dev_s: float, e2e_s: float, lups_per_rank: float, ws: int, device="cuda"):
    """Whole-job throughput of N independent replicas: the slowest rank's
    device and end-to-end times (MAX over ranks), all ranks' lattice updates.
    Returns (value GLUP/s, e2e GLUP/s, dev_s, e2e_s) on every rank."""
    import torch

    times = torch.tensor([dev_s, e2e_s], dtype=torch.float64, device=device)
    if ws > 1:
        torch.distributed.all_reduce(times, op=torch.distributed.ReduceOp.MAX)
    dev_s, e2e_s = times.tolist()
    lups = lups_per_rank * ws
    return lups / dev_s / 1e9, lups / e2e_s / 1e9, dev_s, e2e_s


def run_engine(args):
    import numpy as np
    import torch

    ws, rank, local = dist_info()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    from formura_gb300 import inits, kernels
    from formura_gb300.runtime import load_program

    prog = load_program(WORKLOAD)
    M = prog.steps_per_forward
    prog.init()
    U0, V0 = inits.gray_scott_3d(N, N, N, seed=1 + rank)
    prog.state["U"][...] = U0
    prog.state["V"][...] = V0
    sms = torch.cuda.get_device_properties(local).multi_processor_count

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    # ---- device-resident leg -------------------------------------------------
    prog.upload()
    for _ in range(args.warmup):
        prog.advance(1)
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record()
        for _ in range(args.steps):
            prog.advance(1)
        ev1.record()
        ev1.synchronize()
    dev_s = ev0.elapsed_time(ev1) / 1e3
    barrier()

    # ---- end-to-end leg through Formura_Forward on host globals ---------------
    prog.download()
    prog.forward()  # warm the host-copy path (registration, first copies)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk_e2e:
        t0 = time.perf_counter()
        e0.record()  # the legacy default stream, the one Formura_Forward uses
        for _ in range(args.steps):
            prog.forward()
        e1.record()
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t0
    e2e_dev_s = e0.elapsed_time(e1) / 1e3
    barrier()
    # the host<->device copies of that path on their own (untimed above)
    copies = {}
    for name, fn in (("h2d", prog.upload), ("d2h", prog.download)):
        fn()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        copies[name + "_gbs"] = round(3 * 2 * 8 * N ** 3 / (time.perf_counter() - t) / 1e9, 1)
    copies["host_globals_pinned"] = "%d of 2" % prog.host_pinned()
    # where the end-to-end time goes: the same loop's span on the device, and the
    # SM clock during it (the FP64-bound kernel's time scales with the clock)
    copies["device_span_s"] = round(e2e_dev_s, 4)
    copies["wall_s"] = round(e2e_s, 4)
    copies["clocks"] = clk_e2e.summary()

    # the state after one Formura_Forward from the seeded start (parity, FP32 score)
    U_final = V_final = None
    if rank == 0 and not (args.no_variants and args.no_parity):
        prog.state["U"][...] = U0
        prog.state["V"][...] = V0
        prog.forward()
        U_final = prog.state["U"].copy()
        V_final = prog.state["V"].copy()

    value, e2e, dev_s, e2e_s = aggregate_replicas(dev_s, e2e_s, float(N ** 3) * M * args.steps, ws)
    if rank != 0:
        if ws > 1:
            torch.distributed.destroy_process_group()
        return

    # ---- roofline -----------------------------------------------------------
    launches = M * args.steps
    per_launch = dev_s / launches
    fp64_peak = measure_fma_peak(torch, kernels, True, sms)
    fp32_peak = measure_fma_peak(torch, kernels, False, sms)
    achieved_tf = FLOPS_PER_LUP * N ** 3 / per_launch / 1e12
    peaks = load_peaks()
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    achieved_gbs = BYTES_PER_LUP * N ** 3 / per_launch / 1e9
    traffic = read_profile_traffic()
    clocks = clk.summary()
    cpu = cpu_baseline() if not args.no_cpu else None
    parity = None
    if not args.no_parity:
        parity = run_parity(torch, U_final, V_final, U0, V0)
    variants = None
    if not args.no_variants:
        variants = run_variants(torch, prog, U_final, U0, V0, peaks)

    line = {
        "metric": METRIC,
        "value": round(value, 4), "unit": "GLUP/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dev_s / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded: U=1,V=0 + 8 cubes of side 16 at U=0.5,V=0.25 +-1%)",
        "config": {"workload": "gray_scott_3d: 256^3 FP64 periodic Gray-Scott, pearson-3d.fmr form "
                               "(F=0.04 k=0.06 Du=2e-5 Dv=1e-5 dx=0.01 dt=0.5)",
                   "grid": [N, N, N], "steps_per_bench_step": M,
                   "parallelism": "replicas" if ws > 1 else "1 GPU",
                   "l2": "state 268 MB > 129 MB L2; no flush"},
        "roofline": {"bound": "fp64", "achieved": round(achieved_tf, 4), "peak": round(fp64_peak, 4),
                     "unit": "TFLOP/s", "frac": round(achieved_tf / fp64_peak, 4),
                     "traffic": traffic, "peak_source": "measured in this run (FP64 FMA probe)",
                     "flops_per_lup": FLOPS_PER_LUP,
                     "hbm": {"achieved": round(achieved_gbs, 1), "peak": hbm_peak, "unit": "GB/s",
                             "frac": round(achieved_gbs / hbm_peak, 4),
                             "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback"},
                     "fp32_peak_tflops": round(fp32_peak, 2),
                     "fp64_pipe_ops_per_lup": 26,
                     "integer_pipe_ops_per_lup": "13 divisions by dx (12 + one y-face flux "
                                                 "recomputed) + 5 multiplications by constants, "
                                                 "correctly rounded on the integer pipes",
                     "kernel": "gs3d_f64_row", "ms_per_launch": round(per_launch * 1e3, 4)},
        "e2e": dict({"value": round(e2e, 4), "unit": "GLUP/s",
                     "h2d_bytes_per_step": 2 * 8 * N ** 3, "d2h_bytes_per_step": 2 * 8 * N ** 3},
                    **copies),
        "gpu_launches": 2 * launches,
        "clocks": clocks,
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if parity is not None:
        line["parity"] = parity
    if variants is not None:
        line["variants"] = variants
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_profile_case(args):
    """A few launches of one kernel on a small resident case, for ncu captures
    (nothing is timed or printed as a bench value)."""
    import torch

    from formura_gb300 import inits, kernels

    torch.cuda.set_device(0)
    dev = torch.device("cuda:0")
    from formura_gb300 import _lib

    for kv in args.tune or []:
        k, v = kv.split("=")
        _lib.check(_lib.lib().fm_tune_set(k.encode(), int(v)), "fm_tune_set")
    n = args.profile_n
    if args.profile in ("gs3d_f64", "gs3d_f32k"):
        U0, V0 = inits.gray_scott_3d(n, n, n, seed=1)
        if args.profile == "gs3d_f64":
            U, V = torch.from_numpy(U0).to(dev), torch.from_numpy(V0).to(dev)
            kernels.gs3d_f64_forward(U, V, torch.empty_like(U), torch.empty_like(V),
                                     kernels.gs_params(**GS), args.profile_steps)
        else:
            U = torch.from_numpy(U0.astype("float32")).to(dev)
            V = torch.from_numpy(V0.astype("float32")).to(dev)
            cU, cV = torch.zeros_like(U), torch.zeros_like(V)
            w = torch.empty(4 * U.numel(), dtype=torch.float32, device=dev)
            kernels.gs3d_f32k_forward(U, V, cU, cV, w, kernels.gs_params(**GS),
                                      args.profile_steps, args.profile_tb)
    elif args.profile == "gs3d_f32k_tb":
        U0, V0 = inits.gray_scott_3d(n, n, n, seed=1)
        U = torch.from_numpy(U0.astype("float32")).to(dev)
        V = torch.from_numpy(V0.astype("float32")).to(dev)
        cU, cV = torch.zeros_like(U), torch.zeros_like(V)
        w = torch.empty(4 * U.numel(), dtype=torch.float32, device=dev)
        kernels.gs3d_f32k_tb_forward(U, V, cU, cV, w, kernels.gs_params(**GS),
                                     args.profile_steps, args.profile_tb)
    elif args.profile == "ensemble":
        sizes, F, k = inits.gs2d_ensemble(512, seed=1)
        tile = 1 if args.profile_tile == 0 else args.profile_tile  # 1: wavefront strips
        e = kernels.Ensemble(sizes, F, k, tile=tile, tb=max(args.profile_tb, 1))
        Ue, Ve = inits.gs2d_ensemble_state(sizes, seed=1)
        Ue, Ve = torch.from_numpy(Ue).to(dev), torch.from_numpy(Ve).to(dev)
        e.forward(Ue, Ve, torch.empty_like(Ue), torch.empty_like(Ve), args.profile_steps,
                  use_graph=False)
        e.status()
        e.close()
    elif args.profile in ("mhd", "mhd_f64"):
        dt = torch.float64 if args.profile == "mhd_f64" else torch.float32
        f0 = inits.mhd_3d(n, seed=1)
        t = [torch.from_numpy(x).to(dt).to(dev) for x in f0]
        kernels.mhd_forward(t, torch.empty(18 * n ** 3, dtype=dt, device=dev), args.profile_steps)
    elif args.profile == "diff2d":
        d0 = inits.diffusion_2d(n, n, seed=1)
        d = torch.from_numpy(d0).to(dev)
        kernels.diff2d_f64_forward(d, torch.empty_like(d), 0.4, args.profile_steps)
    elif args.profile == "fmr_gs3d":
        # examples/gray-scott-3d.fmr through the front end: `profile_steps` steps at n^3
        from formura_gb300.fmr import load_program
        from formura_gb300.runtime import load_program as load_lib

        p = load_program(ROOT / "examples" / "gray-scott-3d.fmr", intra_node_shape=[n, n, n],
                         monitor_interval=args.profile_steps)
        prog = load_lib(p)
        prog.init()
        U0, V0 = inits.gray_scott_3d(n, n, n, seed=1)
        prog.state["U"][...] = U0
        prog.state["V"][...] = V0
        prog.upload()
        prog.advance(1)
        prog.download()
        prog.finalize()
    elif args.profile in ("fmr_gs3d_float_tb", "fmr_heat_float_tb", "fmr_heat_float"):
        # examples/gray-scott-3d-float.fmr or heat-3d-float.fmr through the front end,
        # blocked kernel (temporal_blocking_interval 4): `profile_steps` steps at n^3
        import numpy as np

        from formura_gb300.fmr import load_program
        from formura_gb300.runtime import load_program as load_lib

        src = "gray-scott-3d-float" if args.profile == "fmr_gs3d_float_tb" else "heat-3d-float"
        tbk = -1 if args.profile == "fmr_heat_float" else 1  # one step per launch, or blocked
        p = load_program(ROOT / "examples" / (src + ".fmr"), intra_node_shape=[n, n, n],
                         monitor_interval=args.profile_steps, tb_kernel=tbk,
                         name="fmr_%s_prof%d" % (src.replace("-", "_"), tbk + 1))
        prog = load_lib(p)
        prog.init()
        U0, V0 = inits.gray_scott_3d(n, n, n, seed=1)
        for name, a in (("U", U0), ("V", V0), ("u", U0)):
            if name in prog.state:
                prog.state[name][...] = a.astype(np.float32)
        prog.upload()
        prog.advance(1)
        prog.download()
        prog.finalize()
    elif args.profile == "surrogate":
        # `profile_steps` network jumps (and one training step) on `profile_batch` instances of n x n
        from formura_gb300.surrogate import Surrogate

        net = Surrogate(seed=0)
        net.load_npz(ROOT / "formura_gb300" / "weights" / "gs2d_surrogate.npz")
        sizes, F, k = inits.gs2d_ensemble(args.profile_batch, seed=1, sizes=(n,))
        U0, V0 = inits.gs2d_ensemble_state(sizes, seed=1)
        U = torch.from_numpy(U0).to(dev).view(args.profile_batch, n, n)
        V = torch.from_numpy(V0).to(dev).view(args.profile_batch, n, n)
        Ft = torch.tensor(F, dtype=torch.float32, device=dev)
        Kt = torch.tensor(k, dtype=torch.float32, device=dev)
        U1, V1 = U.clone(), V.clone()
        for _ in range(args.profile_steps):
            net.predict(U, V, Ft, Kt)
        if args.profile_train:
            net.train_step(U1, V1, Ft, Kt, U, V, lr=1e-6)
        net.check_errors()
    torch.cuda.synchronize()
    print("profile case %s n=%d steps=%d done" % (args.profile, n, args.profile_steps))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the in-run comparison with the oracle")
    ap.add_argument("--no-variants", action="store_true",
                    help="skip the other forms (FP32 TB, ensemble, diffusion, MHD)")
    ap.add_argument("--profile", choices=["gs3d_f64", "gs3d_f32k", "gs3d_f32k_tb", "ensemble",
                                          "mhd", "mhd_f64", "diff2d", "surrogate", "fmr_gs3d",
                                          "fmr_gs3d_float_tb", "fmr_heat_float_tb",
                                          "fmr_heat_float"],
                    default=None,
                    help="run a small case of one kernel for an ncu capture, then exit")
    ap.add_argument("--profile-n", type=int, default=256)
    ap.add_argument("--profile-steps", type=int, default=4)
    ap.add_argument("--profile-tb", type=int, default=0)
    ap.add_argument("--profile-tile", type=int, default=0,
                    help="ensemble case: 1 wavefront strips (default), 32 or 64 smem tiles")
    ap.add_argument("--profile-batch", type=int, default=8, help="surrogate case: instances")
    ap.add_argument("--profile-train", action="store_true",
                    help="surrogate case: also run one training step")
    ap.add_argument("--tune", action="append", help="KEY=VALUE tuning knob (fm_tune_set)")
    args = ap.parse_args()
    if args.profile:
        run_profile_case(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
