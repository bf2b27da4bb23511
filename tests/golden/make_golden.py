"""Generates the golden vectors under tests/golden/.

pearson_ref.json — outputs of the REFERENCE's own generated C,
    examples-generated/pearson.c (2D Gray-Scott 600x600, periodic), compiled
    from the reference tree by oracle/Makefile into oracle/_ref/.  Seeded
    initial state (formura_gb300.inits.gray_scott_2d_square), then n calls of
    its Formura_Forward (20 steps each).  Stored: SHA-256 of the final U and V
    bytes, time_step, and sampled cells as hex floats.  These pin the oracle.

oracle_regression.json — the oracle's own outputs for the other forms at
    small sizes (3D Gray-Scott FP64, FP32+Kahan, 2D diffusion, 2D Gray-Scott
    FP32).  The reference ships no generated code for these forms, so these are
    regression vectors of the restatement, not reference outputs.

Usage (needs the reference tree, read-only):  python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from formura_gb300 import inits  # noqa: E402
from oracle import oracle  # noqa: E402

HERE = Path(__file__).resolve().parent


def sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def samples(a: np.ndarray, n: int = 24, seed: int = 3):
    idx = (inits.splitmix64(seed, n) % np.uint64(a.size)).astype(np.int64)
    flat = a.reshape(-1)
    return [[int(i), float(flat[i]).hex()] for i in idx]


PEARSON_CASES = [dict(seed=7, n_forward=3), dict(seed=11, n_forward=10)]


def pearson_ref():
    ref = oracle.ReferencePearson()
    out = []
    for case in PEARSON_CASES:
        U0, V0 = inits.gray_scott_2d_square(600, 600, seed=case["seed"], frac=0.05)
        U, V, ts = ref.run(U0, V0, case["n_forward"])
        out.append(dict(case, init_sha256=sha(U0, V0), time_step=ts, sha256=sha(U, V),
                        U_samples=samples(U), V_samples=samples(V, seed=4)))
    return dict(source="examples-generated/pearson.c (reference generated C)",
                constants=oracle.ReferencePearson.CONSTANTS, n=600, cases=out)


GS3D = dict(F=0.04, k=0.06, Du=2e-5, Dv=1e-5, dt=0.5, dx=0.01)


def oracle_regression():
    res = {}
    U0, V0 = inits.gray_scott_3d(32, 32, 32, seed=5, ncubes=2, side=8)
    U, V = oracle.gs3d_f64(U0, V0, 50, **GS3D)
    res["gs3d_f64_32_50"] = dict(init_sha256=sha(U0, V0), sha256=sha(U, V), U_samples=samples(U))
    Z = np.zeros_like(U0, dtype=np.float32)
    out = oracle.gs3d_f32_kahan(U0.astype(np.float32), V0.astype(np.float32), Z, Z, 50, **GS3D)
    res["gs3d_f32k_32_50"] = dict(sha256=sha(*out), U_samples=samples(out[0]))
    d0 = inits.diffusion_2d(64, 64, seed=9)
    d = oracle.diff2d_f64(d0, 100, 0.4, 1.0)
    res["diff2d_64_100"] = dict(init_sha256=sha(d0), sha256=sha(d), samples=samples(d))
    u0, v0 = inits.gray_scott_2d_square(64, 64, seed=13)
    u, v = oracle.gs2d_f32(u0, v0, 100, 0.04, 0.06, 2e-5, 1e-5, 1.0, 0.01)
    res["gs2d_f32_64_100"] = dict(init_sha256=sha(u0, v0), sha256=sha(u, v), samples=samples(u))
    return dict(source="oracle/fmr_oracle.c (regression vectors, not reference outputs)", cases=res)


def main():
    oracle.build(reference=True)
    (HERE / "pearson_ref.json").write_text(json.dumps(pearson_ref(), indent=1) + "\n")
    (HERE / "oracle_regression.json").write_text(json.dumps(oracle_regression(), indent=1) + "\n")
    print("wrote", HERE / "pearson_ref.json", HERE / "oracle_regression.json")


if __name__ == "__main__":
    main()
