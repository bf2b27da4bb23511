"""The oracle against the reference's own generated C, and its regression vectors.

examples-generated/pearson.c is the only generated C the reference ships for a
Jacobi stencil (the reference's tests hold no numerical golden vectors).  Its outputs, recorded in tests/golden/pearson_ref.json by
tests/golden/make_golden.py, pin the oracle's 2D Gray-Scott step bit for bit.
"""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from formura_gb300 import inits
from oracle import oracle

GOLDEN = Path(__file__).resolve().parent / "golden"


def sha(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_oracle_matches_reference_pearson_golden():
    g = json.loads((GOLDEN / "pearson_ref.json").read_text())
    c = g["constants"]
    for case in g["cases"]:
        U0, V0 = inits.gray_scott_2d_square(g["n"], g["n"], seed=case["seed"], frac=0.05)
        assert sha(U0, V0) == case["init_sha256"]
        steps = case["n_forward"] * 20
        assert steps == case["time_step"]
        U, V = oracle.gs2d_f64(U0, V0, steps, **c)
        for i, hx in case["U_samples"]:
            assert U.reshape(-1)[i] == float.fromhex(hx)
        assert sha(U, V) == case["sha256"], "oracle differs from examples-generated/pearson.c"


@pytest.mark.skipif(not oracle.reference_available(), reason="reference tree not present")
def test_oracle_matches_reference_pearson_live():
    ref = oracle.ReferencePearson()
    U0, V0 = inits.gray_scott_2d_square(600, 600, seed=123, frac=0.1)
    U, V, ts = ref.run(U0, V0, 2)
    assert ts == 40
    Uo, Vo = oracle.gs2d_f64(U0, V0, 40, **oracle.ReferencePearson.CONSTANTS)
    assert np.array_equal(U, Uo) and np.array_equal(V, Vo)


def test_oracle_regression_vectors():
    g = json.loads((GOLDEN / "oracle_regression.json").read_text())["cases"]
    GS3D = dict(F=0.04, k=0.06, Du=2e-5, Dv=1e-5, dt=0.5, dx=0.01)
    U0, V0 = inits.gray_scott_3d(32, 32, 32, seed=5, ncubes=2, side=8)
    assert sha(U0, V0) == g["gs3d_f64_32_50"]["init_sha256"]
    assert sha(*oracle.gs3d_f64(U0, V0, 50, **GS3D)) == g["gs3d_f64_32_50"]["sha256"]
    Z = np.zeros_like(U0, dtype=np.float32)
    out = oracle.gs3d_f32_kahan(U0.astype(np.float32), V0.astype(np.float32), Z, Z, 50, **GS3D)
    assert sha(*out) == g["gs3d_f32k_32_50"]["sha256"]
    d0 = inits.diffusion_2d(64, 64, seed=9)
    assert sha(oracle.diff2d_f64(d0, 100, 0.4, 1.0)) == g["diff2d_64_100"]["sha256"]
    u0, v0 = inits.gray_scott_2d_square(64, 64, seed=13)
    assert sha(*oracle.gs2d_f32(u0, v0, 100, 0.04, 0.06, 2e-5, 1e-5, 1.0, 0.01)) == \
        g["gs2d_f32_64_100"]["sha256"]


def test_oracle_fast_build_matches_parity_build():
    # The speed build (timed CPU baseline) computes the same function.
    U0, V0 = inits.gray_scott_3d(16, 16, 32, seed=2, ncubes=1, side=8)
    a = oracle.gs3d_f64(U0, V0, 10, 0.04, 0.06, 2e-5, 1e-5, 0.5, 0.01)
    b = oracle.gs3d_f64(U0, V0, 10, 0.04, 0.06, 2e-5, 1e-5, 0.5, 0.01, fast=True)
    np.testing.assert_allclose(a[0], b[0], rtol=1e-13, atol=0)


def test_uniform_state_is_a_fixed_point():
    # U=1, V=0 is an exact steady state of the Gray-Scott DAG.
    U = np.ones((8, 16, 32))
    V = np.zeros((8, 16, 32))
    U1, V1 = oracle.gs3d_f64(U, V, 5, 0.04, 0.06, 2e-5, 1e-5, 0.5, 0.01)
    assert np.array_equal(U1, U) and np.array_equal(V1, V)


def test_diffusion_conserves_mass():
    d0 = inits.diffusion_2d(32, 64, seed=4)
    d = oracle.diff2d_f64(d0, 200, 0.4, 1.0)
    assert abs(d.sum() - d0.sum()) < 1e-10 * d0.sum()
    assert d.std() < d0.std()


def test_periodic_shift_commutes_with_step():
    U0, V0 = inits.gray_scott_3d(8, 16, 32, seed=6, ncubes=1, side=4)
    a = oracle.gs3d_f64(U0, V0, 6, 0.04, 0.06, 2e-5, 1e-5, 0.5, 0.01)
    sh = (3, 5, 7)
    b = oracle.gs3d_f64(np.roll(U0, sh, (0, 1, 2)), np.roll(V0, sh, (0, 1, 2)), 6,
                        0.04, 0.06, 2e-5, 1e-5, 0.5, 0.01)
    assert np.array_equal(np.roll(a[0], sh, (0, 1, 2)), b[0])


def test_kahan_f32_tracks_f64():
    U0, V0 = inits.gray_scott_3d(16, 16, 32, seed=3, ncubes=1, side=8)
    U, V = oracle.gs3d_f64(U0, V0, 200, 0.04, 0.06, 2e-5, 1e-5, 0.5, 0.01)
    Z = np.zeros(U0.shape, np.float32)
    Uf, Vf, _, _ = oracle.gs3d_f32_kahan(U0.astype(np.float32), V0.astype(np.float32), Z, Z,
                                         200, 0.04, 0.06, 2e-5, 1e-5, 0.5, 0.01)
    err = np.linalg.norm(Uf - U) / np.linalg.norm(U)
    assert err < 1e-5
