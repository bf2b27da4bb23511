"""The exact rewrites behind the packed-pair FP32 blocked kernel
(gs3d_f32k_tbp in formura_gb300/csrc/fm_gs3d_f32k_tb.cu), checked on the host.

The kernel advances a cell's (u, v) as one binary32 pair, so it writes the
scalar fast-form step (gs3d_f32k_tb's cell_step, oracle.gs3d_f32k_fast) as
operations that are the same for both halves:
  inner = fma((F, -Fk), (1 - u, v), (-uvv, uvv))
with 1 - u and u*v*v scalar, and the negations (of uvv, of Fk, and of the
incoming compensation in the Kahan fma) as sign-bit flips.  Each pair
operation rounds like its scalar counterpart (measured on the GPU), so the
form is exact iff it is exact in scalar IEEE binary32.  This test
evaluates both forms in C (fmaf is the correctly rounded fused operation,
-ffp-contract=off keeps every other operation separately rounded) over three
chained steps on random and edge-case operands and requires identical bits,
signed zeros included.  (An earlier form that carried the compensation
negated, y - (t - u), differed from -((t - u) - y) in the sign of zero
compensations; this test found it.)
"""
import ctypes
import shutil
import subprocess

import numpy as np
import pytest

SRC = r"""
#include <math.h>
#include <stdint.h>
#include <string.h>
static uint32_t bits(float x) { uint32_t b; memcpy(&b, &x, 4); return b; }
/* One step of a cell, scalar fast form (cell_step of the scalar kernel). */
static void scalar_step(float u, float v, float lu, float lv, float cu_in, float cv_in,
                        float F, float Fk, float cu, float cv, float dt, float *o) {
  const float uvv = (u * v) * v;
  const float dU = fmaf(cu, lu, fmaf(F, 1.0f - u, -uvv));
  const float dV = fmaf(cv, lv, fmaf(-Fk, v, uvv));
  const float yu = fmaf(dt, dU, -cu_in), tu = u + yu;
  const float yv = fmaf(dt, dV, -cv_in), tv = v + yv;
  o[0] = tu; o[1] = tv; o[2] = (tu - u) - yu; o[3] = (tv - v) - yv;
}
/* -x by flipping the sign bit, as the kernel does */
static float neg(float x) { uint32_t b; memcpy(&b, &x, 4); b ^= 0x80000000u; memcpy(&x, &b, 4); return x; }
/* The same step as the packed kernel writes it, one half at a time: the pair
   constants (F, -Fk), the pair (1 - u, v), the pair (-uvv, uvv). */
static void pair_step(float u, float v, float lu, float lv, float cu_in, float cv_in,
                      float F, float Fk, float cu, float cv, float dt, float *o) {
  const float uvv = (u * v) * v;
  const float nuvv_x = neg(uvv), nuvv_y = uvv;
  const float w_x = 1.0f - u, w_y = v;
  const float kF_x = F, kF_y = neg(Fk);
  const float in_x = fmaf(kF_x, w_x, nuvv_x), in_y = fmaf(kF_y, w_y, nuvv_y);
  const float d_x = fmaf(cu, lu, in_x), d_y = fmaf(cv, lv, in_y);
  const float y_x = fmaf(dt, d_x, neg(cu_in)), y_y = fmaf(dt, d_y, neg(cv_in));
  const float t_x = u + y_x, t_y = v + y_y;
  o[0] = t_x; o[1] = t_y; o[2] = (t_x - u) - y_x; o[3] = (t_y - v) - y_y;
}
/* in[i*10 + 0..9] = u, v, lu, lv, cu_in, cv_in, F, Fk, Du, Dv.  Three chained
   steps (each step's state and compensation feed the next, as the levels of
   a blocked pass do); every output of every step must have identical bits. */
int check(const float *in, int n, float dt, int *first_bad) {
  int bad = 0;
  for (int i = 0; i < n; ++i) {
    const float *p = in + 10 * i;
    float a[4] = {p[0], p[1], p[4], p[5]}, b[4] = {p[0], p[1], p[4], p[5]};
    int diff = 0;
    for (int k = 0; k < 3; ++k) {
      float oa[4], ob[4];
      scalar_step(a[0], a[1], p[2], p[3], a[2], a[3], p[6], p[7], p[8], p[9], dt, oa);
      pair_step(b[0], b[1], p[2], p[3], b[2], b[3], p[6], p[7], p[8], p[9], dt, ob);
      for (int q = 0; q < 4; ++q) {
        diff |= bits(oa[q]) != bits(ob[q]);
        a[q] = oa[q];
        b[q] = ob[q];
      }
    }
    if (diff) {
      if (bad == 0) *first_bad = i;
      ++bad;
    }
  }
  return bad;
}
/* a planted mistake: u*v*v rounded once (as a fused pair multiply-add would
   round it), so the comparison must find differences */
int check_planted(const float *in, int n, float dt) {
  int bad = 0;
  for (int i = 0; i < n; ++i) {
    const float *p = in + 10 * i;
    const float u = p[0], v = p[1], lu = p[2], F = p[6], cu = p[8], cu_in = p[4];
    const float uvv = (u * v) * v;
    const float dU = fmaf(cu, lu, fmaf(F, 1.0f - u, -uvv));
    const float tu = u + fmaf(dt, dU, -cu_in);
    const float uvv1 = (float)((double)u * (double)v * (double)v);
    const float dU1 = fmaf(cu, lu, fmaf(F, fmaf(-1.0f, u, 1.0f), -uvv1));
    const float tu1 = u + fmaf(dt, dU1, cu_in * -1.0f);
    bad += bits(tu) != bits(tu1);
  }
  return bad;
}
"""


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("packed")
    (d / "p.c").write_text(SRC)
    so = d / "p.so"
    subprocess.check_call([cc, "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(so),
                           str(d / "p.c"), "-lm"])
    lib = ctypes.CDLL(str(so))
    lib.check.restype = ctypes.c_int
    lib.check.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_float,
                          ctypes.POINTER(ctypes.c_int)]
    lib.check_planted.restype = ctypes.c_int
    lib.check_planted.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_float]
    return lib


def _run(lib, x, dt):
    x = np.ascontiguousarray(x, dtype=np.float32)
    first = ctypes.c_int(-1)
    bad = lib.check(x.ctypes.data, x.shape[0], float(dt), ctypes.byref(first))
    return bad, first.value


def test_rewrite_exact_on_gray_scott_operands(checker):
    """Operands of the magnitudes a Gray-Scott run produces, and the bench's
    constants: u, v in [0, 1], Laplacians of either sign, small compensations."""
    rng = np.random.default_rng(0)
    n = 400_000
    x = np.empty((n, 10), np.float32)
    x[:, 0] = rng.uniform(0, 1, n)
    x[:, 1] = rng.uniform(0, 1, n) * rng.choice([1, 1e-3, 1e-8, 1e-30], n)
    x[:, 2] = rng.standard_normal(n) * rng.choice([1e-1, 1e-4, 1e-9], n)
    x[:, 3] = rng.standard_normal(n) * rng.choice([1e-1, 1e-4, 1e-9], n)
    x[:, 4] = rng.standard_normal(n) * 1e-8
    x[:, 5] = rng.standard_normal(n) * 1e-9
    x[:, 6] = np.float32(0.04)
    x[:, 7] = np.float32(0.04) + np.float32(0.06)
    x[:, 8] = np.float32(2e-5 / (0.01 * 0.01))
    x[:, 9] = np.float32(1e-5 / (0.01 * 0.01))
    assert _run(checker, x, 0.5) == (0, -1)


def test_rewrite_exact_on_random_bit_patterns(checker):
    """Arbitrary finite operands (random sign, exponent and significand,
    subnormals and signed zeros included) and random constants."""
    rng = np.random.default_rng(1)
    n = 400_000
    b = rng.integers(0, 2 ** 32, size=(n, 10), dtype=np.uint64).astype(np.uint32)
    # exponents spread over a range where products neither overflow nor all vanish
    e = rng.integers(60, 190, size=(n, 10)).astype(np.uint32)
    b = (b & np.uint32(0x807FFFFF)) | (e << np.uint32(23))
    x = b.view(np.float32).copy()
    zero = rng.random((n, 10)) < 0.03
    x[zero] = np.where(rng.random(int(zero.sum())) < 0.5, 0.0, -0.0)
    sub = rng.random((n, 10)) < 0.02
    x[sub] = (rng.integers(1, 2 ** 23, int(sub.sum())).astype(np.uint32)).view(np.float32)
    for dt in (0.5, 1.0, 0.1):
        assert _run(checker, x, dt) == (0, -1), dt


def test_check_finds_a_planted_rounding_difference(checker):
    """The comparison is sensitive: the same step with u*v*v rounded once
    instead of twice (the effect a fused pair multiply-add would have) gives
    different bits on ordinary Gray-Scott operands."""
    rng = np.random.default_rng(2)
    n = 100_000
    x = np.zeros((n, 10), np.float32)
    x[:, 0] = rng.uniform(0, 1, n)
    x[:, 1] = rng.uniform(0, 1, n)
    x[:, 2] = rng.standard_normal(n) * 1e-2
    x[:, 6] = np.float32(0.04)
    x[:, 8] = np.float32(0.2)
    bad = checker.check_planted(np.ascontiguousarray(x).ctypes.data, n, 0.5)
    assert bad > 0
