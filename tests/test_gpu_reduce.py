"""Conserved totals: deterministic, and equal to an exact sum within rounding."""
import math

import numpy as np
import pytest
import torch

from formura_gb300 import kernels

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 255, 4096, 1_000_003, 256 ** 3])
def test_total_f64(cuda_device, n):
    rng = np.random.default_rng(n)
    a = rng.random(n)
    t = torch.from_numpy(a).to(cuda_device)
    s1 = kernels.total(t).item()
    s2 = kernels.total(t).item()
    assert s1 == s2  # same bits every call
    exact = math.fsum(a)
    assert abs(s1 - exact) <= 1e-13 * max(1.0, abs(exact))


def test_total_f32_and_nan(cuda_device):
    a = np.linspace(0, 1, 100_000, dtype=np.float32)
    t = torch.from_numpy(a).to(cuda_device)
    assert abs(kernels.total(t).item() - math.fsum(a.astype(np.float64))) < 1e-9
    b = torch.ones(10_000, dtype=torch.float64, device=cuda_device)
    b[1234] = float("nan")
    assert math.isnan(kernels.total(b).item())
