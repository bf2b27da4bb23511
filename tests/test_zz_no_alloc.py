"""fm_diff2d_f64_forward_noalloc — the entry point that allocates nothing.

It serves callers that cannot call cudaMalloc (a host application that
reserved its device-memory budget up front and lends the library only its own
arrays, or a latency-critical loop that must not hit cudaMalloc's implicit
device synchronization).  Its scratch is a static device array inside the
library.  This file is collected last so that a run stopping at the first
failure has already run every other test; it also passes alone in a fresh
process.  Parity bar: bit-exact against fm_diff2d_f64_forward, the bar of the
other diffusion tests.
"""
import ctypes

import numpy as np
import pytest
import torch

from formura_gb300 import _lib, inits
from tests.bits import same_bits

pytestmark = pytest.mark.gpu


def _existing(d0, coef, steps):
    lib = _lib.lib()
    d = torch.from_numpy(d0).cuda()
    w = torch.empty_like(d)
    st = lib.fm_diff2d_f64_forward(d.shape[0], d.shape[1], ctypes.c_void_p(d.data_ptr()),
                                   ctypes.c_void_p(w.data_ptr()), coef, steps,
                                   ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(st, "fm_diff2d_f64_forward")
    torch.cuda.synchronize()
    return d.cpu().numpy()


def _noalloc(d, coef, steps):
    lib = _lib.lib()
    return lib.fm_diff2d_f64_forward_noalloc(
        d.shape[0], d.shape[1], ctypes.c_void_p(d.data_ptr()), coef, steps,
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


def test_noalloc_matches_existing_entry_point_on_two_calls_in_a_row(cuda_device):
    cases = [((256, 256), 0.1, 37, 3), ((96, 128), 0.05, 20, 4)]
    # both state arrays are allocated before either call; the entry point gets
    # nothing else
    states = [torch.from_numpy(inits.diffusion_2d(*shape, seed=seed)).cuda()
              for shape, _, _, seed in cases]
    torch.cuda.synchronize()
    for d, (shape, coef, steps, seed) in zip(states, cases):
        st = _noalloc(d, coef, steps)
        _lib.check(st, "fm_diff2d_f64_forward_noalloc")
        torch.cuda.synchronize()
        want = _existing(inits.diffusion_2d(*shape, seed=seed), coef, steps)
        assert same_bits(d.cpu().numpy(), want)


def test_noalloc_rejects_sizes_beyond_the_static_scratch(cuda_device):
    lib = _lib.lib()
    nx, ny = 2048, 1024  # 2^21 cells > FM_DIFF2D_NOALLOC_MAX_CELLS = 2^20
    st = lib.fm_diff2d_f64_forward_noalloc(nx, ny, ctypes.c_void_p(0x1000), 0.1, 1, None)
    assert st == 1
    assert b"exceeds" in lib.fm_last_error()


def test_noalloc_result_is_final_on_return_for_another_stream(cuda_device):
    """An odd number of passes leaves the result in the static scratch, and the
    copy back into dens is part of the call: when the call returns, another
    stream may read dens, and a second call on another stream may reuse the
    scratch, with no device-wide synchronization in between."""
    lib = _lib.lib()
    coef, steps = 0.1, 41  # 11 passes of 4 steps: odd
    d0a = inits.diffusion_2d(256, 256, seed=7)
    d0b = inits.diffusion_2d(128, 256, seed=8)
    da, db = torch.from_numpy(d0a).cuda(), torch.from_numpy(d0b).cuda()
    torch.cuda.synchronize()
    sa, sb = torch.cuda.Stream(), torch.cuda.Stream()
    st = lib.fm_diff2d_f64_forward_noalloc(256, 256, ctypes.c_void_p(da.data_ptr()), coef, steps,
                                           ctypes.c_void_p(sa.cuda_stream))
    _lib.check(st, "fm_diff2d_f64_forward_noalloc")
    with torch.cuda.stream(sb):
        seen = da.clone()  # read on stream B right after the call returned
        st = lib.fm_diff2d_f64_forward_noalloc(128, 256, ctypes.c_void_p(db.data_ptr()), coef,
                                               steps, ctypes.c_void_p(sb.cuda_stream))
        _lib.check(st, "fm_diff2d_f64_forward_noalloc")
        got_b = db.clone()
    sb.synchronize()
    assert same_bits(seen.cpu().numpy(), _existing(d0a, coef, steps))
    assert same_bits(got_b.cpu().numpy(), _existing(d0b, coef, steps))
