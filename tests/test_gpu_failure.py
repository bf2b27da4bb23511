"""Failure detection, exercised without faulting, trapping or hanging the GPU.

The reference has none (its generated code aborts through MPI on an error);
this engine reports two failures as status codes.

* A grid-barrier wait of a persistent kernel that runs out.  The tuning knob
  "sync.spin_limit" lowers the number of polls a waiting block makes before it
  gives up; at 1 poll the waits run out during the run, every block returns,
  and the entry point reports FM_ERR_TIMEOUT.  The context stays usable: the
  next call with the default limit is bit-exact again.
* Non-finite state.  A NaN written into a host global (the user's side of the
  generated-code API) reaches the device with Formura_Forward, and
  Formura_Conserved_Totals reports FM_ERR_NONFINITE.
"""
import numpy as np
import pytest
import torch

from formura_gb300 import _lib, inits, kernels
from formura_gb300._lib import FormuraError
from formura_gb300.runtime import load_program
from oracle import oracle
from tests.bits import same_bits

pytestmark = pytest.mark.gpu

FM_ERR_TIMEOUT = 3
FM_ERR_NONFINITE = 4


def _with_spin_limit(limit, fn, tries=3):
    """Runs fn() with "sync.spin_limit" = limit until it raises a timeout (a
    barrier wait can only time out if some block reaches it before the last
    one, so a single short run is allowed to finish); returns the status."""
    L = _lib.lib()
    L.fm_tune_set(b"sync.spin_limit", limit)
    try:
        for _ in range(tries):
            try:
                fn()
            except FormuraError as e:
                return e.status
        return 0
    finally:
        L.fm_tune_set(b"sync.spin_limit", 0)  # 0: the default limit


@pytest.mark.parametrize("tb", [0, 4])
def test_diffusion_barrier_timeout_then_recovers(cuda_device, tb):
    L = _lib.lib()
    d0 = inits.diffusion_2d(256, 256, seed=11)
    try:
        L.fm_tune_set(b"diff2d.tb", tb)

        def run():
            d = torch.from_numpy(d0).cuda()
            kernels.diff2d_f64_forward(d, torch.empty_like(d), 0.1, 400)

        assert _with_spin_limit(1, run) == FM_ERR_TIMEOUT
        assert b"gave up" in L.fm_last_error()
        # the same call with the default limit: no error, bit-exact
        d = torch.from_numpy(d0).cuda()
        kernels.diff2d_f64_forward(d, torch.empty_like(d), 0.1, 400)
        assert same_bits(d.cpu().numpy(), oracle.diff2d_f64(d0, 400, Dt=0.1, Dx=1.0))
    finally:
        L.fm_tune_clear()


@pytest.mark.parametrize("use_graph", [False, True])
def test_ensemble_barrier_timeout_then_recovers(cuda_device, use_graph):
    sizes = [64, 128, 96, 256]
    F = [0.02, 0.04, 0.05, 0.06]
    k = [0.05, 0.06, 0.065, 0.07]
    steps = 200
    U0, V0 = inits.gs2d_ensemble_state(sizes, seed=4)
    e = kernels.Ensemble(sizes, F, k, 2e-5, 1e-5, 1.0, 0.01, tile=1, tb=2)
    try:
        U, V = torch.from_numpy(U0).cuda(), torch.from_numpy(V0).cuda()
        wU, wV = torch.empty_like(U), torch.empty_like(V)

        def run():
            e.forward(U, V, wU, wV, steps, use_graph=use_graph)
            e.status()  # reads the barrier's error word

        assert _with_spin_limit(1, run) == FM_ERR_TIMEOUT
        # a graph captured under the short limit is re-captured with the default
        U.copy_(torch.from_numpy(U0))
        V.copy_(torch.from_numpy(V0))
        e.forward(U, V, wU, wV, steps, use_graph=use_graph)
        e.status()
        Uc, Vc = U.cpu().numpy(), V.cpu().numpy()
        for i, n in enumerate(sizes):
            o = int(e.offsets[i])
            uo, vo = oracle.gs2d_f32(U0[o:o + n * n].reshape(n, n), V0[o:o + n * n].reshape(n, n),
                                     steps, F[i], k[i], 2e-5, 1e-5, 1.0, 0.01)
            assert same_bits(Uc[o:o + n * n].reshape(n, n), uo), i
            assert same_bits(Vc[o:o + n * n].reshape(n, n), vo), i
    finally:
        e.close()


def test_nan_in_host_global_is_reported_by_conserved_totals(cuda_device):
    prog = load_program("diffusion_2d")
    prog.init()
    d0 = inits.diffusion_2d(256, 256, seed=21)
    prog.state["dens"][...] = d0
    prog.state["dens"][17, 33] = np.nan  # injected on the host, between calls
    prog.forward()
    with pytest.raises(FormuraError) as exc:
        prog.conserved_totals()
    assert exc.value.status == FM_ERR_NONFINITE
    assert np.isnan(prog.state["dens"]).any()
    # a finite state afterwards: totals are reported again
    prog.init()
    prog.state["dens"][...] = d0
    prog.forward()
    tot = prog.conserved_totals()
    assert np.isfinite(tot).all() and abs(tot[0] - d0.sum()) < 1e-9 * d0.sum()
