"""Failure detection without a GPU fault: the TMA-staged complex64 Laplacian
bounds every wait for its data.  With a short limit (a launch setting) and
the probe setting on, every block first waits on a barrier of its own that
nothing completes, so the limit runs out whatever the copy latency: the
launch must report ED_ERR_TIMEOUT through the status word, leave the context
usable (every block still drains its own copies in flight before it leaves),
and the next launch with the default settings must be clean and correct."""

import ctypes

import numpy as np
import pytest
import torch

from oracle import restatement as R

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("variant", [2, 1])  # 2: strip-staged (default), 1: input planes staged
def test_staged_laplacian_timeout_is_reported_and_recovers(variant):
    from easydistillation_gb300 import _lib
    from easydistillation_gb300.ops import laplacian, laplacian_config, links_to_soa

    latt = [16, 16, 16, 2]
    V3 = 16 ** 3
    gauge = R.synthetic_gauge(latt, 0.3, 77)
    U = torch.from_numpy(np.ascontiguousarray(gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3])).cuda()
    links = links_to_soa(U, latt, dtype=torch.complex64)
    F = torch.randn((2, 1, 3, V3), dtype=torch.complex64, device="cuda")
    code = ctypes.c_int(0)
    try:
        laplacian_config(variant)
        assert _lib.lib().ed_laplacian_status(ctypes.byref(code), _lib.stream_handle()) == _lib.ED_OK  # clean start
        _lib.check(_lib.lib().ed_laplacian_wait_limit(1000), "ed_laplacian_wait_limit")
        _lib.check(_lib.lib().ed_laplacian_wait_probe(1), "ed_laplacian_wait_probe")
        laplacian(links, F, latt)
        rc = _lib.lib().ed_laplacian_status(ctypes.byref(code), _lib.stream_handle())
        assert rc == _lib.ED_ERR_TIMEOUT and code.value != 0
        assert "gave up" in _lib.last_error()
    finally:
        _lib.lib().ed_laplacian_wait_probe(0)
        _lib.lib().ed_laplacian_wait_limit(0)
        laplacian_config(2)
    # the status word was cleared by the read; the context is usable and the next launch is exact
    out = laplacian(links, F, latt)
    assert _lib.lib().ed_laplacian_status(ctypes.byref(code), _lib.stream_handle()) == _lib.ED_OK and code.value == 0
    U64 = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3]
    for t in range(2):
        f = F[t, 0].cpu().numpy().astype(np.complex128)  # colour planes [3, V3]
        ref = R.laplacian(f.T.reshape(-1), U64[:, t], latt).reshape(V3, 3).T
        got = out[t, 0].cpu().numpy()
        assert np.abs(got - ref).max() < 2e-5 * np.abs(ref).max()


def test_factorised_tensor_core_gemm_timeout_is_reported_and_recovers():
    """The same for the single-SM factorised tcgen05 GEMM (f16x3, the 27
    momenta with |p|^2 <= 3): a short wait limit and the probe (its copy
    issuer issues nothing) make the first operand-stage wait run out before any
    MMA is issued; the run must report ED_ERR_TIMEOUT, every role must leave
    (the drain warps after the MMA issuer's final commit, TMEM released), and
    the next run with the default settings must be clean and within 1e-6 of
    the oracle."""
    from easydistillation_gb300 import _lib
    from easydistillation_gb300.ops import ElementalPlan

    latt, Ne = [8, 4, 4, 1], 6
    V3 = 8 * 4 * 4
    moms = R.mom_dict_to_list(3)
    gauge = R.synthetic_gauge(latt, 0.3, 79)
    evec = R.random_colour_vectors(Ne, latt, 80)
    U = torch.from_numpy(np.ascontiguousarray(gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3])).cuda()
    V = torch.from_numpy(evec.reshape(Ne, -1)).cuda()
    plan = ElementalPlan(latt, Ne, 2, moms, "f16x3", tuning={"tc_pair": 1})
    assert plan.factorised is not None
    out = torch.empty((13, 27, Ne, Ne), dtype=torch.complex128, device="cuda")
    try:
        _lib.check(_lib.lib().ed_elemental_wait_limit(20000), "ed_elemental_wait_limit")
        _lib.check(_lib.lib().ed_elemental_wait_probe(1), "ed_elemental_wait_probe")
        plan.run(U[:, 0], V3 * 9, 9, V, out)
        with pytest.raises(_lib.EDError) as exc:
            plan.check_status()
        assert exc.value.code == _lib.ED_ERR_TIMEOUT and "gave up" in str(exc.value)
    finally:
        _lib.lib().ed_elemental_wait_probe(0)
        _lib.lib().ed_elemental_wait_limit(0)
    # every run clears its status word: the context is usable and the next run is correct
    plan.run(U[:, 0], V3 * 9, 9, V, out)
    assert plan.check_status() == 0
    ref = R.elemental(evec, gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0], latt, 2, moms)
    err = np.linalg.norm(out.cpu().numpy() - ref) / np.linalg.norm(ref)
    assert err < 1e-6
