"""The stacked form of the factorised-phase tensor-core GEMM (the default;
``ED_TUNE_TC_STACK = 1``: B = [Br; Bi] in shared memory, M = 128, N = 256
MMAs A_re [Br | Bi] and A_im [Br | Bi] into two single 256-column TMEM
accumulators, combined into re / im by the drain) against the FP64 oracle
and against the four-product form (``ED_TUNE_TC_STACK = 2``) on the same
inputs.  Shapes cover several M and N tiles, a narrow last column tile
(N = 2 x 16), a batch of timeslices, every split kind, long K over several
lock-step slabs and 1, 2 or 4 k-blocks per accumulator group (including
groups cut short at the end of a step), for both forms.  Tolerances are
those of the split modes: f16x3 and tf32x3 <= 1e-6, bf16x3 <= 1e-4 against
FP64."""

import numpy as np
import pytest
import torch

from oracle import restatement as R
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

TOL = {"f16x3": 1e-6, "tf32x3": 1e-6, "bf16x3": 1e-4}


def _inputs(latt, Ne, seed):
    gauge = R.synthetic_gauge(latt, 0.3, seed)
    evec = np.stack([R.random_colour_vectors(Ne, latt, seed * 10 + t) for t in range(latt[3])])
    U = torch.from_numpy(np.ascontiguousarray(gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3])).cuda()
    V = torch.from_numpy(evec.reshape(latt[3], Ne, -1)).cuda()
    return gauge, evec, U, V


def _run(latt, Ne, moms, mode, tuning, U, V, ts):
    from easydistillation_gb300.ops import ElementalPlan

    Lx, Ly, Lz, Lt = latt
    V3 = Lx * Ly * Lz
    plan = ElementalPlan(latt, Ne, 2, moms, mode, batch=len(ts), tuning=tuning)
    assert plan.factorised is not None
    outs = [torch.empty((13, len(moms), Ne, Ne), dtype=torch.complex128, device="cuda") for _ in ts]
    plan.run_batch([U[:, t] for t in ts], Lt * V3 * 9, 9, [V[t] for t in ts], outs)
    assert plan.check_status() == 0
    return [o.cpu().numpy() for o in outs]


@pytest.mark.parametrize("mode", ["f16x3", "tf32x3", "bf16x3"])
@pytest.mark.parametrize("latt, Ne", [([8, 4, 4, 2], 9), ([8, 8, 4, 1], 150), ([4, 4, 4, 1], 6)])
def test_stacked_gemm_matches_oracle_and_four_product_form(mode, latt, Ne):
    moms = R.mom_dict_to_list(3)
    gauge, evec, U, V = _inputs(latt, Ne, 51)
    ts = list(range(latt[3]))
    stacked = _run(latt, Ne, moms, mode, {"tc_pair": 1, "tc_stack": 1}, U, V, ts)
    four = _run(latt, Ne, moms, mode, {"tc_pair": 1, "tc_stack": 2}, U, V, ts)
    Uh = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3]
    for k, t in enumerate(ts):
        ref = R.elemental(evec[t], Uh[:, t], latt, 2, moms)
        assert rel_err(stacked[k], ref) < TOL[mode]
        assert rel_err(stacked[k], four[k]) < TOL[mode]


@pytest.mark.parametrize("form, kpb", [(1, 1), (1, 2), (1, 4), (2, 1), (2, 2)])
def test_stacked_gemm_long_k_groups_and_slabs(kpb, form):
    """K = 3 * 16*16*12 = 9216 is 288 f16 k-blocks: lock steps of 256 + 32
    (default slab) or 4 x 64 + 32, cut into groups of kpb k-blocks.  (The
    four-product form with 4 k-blocks per buffer adds 48 truncating MMAs per
    accumulator column and measured 1.17e-6 here: not an accurate setting.)"""
    latt, Ne = [16, 16, 12, 1], 30
    moms = R.mom_dict_to_list(3)
    gauge, evec, U, V = _inputs(latt, Ne, 53)
    ref = R.elemental(evec[0], gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0], latt, 2, moms)
    for slab in (0, 64):
        out = _run(latt, Ne, moms, "f16x3", {"tc_stack": form, "tc_kpb": kpb, "tc_slab_kb": slab}, U, V, [0])[0]
        assert rel_err(out, ref) < 1e-6


def test_stacked_gemm_short_group_at_step_end():
    """K = 3 * 4*4*2 = 96 is 3 f16 k-blocks: with 2 or 4 k-blocks per group
    the step ends with a group of one (kpb 2) or three (kpb 4) k-blocks."""
    latt, Ne = [4, 4, 2, 1], 5
    moms = R.mom_dict_to_list(3)
    gauge, evec, U, V = _inputs(latt, Ne, 55)
    ref = R.elemental(evec[0], gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0], latt, 2, moms)
    for form in (1, 2):
        for kpb in (2, 4):
            out = _run(latt, Ne, moms, "f16x3", {"tc_stack": form, "tc_kpb": kpb}, U, V, [0])[0]
            assert rel_err(out, ref) < 1e-6


# ---------------------------------------------------------------- on-chip-phase kernel (tc_pair_gemm.cuh)
def _run_onchip(latt, Ne, num_nabla, moms, mode, tuning, seed):
    from easydistillation_gb300.ops import ElementalPlan

    gauge, evec, U, V = _inputs(latt, Ne, seed)
    V3 = latt[0] * latt[1] * latt[2]
    plan = ElementalPlan(latt, Ne, num_nabla, moms, mode, factorise=False, tuning=tuning)
    assert plan.factorised is None
    nd = {0: 1, 1: 4, 2: 13}[num_nabla]
    out = torch.empty((nd, len(moms), Ne, Ne), dtype=torch.complex128, device="cuda")
    plan.run(U[:, 0], latt[3] * V3 * 9, 9, V[0], out)
    assert plan.check_status() == 0
    ref = R.elemental(evec[0], gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0], latt, num_nabla, moms)
    return out.cpu().numpy(), ref


@pytest.mark.parametrize("mode", ["f16x3", "tf32x3", "bf16x3"])
@pytest.mark.parametrize("tuning", [{}, {"tc_kpb": 1}, {"tc_kpb": 4}, {"tc_stack": 2}])
def test_onchip_phase_kernel_forms(mode, tuning):
    """The on-chip-phase GEMM in the stacked form (default, 2 k-blocks per
    group; 1 and 4) and the four-product form, several ragged M and N tiles,
    27 momenta kept off the factorised path."""
    out, ref = _run_onchip([8, 8, 4, 1], 40, 1, R.mom_dict_to_list(3), mode, tuning, 71)
    assert rel_err(out, ref) < TOL[mode]


@pytest.mark.parametrize("kpb", [1, 2, 4])
def test_onchip_phase_stacked_long_k_and_short_group(kpb):
    """K = 3 * 16^3 = 12288 (384 k-blocks: flushes after k-block 255 and at
    the end) with an open momentum list, and K = 3 * 4*4*2 = 96 (3 k-blocks:
    the last group is short)."""
    moms = [(0, 0, 0), (0, 0, 1), (0, 1, 1), (1, 1, 1), (0, 0, 2), (0, 1, 2), (1, 1, 2)]
    out, ref = _run_onchip([16, 16, 16, 1], 24, 1, moms, "f16x3", {"tc_kpb": kpb}, 73)
    assert rel_err(out, ref) < 1e-6
    out, ref = _run_onchip([4, 4, 2, 1], 5, 2, R.mom_dict_to_list(3)[:7], "f16x3", {"tc_kpb": kpb}, 75)
    assert rel_err(out, ref) < 1e-6
