"""The factorised-phase tensor-core GEMMs on SM pairs (two-CTA clusters,
tcgen05.mma.cta_group::2): the four-product form with 256 x 128 tiles
(ED_TUNE_TC_PAIR = 2) and the stacked form with the re / im planes of both
operands spread over the pair (ED_TUNE_TC_PAIR = 3, two TMEM buffers per
CTA, two double-float planes), against the FP64 oracle and against the
single-SM form on the same inputs.  Shapes cover several M and N
tiles, a narrow last column tile, a batch of timeslices and every split
kind.  Tolerances are those of the split modes: f16x3 and tf32x3 <= 1e-6,
bf16x3 <= 1e-4 against FP64."""

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


def _run(latt, Ne, moms, mode, pair, batch, U, V, ts):
    from easydistillation_gb300.ops import ElementalPlan

    Lx, Ly, Lz, Lt = latt
    V3 = Lx * Ly * Lz
    plan = ElementalPlan(latt, Ne, 2, moms, mode, batch=batch, tuning={"tc_pair": pair})
    assert plan.factorised is not None
    outs = [torch.empty((13, len(moms), Ne, Ne), dtype=torch.complex128, device="cuda") for _ in ts]
    plan.run_batch([U[:, t] for t in ts], Lt * V3 * 9, 9, [V[t] for t in ts], outs)
    assert plan.check_status() == 0
    return [o.cpu().numpy() for o in outs]


@pytest.mark.parametrize("form", [2, 3])
@pytest.mark.parametrize("mode", ["f16x3", "tf32x3", "bf16x3"])
@pytest.mark.parametrize("latt, Ne", [([8, 4, 4, 2], 9), ([8, 8, 4, 1], 150), ([4, 4, 4, 1], 6)])
def test_pair_gemm_matches_oracle_and_single_sm(mode, latt, Ne, form):
    moms = R.mom_dict_to_list(3)
    gauge, evec, U, V = _inputs(latt, Ne, 41)
    ts = list(range(latt[3]))
    pair = _run(latt, Ne, moms, mode, form, len(ts), U, V, ts)
    single = _run(latt, Ne, moms, mode, 1, len(ts), U, V, ts)
    Uh = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3]
    for k, t in enumerate(ts):
        ref = R.elemental(evec[t], Uh[:, t], latt, 2, moms)
        assert rel_err(pair[k], ref) < TOL[mode]
        assert rel_err(pair[k], single[k]) < TOL[mode]


@pytest.mark.parametrize("form", [2, 3])
def test_pair_gemm_long_k_and_slabs(form):
    """K = 3 * 16^3 = 12288 (384 f16 k-blocks: lock steps of 256 + 128 with
    the default slab; 64-k-block slabs give several lock steps per tile)."""
    latt, Ne = [16, 16, 16, 1], 24
    moms = R.mom_dict_to_list(3)
    gauge, evec, U, V = _inputs(latt, Ne, 43)
    from easydistillation_gb300.ops import ElementalPlan

    V3 = 16 ** 3
    out = torch.empty((13, 27, Ne, Ne), dtype=torch.complex128, device="cuda")
    plan = ElementalPlan(latt, Ne, 2, moms, "f16x3", tuning={"tc_pair": form, "tc_slab_kb": 64})
    plan.run(U[:, 0], V3 * 9, 9, V[0], out)
    assert plan.check_status() == 0
    ref = R.elemental(evec[0], gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0], latt, 2, moms)
    assert rel_err(out.cpu().numpy(), ref) < 1e-6


@pytest.mark.parametrize("pair", [1, 2, 3])
def test_two_kblocks_per_tmem_buffer(pair):
    """ED_TUNE_TC_KPB = 2: each TMEM buffer accumulates two k-blocks before it
    is drained; still within 1e-6 of FP64.  K = 3 * 16*16*12 = 9216 is 288
    f16 k-blocks: lock steps of 256 + 32 (default slab) or 4 x 64 + 32."""
    from easydistillation_gb300.ops import ElementalPlan

    latt, Ne = [16, 16, 12, 1], 30
    moms = R.mom_dict_to_list(3)
    gauge, evec, U, V = _inputs(latt, Ne, 47)
    V3 = 16 * 16 * 12
    ref = R.elemental(evec[0], gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0], latt, 2, moms)
    for slab in (0, 64):
        out = torch.empty((13, 27, Ne, Ne), dtype=torch.complex128, device="cuda")
        plan = ElementalPlan(latt, Ne, 2, moms, "f16x3", tuning={"tc_pair": pair, "tc_kpb": 2, "tc_slab_kb": slab})
        plan.run(U[:, 0], V3 * 9, 9, V[0], out)
        assert plan.check_status() == 0
        assert rel_err(out.cpu().numpy(), ref) < 1e-6


def test_two_kblocks_per_buffer_odd_block_count():
    """An odd number of k-blocks per lock step: K = 3 * 4*4*2 = 96 is 3 f16
    k-blocks, so the step ends with a buffer of one k-block."""
    from easydistillation_gb300.ops import ElementalPlan

    latt, Ne = [4, 4, 2, 1], 5
    moms = R.mom_dict_to_list(3)
    gauge, evec, U, V = _inputs(latt, Ne, 49)
    ref = R.elemental(evec[0], gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0], latt, 2, moms)
    for pair in (1, 2, 3):
        out = torch.empty((13, 27, Ne, Ne), dtype=torch.complex128, device="cuda")
        plan = ElementalPlan(latt, Ne, 2, moms, "f16x3", tuning={"tc_pair": pair, "tc_kpb": 2})
        plan.run(U[:, 0], 32 * 9, 9, V[0], out)
        assert plan.check_status() == 0
        assert rel_err(out.cpu().numpy(), ref) < 1e-6
