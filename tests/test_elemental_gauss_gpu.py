"""The Gauss three-multiplication form of the factorised-phase tensor-core
GEMM (``ED_MODE_FLAG_GAUSS``: X = Ar Br, Y = Ai Bi, Z = (Ar + Ai)(Br + Bi),
re = X - Y, im = Z - X - Y, with the re + im planes written by the split)
against the FP64 oracle and against the default (stacked) form on the same
inputs.  Shapes cover several M and N tiles, a narrow last column tile, a
batch of timeslices, every split kind, long K over several lock-step slabs
and 1, 2 or 4 k-blocks per accumulator group (including a group cut short
at the end of a step).  Tolerances are those of the split modes: f16x3 and
tf32x3 <= 1e-6, bf16x3 <= 1e-4 against FP64."""

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


def _run(latt, Ne, moms, mode, gauss, tuning, U, V, ts):
    from easydistillation_gb300.ops import ElementalPlan

    Lx, Ly, Lz, Lt = latt
    V3 = Lx * Ly * Lz
    plan = ElementalPlan(latt, Ne, 2, moms, mode, batch=len(ts), tuning=tuning, gauss=gauss)
    assert plan.factorised is not None
    outs = [torch.empty((13, len(moms), Ne, Ne), dtype=torch.complex128, device="cuda") for _ in ts]
    plan.run_batch([U[:, t] for t in ts], Lt * V3 * 9, 9, [V[t] for t in ts], outs)
    assert plan.check_status() == 0
    return [o.cpu().numpy() for o in outs]


@pytest.mark.parametrize("mode", ["f16x3", "tf32x3", "bf16x3"])
@pytest.mark.parametrize("latt, Ne", [([8, 4, 4, 2], 9), ([8, 8, 4, 1], 150), ([4, 4, 4, 1], 6)])
def test_gauss_gemm_matches_oracle_and_stacked_form(mode, latt, Ne):
    moms = R.mom_dict_to_list(3)
    gauge, evec, U, V = _inputs(latt, Ne, 57)
    ts = list(range(latt[3]))
    gauss = _run(latt, Ne, moms, mode, True, {}, U, V, ts)
    stacked = _run(latt, Ne, moms, mode, False, {}, U, V, ts)
    Uh = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3]
    for k, t in enumerate(ts):
        ref = R.elemental(evec[t], Uh[:, t], latt, 2, moms)
        assert rel_err(gauss[k], ref) < TOL[mode]
        assert rel_err(gauss[k], stacked[k]) < TOL[mode]


@pytest.mark.parametrize("kpb", [1, 2, 4])
def test_gauss_gemm_long_k_groups_and_slabs(kpb):
    """K = 3 * 16*16*12 = 9216 is 288 f16 k-blocks: lock steps of 256 + 32
    (default slab) or 4 x 64 + 32, cut into groups of kpb k-blocks."""
    latt, Ne = [16, 16, 12, 1], 30
    moms = R.mom_dict_to_list(3)
    gauge, evec, U, V = _inputs(latt, Ne, 59)
    ref = R.elemental(evec[0], gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0], latt, 2, moms)
    for slab in (0, 64):
        out = _run(latt, Ne, moms, "f16x3", True, {"tc_kpb": kpb, "tc_slab_kb": slab}, U, V, [0])[0]
        assert rel_err(out, ref) < 1e-6


def test_gauss_gemm_short_group_and_ignored_pairing():
    """K = 3 * 4*4*2 = 96 is 3 f16 k-blocks (a group of one k-block ends the
    step with 2 per group); SM pairing is ignored by the Gauss form."""
    latt, Ne = [4, 4, 2, 1], 5
    moms = R.mom_dict_to_list(3)
    gauge, evec, U, V = _inputs(latt, Ne, 61)
    ref = R.elemental(evec[0], gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0], latt, 2, moms)
    for tuning in ({"tc_kpb": 2}, {"tc_pair": 2}, {"tc_stages": 3}):
        out = _run(latt, Ne, moms, "f16x3", True, tuning, U, V, [0])[0]
        assert rel_err(out, ref) < 1e-6
