"""Batched elementals (several timeslices, one pair-contraction launch)
against per-timeslice runs and the oracle."""

import numpy as np
import pytest
import torch

from oracle import restatement as R
from tests.helpers import MemEigen, MemGauge, rel_err

pytestmark = pytest.mark.gpu


def _gen(latt, Ne, num_nabla, moms, precision, seed=9):
    from easydistillation_gb300 import ElementalGenerator

    gauge = R.synthetic_gauge(latt, 0.3, seed)
    evec = np.stack([R.random_colour_vectors(Ne, latt, seed * 7 + t) for t in range(latt[3])])
    gen = ElementalGenerator(latt, MemGauge(gauge), MemEigen(evec, Ne), num_nabla, moms, precision=precision)
    gen.load("k")
    return gen, gauge, evec


@pytest.mark.parametrize("batch", [2, 3])
def test_batch_fp64_equals_single_timeslices(batch):
    latt = [4, 4, 4, 5]
    moms = R.mom_dict_to_list(3)[:7]
    gen, gauge, evec = _gen(latt, 6, 2, moms, "fp64")
    ts = [4, 0, 2, 3, 1]
    out = gen.calc_batch(ts, batch=batch).cpu().numpy()
    for k, t in enumerate(ts):
        single = gen.calc(t).cpu().numpy()
        assert rel_err(out[k], single) < 1e-14


def test_batch_f16x3_vs_oracle():
    latt = [8, 4, 4, 3]
    moms = R.mom_dict_to_list(3)
    gen, gauge, evec = _gen(latt, 20, 2, moms, "f16x3")
    out = gen.calc_batch(range(3), batch=3).cpu().numpy()
    U = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3]
    for t in range(3):
        ref = R.elemental(evec[t], U[:, t], latt, 2, moms)
        assert rel_err(out[t], ref) < 1e-6


def test_admit_batch_respects_memory():
    from easydistillation_gb300.generator.elemental import admit_batch

    b = admit_batch([4, 4, 4, 8], 6, 2, [(0, 0, 0)], "fp64", max_batch=4)
    assert 1 <= b <= 4
