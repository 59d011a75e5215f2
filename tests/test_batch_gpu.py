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


@pytest.mark.parametrize("source", ["numpy", "pinned"])
def test_pipelined_batches_into_host_output(source):
    """calc_batch over several batches with a pinned host output (copies of
    batch k+-1 overlap batch k) against the oracle, for numpy and
    pinned-tensor eigenvector sources."""
    from easydistillation_gb300 import ElementalGenerator

    latt = [8, 4, 4, 6]
    moms = R.mom_dict_to_list(3)
    Ne = 10
    gauge = R.synthetic_gauge(latt, 0.3, 13)
    evec = np.stack([R.random_colour_vectors(Ne, latt, 40 + t) for t in range(latt[3])])

    class _T:
        def __init__(self, t):
            self.t, self.Ne = t, Ne

        def load(self, key):
            return self.t

    src = MemEigen(evec, Ne) if source == "numpy" else _T(torch.from_numpy(evec).pin_memory())
    gen = ElementalGenerator(latt, MemGauge(gauge), src, 2, moms, precision="f16x3")
    gen.load("k")
    ts = [5, 1, 3, 0, 2]
    host = torch.empty((len(ts), 13, 27, Ne, Ne), dtype=torch.complex128).pin_memory()
    out = gen.calc_batch(ts, out=host, batch=2)
    assert out is host
    U = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3]
    for k, t in enumerate(ts):
        ref = R.elemental(evec[t], U[:, t], latt, 2, moms)
        assert rel_err(host[k].numpy(), ref) < 1e-6
