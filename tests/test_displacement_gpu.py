"""DisplacementElementalGenerator on the GPU against the reference's own output
(golden fixture) and the oracle; FP64 to 1e-12 relative."""

import numpy as np
import pytest

from oracle import restatement as R
from tests.conftest import golden
from tests.helpers import MemEigen, MemGauge, rel_err

pytestmark = pytest.mark.gpu


def test_displacement_golden():
    from easydistillation_gb300 import DisplacementElementalGenerator

    g = golden("displacement_d2.npz")
    latt = [int(v) for v in g["latt"]]
    gen = DisplacementElementalGenerator(latt, MemGauge(g["gauge"]), MemEigen(g["evec"], 4), 2,
                                         [tuple(int(v) for v in p) for p in g["moms"]])
    gen.load("mem")
    assert rel_err(gen.calc(0).cpu().numpy(), g["E"]) < 1e-12


@pytest.mark.parametrize("distance", [0, 1, 3])
def test_displacement_vs_oracle_nonsymmetric(distance):
    from easydistillation_gb300 import DisplacementElementalGenerator

    latt = [6, 4, 8, 2]
    Ne = 5
    moms = R.mom_dict_to_list(3)[:5]
    gauge = R.synthetic_gauge(latt, 0.3, 61)
    evec = np.stack([R.random_colour_vectors(Ne, latt, 70 + t) for t in range(2)])
    gen = DisplacementElementalGenerator(latt, MemGauge(gauge), MemEigen(evec, Ne), distance, moms)
    gen.load("k")
    U = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3]
    for t in range(2):
        ref = R.displacement_elemental(evec[t], U[:, t], latt, distance, moms)
        assert rel_err(gen.calc(t).cpu().numpy(), ref) < 1e-12
