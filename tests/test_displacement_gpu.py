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


def test_displacement_after_stout_smear_and_projection():
    """``stout_smear`` and ``project_SU3`` on the generator's own links
    (``displacement_elemental.py:98-108, 202-214``) change what ``calc``
    transports with: against the oracle's smearing followed by the oracle's
    displacement elemental, and the projection against the reference's own
    result (tests/golden/project_su3.npz)."""
    from easydistillation_gb300 import DisplacementElementalGenerator

    latt = [6, 4, 8, 2]
    Ne, distance = 4, 2
    moms = R.mom_dict_to_list(3)[:3]
    gauge = R.synthetic_gauge(latt, 0.4, 83)
    evec = np.stack([R.random_colour_vectors(Ne, latt, 90 + t) for t in range(2)])
    gen = DisplacementElementalGenerator(latt, MemGauge(gauge), MemEigen(evec, Ne), distance, moms)
    with pytest.raises(RuntimeError):
        gen.stout_smear(1, 0.1)
    gen.load("k")
    before = gen.calc(1).cpu().numpy().copy()
    gen.stout_smear(2, 0.12)
    Us = R.stout_smear(gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3].copy(), 2, 0.12)
    assert np.abs(gen._U.cpu().numpy() - Us).max() < 1e-13
    for t in range(2):
        ref = R.displacement_elemental(evec[t], Us[:, t], latt, distance, moms)
        assert rel_err(gen.calc(t).cpu().numpy(), ref) < 1e-12
    assert rel_err(before, R.displacement_elemental(evec[1], Us[:, 1], latt, distance, moms)) > 1e-6

    z = golden("project_su3.npz")
    latt = [int(v) for v in z["latt"]]
    evec = np.stack([R.random_colour_vectors(Ne, latt, 95 + t) for t in range(latt[3])])
    gen = DisplacementElementalGenerator(latt, MemGauge(z["gauge"]), MemEigen(evec, Ne), 1, moms)
    gen.load("k")
    gen.project_SU3()
    P = gen._U.cpu().numpy()
    assert np.abs(P - z["projected"]).max() < 1e-13
    ref = R.displacement_elemental(evec[0], z["projected"][:, 0], latt, 1, moms)
    assert rel_err(gen.calc(0).cpu().numpy(), ref) < 1e-12
