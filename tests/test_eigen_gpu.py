"""EigenvectorGenerator (GPU thick-restart Lanczos around the stencil kernel)
against the reference's scipy/ARPACK eigensolve: eigenvalues to 1e-10
relative, eigen-residuals ||L v - lambda v|| < 1e-9 with the FP64 oracle
operator, and agreement of the projector V V^dagger (phases and rotations
inside degenerate subspaces are arbitrary)."""

import numpy as np
import pytest

from oracle import restatement as R
from tests.conftest import golden
from tests.helpers import MemGauge

pytestmark = pytest.mark.gpu


def _check(evecs, evals, ref_vecs, ref_vals, U_t, latt, Ne):
    np.testing.assert_allclose(evals, ref_vals, rtol=1e-10, atol=1e-12)
    X = evecs.reshape(Ne, -1)
    LX = R.laplacian(X.T, U_t, latt).T
    res = np.linalg.norm(LX - evals[:, None] * X, axis=1)
    assert res.max() < 1e-9
    P = lambda v: v.reshape(Ne, -1).T @ v.reshape(Ne, -1).conj()
    assert np.abs(P(evecs) - P(ref_vecs)).max() < 1e-8
    # renormalisation phase: first component real and positive
    first = X[:, 0]
    assert np.all(np.abs(first.imag) < 1e-12) and np.all(first.real >= 0)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_eigen_golden(prec):
    from easydistillation_gb300 import EigenvectorGenerator

    g = golden("eigen_443.npz")
    latt = [int(v) for v in g["latt"]]
    Ne = int(g["Ne"])
    gen = EigenvectorGenerator(latt, MemGauge(g["gauge"]), Ne, 1e-10, stencil_precision=prec)
    gen.load("mem")
    evecs, evals = gen.calc(0)
    U = g["gauge"].transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0]
    _check(evecs.cpu().numpy(), evals.cpu().numpy(), g["evecs0"], g["evals0"], U, latt, Ne)


def test_eigen_batched_timeslices_match_scipy():
    from easydistillation_gb300 import EigenvectorGenerator

    latt = [6, 4, 4, 3]
    Ne = 10
    gauge = R.synthetic_gauge(latt, 0.3, 3)
    gen = EigenvectorGenerator(latt, MemGauge(gauge), Ne, 1e-10)
    gen.load("k")
    evecs, evals = gen.calc_batch(range(3))
    U = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3]
    for t in range(3):
        rv, re = R.eigensolve(U[:, t], latt, Ne, 1e-10)
        _check(evecs[t].cpu().numpy(), evals[t].cpu().numpy(), rv, re, U[:, t], latt, Ne)


@pytest.mark.parametrize("deg", [10, 7])
def test_eigen_chebyshev_acceleration(deg):
    """calc(t, True, polynomial_degree, lambda_cut) as the reference's test
    calls it (tests/test_eigenvector.py:54): cut at 1.1 x the largest wanted
    eigenvalue; same eigenpairs as the unaccelerated solve."""
    from easydistillation_gb300 import EigenvectorGenerator

    g = golden("eigen_443.npz")
    latt = [int(v) for v in g["latt"]]
    Ne = int(g["Ne"])
    gen = EigenvectorGenerator(latt, MemGauge(g["gauge"]), Ne, 1e-10)
    gen.load("mem")
    evecs, evals = gen.calc(0, True, deg, float(g["evals0"][-1]) * 1.1)
    U = g["gauge"].transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0]
    _check(evecs.cpu().numpy(), evals.cpu().numpy(), g["evecs0"], g["evals0"], U, latt, Ne)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_eigen_larger_volume_against_scipy(prec):
    """12^3 (n = 5184), Ne = 40, tol 1e-10, two timeslices in one batch: several
    thick restarts, so the reorthogonalisation is exercised over many steps."""
    from easydistillation_gb300 import EigenvectorGenerator

    latt = [12, 12, 12, 2]
    Ne = 40
    gauge = R.synthetic_gauge(latt, 0.3, 17)
    gen = EigenvectorGenerator(latt, MemGauge(gauge), Ne, 1e-10, stencil_precision=prec)
    gen.load("k")
    evecs, evals = gen.calc_batch(range(2))
    assert gen.last_stats["converged"]
    U = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3]
    for t in range(2):
        rv, re = R.eigensolve(U[:, t], latt, Ne, 1e-10)
        _check(evecs[t].cpu().numpy(), evals[t].cpu().numpy(), rv, re, U[:, t], latt, Ne)
