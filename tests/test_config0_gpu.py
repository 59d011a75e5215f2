"""The plain-FP64 CPU configuration end to end against the reference's own
chain (tests/golden/config0_chain.npz, made by running the reference's
EigenvectorGenerator and then its ElementalGenerator on those eigenvectors):
4^3 x 8, links exp(i 0.1 A), Ne = 20, tol 1e-10, num_nabla = 1 (operators
1, nabla_x, nabla_y, nabla_z), the 7 momenta with |p|^2 <= 1.

(a) the eigensolve on every timeslice: eigenvalues to 1e-10 relative,
    residuals ||L v - lambda v|| < 1e-9, and the projector V V^dagger against
    the reference's (eigenvector phases and rotations are arbitrary).  The
    20th and 21st eigenvalues of these fields are ~0.01 apart, so a residual
    of 1e-9 moves the projector by at most ~1e-7 (Davis-Kahan);
(b) the elementals of all 8 timeslices computed from the REFERENCE's
    eigenvectors: FP64 to 1e-12 relative, the split-precision modes to 1e-6."""

import numpy as np
import pytest

from oracle import restatement as R
from tests.conftest import golden
from tests.helpers import MemEigen, MemGauge, rel_err

pytestmark = pytest.mark.gpu

EVAL_RTOL = 1e-10
RESID_MAX = 1e-9
PROJ_TOL = 1e-7
FP64_TOL = 1e-12
SPLIT_TOL = 1e-6


def test_config0_eigensolve_all_timeslices():
    from easydistillation_gb300 import EigenvectorGenerator

    z = golden("config0_chain.npz")
    latt = [int(v) for v in z["latt"]]
    Ne, tol = int(z["Ne"]), float(z["tol"])
    gen = EigenvectorGenerator(latt, MemGauge(z["gauge"]), Ne, tol)
    gen.load("cfg0")
    evecs, evals = gen.calc_batch(range(latt[3]))
    U = z["gauge"].transpose(4, 0, 1, 2, 3, 5, 6)[:3]
    P = lambda v: v.reshape(Ne, -1).T @ v.reshape(Ne, -1).conj()
    for t in range(latt[3]):
        X, lam = evecs[t].cpu().numpy(), evals[t].cpu().numpy()
        np.testing.assert_allclose(lam, z["evals"][t], rtol=EVAL_RTOL, atol=0)
        Xf = X.reshape(Ne, -1)
        res = np.linalg.norm(R.laplacian(Xf.T, U[:, t], latt).T - lam[:, None] * Xf, axis=1)
        assert res.max() < RESID_MAX
        assert np.abs(P(X) - P(z["evecs"][t])).max() < PROJ_TOL
        first = Xf[:, 0]  # the renormalisation phase of eigenvector.py:249-257
        assert np.all(np.abs(first.imag) < 1e-12) and np.all(first.real >= 0)


@pytest.mark.parametrize("mode", ["fp64", "f16x3", "tf32x3"])
def test_config0_elementals_from_reference_eigenvectors(mode):
    from easydistillation_gb300 import ElementalGenerator

    z = golden("config0_chain.npz")
    latt = [int(v) for v in z["latt"]]
    Ne = int(z["Ne"])
    moms = [tuple(int(v) for v in p) for p in z["moms"]]
    gen = ElementalGenerator(latt, MemGauge(z["gauge"]), MemEigen(z["evecs"], Ne), 1, moms, precision=mode)
    gen.load("cfg0")
    tol = FP64_TOL if mode == "fp64" else SPLIT_TOL
    for t in range(latt[3]):
        E = gen.calc(t).cpu().numpy()
        assert E.shape == (4, 7, Ne, Ne)
        assert rel_err(E, z["E"][t]) < tol, (t, rel_err(E, z["E"][t]))


def test_config0_reference_loop_with_numpy_backend():
    """The reference's own driver loop (tests/test_elemental.py:37-45):
    data = backend.zeros(...); data[t] = elemental.calc(t), with the numpy
    backend selected."""
    import easydistillation_gb300 as ed
    from easydistillation_gb300 import ElementalGenerator

    z = golden("config0_chain.npz")
    latt = [int(v) for v in z["latt"]]
    Ne = int(z["Ne"])
    moms = [tuple(int(v) for v in p) for p in z["moms"]]
    try:
        ed.set_backend("numpy")
        backend = ed.get_backend()
        gen = ElementalGenerator(latt, MemGauge(z["gauge"]), MemEigen(z["evecs"], Ne), 1, moms)
        gen.load("cfg0")
        data = backend.zeros((latt[3], 4, 7, Ne, Ne), "<c16")
        for t in range(latt[3]):
            data[t] = gen.calc(t)
    finally:
        ed.set_backend("torch")
    assert rel_err(data, z["E"]) < FP64_TOL
