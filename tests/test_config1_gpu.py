"""Plain FP64 at the 24^3 configuration (24^3, links exp(i 0.3 A), Ne = 100,
tol 1e-10), one timeslice:

* the eigensolve against scipy/ARPACK (the reference's solver) on the host:
  eigenvalues to 1e-10 relative, residuals ||L v - lambda v|| < 1e-9, the
  projector V V^dagger (to 1e-7, bounded by residual / eigenvalue gap),
  orthonormality to 1e-12, and the Chebyshev-accelerated solve giving the
  same eigenpairs;
* the FP64 elementals (13 operators) against the oracle for a subset of
  momenta closed under p -> -p, to 1e-12, and the split-precision f16x3
  path with all 27 momenta against the FP64 GPU path, to 1e-6."""

import numpy as np
import pytest
import torch

from oracle import restatement as R
from tests.helpers import MemGauge, rel_err

pytestmark = pytest.mark.gpu

LATT = [24, 24, 24, 1]
NE = 100


def _gauge(seed=1001):
    return R.synthetic_gauge(LATT, 0.3, seed)


def test_config1_eigensolve_against_arpack():
    from easydistillation_gb300 import EigenvectorGenerator

    gauge = _gauge()
    gen = EigenvectorGenerator(LATT, MemGauge(gauge), NE, 1e-10)
    gen.load("cfg1")
    X, lam = (a.cpu().numpy() for a in gen.calc(0))
    assert gen.last_stats["converged"]
    U = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0]
    rv, re = R.eigensolve(U, LATT, NE, 1e-10)
    np.testing.assert_allclose(lam, re, rtol=1e-10, atol=0)
    Xf = X.reshape(NE, -1)
    res = np.linalg.norm(R.laplacian(Xf.T, U, LATT).T - lam[:, None] * Xf, axis=1)
    assert res.max() < 1e-9
    G = Xf.conj() @ Xf.T
    assert np.abs(G - np.eye(NE)).max() < 1e-12
    Xt = torch.from_numpy(Xf).cuda()
    Rt = torch.from_numpy(np.ascontiguousarray(rv.reshape(NE, -1))).cuda()
    Pd = Xt.T @ Xt.conj() - Rt.T @ Rt.conj()
    assert float(Pd.abs().max()) < 1e-7
    # Chebyshev acceleration (the reference's QUDA option): the same eigenpairs
    Xc, lc = (a.cpu().numpy() for a in gen.calc(0, True, 16, 1.15 * float(lam[-1])))
    np.testing.assert_allclose(lc, lam, rtol=1e-10, atol=0)
    Xcf = Xc.reshape(NE, -1)
    resc = np.linalg.norm(R.laplacian(Xcf.T, U, LATT).T - lc[:, None] * Xcf, axis=1)
    assert resc.max() < 1e-9


def test_config1_elementals():
    from easydistillation_gb300.insertion import mom_dict_to_list
    from easydistillation_gb300.ops import ElementalPlan

    gauge = _gauge()
    V = R.random_colour_vectors(NE, LATT, 1101)  # [Ne, Lz, Ly, Lx, 3], orthonormal
    U = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0]
    Ud = torch.from_numpy(np.ascontiguousarray(U)).cuda()
    Vd = torch.from_numpy(V.reshape(NE, -1)).cuda()
    V3 = LATT[0] * LATT[1] * LATT[2]
    moms = [(0, 0, 0), (1, 0, -1), (-1, 0, 1)]
    plan = ElementalPlan(LATT, NE, 2, moms, "fp64", tuning={"f64_tile": 3})
    out = torch.empty((13, 3, NE, NE), dtype=torch.complex128, device="cuda")
    plan.run(Ud, V3 * 9, 9, Vd, out)
    ref = R.elemental(V, U, LATT, 2, moms)
    assert rel_err(out.cpu().numpy(), ref) < 1e-12
    moms27 = mom_dict_to_list(3)
    res = {}
    for mode in ("fp64", "f16x3"):
        p = ElementalPlan(LATT, NE, 2, moms27, mode, tuning={"f64_tile": 3} if mode == "fp64" else None)
        o = torch.empty((13, 27, NE, NE), dtype=torch.complex128, device="cuda")
        p.run(Ud, V3 * 9, 9, Vd, o)
        if mode != "fp64":
            p.check_status()
        res[mode] = o
    err = float(torch.linalg.vector_norm(res["f16x3"] - res["fp64"]) / torch.linalg.vector_norm(res["fp64"]))
    assert err <= 1e-6, err


def test_config1_mixed_precision_eigensolve():
    """The complex64 stencil inside the native thick-restart iteration, then the
    FP64 Chebyshev refinement (ed_lanczos_tr_ex): the same eigenpairs as ARPACK
    to check (a)'s tolerances, and fewer FP64 operator applications than the
    plain FP64 solve needs."""
    from easydistillation_gb300 import EigenvectorGenerator

    gauge = _gauge()
    U = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0]
    gen = EigenvectorGenerator(LATT, MemGauge(gauge), NE, 1e-10, stencil_precision="fp32")
    gen.load("cfg1")
    X, lam = (a.cpu().numpy() for a in gen.calc(0))
    st = gen.last_stats
    assert st["converged"] and st["matvecs_fp32"] > 0 and st["matvecs_fp64"] > 0
    rv, re = R.eigensolve(U, LATT, NE, 1e-10)
    np.testing.assert_allclose(lam, re, rtol=1e-10, atol=0)
    Xf = X.reshape(NE, -1)
    res = np.linalg.norm(R.laplacian(Xf.T, U, LATT).T - lam[:, None] * Xf, axis=1)
    assert res.max() < 1e-9
    assert np.abs(Xf.conj() @ Xf.T - np.eye(NE)).max() < 1e-12
    Xt = torch.from_numpy(Xf).cuda()
    Rt = torch.from_numpy(np.ascontiguousarray(rv.reshape(NE, -1))).cuda()
    assert float((Xt.T @ Xt.conj() - Rt.T @ Rt.conj()).abs().max()) < 1e-7


@pytest.mark.parametrize("stencil", ["fp64", "fp32"])
def test_config1_double_float_gram_schmidt(stencil):
    """Gram-Schmidt in double-float arithmetic on the FP32 pipe
    (gs_precision="df", ED_LANCZOS_GS_DF), with the FP64 and the mixed
    stencil: the same checks against ARPACK as the FP64 passes."""
    from easydistillation_gb300 import EigenvectorGenerator

    gauge = _gauge()
    U = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0]
    gen = EigenvectorGenerator(LATT, MemGauge(gauge), NE, 1e-10, stencil_precision=stencil, gs_precision="df")
    gen.load("cfg1")
    X, lam = (a.cpu().numpy() for a in gen.calc(0))
    assert gen.last_stats["converged"]
    rv, re = R.eigensolve(U, LATT, NE, 1e-10)
    np.testing.assert_allclose(lam, re, rtol=1e-10, atol=0)
    Xf = X.reshape(NE, -1)
    res = np.linalg.norm(R.laplacian(Xf.T, U, LATT).T - lam[:, None] * Xf, axis=1)
    assert res.max() < 1e-9
    assert np.abs(Xf.conj() @ Xf.T - np.eye(NE)).max() < 1e-12
    Xt = torch.from_numpy(Xf).cuda()
    Rt = torch.from_numpy(np.ascontiguousarray(rv.reshape(NE, -1))).cuda()
    assert float((Xt.T @ Xt.conj() - Rt.T @ Rt.conj()).abs().max()) < 1e-7
