"""The native thick-restart Lanczos (``ed_lanczos_tr``) against the Python
driver of the same kernels and against itself with Chebyshev acceleration:
eigenvalues to 1e-10 relative, residuals ||L x - lambda x|| < 1e-9, the same
eigenspace, orthonormal vectors."""

import numpy as np
import pytest
import torch

from oracle import restatement as R

pytestmark = pytest.mark.gpu


def _links(latt, seed):
    from easydistillation_gb300.ops import links_to_soa

    g = R.synthetic_gauge(latt, 0.3, seed)
    U = torch.from_numpy(np.ascontiguousarray(g.transpose(4, 0, 1, 2, 3, 5, 6))).cuda()
    return links_to_soa(U, latt)


def _check_pairs(L, latt, evals, X):
    from easydistillation_gb300.ops import laplacian

    nt, Ne = evals.shape
    V3 = latt[0] * latt[1] * latt[2]
    LX = laplacian(L, X, latt)  # [nt, Ne, 3, V3]
    res = torch.linalg.vector_norm((LX - evals[:, :, None, None].to(X.dtype) * X).reshape(nt, Ne, -1), dim=2)
    assert float(res.max()) < 1e-9
    G = torch.einsum("tia,tja->tij", X.reshape(nt, Ne, -1).conj(), X.reshape(nt, Ne, -1))
    assert float((G - torch.eye(Ne, dtype=G.dtype, device=G.device)).abs().max()) < 1e-12
    assert bool((evals[:, 1:] >= evals[:, :-1]).all())


def test_native_matches_python_driver():
    from easydistillation_gb300.lanczos import trlanczos
    from easydistillation_gb300.ops import lanczos_tr, laplacian

    latt = [6, 6, 6, 2]
    V3 = 216
    L = _links(latt, 5)
    evals, X, st = lanczos_tr(L, latt, 16, 1e-11, ncv=40)
    assert st["converged"] and st["restarts"] > 1 and st["matvecs"] >= 40
    _check_pairs(L, latt, evals, X)

    def mv(Z):
        return laplacian(L, Z.contiguous().view(2, 1, 3, V3), latt).view(2, 3 * V3)

    ref = trlanczos(mv, 2, 3 * V3, 16, 1e-11, ncv=40)
    assert torch.allclose(evals, ref.evals, rtol=1e-10, atol=0)
    # same eigenspace: ||X_ref^H X||_F^2 = Ne
    M = torch.einsum("tia,tja->tij", ref.evecs.conj(), X.reshape(2, 16, -1))
    assert float((torch.linalg.matrix_norm(M) ** 2 - 16).abs().max()) < 1e-8


def test_native_chebyshev_and_batch_of_four():
    from easydistillation_gb300.ops import lanczos_tr

    latt = [8, 8, 6, 4]
    L = _links(latt, 6)
    ev0, X0, st0 = lanczos_tr(L, latt, 20, 1e-11)
    assert st0["converged"]
    _check_pairs(L, latt, ev0, X0)
    cut = 1.15 * float(ev0[:, -1].max())
    ev1, X1, st1 = lanczos_tr(L, latt, 20, 1e-12, poly_deg=8, lambda_cut=cut)
    assert st1["converged"]
    assert torch.allclose(ev1, ev0, rtol=1e-10, atol=0)
    _check_pairs(L, latt, ev1, X1)


def test_generator_native_and_python_drivers_agree():
    from easydistillation_gb300 import EigenvectorGenerator
    from tests.helpers import MemGauge

    latt = [6, 6, 4, 3]
    gauge = R.synthetic_gauge(latt, 0.3, 7)
    out = {}
    for drv in ("native", "python"):
        gen = EigenvectorGenerator(latt, MemGauge(gauge), 12, 1e-11, driver=drv)
        gen.load("k")
        out[drv] = gen.calc_batch([0, 2])
        assert gen.last_stats["converged"]
    vn, en = out["native"]
    vp, ep = out["python"]
    assert torch.allclose(en, ep, rtol=1e-10, atol=0)
    # renormalised phases: vectors of non-degenerate eigenvalues agree up to rounding
    gaps = (en[:, 1:] - en[:, :-1]).min()
    if float(gaps) > 1e-3:  # vector error ~ residual / gap
        assert float((vn - vp).abs().max()) < 1e-6
