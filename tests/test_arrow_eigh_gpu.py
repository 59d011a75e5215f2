"""The batched arrowhead + tridiagonal eigensolver (``ed_arrow_eigh``, the
projected eigenproblem of thick-restart Lanczos) against numpy's dense
eigh: eigenvalues to 1e-13 ||T||, residuals ||T y - lambda y|| and the
orthonormality of the vectors to 1e-12, including exactly degenerate and
nearly degenerate (Wilkinson) spectra; and Lanczos with it against Lanczos
with the dense eigh."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _dense(d, e, s):
    B, m = d.shape
    T = np.zeros((B, m, m))
    ka = 0 if s is None else s.shape[1]
    for b in range(B):
        T[b][np.arange(m), np.arange(m)] = d[b]
        for j in range(ka, m - 1):
            T[b, j, j + 1] = T[b, j + 1, j] = e[b, j]
        for j in range(ka):
            T[b, j, ka] = T[b, ka, j] = s[b, j]
    return T


def _check(d, e, s, nwant):
    from easydistillation_gb300.ops import arrow_eigh

    T = _dense(d, e, s)
    dev = lambda a: None if a is None else torch.from_numpy(np.ascontiguousarray(a)).cuda()
    lam, Y = arrow_eigh(dev(d), dev(e), dev(s), nwant=nwant)
    lam, Y = lam.cpu().numpy(), Y.cpu().numpy()
    for b in range(T.shape[0]):
        ref = np.linalg.eigvalsh(T[b])[:nwant]
        tn = np.abs(ref).max() + np.abs(T[b]).sum(1).max()
        assert np.abs(lam[b] - ref).max() <= 1e-13 * tn
        R = T[b] @ Y[b] - Y[b] * lam[b]
        assert np.linalg.norm(R, axis=0).max() <= 1e-12 * tn
        assert np.abs(Y[b].T @ Y[b] - np.eye(nwant)).max() <= 1e-12
    return lam, Y


@pytest.mark.parametrize("m,ka,nwant", [(1, 0, 1), (2, 0, 2), (60, 0, 60), (60, 0, 25), (80, 30, 45), (300, 200, 200),
                                        (64, 63, 40)])
def test_random_arrow_matrices(m, ka, nwant):
    rng = np.random.default_rng(m + ka)
    B = 3
    d = rng.uniform(0.0, 12.0, (B, m))
    d[:, :ka] = np.sort(rng.uniform(0.2, 0.6, (B, ka)), axis=1)  # kept Ritz values
    e = np.zeros((B, m - 1))
    e[:, ka:] = rng.uniform(0.5, 3.0, (B, m - 1 - ka))
    s = rng.standard_normal((B, ka)) * np.logspace(-12, -1, ka) if ka else None  # converged ones have tiny borders
    _check(d, e, s, nwant)


def test_degenerate_and_clustered_spectra():
    """Exactly repeated decoupled Ritz values (zero border), borders at the
    rounding level, and the Wilkinson matrix W21+ (pairs of eigenvalues
    1e-14 .. 1e-6 apart)."""
    m, ka = 50, 12
    d = np.zeros((2, m))
    e = np.zeros((2, m - 1))
    d[0, :ka] = [0.5] * 4 + [0.7] * 3 + [0.9, 0.9, 1.1, 1.1, 1.3]
    s0 = np.zeros((2, ka))
    s0[0, 4:7] = 1e-17
    d[0, ka:] = np.linspace(0.1, 5.0, m - ka)
    e[0, ka:] = 0.8
    d[1, :ka] = np.linspace(0.3, 0.8, ka)
    s0[1] = 1e-9
    d[1, ka:] = 2.0
    e[1, ka:] = 1.0
    _check(d, e, s0, 40)
    w = np.abs(np.arange(-10, 11)).astype(float)
    _check(w[None], np.ones((1, 20)), None, 21)


def test_lanczos_arrow_matches_dense_eigh():
    """Thick-restart Lanczos on the 6^3 covariant Laplacian (several restarts)
    with the arrow eigensolver against the same run with torch's dense eigh."""
    from easydistillation_gb300.lanczos import trlanczos
    from easydistillation_gb300.ops import laplacian, links_to_soa
    from oracle import restatement as R

    latt = [6, 6, 6, 2]
    V3 = 216
    g = R.synthetic_gauge(latt, 0.3, 3)
    U = torch.from_numpy(np.ascontiguousarray(g.transpose(4, 0, 1, 2, 3, 5, 6))).cuda()
    L = links_to_soa(U, latt)

    def mv(X):  # colour-plane vectors [2, 3*V3], one per timeslice
        return laplacian(L, X.contiguous().view(2, 1, 3, V3), latt).view(2, 3 * V3)

    a = trlanczos(mv, 2, 3 * V3, 20, 1e-11, ncv=36, small_eigh="arrow")
    b = trlanczos(mv, 2, 3 * V3, 20, 1e-11, ncv=36, small_eigh="dense")
    assert a.converged and b.converged and a.restarts > 2
    assert torch.allclose(a.evals, b.evals, rtol=1e-11, atol=0)
    x0 = a.evecs[:, 0]
    res = torch.linalg.vector_norm(mv(x0) - a.evals[:, :1].to(x0.dtype) * x0, dim=1)
    assert float(res.max()) < 1e-9


@pytest.mark.parametrize("B,rows,r,n", [(3, 9, 7, 1000), (2, 40, 33, 3 * 216), (1, 5, 5, 17), (2, 1500, 1100, 64)])
def test_cgs_pass_matches_torch(B, rows, r, n):
    """The batched Gram-Schmidt kernel against torch GEMVs, on a basis view
    whose batch stride exceeds r*n (rows beyond r are never read)."""
    from easydistillation_gb300.ops import cgs_pass

    g = torch.Generator(device="cuda").manual_seed(r)
    V = torch.randn((B, rows + 1, n), dtype=torch.complex128, device="cuda", generator=g)
    w = torch.randn((B, n), dtype=torch.complex128, device="cuda", generator=g)
    Vj = V[:, :r]
    h_ref = torch.bmm(w.unsqueeze(1).conj(), Vj.transpose(1, 2)).conj().squeeze(1)
    w_ref = w - torch.bmm(h_ref.unsqueeze(1), Vj).squeeze(1)
    w2 = w.clone()
    h, nrm = cgs_pass(Vj, r, w2, norm=True)
    scale = float(torch.linalg.vector_norm(w)) * float(torch.linalg.vector_norm(Vj))
    assert float(torch.linalg.vector_norm(h - h_ref)) <= 1e-13 * scale
    assert float(torch.linalg.vector_norm(w2 - w_ref)) <= 1e-13 * scale * r ** 0.5
    assert torch.allclose(nrm, torch.linalg.vector_norm(w2, dim=1), rtol=1e-13, atol=0)


@pytest.mark.parametrize("B,rows,r,n", [(3, 9, 7, 1000), (2, 40, 33, 3 * 216), (1, 5, 5, 17), (2, 1500, 1100, 64)])
def test_cgs_pass_df_matches_torch(B, rows, r, n):
    """The double-float Gram-Schmidt pass (FP32 pipe, values split into two
    complex64 parts, (hi, lo) sums) against torch's FP64 GEMVs: products err by
    ~2^-47 relative, so the pass agrees to ~1e-13 of the scale."""
    from easydistillation_gb300.ops import cgs_pass

    g = torch.Generator(device="cuda").manual_seed(r + 1)
    V = torch.randn((B, rows + 1, n), dtype=torch.complex128, device="cuda", generator=g)
    w = torch.randn((B, n), dtype=torch.complex128, device="cuda", generator=g)
    Vj = V[:, :r]
    h_ref = torch.bmm(w.unsqueeze(1).conj(), Vj.transpose(1, 2)).conj().squeeze(1)
    w_ref = w - torch.bmm(h_ref.unsqueeze(1), Vj).squeeze(1)
    w2 = w.clone()
    h, nrm = cgs_pass(Vj, r, w2, norm=True, precision="df")
    scale = float(torch.linalg.vector_norm(w)) * float(torch.linalg.vector_norm(Vj))
    assert float(torch.linalg.vector_norm(h - h_ref)) <= 2e-13 * scale
    assert float(torch.linalg.vector_norm(w2 - w_ref)) <= 2e-13 * scale * r ** 0.5
    assert torch.allclose(nrm, torch.linalg.vector_norm(w2, dim=1), rtol=1e-13, atol=0)


def test_lanczos_gs_kernel_matches_torch_gemv():
    from easydistillation_gb300.lanczos import trlanczos
    from easydistillation_gb300.ops import laplacian, links_to_soa
    from oracle import restatement as R

    latt = [6, 6, 6, 2]
    V3 = 216
    g = R.synthetic_gauge(latt, 0.3, 4)
    U = torch.from_numpy(np.ascontiguousarray(g.transpose(4, 0, 1, 2, 3, 5, 6))).cuda()
    L = links_to_soa(U, latt)

    def mv(X):
        return laplacian(L, X.contiguous().view(2, 1, 3, V3), latt).view(2, 3 * V3)

    a = trlanczos(mv, 2, 3 * V3, 16, 1e-11, ncv=40, gs_kernel=True)
    b = trlanczos(mv, 2, 3 * V3, 16, 1e-11, ncv=40, gs_kernel=False)
    assert a.converged and b.converged
    assert torch.allclose(a.evals, b.evals, rtol=1e-11, atol=0)
