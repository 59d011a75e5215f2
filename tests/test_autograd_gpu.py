"""Hand-written adjoints (torch.autograd.Function) against an einsum/roll
autograd reference of the same FP64 forward, and the correlator-based loss
against FP64 central finite differences (h = 1e-6) in the links and in the
profile weights.  Also the GPU correlator against the oracle's restatement
of lattice/correlator/one_particle.py."""

import numpy as np
import pytest
import torch

from oracle import restatement as R

pytestmark = pytest.mark.gpu


def _torch_hop(V, U, d):
    # V [Ne, Lz, Ly, Lx, 3], U [3, Lz, Ly, Lx, 3, 3]  (elemental.py:282-287)
    axis = 3 - d
    Vf = torch.roll(V, -1, axis)
    UVf = torch.einsum("zyxab,ezyxb->ezyxa", U[d], Vf)
    UdV = torch.einsum("zyxba,ezyxb->ezyxa", U[d].conj(), V)
    return UVf - torch.roll(UdV, 1, axis)


def _torch_elemental(U, V, latt, d, p):
    Ne = V.shape[0]
    ph = torch.from_numpy(R.momentum_phase(latt, p)).to(V.device)
    E = torch.zeros((Ne, Ne), dtype=torch.complex128, device=V.device)
    for coeff, lseq, rseq in R.elemental_pair_terms(R.derivative(d)):
        L, Rr = V, V
        for dd in lseq:
            L = _torch_hop(L, U, dd)
        for dd in rseq:
            Rr = _torch_hop(Rr, U, dd)
        E = E + coeff * torch.einsum("zyx,ezyxc,fzyxc->ef", ph, L.conj(), Rr)
    return E


@pytest.mark.parametrize("d", [0, 2, 5, 12])
@pytest.mark.parametrize("p", [(0, 0, 0), (1, 0, -1)])
def test_elemental_adjoint_matches_einsum_autograd(d, p):
    from easydistillation_gb300.autograd import elemental_op

    latt = [6, 4, 4, 1]
    Ne = 5
    U = torch.from_numpy(R.synthetic_gauge(latt, 0.3, 3).transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0].copy()).cuda()
    V = torch.from_numpy(R.random_colour_vectors(Ne, latt, 4)).cuda()
    Vr = V.to(torch.complex64).to(torch.complex128)
    G = torch.randn((Ne, Ne), dtype=torch.complex128, device="cuda")
    U1 = U.clone().requires_grad_(True)
    E1 = elemental_op(U1, V, latt, d, p)
    U2 = U.clone().requires_grad_(True)
    E2 = _torch_elemental(U2, Vr, latt, d, p)
    assert torch.linalg.vector_norm(E1 - E2) / torch.linalg.vector_norm(E2) < 1e-12
    (E1 * G.conj()).real.sum().backward()
    if d == 0:  # no derivative: the elemental does not depend on the links
        assert U1.grad is None or torch.count_nonzero(U1.grad) == 0
        return
    (E2 * G.conj()).real.sum().backward()
    g1, g2 = U1.grad, U2.grad
    assert torch.linalg.vector_norm(g1 - g2) / torch.linalg.vector_norm(g2) < 1e-11


def test_all_elementals_adjoint_matches_einsum_autograd():
    """Every operator of num_nabla = 2 and a momentum list closed under p -> -p
    (the plan then takes half the pairs from hermiticity): forward through the
    library's elemental plan, backward through the library's adjoint kernels,
    against torch autograd of the einsum/roll form of the reference."""
    from easydistillation_gb300.autograd import elementals

    latt = [4, 6, 4, 1]
    Ne = 4
    moms = [(0, 0, 0), (1, 0, -1), (-1, 0, 1), (0, 1, 0), (0, -1, 0)]
    U = torch.from_numpy(R.synthetic_gauge(latt, 0.3, 13).transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0].copy()).cuda()
    V = torch.from_numpy(R.random_colour_vectors(Ne, latt, 14)).cuda()
    Vr = V.to(torch.complex64).to(torch.complex128)
    G = torch.randn((13, len(moms), Ne, Ne), dtype=torch.complex128, device="cuda")
    U1 = U.clone().requires_grad_(True)
    E1 = elementals(U1, V, latt, 2, moms)
    U2 = U.clone().requires_grad_(True)
    E2 = torch.stack([torch.stack([_torch_elemental(U2, Vr, latt, d, p) for p in moms]) for d in range(13)])
    assert torch.linalg.vector_norm(E1 - E2) / torch.linalg.vector_norm(E2) < 1e-12
    (E1 * G.conj()).real.sum().backward()
    (E2 * G.conj()).real.sum().backward()
    assert torch.linalg.vector_norm(U1.grad - U2.grad) / torch.linalg.vector_norm(U2.grad) < 1e-11


def test_correlator_loss_gradients_vs_finite_differences():
    from easydistillation_gb300.autograd import correlator_log_ratio
    from easydistillation_gb300.correlator import gamma

    latt = [4, 4, 4, 16]
    Ne = 6
    gauge = R.synthetic_gauge(latt, 0.3, 21)
    U = torch.from_numpy(gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3].copy()).cuda()
    V = torch.from_numpy(np.stack([R.random_colour_vectors(Ne, latt, 30 + t) for t in range(latt[3])])).cuda()
    rng = np.random.default_rng(5)
    evals = torch.from_numpy(np.sort(rng.uniform(0.1, 1.0, (latt[3], Ne)), axis=1)).cuda()
    tau = torch.from_numpy(rng.standard_normal((latt[3], 4, 4, Ne, Ne)) +
                           1j * rng.standard_normal((latt[3], 4, 4, Ne, Ne))).cuda()
    w = torch.from_numpy(rng.uniform(0.5, 1.5, Ne)).cuda()
    g5 = gamma(15, "cuda")

    def loss(U_, w_):
        return correlator_log_ratio(U_, V, evals, w_, tau, latt, g5, d=1, t1=6, t2=12)

    U1 = U.clone().requires_grad_(True)
    w1 = w.clone().requires_grad_(True)
    L = loss(U1, w1)
    L.backward()
    h = 1e-6
    # links: a random complex direction
    dU = torch.randn_like(U)
    with torch.no_grad():
        fd = (loss(U + h * dU, w) - loss(U - h * dU, w)) / (2 * h)
    an = (U1.grad.conj() * dU).real.sum()
    assert abs(float(fd - an)) <= 1e-6 * max(1.0, abs(float(an)))
    # profile weights
    dw = torch.randn_like(w)
    with torch.no_grad():
        fdw = (loss(U, w + h * dw) - loss(U, w - h * dw)) / (2 * h)
    anw = (w1.grad * dw).sum()
    assert abs(float(fdw - anw)) <= 1e-6 * max(1.0, abs(float(anw)))


def test_twopoint_matches_oracle():
    from easydistillation_gb300.correlator import gamma, twopoint_assembled

    rng = np.random.default_rng(7)
    Lt, Ne, X = 6, 4, 2
    g = np.stack([R.gamma(15), R.gamma(1)])
    e = rng.standard_normal((X, Lt, Ne, Ne)) + 1j * rng.standard_normal((X, Lt, Ne, Ne))
    peram = rng.standard_normal((Lt, Lt, 4, 4, Ne, Ne)) + 1j * rng.standard_normal((Lt, Lt, 4, 4, Ne, Ne))
    ref = R.twopoint([(g, e)], peram, range(Lt), Lt)
    out = twopoint_assembled([(torch.from_numpy(g).cuda(), torch.from_numpy(e).cuda())],
                             torch.from_numpy(peram).cuda(), range(Lt), Lt)
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-11, atol=1e-11)
    np.testing.assert_allclose(gamma(7).numpy(), R.gamma(7), atol=0)
