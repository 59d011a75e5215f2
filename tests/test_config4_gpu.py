"""Differentiation at its real size: 24^3 x 48, links exp(i 0.3 A),
Ne = 100, profile weights f(lambda_k) = exp(-lambda_k / sigma) w_k with
w_k ~ U(0.5, 1.5) and sigma = 1, a complex Gaussian perambulator
[48, 4, 4, 100, 100], and the loss log(C(6) / C(12)) of the meson two-point
function built from the elementals.  The gradients with respect to w and to
the gauge links, through the hand-written adjoints, must match central
finite differences (h = 1e-6) along random directions:
|fd - analytic| <= 1e-6 max(1, |analytic|)."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

REL = 1e-6


def test_correlator_loss_gradient_full_size_vs_finite_differences():
    from easydistillation_gb300.autograd import correlator_log_ratio
    from easydistillation_gb300.correlator import gamma
    from easydistillation_gb300.generator.elemental import links_to_device
    from easydistillation_gb300.synthetic import gauge_field

    dev = torch.device("cuda")
    latt = [24, 24, 24, 48]
    Lx, Ly, Lz, Lt = latt
    V3 = Lx * Ly * Lz
    Ne = 100
    g = gauge_field([Lx, Ly, Lz, 4], 0.3, 1004)
    U4 = links_to_device(g, [Lx, Ly, Lz, 4], dev)
    U = U4[:, torch.arange(Lt, device=dev) % 4].contiguous()
    gen = torch.Generator(device=dev).manual_seed(4006)
    V = torch.complex(torch.randn((Lt, Ne, V3 * 3), generator=gen, device=dev, dtype=torch.float64),
                      torch.randn((Lt, Ne, V3 * 3), generator=gen, device=dev, dtype=torch.float64))
    V /= (2 * V3 * 3) ** 0.5
    rng = np.random.default_rng(4004)
    w = torch.from_numpy(rng.uniform(0.5, 1.5, Ne)).to(dev)
    evals = torch.from_numpy(np.sort(rng.uniform(0.2, 0.6, (Lt, Ne)), axis=1)).to(dev)
    rng5 = np.random.default_rng(4005)
    tau = torch.from_numpy(rng5.standard_normal((Lt, 4, 4, Ne, Ne)) +
                           1j * rng5.standard_normal((Lt, 4, 4, Ne, Ne))).to(dev)
    g5 = gamma(15, dev)

    def loss(U_, w_):
        return correlator_log_ratio(U_, V, evals, w_, tau, latt, g5, d=1, t1=6, t2=12)

    U1 = U.clone().requires_grad_(True)
    w1 = w.clone().requires_grad_(True)
    L = loss(U1, w1)
    L.backward()
    assert torch.isfinite(L)
    h = 1e-6
    dU = torch.randn(U.shape, generator=gen, device=dev, dtype=torch.complex128)
    dw = torch.randn(w.shape, generator=gen, device=dev, dtype=torch.float64)
    with torch.no_grad():
        fdU = float((loss(U + h * dU, w) - loss(U - h * dU, w)) / (2 * h))
        fdw = float((loss(U, w + h * dw) - loss(U, w - h * dw)) / (2 * h))
    anU = float((U1.grad.conj() * dU).real.sum())
    anw = float((w1.grad * dw).sum())
    assert abs(anU - fdU) <= REL * max(1.0, abs(anU)), (anU, fdU)
    assert abs(anw - fdw) <= REL * max(1.0, abs(anw)), (anw, fdw)
