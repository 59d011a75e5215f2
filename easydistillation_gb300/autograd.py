"""Differentiable elementals with hand-written adjoints (torch.autograd.Function).

``elemental_op(U_t, V, latt, d, p)`` returns the ``[Ne, Ne]`` elemental of
derivative operator ``d`` and momentum ``p`` on one timeslice
(``lattice/generator/elemental.py:290-338``), differentiable with respect to
the spatial links ``U_t`` (``[3, Lz, Ly, Lx, 3, 3]`` complex128).  The
eigenvectors are held fixed.  The backward pass is hand-written:

* for each left/right subset term ``c <L | phase_p | R>`` the adjoint seeds of
  the two chains are ``A = conj(phase) (G^T L)`` (right chain) and
  ``B = phase (conj(G) R)`` (left chain) -- two plain complex GEMMs;
* each chain ``F_m = D_{d_m} F_{m-1}`` is recomputed from ``V`` with the
  library's hop kernel (``D_op V`` is not stored), then walked backwards:
  the link-gradient kernel ``ed_link_grad`` adds
  ``Abar(x) F(x+d)^dag - F(x) Abar(x+d)^dag`` and the seed moves on as
  ``-D_d Abar`` (the covariant central difference is anti-Hermitian).

Gradients follow torch's complex convention, ``dL = Re sum conj(grad) dU``.
"""

from __future__ import annotations

from typing import Sequence

import torch

from . import _lib
from .insertion import derivative
from .ops import covariant_derivative, links_to_soa, momentum_phases, vectors_to_planes

NC = 3


def _subset_terms(deriv):
    """(coeff, left chain, right chain) of the reference's symmetric split
    (``elemental.py:309-321``)."""
    out = []
    for pick in range(2 ** len(deriv)):
        right, left = [], []
        for k, direction in enumerate(deriv):
            (right if (pick >> k) & 1 else left).append(direction)
        out.append(((-1) ** len(right), tuple(left[::-1]), tuple(right)))
    return out


def _chain(links_soa, V, latt, seq):
    """[F_0 = V, F_1, ..., F_n] with F_m = D_{seq[m-1]} F_{m-1}."""
    Fs = [V]
    for d in seq:
        Fs.append(covariant_derivative(links_soa, Fs[-1], latt, d))
    return Fs


def _backprop_chain(links_soa, Fs, seq, seed, grad_soa, latt):
    Lx, Ly, Lz = latt[0], latt[1], latt[2]
    Ne = seed.shape[0]
    abar = seed.contiguous()
    for m in range(len(seq) - 1, -1, -1):
        d = seq[m]
        _lib.call("ed_link_grad", Lx, Ly, Lz, d, Ne, 1.0, -1.0, _lib.ptr(abar), _lib.ptr(Fs[m]), _lib.ptr(grad_soa),
                  _lib.stream_handle())
        if m > 0:
            abar = -covariant_derivative(links_soa, abar, latt, d)


def _soa_to_links(grad_soa, latt):
    """[27, V3] SoA -> [3, Lz, Ly, Lx, 3, 3]."""
    Lx, Ly, Lz = latt[0], latt[1], latt[2]
    return grad_soa.view(3, 3, 3, Lz, Ly, Lx).permute(0, 3, 4, 5, 1, 2).contiguous()


def _forward_elemental(U_t, Vp, latt, d, p):
    links = links_to_soa(U_t.unsqueeze(1).contiguous(), list(latt[:3]) + [1])[0]
    ph = momentum_phases(latt, [p])[0].reshape(-1)  # [V3]
    Ne = Vp.shape[0]
    E = torch.zeros((Ne, Ne), dtype=torch.complex128, device=Vp.device)
    for coeff, lseq, rseq in _subset_terms(derivative(d)):
        L = _chain(links, Vp, latt, lseq)[-1]
        R = _chain(links, Vp, latt, rseq)[-1]
        Lp = (L * ph.view(1, 1, -1).conj()).reshape(Ne, -1)  # conj(L) phase = conj(L conj(phase))
        E += coeff * (Lp.conj() @ R.reshape(Ne, -1).T)
    return E, links, ph


class ElementalOpFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, U_t, Vp, latt, d, p):
        E, links, ph = _forward_elemental(U_t, Vp, latt, d, p)
        ctx.save_for_backward(U_t, Vp)
        ctx.latt, ctx.d, ctx.p = list(latt), d, tuple(p)
        return E

    @staticmethod
    def backward(ctx, G):
        U_t, Vp = ctx.saved_tensors
        latt, d, p = ctx.latt, ctx.d, ctx.p
        Lx, Ly, Lz = latt[0], latt[1], latt[2]
        V3 = Lx * Ly * Lz
        links = links_to_soa(U_t.unsqueeze(1).contiguous(), list(latt[:3]) + [1])[0]
        ph = momentum_phases(latt, [p])[0].reshape(1, 1, V3)
        Ne = Vp.shape[0]
        grad_soa = torch.zeros((27, V3), dtype=torch.complex128, device=Vp.device)
        G = G.contiguous()
        for coeff, lseq, rseq in _subset_terms(derivative(d)):
            Ls = _chain(links, Vp, latt, lseq)  # recomputed, not stored by the forward pass
            Rs = _chain(links, Vp, latt, rseq)
            Gc = coeff * G
            A = (Gc.T @ Ls[-1].reshape(Ne, -1)).reshape(Ne, NC, V3) * ph.conj()
            Bs = (Gc.conj() @ Rs[-1].reshape(Ne, -1)).reshape(Ne, NC, V3) * ph
            if rseq:
                _backprop_chain(links, Rs, rseq, A, grad_soa, latt)
            if lseq:
                _backprop_chain(links, Ls, lseq, Bs, grad_soa, latt)
        return _soa_to_links(grad_soa, latt), None, None, None, None


def elemental_op(U_t: torch.Tensor, V_ref: torch.Tensor, latt: Sequence[int], d: int, p: Sequence[int]):
    """Differentiable ``E[d, p]`` of one timeslice.  ``U_t``: ``[3, Lz, Ly, Lx, 3, 3]``
    complex128 (may require grad); ``V_ref``: ``[Ne, Lz, Ly, Lx, 3]`` (or
    ``[Ne, V3*3]``) eigenvectors, rounded to complex64 like the reference."""
    Lx, Ly, Lz = latt[0], latt[1], latt[2]
    V3 = Lx * Ly * Lz
    Ne = V_ref.shape[0]
    Vp = vectors_to_planes(V_ref.reshape(Ne, V3, NC).contiguous(), V3, torch.complex128, round_c64=True)
    return ElementalOpFunction.apply(U_t, Vp, list(latt), int(d), tuple(int(v) for v in p))


def profile_weights(evals: torch.Tensor, w: torch.Tensor, sigma: float = 1.0) -> torch.Tensor:
    """Distillation profile ``f(lambda_k) = exp(-lambda_k / sigma) * w_k``."""
    return torch.exp(-evals / sigma) * w


def correlator_log_ratio(U: torch.Tensor, V: torch.Tensor, evals: torch.Tensor, w: torch.Tensor, tau: torch.Tensor,
                         latt, gamma_op: torch.Tensor, d: int, p=(0, 0, 0), t_src: int = 0, t1: int = 6,
                         t2: int = 12, sigma: float = 1.0):
    """``log|C(t1)| - log|C(t2)|`` for a one-part meson operator (``gamma_op``,
    elemental ``d``/``p``) with profile-weighted elementals
    ``f_i E_t[i, j] f_j`` and the perambulator ``tau [Lt, 4, 4, Ne, Ne]`` of
    source ``t_src`` (the contraction of ``one_particle.py:64-72``).  Only the
    timeslices t_src, t_src+t1, t_src+t2 enter.  Differentiable in ``U``
    (``[3, Lt, Lz, Ly, Lx, 3, 3]``) and ``w``."""
    from .correlator import twopoint_source

    Lt = latt[3]
    Ne = V.shape[1]
    need = sorted({t_src % Lt, (t_src + t1) % Lt, (t_src + t2) % Lt})
    Es = {}
    for t in need:
        f = profile_weights(evals[t], w, sigma).to(torch.complex128)
        Es[t] = f[:, None] * elemental_op(U[:, t], V[t], latt, d, p) * f[None, :]
    zero = torch.zeros((Ne, Ne), dtype=torch.complex128, device=V.device)
    el = torch.stack([Es.get(t, zero) for t in range(Lt)]).unsqueeze(0)  # [1, Lt, Ne, Ne]
    ret = -twopoint_source(tau, gamma_op.unsqueeze(0), el, t_src)
    c1, c2 = ret[t1 % Lt], ret[t2 % Lt]
    return 0.5 * torch.log((c1 * c1.conj()).real) - 0.5 * torch.log((c2 * c2.conj()).real)
