"""Differentiable elementals with hand-written adjoints (torch.autograd.Function).

``elementals(U_t, V, latt, num_nabla, momenta)`` returns every elemental
``E[d, p]`` (``[Nderiv, Nmom, Ne, Ne]``) of one timeslice
(``lattice/generator/elemental.py:290-338``), differentiable with respect to
the spatial links ``U_t`` (``[3, Lz, Ly, Lx, 3, 3]`` complex128); the
eigenvectors are held fixed.  ``elemental_op(U_t, V, latt, d, p)`` is one
``[Ne, Ne]`` block of it.

Forward: the library's FP64 elemental plan (``ed_elemental_run``: every
derivative chain built once, the distinct (left, right) chain pairs
contracted by the library's pair GEMM, the operator terms combined).

Backward, all in the library's kernels, with ``D_op V`` recomputed rather
than stored:

* the loss gradient of each ordered chain pair (X, Y) is
  ``Gbar_p(X, Y) = sum over the operator terms c * Ebar[d, p]`` of the
  reference's left/right split (``elemental.py:309-321``);
* the adjoint seed of every chain C, ``sum_p (Gbar_p(X, C)^T X) conj(phase_p)``
  over its left partners plus ``sum_p (conj(Gbar_p(C, Y)) Y) phase_p`` over
  its right partners, is one gather-GEMM launch (``ed_chain_adjoint``);
* the chains are rebuilt from V with the hop kernel and the seeds walked down
  the chain tree from the longest chains: each chain
  ``F_C = D_dir F_parent`` adds ``seed(x) F_parent(x+dir)^dag -
  F_parent(x) seed(x+dir)^dag`` to the link gradient (``ed_link_grad``) and
  passes ``-D_dir seed`` to its parent (the covariant central difference is
  anti-Hermitian).

Gradients follow torch's complex convention, ``dL = Re sum conj(grad) dU``.
"""

from __future__ import annotations

from typing import Dict, Sequence, Tuple

import torch

from . import _lib
from .insertion import derivative, num_derivative
from .ops import ElementalPlan, covariant_derivative, links_to_soa, momentum_phases, vectors_to_planes

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


def _chain_id(seq) -> int:
    """Index of a direction sequence in the derivative numbering (``derivative.py:23-33``)."""
    base, p3, v = 0, 1, 0
    for _ in seq:
        base += p3
        p3 *= 3
    for d in seq:
        v = v * 3 + d
    return base + v


def _soa_to_links(grad_soa, latt):
    """[27, V3] SoA -> [3, Lz, Ly, Lx, 3, 3]."""
    Lx, Ly, Lz = latt[0], latt[1], latt[2]
    return grad_soa.view(3, 3, 3, Lz, Ly, Lx).permute(0, 3, 4, 5, 1, 2).contiguous()


_PLANS: Dict[Tuple, ElementalPlan] = {}


def _plan(latt, Ne, num_nabla, moms, device) -> ElementalPlan:
    key = (tuple(latt[:3]), Ne, num_nabla, tuple(moms), str(device))
    if key not in _PLANS:
        _PLANS[key] = ElementalPlan(list(latt[:3]) + [1], Ne, num_nabla, list(moms), "fp64", device)
    return _PLANS[key]


def _chains(links_soa, V_ref, latt, nchain):
    """Colour-plane chains [nchain, Ne, 3, V3] (complex128; chain 0 is V rounded
    to complex64, chain c = D_dir(c) chain parent(c))."""
    Lx, Ly, Lz = latt[0], latt[1], latt[2]
    V3 = Lx * Ly * Lz
    Ne = V_ref.shape[0]
    out = torch.empty((nchain, Ne, NC, V3), dtype=torch.complex128, device=V_ref.device)
    out[0] = vectors_to_planes(V_ref.reshape(Ne, V3, NC).contiguous(), V3, torch.complex128, round_c64=True)
    for c in range(1, nchain):
        seq = derivative(c)
        out[c] = covariant_derivative(links_soa, out[_chain_id(seq[:-1])], latt, seq[-1])
    return out


class ElementalsFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, U_t, V_ref, latt, num_nabla, moms):
        Lx, Ly, Lz = latt[0], latt[1], latt[2]
        V3 = Lx * Ly * Lz
        Ne = V_ref.shape[0]
        plan = _plan(latt, Ne, num_nabla, moms, U_t.device)
        E = torch.empty((num_derivative(num_nabla), len(moms), Ne, Ne), dtype=torch.complex128, device=U_t.device)
        plan.run(U_t.detach().contiguous(), V3 * 9, 9, V_ref.reshape(Ne, V3 * NC).contiguous(), E)
        ctx.save_for_backward(U_t, V_ref)
        ctx.latt, ctx.num_nabla, ctx.moms = list(latt), num_nabla, list(moms)
        return E

    @staticmethod
    def backward(ctx, Ebar):
        U_t, V_ref = ctx.saved_tensors
        latt, num_nabla, moms = ctx.latt, ctx.num_nabla, ctx.moms
        Lx, Ly, Lz = latt[0], latt[1], latt[2]
        V3 = Lx * Ly * Lz
        Ne, nmom, dev = V_ref.shape[0], len(moms), V_ref.device
        nchain = num_derivative(num_nabla)
        Ebar = Ebar.contiguous()
        links = links_to_soa(U_t.detach().unsqueeze(1).contiguous(), list(latt[:3]) + [1])[0]
        chains = _chains(links, V_ref, latt, nchain)  # recomputed, not stored by the forward pass
        phases = momentum_phases(latt, moms, dev).reshape(nmom, V3)
        # loss gradient of every ordered chain pair, summed over the operator terms that use it; operators whose
        # gradient is zero (a loss built from a few elementals) contribute no pairs
        live = (Ebar.abs().amax(dim=(1, 2, 3)) > 0).tolist()
        gbar: Dict[Tuple[int, int], torch.Tensor] = {}
        for d in range(nchain):
            if not live[d]:
                continue
            for coeff, lseq, rseq in _subset_terms(derivative(d)):
                key = (_chain_id(lseq), _chain_id(rseq))
                term = coeff * Ebar[d]
                gbar[key] = term if key not in gbar else gbar[key] + term
        seeds = torch.zeros((nchain, Ne, NC, V3), dtype=torch.complex128, device=dev)
        ar_p = torch.arange(nmom, dtype=torch.int32).repeat_interleave(Ne)
        ar_i = torch.arange(Ne, dtype=torch.int32).repeat(nmom)
        for c in range(nchain):
            Ms, cxs, irs, prs = [], [], [], []
            for (X, Y), gb in gbar.items():
                if Y == c:  # c as the right chain: rows (X, p, i), M = Gbar_p[i][.], conj phases
                    Ms.append(gb.reshape(nmom * Ne, Ne))
                    cxs.append(torch.full((nmom * Ne,), X, dtype=torch.int32))
                    irs.append(ar_i)
                    prs.append(-ar_p - 1)
                if X == c:  # c as the left chain: rows (Y, p, j), M = conj(Gbar_p[.][j]), phases
                    Ms.append(gb.conj().transpose(1, 2).reshape(nmom * Ne, Ne))
                    cxs.append(torch.full((nmom * Ne,), Y, dtype=torch.int32))
                    irs.append(ar_i)
                    prs.append(ar_p)
            if not Ms:
                continue
            M = torch.cat(Ms).contiguous()
            idx = torch.stack([torch.cat(cxs), torch.cat(irs), torch.cat(prs)]).to(dev)
            _lib.call("ed_chain_adjoint", Lx, Ly, Lz, Ne, nchain, nmom, M.shape[0], _lib.ptr(M),
                      _lib.ptr(idx[0]), _lib.ptr(idx[1]), _lib.ptr(idx[2]), _lib.ptr(chains), _lib.ptr(phases),
                      _lib.ptr(seeds[c]), _lib.stream_handle())
        grad_soa = torch.zeros((27, V3), dtype=torch.complex128, device=dev)
        for c in range(nchain - 1, 0, -1):  # children have larger indices than their parents
            seq = derivative(c)
            parent, d = _chain_id(seq[:-1]), seq[-1]
            _lib.call("ed_link_grad", Lx, Ly, Lz, d, Ne, 1.0, -1.0, _lib.ptr(seeds[c]), _lib.ptr(chains[parent]),
                      _lib.ptr(grad_soa), _lib.stream_handle())
            if parent > 0:
                seeds[parent] -= covariant_derivative(links, seeds[c], latt, d)
        return _soa_to_links(grad_soa, latt), None, None, None, None


def elementals(U_t: torch.Tensor, V_ref: torch.Tensor, latt: Sequence[int], num_nabla: int, momenta):
    """Differentiable ``E[d, p]`` of one timeslice for every derivative operator
    of ``num_nabla`` and every momentum: ``[Nderiv, Nmom, Ne, Ne]``.  ``U_t``:
    ``[3, Lz, Ly, Lx, 3, 3]`` complex128 (may require grad); ``V_ref``:
    ``[Ne, Lz, Ly, Lx, 3]`` (or ``[Ne, V3*3]``) complex128 eigenvectors, rounded
    to complex64 like the reference."""
    moms = [tuple(int(v) for v in p) for p in momenta]
    return ElementalsFunction.apply(U_t, V_ref, list(latt), int(num_nabla), moms)


def elemental_op(U_t: torch.Tensor, V_ref: torch.Tensor, latt: Sequence[int], d: int, p: Sequence[int]):
    """Differentiable ``E[d, p]`` of one timeslice (one ``[Ne, Ne]`` block of
    :func:`elementals` with the smallest ``num_nabla`` that holds ``d``)."""
    return elementals(U_t, V_ref, latt, len(derivative(int(d))), [p])[int(d), 0]


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
