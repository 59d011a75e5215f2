"""Plain numpy/scipy restatement of the reference hot path (test infrastructure).

Every function names the reference file:line range it restates; paths are
relative to the EasyDistillation source tree (``lattice/...``).  Layout
conventions follow the reference exactly:

* gauge field as loaded: ``[Lt, Lz, Ly, Lx, Nd, 3, 3]`` (ILDG/Chroma order),
  transposed by the generators to ``[Nd, Lt, Lz, Ly, Lx, 3, 3]``
  (``lattice/generator/eigenvector.py:50``, ``elemental.py:103``);
* one timeslice of spatial links: ``U_t = U[:3, t]`` with shape
  ``[3, Lz, Ly, Lx, 3, 3]`` (direction 0 = x, 1 = y, 2 = z);
* colour vectors: ``[Ne, Lz, Ly, Lx, 3]``, lexicographic with x fastest;
* elementals per timeslice: ``[Nderiv, Nmom, Ne, Ne]`` complex128.

This module is imported only by tests, the smoke check and the CPU-baseline
leg of the benchmark.
"""

from __future__ import annotations

import math
from typing import List, Optional, Sequence, Tuple

import numpy as np

NC = 3
ND = 4

__all__ = [
    "NC",
    "ND",
    "derivative",
    "num_derivative",
    "mom_dict_to_list",
    "momentum_phase",
    "laplacian",
    "nD",
    "covariant_derivative",
    "elemental",
    "elemental_pair_terms",
    "elemental_items",
    "elemental_item_into",
    "blending_coeff",
    "displacement_elemental",
    "eigensolve",
    "synthetic_gauge",
    "gell_mann",
    "stout_smear",
    "random_colour_vectors",
    "gamma",
    "twopoint",
    "operator_parts",
    "elemental_data",
    "twopoint_operators",
    "twopoint_profile_operators",
    "project_su3",
]


# ---------------------------------------------------------------------------
# operator metadata
# ---------------------------------------------------------------------------


def derivative(n: int) -> Tuple[int, ...]:
    """Index -> direction tuple (``lattice/insertion/derivative.py:23-33``).

    0 -> (); 1,2,3 -> (0,),(1,),(2,); 4+3a+b -> (a, b).  The base-3 digits of
    ``n - (1 + 3 + ... )`` read most-significant first.
    """
    if n < 0:
        raise ValueError("derivative index must be >= 0")
    length = 0
    block = 1
    while n >= block:
        n -= block
        length += 1
        block *= 3
    digits = []
    for _ in range(length):
        digits.append(n % 3)
        n //= 3
    return tuple(digits[::-1])


def num_derivative(num_nabla: int) -> int:
    """``(3**(num_nabla+1) - 1) // 2`` operators (``elemental.py:48``)."""
    return (3 ** (num_nabla + 1) - 1) // 2


_MOM3 = [
    "0 0 0", "0 0 1", "0 0 -1", "0 1 0", "0 -1 0", "1 0 0", "-1 0 0",
    "0 1 1", "0 1 -1", "0 -1 1", "0 -1 -1", "1 0 1", "1 0 -1", "-1 0 1",
    "-1 0 -1", "1 1 0", "1 -1 0", "-1 1 0", "-1 -1 0", "1 1 1", "1 1 -1",
    "1 -1 1", "1 -1 -1", "-1 1 1", "-1 1 -1", "-1 -1 1", "-1 -1 -1",
]


def mom_dict_to_list(mom: int = 3) -> List[Tuple[int, int, int]]:
    """The |p|^2 <= 3 momentum list in the reference's order
    (``lattice/insertion/mom_dict.py:5-33,162-175``).  Only ``mom`` 1 and 3
    are restated (the hot path uses these)."""
    if mom == 1:
        return [(0, 0, 0)]
    if mom == 3:
        return [tuple(int(v) for v in s.split(" ")) for s in _MOM3]
    raise ValueError(f"Unknown mom max = {mom}")


def momentum_phase(latt_size: Sequence[int], p: Sequence[int]) -> np.ndarray:
    """``exp(+2*pi*i*(px*x/Lx + py*y/Ly + pz*z/Lz))`` on ``[Lz, Ly, Lx]``.

    Restates ``lattice/insertion/phase.py:11-13`` (coordinate tables scaled
    by ``2j*pi/L``) and ``:41-46`` (``exp(npx*x + npy*y + npz*z)``).  The sign
    is +i, as in the reference.
    """
    Lx, Ly, Lz = latt_size[0], latt_size[1], latt_size[2]
    x = np.arange(Lx).reshape(1, 1, Lx) * 2j * np.pi / Lx
    y = np.arange(Ly).reshape(1, Ly, 1) * 2j * np.pi / Ly
    z = np.arange(Lz).reshape(Lz, 1, 1) * 2j * np.pi / Lz
    x = np.broadcast_to(x, (Lz, Ly, Lx))
    y = np.broadcast_to(y, (Lz, Ly, Lx))
    z = np.broadcast_to(z, (Lz, Ly, Lx))
    px, py, pz = p
    return np.exp(px * x + py * y + pz * z)


# ---------------------------------------------------------------------------
# stencils
# ---------------------------------------------------------------------------


def _mat_vec(U: np.ndarray, F: np.ndarray) -> np.ndarray:
    """site-wise ``U[z,y,x] @ F[z,y,x,:,...]`` for F ``[Lz,Ly,Lx,3,n]``."""
    return np.einsum("zyxab,zyxbn->zyxan", U, F)


def laplacian(F: np.ndarray, U_t: np.ndarray, latt_size: Sequence[int]) -> np.ndarray:
    """3D covariant Laplacian (``lattice/generator/eigenvector.py:11-26``).

    ``L F = 6 F - sum_mu [ U_mu(x) F(x+mu) + U_mu(x-mu)^dag F(x-mu) ]`` with
    periodic boundaries.  ``F`` is ``[V3*3, nvec]`` (site-major, colour, then
    vector index fastest) or anything reshapeable to it; returns the same
    ``[V3*3, nvec]`` shape.  ``U_t`` is ``[3, Lz, Ly, Lx, 3, 3]``.
    """
    Lx, Ly, Lz = latt_size[0], latt_size[1], latt_size[2]
    F = np.asarray(F).reshape(Lz, Ly, Lx, NC, -1)
    U_dag = U_t.transpose(0, 1, 2, 3, 5, 4).conj()
    acc = 6 * F
    for mu, axis in ((0, 2), (1, 1), (2, 0)):
        acc = acc - _mat_vec(U_t[mu], np.roll(F, -1, axis))
        acc = acc - np.roll(_mat_vec(U_dag[mu], F), 1, axis)
    return acc.reshape(Lz * Ly * Lx * NC, -1)


def covariant_derivative(V: np.ndarray, U_t: np.ndarray, d: int) -> np.ndarray:
    """One hop ``D_d V(x) = U_d(x) V(x+d) - U_d(x-d)^dag V(x-d)`` with no 1/2
    (``lattice/generator/elemental.py:282-287``).  ``V`` is ``[Ne,Lz,Ly,Lx,3]``."""
    axis = 3 - d
    Vf = np.roll(V, -1, axis)
    UVf = np.einsum("zyxab,ezyxb->ezyxa", U_t[d], Vf)
    UdV = np.einsum("zyxba,ezyxb->ezyxa", U_t[d].conj(), V)
    return UVf - np.roll(UdV, 1, axis)


def nD(V: np.ndarray, U_t: np.ndarray, deriv: Sequence[int]) -> np.ndarray:
    """Chain of hops applied left to right in tuple order
    (``lattice/generator/elemental.py:279-288``)."""
    for d in deriv:
        V = covariant_derivative(V, U_t, d)
    return V


# ---------------------------------------------------------------------------
# elementals
# ---------------------------------------------------------------------------


def elemental_pair_terms(deriv: Sequence[int]):
    """The symmetric left/right split of one derivative tuple
    (``lattice/generator/elemental.py:309-321``).

    Yields ``(coeff, left_chain, right_chain)``: for each of the ``2**len``
    subsets (bit k of the subset picks direction k for the right side), the
    right chain keeps its directions in order, the left chain takes the rest
    in reversed order, and ``coeff = (-1)**len(right)``.
    """
    out = []
    for pick_nabla in range(2 ** len(deriv)):
        pick_right, pick_left = [], []
        pick = pick_nabla
        for direction in deriv:
            if pick & 1:
                pick_right.append(direction)
            else:
                pick_left.append(direction)
            pick >>= 1
        out.append(((-1) ** len(pick_right), tuple(pick_left[::-1]), tuple(pick_right)))
    return out


def blending_coeff(Ne: int, dilution) -> np.ndarray:
    """Stochastic blending coefficients (``lattice/generator/elemental.py:61-95``)."""
    totNe_list = dilution[0]
    if isinstance(dilution[1], int):
        usedNe_list = [dilution[1]] * len(dilution[0])
    else:
        usedNe_list = list(dilution[1])
    assert len(usedNe_list) == len(totNe_list)
    assert all(u <= t for u, t in zip(usedNe_list, totNe_list))
    assert sum(usedNe_list) == Ne
    coeff = np.zeros((Ne, Ne))
    s1 = 0
    for nv1, (u1, t1) in enumerate(zip(usedNe_list, totNe_list)):
        s2 = 0
        for nv2, (u2, t2) in enumerate(zip(usedNe_list, totNe_list)):
            if nv1 != nv2:
                coeff[s1 : s1 + u1, s2 : s2 + u2] = t1 * t2 / u1 / u2
            else:
                c1 = t1 / u1
                c2 = c1 * (t1 - 1) / (u1 - 1)
                block = np.full((u1, u2), c2)
                np.fill_diagonal(block, c1)
                coeff[s1 : s1 + u1, s2 : s2 + u2] = block
            s2 += u2
        s1 += u1
    return coeff


def elemental_items(num_nabla: int):
    """The work items of one reference timeslice in its loop order
    (``lattice/generator/elemental.py:299-321``): one ``(operator, coeff,
    left_chain, right_chain)`` per derivative operator and left/right subset
    (43 items for ``num_nabla = 2``)."""
    return [(di, coeff, left, right) for di in range(num_derivative(num_nabla))
            for coeff, left, right in elemental_pair_terms(derivative(di))]


def elemental_item_into(out, Vc, U_t, item, phases, stocastic_coeff=None):
    """Add one work item of ``ElementalGenerator.calc`` into ``out``
    (``lattice/generator/elemental.py:320-337``): build its two chains from the
    (complex64-rounded, complex128) vectors ``Vc`` as the reference does, then
    one phase-weighted zgemm per momentum."""
    di, coeff, left_chain, right_chain = item
    Ne = Vc.shape[0]
    right = nD(Vc, U_t, right_chain).reshape(Ne, -1)
    left = nD(Vc, U_t, left_chain)
    for pi, ph in enumerate(phases):
        # opt_einsum evaluates "zyx,ezyxc,fzyxc->ef" as an elementwise
        # phase * conj(left) followed by a tensordot (zgemm).
        lp = (coeff * ph[None, :, :, :, None] * left.conj()).reshape(Ne, -1)
        blk = lp @ right.T
        if stocastic_coeff is not None:
            blk = blk * stocastic_coeff
        out[di, pi] += blk


def elemental(
    V: np.ndarray,
    U_t: np.ndarray,
    latt_size: Sequence[int],
    num_nabla: int,
    momentum_list: Sequence[Sequence[int]],
    stocastic_coeff: Optional[np.ndarray] = None,
    round_to_c64: bool = True,
) -> np.ndarray:
    """One timeslice of ``ElementalGenerator.calc``
    (``lattice/generator/elemental.py:290-338``).

    ``V`` is ``[Ne, Lz, Ly, Lx, 3]``; the reference stores it in a complex64
    buffer (``elemental.py:55,297-298``), so it is rounded to c64 first and
    all later arithmetic is complex128 (links and phases are c128).
    Returns ``[Nderiv, Nmom, Ne, Ne]`` complex128 with
    ``E[d,p,i,j] = sum_subsets coeff * sum_x phase_p(x) conj(L_i(x)) . R_j(x)``.
    """
    if round_to_c64:
        V = np.asarray(V).astype(np.complex64)
    Vc = V.astype(np.complex128)
    Ne = V.shape[0]
    nmom = len(momentum_list)
    phases = [momentum_phase(latt_size, p) for p in momentum_list]
    out = np.zeros((num_derivative(num_nabla), nmom, Ne, Ne), np.complex128)
    for item in elemental_items(num_nabla):
        elemental_item_into(out, Vc, U_t, item, phases, stocastic_coeff)
    return out


def displacement_elemental(
    V: np.ndarray,
    U_t: np.ndarray,
    latt_size: Sequence[int],
    distance: int,
    momentum_list: Sequence[Sequence[int]],
) -> np.ndarray:
    """``DisplacementElementalGenerator.calc`` for one timeslice
    (``lattice/generator/displacement_elemental.py:53-96``).

    ``right = mean over the 6 straight-line displacements by `dist` hops``;
    returns ``[distance+1, Nmom, Ne, Ne]``.
    """
    V = np.asarray(V).astype(np.complex64).astype(np.complex128)
    Ne = V.shape[0]
    out = np.zeros((distance + 1, len(momentum_list), Ne, Ne), np.complex128)
    Vd = np.zeros((6,) + V.shape, np.complex128)
    for dist in range(distance + 1):
        if dist == 0:
            right = V
        else:
            for d in range(3):
                axis = 3 - d
                src_f = V if dist == 1 else Vd[d]
                src_b = V if dist == 1 else Vd[-d - 1]
                Vd[d] = np.einsum("zyxab,ezyxb->ezyxa", U_t[d], np.roll(src_f, -1, axis))
                UdV = np.einsum("zyxba,ezyxb->ezyxa", U_t[d].conj(), src_b)
                Vd[-d - 1] = np.roll(UdV, 1, axis)
            right = Vd.mean(0)
        for pi, p in enumerate(momentum_list):
            ph = momentum_phase(latt_size, p)
            lp = (ph[None, :, :, :, None] * V.conj()).reshape(Ne, -1)
            out[dist, pi] += lp @ right.reshape(Ne, -1).T
    return out


# ---------------------------------------------------------------------------
# eigensolve
# ---------------------------------------------------------------------------


def eigensolve(
    U_t: np.ndarray,
    latt_size: Sequence[int],
    Ne: int,
    tol: float,
    apply_renorm_phase: bool = True,
):
    """``EigenvectorGenerator.laplacian_cupy_numpy`` on the numpy backend
    (``lattice/generator/eigenvector.py:234-257``).

    scipy ``eigsh(LinearOperator, Ne, which="SA", tol)`` (ARPACK, third-party),
    eigenvalues sorted ascending, then each vector multiplied by
    ``exp(-i*angle(v[0]))`` so that site 0 colour 0 is real and positive.
    Returns ``(evecs [Ne, Lz, Ly, Lx, 3] c128, evals [Ne] f64)``.
    """
    from scipy.sparse import linalg

    Lx, Ly, Lz = latt_size[0], latt_size[1], latt_size[2]
    n = Lz * Ly * Lx * NC

    def mv(F):
        return laplacian(F, U_t, latt_size)

    A = linalg.LinearOperator((n, n), matvec=mv, matmat=mv, dtype=np.complex128)
    evals, evecs = linalg.eigsh(A, Ne, which="SA", tol=tol)
    evecs = evecs.transpose(1, 0).reshape(Ne, -1)
    order = np.argsort(evals)
    evals, evecs = evals[order], evecs[order]
    if apply_renorm_phase:
        evecs = evecs * np.exp(-1.0j * np.angle(evecs[:, 0]))[:, None]
    return evecs.reshape(Ne, Lz, Ly, Lx, NC), evals


# ---------------------------------------------------------------------------
# synthetic inputs
# ---------------------------------------------------------------------------


def gell_mann() -> np.ndarray:
    """The 8 Gell-Mann matrices, ``[8, 3, 3]`` complex128."""
    l = np.zeros((8, 3, 3), np.complex128)
    l[0, 0, 1] = l[0, 1, 0] = 1
    l[1, 0, 1], l[1, 1, 0] = -1j, 1j
    l[2, 0, 0], l[2, 1, 1] = 1, -1
    l[3, 0, 2] = l[3, 2, 0] = 1
    l[4, 0, 2], l[4, 2, 0] = -1j, 1j
    l[5, 1, 2] = l[5, 2, 1] = 1
    l[6, 1, 2], l[6, 2, 1] = -1j, 1j
    l[7, 0, 0] = l[7, 1, 1] = 1 / math.sqrt(3)
    l[7, 2, 2] = -2 / math.sqrt(3)
    return l


def synthetic_gauge(latt_size: Sequence[int], eps: float, seed: int) -> np.ndarray:
    """Seeded SU(3) field ``U = exp(i*eps*A)``, ``A = sum_a w_a lambda_a / 2``,
    ``w_a ~ N(0,1)``, computed through ``eigh`` (unitary to ~1e-15).

    Returned in the on-disk ILDG order ``[Lt, Lz, Ly, Lx, 4, 3, 3]`` c128,
    timeslice-major fill from ``numpy.random.default_rng(seed)``.
    """
    Lx, Ly, Lz, Lt = latt_size
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((Lt, Lz, Ly, Lx, ND, 8))
    A = np.einsum("...a,aij->...ij", w, gell_mann() / 2)
    ev, Q = np.linalg.eigh(A)
    ph = np.exp(1j * eps * ev)
    return np.einsum("...ik,...k,...jk->...ij", Q, ph, Q.conj())


def random_colour_vectors(Ne: int, latt_size: Sequence[int], seed: int, orthonormal: bool = True) -> np.ndarray:
    """Seeded complex Gaussian colour vectors ``[Ne, Lz, Ly, Lx, 3]`` c128,
    optionally orthonormalised (QR), standing in for eigenvectors where only
    the elemental arithmetic is exercised."""
    Lx, Ly, Lz = latt_size[0], latt_size[1], latt_size[2]
    rng = np.random.default_rng(seed)
    n = Lz * Ly * Lx * NC
    X = rng.standard_normal((n, Ne)) + 1j * rng.standard_normal((n, Ne))
    if orthonormal:
        X, _ = np.linalg.qr(X)
    else:
        X = X / np.sqrt(n)
    return np.ascontiguousarray(X.T).reshape(Ne, Lz, Ly, Lx, NC)


# ---------------------------------------------------------------------------
# stout smearing (numpy path)
# ---------------------------------------------------------------------------


def stout_smear(U_spatial: np.ndarray, nstep: int, rho: float) -> np.ndarray:
    """3D stout smearing of the spatial links, numpy form
    (``lattice/generator/eigenvector.py:123-190``).

    ``U_spatial`` is ``[3, Lt, Lz, Ly, Lx, 3, 3]``; staples over the two other
    spatial directions, ``Q = (i/2)(Omega^dag - Omega) - trace/3`` with
    ``Omega = rho * C U^dag``, and ``exp(iQ)`` through the Cayley-Hamilton
    coefficients f0, f1, f2 (Morningstar-Peardon).  Returns the smeared links.
    """
    U = np.ascontiguousarray(U_spatial)
    eye = np.eye(3)
    for _ in range(nstep):
        Q = np.zeros_like(U)
        U_dag = U.transpose(0, 1, 2, 3, 4, 6, 5).conj()
        for mu in range(3):
            for nu in range(3):
                if mu == nu:
                    continue
                Q[mu] += U[nu] @ np.roll(U[mu], -1, 3 - nu) @ np.roll(U_dag[nu], -1, 3 - mu)
                Q[mu] += (
                    np.roll(U_dag[nu], +1, 3 - nu)
                    @ np.roll(U[mu], +1, 3 - nu)
                    @ np.roll(np.roll(U[nu], +1, 3 - nu), -1, 3 - mu)
                )
        Q = rho * Q @ U_dag
        Q = 0.5j * (Q.transpose(0, 1, 2, 3, 4, 6, 5).conj() - Q)
        tr = np.einsum("...aa->...", Q)
        Q = Q - (tr / 3)[..., None, None] * eye
        Q_sq = Q @ Q
        c0 = np.einsum("...aa->...", Q @ Q_sq).real / 3
        c1 = np.einsum("...aa->...", Q_sq).real / 2
        c0_max = 2 * (c1 / 3) ** 1.5
        parity = c0 < 0
        c0 = np.abs(c0)
        with np.errstate(invalid="ignore", divide="ignore"):
            theta = np.arccos(np.clip(c0 / c0_max, -1.0, 1.0))
        theta = np.where(c0_max > 0, theta, 0.0)
        u = np.sqrt(c1 / 3) * np.cos(theta / 3)
        w = np.sqrt(c1) * np.sin(theta / 3)
        u_sq, w_sq = u * u, w * w
        e_iu = np.exp(-1j * u)
        e_2iu = np.exp(2j * u)
        cos_w = np.cos(w)
        sinc_w = 1 - w_sq / 6 * (1 - w_sq / 20 * (1 - w_sq / 42 * (1 - w_sq / 72)))
        large = np.abs(w) > 0.05
        sinc_w = np.where(large, np.sin(w) / np.where(large, w, 1.0), sinc_w)
        f_denom = 1 / (9 * u_sq - w_sq)
        f0 = ((u_sq - w_sq) * e_2iu + e_iu * (8 * u_sq * cos_w + 2j * u * (3 * u_sq + w_sq) * sinc_w)) * f_denom
        f1 = (2 * u * e_2iu - e_iu * (2 * u * cos_w - 1j * (3 * u_sq - w_sq) * sinc_w)) * f_denom
        f2 = (e_2iu - e_iu * (cos_w + 3j * u * sinc_w)) * f_denom
        f0 = np.where(parity, f0.conj(), f0)
        f1 = np.where(parity, -f1.conj(), f1)
        f2 = np.where(parity, f2.conj(), f2)
        f = f2[..., None, None] * Q_sq + f1[..., None, None] * Q + f0[..., None, None] * eye
        U = f @ U
    return U


# ---------------------------------------------------------------------------
# correlators
# ---------------------------------------------------------------------------

_GAMMA_BASIS = {
    0: [[0, 0, 0, 1j], [0, 0, 1j, 0], [0, -1j, 0, 0], [-1j, 0, 0, 0]],
    1: [[0, 0, 0, -1], [0, 0, 1, 0], [0, 1, 0, 0], [-1, 0, 0, 0]],
    2: [[0, 0, 1j, 0], [0, 0, 0, -1j], [-1j, 0, 0, 0], [0, 1j, 0, 0]],
    3: [[0, 0, 1, 0], [0, 0, 0, 1], [1, 0, 0, 0], [0, 1, 0, 0]],
}


def gamma(n: int) -> np.ndarray:
    """``gamma(n) = g0^(n&1) g1^(n&2) g2^(n&4) g3^(n&8)``
    (``lattice/insertion/gamma.py:20-68,101-110``)."""
    m = np.eye(4, dtype=np.complex128)
    for bit in range(4):
        if n & (1 << bit):
            m = m @ np.array(_GAMMA_BASIS[bit], dtype=np.complex128)
    return m


def twopoint(phis, perambulator, timeslices, Lt, usedNe=None, is_sum_over_source_t=True):
    """Meson two-point function (``lattice/correlator/one_particle.py:12-77``)
    with the operator data already assembled: ``phis`` is a list of
    ``(gammas [X,4,4], elementals [X, Lt, Ne, Ne])``; ``perambulator[t_src]`` is
    ``[Lt, 4, 4, Ne, Ne]``."""
    Nop = len(phis)
    ts = list(timeslices)
    ret = np.zeros((Nop, len(ts), Lt), np.complex128)
    for it, t_src in enumerate(ts):
        tau = np.asarray(perambulator[t_src])
        if usedNe is not None:
            tau = tau[..., :usedNe, :usedNe]
        tau_bw = np.einsum("ii,tjiba,jj->tijab", gamma(15), tau.conj(), gamma(15))
        for idx, (g, e) in enumerate(phis):
            if usedNe is not None:
                e = e[..., :usedNe, :usedNe]
            gamma_src = np.einsum("ij,xkj,kl->xil", gamma(8), g.conj(), gamma(8))
            ret[idx, it] = np.einsum(
                "tijab,xjk,xtbc,tklcd,yli,yad->t", tau_bw, g, np.roll(e, -t_src, 1), tau, gamma_src,
                e[:, t_src].conj(), optimize=True,
            )
    return -ret.mean(1) if is_sum_over_source_t else -ret


def operator_parts(rows, coefficients):
    """``Operator(name, insertion_rows, coefficients).parts``
    (``lattice/insertion/__init__.py:116-145``): ``rows`` is a list of
    ``(row, momentum)`` with ``row = [gamma, [(coeff, derivative), ...], ...]``;
    every part becomes ``[gamma, [[coefficient*coeff, derivative, momentum], ...]]``
    with the coefficient negated for gamma 5 and 13."""
    parts = []
    for (row, momentum), c in zip(rows, coefficients):
        for i in range(len(row) // 2):
            g = row[2 * i]
            parts.append(g)
            sign = -1 if g in (5, 13) else 1
            parts.append([[c * dc * sign, d, momentum] for dc, d in row[2 * i + 1]])
    return parts


def elemental_data(parts_list, elemental, usedNe):
    """``get_elemental_data`` (``lattice/data.py:7-33``): per operator the
    gammas ``[X, 4, 4]`` of its parts and the coefficient sums of its
    elementals ``elemental[d, p, :, :usedNe, :usedNe]`` (``[X, Lt, Ne', Ne']``)."""
    out = []
    for parts in parts_list:
        gs, es = [], []
        for i in range(len(parts) // 2):
            gs.append(gamma(parts[2 * i]))
            acc = None
            for coeff, d, p in parts[2 * i + 1]:
                term = coeff * np.asarray(elemental[d, p, :, :usedNe, :usedNe])
                acc = term if acc is None else acc + term
            es.append(acc)
        out.append((np.array(gs), np.array(es)))
    return out


def twopoint_operators(parts_list, elemental, perambulator, timeslices, Lt, usedNe=None, perambulator_bw=None,
                       is_sum_over_source_t=True):
    """``twopoint`` on the reference interface (``lattice/correlator/one_particle.py:12-77``):
    operators given by their ``parts``, elementals ``[Nderiv, Nmom, Lt, Ne, Ne]``,
    perambulators ``[Lt_src, Lt, 4, 4, Ne, Ne]``; ``perambulator_bw`` replaces
    the backward propagator ``g5 tau^dag g5`` by ``g5 tau_bw^dag g5``."""
    phis = elemental_data(parts_list, elemental, usedNe)
    ts = list(timeslices)
    ret = np.zeros((len(phis), len(ts), Lt), np.complex128)
    g15, g8 = gamma(15), gamma(8)
    for it, t_src in enumerate(ts):
        tau = np.asarray(perambulator[t_src, :, :, :, :usedNe, :usedNe])
        src_bw = tau if perambulator_bw is None else np.asarray(perambulator_bw[t_src, :, :, :, :usedNe, :usedNe])
        tau_bw = np.einsum("ii,tjiba,jj->tijab", g15, src_bw.conj(), g15)
        for idx, (g, e) in enumerate(phis):
            gamma_src = np.einsum("ij,xkj,kl->xil", g8, g.conj(), g8)
            ret[idx, it] = np.einsum("tijab,xjk,xtbc,tklcd,yli,yad->t", tau_bw, g, np.roll(e, -t_src, 1), tau,
                                     gamma_src, e[:, t_src].conj(), optimize=True)
    return -ret.mean(1) if is_sum_over_source_t else -ret


def twopoint_profile_operators(parts_list, elemental, perambulator, timeslices, delta_t_slices, usedNe=None,
                               perambulator_bw=None, is_sum_over_source_t=True, is_diagonal=False):
    """``twopoint_profile`` (``lattice/correlator/one_particle.py:80-135``): the
    two-point function at the sink separations ``delta_t_slices`` resolved in
    the eigenvector indices, ``[Nop, Ndt, Ne', Ne']`` (``[Nop, Ndt, Ne']`` with
    ``is_diagonal``).  The reference reads the backward propagator at every
    sink time (``:100-101``), so ``perambulator_bw`` needs ``delta_t_slices``
    to cover all of them, as there."""
    phis = elemental_data(parts_list, elemental, usedNe)
    ts, dts = list(timeslices), list(delta_t_slices)
    ne = np.asarray(elemental[0, 0, 0, :usedNe, :usedNe]).shape[-1]
    shape = (len(phis), len(ts), len(dts), ne) if is_diagonal else (len(phis), len(ts), len(dts), ne, ne)
    ret = np.zeros(shape, np.complex128)
    g15, g8 = gamma(15), gamma(8)
    for it, t_src in enumerate(ts):
        tau = np.asarray(perambulator[t_src, dts, :, :, :usedNe, :usedNe])
        src_bw = tau if perambulator_bw is None else np.asarray(perambulator_bw[t_src, :, :, :, :usedNe, :usedNe])
        tau_bw = np.einsum("ii,tjiba,jj->tijab", g15, src_bw.conj(), g15)
        for idx, (g, e) in enumerate(phis):
            gamma_src = np.einsum("ij,xkj,kl->xil", g8, g.conj(), g8)
            sink = np.roll(e, -t_src, 1)[:, dts]
            if is_diagonal:
                ret[idx, it] = np.einsum("tijab,xjk,xtbb,tklba,yli,yaa->ta", tau_bw, g, sink, tau, gamma_src,
                                         e[:, t_src].conj(), optimize=True)
            else:
                ret[idx, it] = np.einsum("tijab,xjk,xtbc,tklcd,yli,yad->tad", tau_bw, g, sink, tau, gamma_src,
                                         e[:, t_src].conj(), optimize=True)
    return -ret.mean(1) if is_sum_over_source_t else -ret


def project_su3(U: np.ndarray, tol: float = 1e-15) -> np.ndarray:
    """``EigenvectorGenerator.project_SU3`` (``lattice/generator/eigenvector.py:55-65``):
    ``U <- (U + U^-dag) / 2`` over the whole field until ``max|U - U^-dag|``
    and ``max|U U^dag - 1|`` are both <= tol.  ``U``: ``[..., 3, 3]``."""
    U = np.array(U, dtype=np.complex128)
    eye = np.eye(3)
    while True:
        Uid = np.linalg.inv(U).conj().swapaxes(-1, -2)
        if np.abs(U - Uid).max() <= tol and np.abs(U @ U.conj().swapaxes(-1, -2) - eye).max() <= tol:
            return U
        U = 0.5 * (U + Uid)
