"""Meson two-point correlators from elementals and perambulators (GPU).

Same interface as ``lattice/correlator/one_particle.py``:

* :class:`InsertionRowMom` and :class:`Operator` build an operator's
  ``parts`` exactly like ``lattice/insertion/__init__.py:109-145`` (a gamma
  index, then ``[coefficient, derivative, momentum]`` triples; the
  coefficient is negated for gamma 5 and 13, the reference's sign
  convention);
* :func:`get_elemental_data` assembles, per operator, the gammas of its parts
  and the coefficient sums of ``elemental[d, p, :, :usedNe, :usedNe]``
  (``lattice/data.py:7-33``);
* :func:`twopoint` (``one_particle.py:12-77``) and :func:`twopoint_profile`
  (``one_particle.py:80-135``) take the operators, the elemental and
  perambulator file data (anything indexable like
  ``elemental[d, p, :, :Ne, :Ne]`` / ``perambulator[t_src, ...]``: the
  reference's ``FileData``, this package's readers, numpy arrays or torch
  tensors) and return ``C[op, t]`` / ``C[op, t, a, d]`` (``C[op, t, a]``
  with ``is_diagonal``), averaged over the source timeslices unless
  ``is_sum_over_source_t`` is False, with the reference's overall minus sign.

Results are complex128 device tensors (host numpy arrays after
``set_backend("numpy")``).  The gamma matrices follow
``lattice/insertion/gamma.py`` (``gamma(n) = g0^(n&1) g1^(n&2) g2^(n&4)
g3^(n&8)``); every one of them is monomial (one non-zero per row), which the
contraction uses: with ``tau_bw = g5 tau^dag g5`` (``one_particle.py:59-63``)
and the source gamma ``G = g4 Gamma^dag g4`` (``:66``),

    C(t) = sum_{x,y} Tr[ tau_bw(t) (Gamma_x (x) phi_x(t)) tau(t) (G_y (x) psi_y) ]

is a sum of terms coef Tr[A phi_x(t) B psi_y^T] with A, B single Ne x Ne spin
blocks of tau_bw(t) and tau(t) (one per part pair and spin pair, j and l fixed
by the gammas): ``twopoint`` evaluates them in the library's
``ed_twopoint_trace`` (both products per 32 x 32 tile in shared memory, never
written to HBM); ``twopoint_profile`` in ``ed_twopoint_profile`` (the 16 left
blocks L[i][k] = sum_x c A phi_x, then sum_k L[i][k] B weighted by psi_y, the
output tile kept in registers) or ``ed_twopoint_profile_diag``.  All FP64.
"""

from __future__ import annotations

from functools import lru_cache
from typing import Iterable, List, Sequence, Tuple

import numpy as np
import torch

from .backend import to_backend

_G = {
    0: [[0, 0, 0, 1j], [0, 0, 1j, 0], [0, -1j, 0, 0], [-1j, 0, 0, 0]],
    1: [[0, 0, 0, -1], [0, 0, 1, 0], [0, 1, 0, 0], [-1, 0, 0, 0]],
    2: [[0, 0, 1j, 0], [0, 0, 0, -1j], [-1j, 0, 0, 0], [0, 1j, 0, 0]],
    3: [[0, 0, 1, 0], [0, 0, 0, 1], [1, 0, 0, 0], [0, 1, 0, 0]],
}


@lru_cache(maxsize=None)
def _gamma_cpu(n: int) -> torch.Tensor:
    if not (0 <= n <= 15):
        raise ValueError("gamma index must be in 0..15")
    m = torch.eye(4, dtype=torch.complex128)
    for bit in range(4):
        if n & (1 << bit):
            m = m @ torch.tensor(_G[bit], dtype=torch.complex128)
    return m


def gamma(n: int, device=None) -> torch.Tensor:
    """The 4x4 matrix ``gamma(n)`` of the reference's insertion table."""
    return _gamma_cpu(n).to(device or "cpu")


# ---------------------------------------------------------------- operators


class InsertionRowMom:
    """One insertion row at one momentum (``lattice/insertion/__init__.py:103-106``):
    ``row = [gamma, [(coeff, derivative), ...], gamma, [...], ...]`` and the
    momentum index into the elementals' momentum axis."""

    def __init__(self, row, momentum) -> None:
        self.row = row
        self.momentum = momentum


class Operator:
    """An interpolating operator: a sum of insertion rows with coefficients
    (``lattice/insertion/__init__.py:109-145``).  ``parts`` alternates a gamma
    index and its elemental terms ``[coefficient * coeff, derivative, momentum]``."""

    def __init__(self, name: str, insertion_rows: List[InsertionRowMom], coefficients: List[float]) -> None:
        assert len(insertion_rows) == len(coefficients), (
            f"Unmatched numbers of insertion rows {len(insertion_rows)} and coefficients {len(coefficients)}"
        )
        parts = []
        for ins, coefficient in zip(insertion_rows, coefficients):
            row, momentum = ins.row, ins.momentum
            for i in range(len(row) // 2):
                g = row[2 * i]
                parts.append(g)
                # gamma_3 gamma_1 = -gamma(5) and gamma_3 gamma_1 gamma_4 = -gamma(13) in the reference's table
                sign = -1 if g in (5, 13) else 1
                parts.append([[coefficient * dc * sign, d, momentum] for dc, d in row[2 * i + 1]])
        self.name = name
        self.parts = parts

    def __str__(self) -> str:
        return f"Operator({self.name!r}, parts={self.parts})"


def _fetch(data, key, device) -> torch.Tensor:
    x = data[key]
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=torch.complex128)
    if hasattr(x, "get") and not isinstance(x, np.ndarray):  # cupy
        x = x.get()
    arr = np.ascontiguousarray(np.asarray(x)).astype(np.complex128, copy=False)
    return torch.from_numpy(arr).to(device)


def _cuda(device) -> torch.device:
    device = torch.device(device or "cuda")
    if device.type != "cuda":
        raise ValueError("the correlator contractions run on a CUDA device (there is no CPU path)")
    return device


def get_elemental_data(operators: Sequence[Operator], elemental, usedNe: int = None, device=None):
    """Per operator ``(gammas [X, 4, 4], elementals [X, Lt, Ne', Ne'])`` on the
    device: the gammas of its X parts and the coefficient sums of their
    elementals ``elemental[d, p, :, :usedNe, :usedNe]``, each (d, p) read once
    (``lattice/data.py:7-33``)."""
    device = _cuda(device)
    cache = {}
    out = []
    for op in operators:
        parts = op.parts
        gs, es = [], []
        for i in range(len(parts) // 2):
            gs.append(gamma(parts[2 * i], device))
            acc = None
            for coeff, d, p in parts[2 * i + 1]:
                key = (d, p)
                if key not in cache:
                    cache[key] = _fetch(elemental, (d, p, slice(None), slice(None, usedNe), slice(None, usedNe)),
                                        device)
                term = coeff * cache[key]
                acc = term if acc is None else acc + term
            es.append(acc)
        out.append((torch.stack(gs), torch.stack(es)))
    return out


# ---------------------------------------------------------------- contraction


@lru_cache(maxsize=None)
def _monomial(n: int, conj_src: bool) -> Tuple[Tuple[int, ...], Tuple[complex, ...]]:
    """gamma(n) (or the source form g4 gamma(n)^dag g4 of ``one_particle.py:66``)
    as (column of the non-zero in each row, its value)."""
    g = _gamma_cpu(n)
    if conj_src:
        g8 = _gamma_cpu(8)
        g = g8 @ g.conj().T @ g8
    cols, vals = [], []
    for r in range(4):
        nz = [c for c in range(4) if abs(complex(g[r, c])) > 0]
        if len(nz) != 1:
            raise AssertionError("gamma matrices of the insertion table are monomial")
        cols.append(nz[0])
        vals.append(complex(g[r, nz[0]]))
    return tuple(cols), tuple(vals)


def _gamma_index(g: torch.Tensor) -> int:
    for n in range(16):
        if torch.equal(_gamma_cpu(n), g.detach().cpu()):
            return n
    raise ValueError("not a gamma matrix of the insertion table")


_G5 = (1.0, 1.0, -1.0, -1.0)  # the diagonal of gamma(15) in the reference's basis


def _term_table(gid):
    """The terms of one operator (parts with gamma indices ``gid``): one per
    (sink part x, source part y, spin i, spin k) with j the row of gamma_x
    holding column k, l the row of the source gamma holding column i, coef =
    gamma_x[j][k] G_y[l][i] g5[i] g5[j]."""
    idx, coef = [], []
    for x, gx in enumerate(gid):
        cx, vx = _monomial(gx, False)
        for y, gy in enumerate(gid):
            cy, vy = _monomial(gy, True)
            for i in range(4):
                l = cy.index(i)
                for k in range(4):
                    j = cx.index(k)
                    c = vx[j] * vy[l] * _G5[i] * _G5[j]
                    idx.append((x, y, i, j, k, l))
                    coef.append((c.real, c.imag))
    return idx, coef


def _trace_terms(tau, taub, el, gid, t_src):
    """``out[t]`` of one operator through ``ed_twopoint_trace``."""
    from . import _lib

    T, Ne, Lt = tau.shape[0], tau.shape[-1], el.shape[1]
    idx, coef = _term_table(gid)
    dev = tau.device
    idx_t = torch.tensor(idx, dtype=torch.int32, device=dev)
    coef_t = torch.tensor(coef, dtype=torch.float64, device=dev)
    out = torch.zeros(T, dtype=torch.complex128, device=dev)
    tau, taub = tau.contiguous(), taub.contiguous()
    _lib.call("ed_twopoint_trace", T, Ne, Lt, int(t_src), len(gid), len(idx), _lib.ptr(idx_t), _lib.ptr(coef_t),
              _lib.ptr(tau), _lib.ptr(taub), _lib.ptr(el), _lib.ptr(out), _lib.stream_handle())
    return out


def _profile_terms(tau, taub, el, gid, t_src, sink_t, diagonal):
    """``out[t, a, d]`` (or ``out[t, a]`` with ``diagonal``) of one operator
    through ``ed_twopoint_profile`` / ``ed_twopoint_profile_diag``; the
    coefficient of a term factorises into gamma_x[j][k] g5[j] (sink part x,
    spin k) times G_y[l][i] g5[i] (source part y, spin i)."""
    from . import _lib

    T, Ne, Lt, X = tau.shape[0], tau.shape[-1], el.shape[1], len(gid)
    dev = tau.device
    tau, taub, el = tau.contiguous(), taub.contiguous(), el.contiguous()
    st = torch.tensor(sink_t, dtype=torch.int32, device=dev)
    if diagonal:
        idx, coef = _term_table(gid)
        idx_t = torch.tensor(idx, dtype=torch.int32, device=dev)
        coef_t = torch.tensor(coef, dtype=torch.float64, device=dev)
        out = torch.empty((T, Ne), dtype=torch.complex128, device=dev)
        _lib.call("ed_twopoint_profile_diag", T, Ne, Lt, int(t_src), X, len(idx), _lib.ptr(st), _lib.ptr(idx_t),
                  _lib.ptr(coef_t), _lib.ptr(tau), _lib.ptr(taub), _lib.ptr(el), _lib.ptr(out), _lib.stream_handle())
        return out
    ltab, lcoef, rtab, rcoef = [], [], [], []
    for k in range(4):
        for x in range(X):
            cx, vx = _monomial(gid[x], False)
            j = cx.index(k)
            c = vx[j] * _G5[j]
            ltab.append(j)
            lcoef.append((c.real, c.imag))
    for i in range(4):
        for y in range(X):
            cy, vy = _monomial(gid[y], True)
            l = cy.index(i)
            c = vy[l] * _G5[i]
            rtab.append(l)
            rcoef.append((c.real, c.imag))
    lt = torch.tensor(ltab, dtype=torch.int32, device=dev)
    lc = torch.tensor(lcoef, dtype=torch.float64, device=dev)
    rt = torch.tensor(rtab, dtype=torch.int32, device=dev)
    rc = torch.tensor(rcoef, dtype=torch.float64, device=dev)
    work = torch.empty((T, 16, Ne, Ne), dtype=torch.complex128, device=dev)
    out = torch.empty((T, Ne, Ne), dtype=torch.complex128, device=dev)
    _lib.call("ed_twopoint_profile", T, Ne, Lt, int(t_src), X, _lib.ptr(st), _lib.ptr(lt), _lib.ptr(lc), _lib.ptr(rt),
              _lib.ptr(rc), _lib.ptr(tau), _lib.ptr(taub), _lib.ptr(el), _lib.ptr(work), _lib.ptr(out),
              _lib.stream_handle())
    return out


def _source_terms(tau, taub, phis, t_src, dts=None, mode="trace"):
    """All operators for one source timeslice.  ``tau``: the source's
    perambulator ``[T, 4, 4, Ne, Ne]`` at the sink times, ``taub`` the one of
    the backward propagator (``tau`` itself or ``perambulator_bw``); ``phis``:
    per operator ``(gammas, elementals)`` with elementals ``[X, Lt, Ne, Ne]``.
    mode "trace" (the library's ``ed_twopoint_trace``): ``[Nop, T]``;
    "profile": ``[Nop, T, Ne, Ne]`` (indices a, d); "diagonal": ``[Nop, T, Ne]``."""
    out = []
    Lt = phis[0][1].shape[1]
    sink_t = [(t_src + int(dt)) % Lt for dt in (dts if dts is not None else range(tau.shape[0]))]
    for gammas, el in phis:
        gid = [_gamma_index(g) for g in gammas]
        if mode == "trace":
            out.append(_trace_terms(tau, taub, el.contiguous(), gid, t_src))
        else:
            out.append(_profile_terms(tau, taub, el, gid, t_src, sink_t, mode == "diagonal"))
    return torch.stack(out)


def _peram_block(perambulator, t_src, tsel, usedNe, device):
    key = (t_src, tsel, slice(None), slice(None), slice(None, usedNe), slice(None, usedNe))
    return _fetch(perambulator, key, device)


def twopoint(operators: List[Operator], elemental, perambulator, timeslices: Iterable[int], Lt: int,
             usedNe: int = None, perambulator_bw=None, is_sum_over_source_t: bool = True, *, device=None):
    """Two-point functions ``C[op, t]`` (``lattice/correlator/one_particle.py:12-77``):
    ``-mean over t_src`` of the contraction, or ``[Nop, Nsrc, Lt]`` per source
    with ``is_sum_over_source_t=False``.  ``perambulator_bw`` replaces the
    backward quark propagator (``tau_bw = g5 perambulator_bw^dag g5``)."""
    device = _cuda(device)
    ts = list(timeslices)
    phis = get_elemental_data(operators, elemental, usedNe, device)
    ret = torch.zeros((len(operators), len(ts), Lt), dtype=torch.complex128, device=device)
    for it, t_src in enumerate(ts):
        tau = _peram_block(perambulator, t_src, slice(None), usedNe, device)
        src_bw = tau if perambulator_bw is None else _peram_block(perambulator_bw, t_src, slice(None), usedNe, device)
        ret[:, it] = _source_terms(tau, src_bw, phis, t_src)
    ret = -ret.mean(1) if is_sum_over_source_t else -ret
    return to_backend(ret)


def twopoint_profile(operators: List[Operator], elemental, perambulator, timeslices: Iterable[int],
                     delta_t_slices: Iterable[int], usedNe: int = None, perambulator_bw=None,
                     is_sum_over_source_t: bool = True, is_diagonal: bool = False, *, device=None):
    """Two-point functions at the sink separations ``delta_t_slices``, resolved
    in the eigenvector indices (``lattice/correlator/one_particle.py:80-135``):
    ``C[op, dt, a, d]``, or ``C[op, dt, a]`` with ``is_diagonal``.
    ``perambulator_bw`` is read at the same sink separations (the reference
    reads it at every sink time, ``:100-101``, which agrees when
    ``delta_t_slices`` covers all of them and fails otherwise)."""
    device = _cuda(device)
    ts, dts = list(timeslices), [int(v) for v in delta_t_slices]
    phis = get_elemental_data(operators, elemental, usedNe, device)
    ne = phis[0][1].shape[-1]
    shape = (len(operators), len(ts), len(dts)) + ((ne,) if is_diagonal else (ne, ne))
    ret = torch.zeros(shape, dtype=torch.complex128, device=device)
    for it, t_src in enumerate(ts):
        tau = _peram_block(perambulator, t_src, dts, usedNe, device)
        src_bw = tau if perambulator_bw is None else _peram_block(perambulator_bw, t_src, dts, usedNe, device)
        ret[:, it] = _source_terms(tau, src_bw, phis, t_src, dts, "diagonal" if is_diagonal else "profile")
    ret = -ret.mean(1) if is_sum_over_source_t else -ret
    return to_backend(ret)


def twopoint_source(tau: torch.Tensor, gammas: torch.Tensor, elementals: torch.Tensor, t_src: int,
                    tau_bw: torch.Tensor = None) -> torch.Tensor:
    """``ret[t]`` of one source timeslice and one assembled operator (before
    the overall minus sign), differentiable through torch autograd: the form
    the correlator loss of :mod:`easydistillation_gb300.autograd` uses.

    ``tau``: perambulator of this source ``[Lt, 4, 4, Ne, Ne]``; ``gammas``
    ``[X, 4, 4]``; ``elementals`` ``[X, Lt, Ne, Ne]``."""
    dev = tau.device
    g15, g8 = gamma(15, dev), gamma(8, dev)
    if tau_bw is None:
        tau_bw = torch.einsum("ii,tjiba,jj->tijab", g15, tau.conj(), g15)
    gamma_src = torch.einsum("ij,xkj,kl->xil", g8, gammas.conj(), g8)
    phi_t = torch.roll(elementals, -t_src, 1)
    phi_src = elementals[:, t_src].conj()
    left = torch.einsum("tijab,xjk,xtbc->tikac", tau_bw, gammas, phi_t)
    right = torch.einsum("tklcd,yli,yad->tkica", tau, gamma_src, phi_src)
    return torch.einsum("tikac,tkica->t", left, right)


def twopoint_assembled(phis: Sequence[Tuple[torch.Tensor, torch.Tensor]], perambulator, timeslices: Iterable[int],
                       Lt: int, usedNe: int = None, is_sum_over_source_t: bool = True) -> torch.Tensor:
    """``C[op, t]`` from operators already assembled as ``(gammas [X,4,4],
    elementals [X, Lt, Ne, Ne])`` device tensors (the output of
    :func:`get_elemental_data`); ``perambulator[t_src]`` -> ``[Lt, 4, 4, Ne, Ne]``."""
    ts = list(timeslices)
    dev = phis[0][1].device
    phis = [(g.to(dev), e if usedNe is None else e[..., :usedNe, :usedNe]) for g, e in phis]
    ret = torch.zeros((len(phis), len(ts), Lt), dtype=torch.complex128, device=dev)
    for it, t_src in enumerate(ts):
        tau = torch.as_tensor(perambulator[t_src]).to(dev)
        if usedNe is not None:
            tau = tau[..., :usedNe, :usedNe]
        ret[:, it] = _source_terms(tau, tau, phis, t_src)
    return -ret.mean(1) if is_sum_over_source_t else -ret
