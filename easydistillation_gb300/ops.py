"""Torch-facing wrappers of the C ABI (device tensors in, device tensors out).

Every function here launches the library's own CUDA kernels on the current
torch stream; none has a CPU path.
"""

from __future__ import annotations

import ctypes
import sys
from typing import Sequence

import torch

from . import _lib
from ._lib import ED_C64, ED_C128, ED_DF, ED_LANCZOS_GS_DF, call, ptr, require_cuda, stream_handle

_PREC = {torch.complex128: ED_C128, torch.complex64: ED_C64}
_NATIVE_LITTLE = sys.byteorder == "little"
_DTYPE = {ED_C128: torch.complex128, ED_C64: torch.complex64}


def prec_of(t: torch.Tensor) -> int:
    try:
        return _PREC[t.dtype]
    except KeyError:
        raise ValueError(f"unsupported dtype {t.dtype}; expected complex128 or complex64") from None


def links_to_soa(U: torch.Tensor, latt_size: Sequence[int], dtype=torch.complex128, layout: str = "reference"):
    """Spatial links of every timeslice -> SoA ``[Lt, 27, V3]``.

    ``U`` is complex128 on the device, either the generators' transposed
    layout ``[Nd, Lt, Lz, Ly, Lx, 3, 3]`` (``layout="reference"``,
    ``lattice/generator/eigenvector.py:50``) or the on-disk ILDG order
    ``[Lt, Lz, Ly, Lx, Nd, 3, 3]`` (``layout="ildg"``)."""
    require_cuda(U, "U")
    if U.dtype != torch.complex128:
        raise ValueError("links must be complex128")
    Lx, Ly, Lz, Lt = latt_size
    V3 = Lx * Ly * Lz
    if layout == "reference":
        nt = U.shape[1]
        ts, ds, ss = V3 * 9, nt * V3 * 9, 9
    elif layout == "ildg":
        nt = U.shape[0]
        ts, ds, ss = V3 * U.shape[4] * 9, 9, U.shape[4] * 9
    else:
        raise ValueError(f"unknown link layout {layout!r}")
    out = torch.empty((nt, 27, V3), dtype=dtype, device=U.device)
    call("ed_links_to_soa", _PREC[dtype], Lx, Ly, Lz, nt, ptr(U), ts, ds, ss, ptr(out), stream_handle())
    return out


def file_prec(dtype) -> int:
    """Source precision code of ``ed_decode_*`` for a stored complex numpy
    dtype (``">c16"``, ``"<c8"`` ...): ED_C128 / ED_C64, plus ED_BIG_ENDIAN
    when the bytes are big-endian."""
    import numpy as np

    dt = np.dtype(dtype)
    if dt.kind != "c" or dt.itemsize not in (8, 16):
        raise ValueError(f"not a complex64/complex128 dtype: {dtype!r}")
    big = dt.byteorder == ">" or (dt.byteorder == "=" and not _NATIVE_LITTLE)
    return (ED_C128 if dt.itemsize == 16 else ED_C64) | (_lib.ED_BIG_ENDIAN if big else 0)


def decode_complex(raw: torch.Tensor, file_dtype, dtype=torch.complex128, out: torch.Tensor = None) -> torch.Tensor:
    """Complex numbers from a file's byte image on the device.

    ``raw`` holds the stored bytes (any dtype, contiguous, on the device);
    ``file_dtype`` is their numpy dtype (e.g. ``">c16"`` for ILDG, ``">c8"``
    for QDP eigenvectors).  Returns (or fills ``out``) a flat ``dtype``
    tensor: the byte order swapped and the precision converted on the device,
    bit-identical to numpy's ``astype`` (``lattice/filedata/ildg.py:70``,
    ``timeslice.py:96``)."""
    require_cuda(raw, "raw")
    if not raw.is_contiguous():
        raise ValueError("raw bytes must be contiguous")
    src = file_prec(file_dtype)
    esz = 16 if (src & ~_lib.ED_BIG_ENDIAN) == ED_C128 else 8
    nbytes = raw.numel() * raw.element_size()
    if nbytes % esz:
        raise ValueError(f"{nbytes} bytes is not a whole number of {esz}-byte complex numbers")
    n = nbytes // esz
    if out is None:
        out = torch.empty(n, dtype=dtype, device=raw.device)
    elif out.numel() != n or out.dtype != dtype or not out.is_contiguous():
        raise ValueError("out must be a contiguous tensor of the decoded size and dtype")
    call("ed_decode_complex", src, n, ptr(raw), _PREC[dtype], ptr(out), stream_handle())
    return out


def decode_links(raw: torch.Tensor, file_dtype, latt_size: Sequence[int]) -> torch.Tensor:
    """Links in the ILDG order ``[Lt, Lz, Ly, Lx, 4, 3, 3]`` (the file's byte
    image on the device) -> the generators' spatial links
    ``[3, Lt, Lz, Ly, Lx, 3, 3]`` complex128 (``elemental.py:103``,
    ``eigenvector.py:50``), in one device pass."""
    require_cuda(raw, "raw")
    if not raw.is_contiguous():
        raise ValueError("raw bytes must be contiguous")
    Lx, Ly, Lz, Lt = latt_size
    sites = Lx * Ly * Lz * Lt
    src = file_prec(file_dtype)
    esz = 16 if (src & ~_lib.ED_BIG_ENDIAN) == ED_C128 else 8
    if raw.numel() * raw.element_size() != sites * 36 * esz:
        raise ValueError("raw bytes do not hold [Lt, Lz, Ly, Lx, 4, 3, 3] complex numbers")
    out = torch.empty((3, Lt, Lz, Ly, Lx, 3, 3), dtype=torch.complex128, device=raw.device)
    call("ed_decode_links", src, sites, ptr(raw), ptr(out), stream_handle())
    return out


def vectors_to_planes(V: torch.Tensor, V3: int, dtype=torch.complex128, round_c64: bool = False):
    """``[..., V3, 3]`` -> colour planes ``[..., 3, V3]``."""
    require_cuda(V, "V")
    nvec = V.numel() // (3 * V3)
    out = torch.empty(V.shape[:-2] + (3, V3) if V.dim() >= 2 else (nvec, 3, V3), dtype=dtype, device=V.device)
    call("ed_vectors_to_planes", prec_of(V), _PREC[dtype], int(round_c64), nvec, V3, ptr(V), ptr(out), stream_handle())
    return out


def vectors_from_planes(P: torch.Tensor, V3: int, dtype=torch.complex128):
    """Colour planes ``[..., 3, V3]`` -> ``[..., V3, 3]``."""
    require_cuda(P, "P")
    nvec = P.numel() // (3 * V3)
    out = torch.empty(P.shape[:-2] + (V3, 3), dtype=dtype, device=P.device)
    call("ed_vectors_from_planes", prec_of(P), _PREC[dtype], nvec, V3, ptr(P), ptr(out), stream_handle())
    return out


def momentum_phases(latt_size: Sequence[int], momenta, device=None) -> torch.Tensor:
    """FP64 phase tables ``[Nmom, Lz, Ly, Lx]`` = ``exp(+2 pi i p.x / L)``
    (``lattice/insertion/phase.py:11-13,41-46``)."""
    Lx, Ly, Lz = latt_size[0], latt_size[1], latt_size[2]
    moms = [int(v) for p in momenta for v in p]
    nmom = len(moms) // 3
    arr = (ctypes.c_int * len(moms))(*moms)
    out = torch.empty((nmom, Lz, Ly, Lx), dtype=torch.complex128, device=device or "cuda")
    call("ed_momentum_phases", Lx, Ly, Lz, arr, nmom, ptr(out), stream_handle())
    return out


def laplacian(links_soa: torch.Tensor, F: torch.Tensor, latt_size: Sequence[int], out: torch.Tensor = None):
    """3D covariant Laplacian (``lattice/generator/eigenvector.py:11-26``).

    ``links_soa``: ``[nt, 27, V3]``; ``F``: colour planes ``[nt, nvec, 3, V3]``
    (any leading view whose timeslice stride is uniform).  Precision follows
    the tensors (complex128 or complex64, both the same)."""
    Lx, Ly, Lz = latt_size[0], latt_size[1], latt_size[2]
    V3 = Lx * Ly * Lz
    require_cuda(links_soa, "links")
    if F.dim() == 2:
        F = F.unsqueeze(0).unsqueeze(0)
    elif F.dim() == 3:
        F = F.unsqueeze(1)
    nt, nvec = F.shape[0], F.shape[1]
    if links_soa.dtype != F.dtype:
        raise ValueError("links and vectors must share a precision")
    if tuple(F.shape[2:]) != (3, V3) or F.stride(-1) != 1 or F.stride(-2) != V3 or F.stride(1) != 3 * V3:
        raise ValueError("F must be colour planes [nt, nvec, 3, V3] with contiguous vectors")
    if links_soa.shape[0] != nt:
        raise ValueError("links and vectors disagree on the number of timeslices")
    if out is None:
        out = torch.empty((nt, nvec, 3, V3), dtype=F.dtype, device=F.device)
    call(
        "ed_laplacian",
        prec_of(F),
        Lx,
        Ly,
        Lz,
        nt,
        nvec,
        ptr(links_soa),
        ptr(F),
        F.stride(0),
        ptr(out),
        out.stride(0),
        stream_handle(),
    )
    return out


def split_c128(x: torch.Tensor) -> torch.Tensor:
    """Double-float form of a complex128 tensor: float32 ``[..., 4]`` =
    (re_hi, im_hi, re_lo, im_lo) with hi the value rounded to FP32 and lo the
    rest (``ed_split_c128``)."""
    require_cuda(x, "x")
    if x.dtype != torch.complex128 or not x.is_contiguous():
        raise ValueError("x must be a contiguous complex128 tensor")
    out = torch.empty(tuple(x.shape) + (4,), dtype=torch.float32, device=x.device)
    call("ed_split_c128", x.numel(), ptr(x), ptr(out), stream_handle())
    return out


def laplacian_df(links_split: torch.Tensor, F: torch.Tensor, latt_size: Sequence[int], out: torch.Tensor = None):
    """The 3D covariant Laplacian of complex128 colour planes ``F`` ``[nt,
    nvec, 3, V3]`` in double-float arithmetic on the FP32 pipe (``ed_laplacian``
    with ``ED_DF``): ``links_split`` = ``split_c128`` of the SoA links ``[nt,
    27, V3]``.  ~2^-47 relative per product, the FP64 kernel's results to
    about 1e-14."""
    Lx, Ly, Lz = latt_size[0], latt_size[1], latt_size[2]
    V3 = Lx * Ly * Lz
    require_cuda(links_split, "links")
    if F.dim() == 3:
        F = F.unsqueeze(1)
    nt, nvec = F.shape[0], F.shape[1]
    if F.dtype != torch.complex128 or links_split.dtype != torch.float32:
        raise ValueError("F must be complex128 and the links split into float32 parts")
    if tuple(links_split.shape) != (nt, 27, V3, 4) or not links_split.is_contiguous():
        raise ValueError("links_split must be split_c128 of SoA links [nt, 27, V3]")
    if tuple(F.shape[2:]) != (3, V3) or F.stride(-1) != 1 or F.stride(-2) != V3 or F.stride(1) != 3 * V3:
        raise ValueError("F must be colour planes [nt, nvec, 3, V3] with contiguous vectors")
    if out is None:
        out = torch.empty((nt, nvec, 3, V3), dtype=F.dtype, device=F.device)
    call("ed_laplacian", ED_DF, Lx, Ly, Lz, nt, nvec, ptr(links_split), ptr(F), F.stride(0), ptr(out),
         out.stride(0), stream_handle())
    return out


def laplacian_config(use_tma=2):
    """Select the complex64 Laplacian kernel process-wide: 0 / False = the
    kernel reading every neighbour through L1/L2; 1 / True = input planes
    staged by TMA; 2 (the default) = strips whose links and inputs are all
    staged by TMA.  The staged kernels are used where their shape limits
    allow."""
    mode = int(use_tma) if not isinstance(use_tma, bool) else (1 if use_tma else 0)
    call("ed_laplacian_config", mode)


def laplacian_status():
    """Synchronise the current stream and raise if a bounded wait of the
    TMA-staged Laplacian gave up since the last check."""
    code = ctypes.c_int()
    call("ed_laplacian_status", ctypes.byref(code), stream_handle())
    return code.value


def lanczos_tr(links_soa: torch.Tensor, latt_size, Ne: int, tol: float, ncv: int = None, max_restarts: int = None,
               poly_deg: int = 0, lambda_cut: float = 0.0, stencil_precision: str = "fp64",
               links_c64: torch.Tensor = None, gs_precision: str = "fp64"):
    """Native batched thick-restart Lanczos (``ed_lanczos_tr`` /
    ``ed_lanczos_tr_ex``) for the lowest ``Ne`` eigenpairs of the FP64
    Laplacian of every timeslice of ``links_soa`` (complex128 ``[nt, 27, V3]``).

    ``stencil_precision="fp32"`` runs the mixed solve: the complex64 stencil
    on ``links_c64`` (complex64 SoA of the same links) inside a loose FP64
    thick-restart iteration, then an FP64 Chebyshev-filtered refinement whose
    cut comes from it (``poly_deg``: its degree, 0 = 16; ``lambda_cut`` <= 0:
    automatic).  ``gs_precision="df"`` runs the Gram-Schmidt passes in
    double-float arithmetic on the FP32 pipe (``ED_LANCZOS_GS_DF``; products
    to ~2^-47 relative, the basis streamed at HBM speed) instead of FP64.
    Returns (evals ``[nt, Ne]`` float64 ascending, evecs
    ``[nt, Ne, 3, V3]`` complex128 colour planes, stats ``{"converged",
    "restarts", "matvecs", ...}``)."""
    require_cuda(links_soa, "links")
    if links_soa.dtype != torch.complex128:
        raise ValueError("the native Lanczos works on complex128 links")
    if stencil_precision not in ("fp64", "fp32"):
        raise ValueError("stencil_precision must be 'fp64' or 'fp32'")
    if gs_precision not in ("fp64", "df"):
        raise ValueError("gs_precision must be 'fp64' or 'df'")
    gs_flag = ED_LANCZOS_GS_DF if gs_precision == "df" else 0
    Lx, Ly, Lz = (int(v) for v in latt_size[:3])
    nt, V3 = links_soa.shape[0], Lx * Ly * Lz
    if tuple(links_soa.shape[1:]) != (27, V3):
        raise ValueError("links must be [nt, 27, Lx*Ly*Lz]")
    n = 3 * V3
    mixed = stencil_precision == "fp32"
    if ncv is None:
        ncv = min(max(2 * Ne if (poly_deg > 0 and not mixed) else 9 * Ne // 4, Ne + 32), n - 1)
    if max_restarts is None:
        max_restarts = max(30, 10 * n // max(1, ncv - Ne))
    evecs = torch.empty((nt, Ne, 3, V3), dtype=torch.complex128, device=links_soa.device)
    evals = torch.empty((nt, Ne), dtype=torch.float64, device=links_soa.device)
    nbytes = ctypes.c_size_t()
    if not mixed and gs_flag:
        call("ed_lanczos_workspace_ex", Lx, Ly, Lz, nt, Ne, ncv, ED_C128 | gs_flag, ctypes.byref(nbytes))
        ws = torch.empty(nbytes.value, dtype=torch.uint8, device=links_soa.device)
        st = (ctypes.c_int * 6)()
        call("ed_lanczos_tr_ex", Lx, Ly, Lz, nt, ptr(links_soa), None, ED_C128 | gs_flag, Ne, float(tol), ncv,
             max_restarts, int(poly_deg), float(lambda_cut), ptr(evecs), ptr(evals), st, ptr(ws), ws.numel(),
             stream_handle())
        return evals, evecs, {"converged": bool(st[0]), "restarts": int(st[1]), "matvecs": int(st[2]), "ncv": ncv,
                              "gs_precision": gs_precision}
    if not mixed:
        call("ed_lanczos_workspace", Lx, Ly, Lz, nt, Ne, ncv, ctypes.byref(nbytes))
        ws = torch.empty(nbytes.value, dtype=torch.uint8, device=links_soa.device)
        st = (ctypes.c_int * 3)()
        call("ed_lanczos_tr", Lx, Ly, Lz, nt, ptr(links_soa), Ne, float(tol), ncv, max_restarts, int(poly_deg),
             float(lambda_cut), ptr(evecs), ptr(evals), st, ptr(ws), ws.numel(), stream_handle())
        return evals, evecs, {"converged": bool(st[0]), "restarts": int(st[1]), "matvecs": int(st[2]), "ncv": ncv}
    if links_c64 is None or links_c64.dtype != torch.complex64 or tuple(links_c64.shape) != tuple(links_soa.shape):
        raise ValueError("the fp32 stencil needs links_c64: complex64 SoA links of the same shape")
    require_cuda(links_c64, "links_c64")
    call("ed_lanczos_workspace_ex", Lx, Ly, Lz, nt, Ne, ncv, ED_C64 | gs_flag, ctypes.byref(nbytes))
    ws = torch.empty(nbytes.value, dtype=torch.uint8, device=links_soa.device)
    st = (ctypes.c_int * 6)()
    call("ed_lanczos_tr_ex", Lx, Ly, Lz, nt, ptr(links_soa), ptr(links_c64), ED_C64 | gs_flag, Ne, float(tol), ncv,
         max_restarts, int(poly_deg), float(lambda_cut), ptr(evecs), ptr(evals), st, ptr(ws), ws.numel(),
         stream_handle())
    return evals, evecs, {"converged": bool(st[0]), "restarts": int(st[1]), "matvecs": int(st[2]), "ncv": ncv,
                          "matvecs_fp32": int(st[3]), "matvecs_fp64": int(st[4]), "restarts_fp32": int(st[5])}


def cgs_pass(V: torch.Tensor, r: int, w: torch.Tensor, h: torch.Tensor = None, norm: bool = False,
             precision: str = "fp64"):
    """One classical Gram-Schmidt pass (``ed_cgs_pass``): ``h = V[:, :r]^H w``,
    ``w -= V[:, :r] h`` in place.  ``V``: complex128 [B, rows, n] with
    contiguous rows (any batch stride), ``w``: contiguous complex128 [B, n].
    Returns ``h`` [B, r], and with ``norm`` also ``||w||`` [B] float64 of the
    updated w (from the kernel's per-block partial sums).  ``precision="df"``:
    the double-float pass on the FP32 pipe (``ed_cgs_pass_df``)."""
    if precision not in ("fp64", "df"):
        raise ValueError("precision must be 'fp64' or 'df'")
    if V.dtype != torch.complex128 or w.dtype != torch.complex128:
        raise ValueError("cgs_pass works on complex128")
    if not (V.is_cuda and w.is_cuda) or not w.is_contiguous():
        raise ValueError("V and w must be CUDA tensors, w contiguous")
    B, rows, n = V.shape
    if V.stride(2) != 1 or V.stride(1) != n or not (0 < r <= rows) or tuple(w.shape) != (B, n):
        raise ValueError("V must be [B, rows, n] with contiguous rows, w [B, n], 0 < r <= rows")
    if h is None:
        h = torch.empty((B, r), dtype=torch.complex128, device=w.device)
    part = torch.empty((B, (n + 255) // 256), dtype=torch.float64, device=w.device) if norm else None
    if precision == "df":
        ws = torch.empty(B * (r + 1) * n * 16, dtype=torch.uint8, device=w.device)
        call("ed_cgs_pass_df", B, r, n, ptr(V), V.stride(0), ptr(w), ptr(h), h.stride(0),
             None if part is None else ptr(part), ptr(ws), ws.numel(), stream_handle())
    else:
        call("ed_cgs_pass", B, r, n, ptr(V), V.stride(0), ptr(w), ptr(h), h.stride(0),
             None if part is None else ptr(part), stream_handle())
    if norm:
        return h, torch.sqrt(part.sum(dim=1))
    return h


def arrow_eigh(d: torch.Tensor, e: torch.Tensor, s: torch.Tensor = None, nwant: int = None):
    """Lowest ``nwant`` eigenpairs of the batched arrowhead + tridiagonal
    matrices of thick-restart Lanczos (``ed_arrow_eigh``): ``d`` [B, m] the
    diagonal, ``e`` [B, m-1] the off-diagonal ``T[j, j+1]`` (used from row
    ``ka`` on), ``s`` [B, ka] the border ``T[j, ka]`` (None: tridiagonal).
    FP64 device tensors.  Returns (evals [B, nwant] ascending, evecs [B, m, nwant])."""
    if d.dim() != 2 or d.dtype != torch.float64:
        raise ValueError("d must be float64 [B, m]")
    d = d.contiguous()
    require_cuda(d, "d")
    B, m = d.shape
    nwant = m if nwant is None else int(nwant)
    ka = 0 if s is None else s.shape[1]
    e = e.contiguous() if m > 1 else torch.zeros((B, 1), dtype=torch.float64, device=d.device)
    if e.dtype != torch.float64 or e.shape[0] != B or (m > 1 and e.shape[1] != m - 1):
        raise ValueError("e must be float64 [B, m-1]")
    if s is not None:
        s = s.contiguous()
        if s.dtype != torch.float64 or s.shape[0] != B:
            raise ValueError("s must be float64 [B, ka]")
    nbytes = ctypes.c_size_t()
    call("ed_arrow_eigh_workspace", B, m, nwant, ctypes.byref(nbytes))
    ws = torch.empty(nbytes.value // 8 + 1, dtype=torch.float64, device=d.device)
    evals = torch.empty((B, nwant), dtype=torch.float64, device=d.device)
    evecs = torch.empty((B, m, nwant), dtype=torch.float64, device=d.device)
    call("ed_arrow_eigh", B, m, ka, nwant, ptr(d), None if s is None else ptr(s), ptr(e), ptr(evals), ptr(evecs),
         ptr(ws), ws.numel() * 8, stream_handle())
    return evals, evecs


def covariant_derivative(links_soa_c128: torch.Tensor, F: torch.Tensor, latt_size, direction: int, out_dtype=None):
    """One hop ``D_d F = U_d(x) F(x+d) - U_d(x-d)^dag F(x-d)``
    (``lattice/generator/elemental.py:282-287``); ``F`` colour planes ``[nvec, 3, V3]``."""
    Lx, Ly, Lz = latt_size[0], latt_size[1], latt_size[2]
    require_cuda(F, "F")
    require_cuda(links_soa_c128, "links")
    out_dtype = out_dtype or F.dtype
    nvec = F.numel() // (3 * Lx * Ly * Lz)
    out = torch.empty_like(F, dtype=out_dtype)
    call(
        "ed_covariant_derivative",
        prec_of(F),
        _PREC[out_dtype],
        Lx,
        Ly,
        Lz,
        int(direction),
        nvec,
        ptr(links_soa_c128),
        ptr(F),
        ptr(out),
        stream_handle(),
    )
    return out


def parallel_transport(links_soa_c128: torch.Tensor, F: torch.Tensor, latt_size, direction: int, sign: int,
                       out: torch.Tensor = None):
    """``U_d(x) F(x+d)`` (sign +1) or ``U_d(x-d)^dag F(x-d)`` (sign -1) on c128
    colour planes ``[nvec, 3, V3]`` (``displacement_elemental.py:53-71``)."""
    Lx, Ly, Lz = latt_size[0], latt_size[1], latt_size[2]
    require_cuda(F, "F")
    nvec = F.numel() // (3 * Lx * Ly * Lz)
    out = torch.empty_like(F) if out is None else out
    call("ed_parallel_transport", Lx, Ly, Lz, int(direction), int(sign), nvec, ptr(links_soa_c128), ptr(F), ptr(out),
         stream_handle())
    return out


def mean_c128(stack: torch.Tensor, out: torch.Tensor = None):
    """Mean over the leading axis of a contiguous complex128 stack."""
    require_cuda(stack, "stack")
    n = stack[0].numel()
    out = torch.empty_like(stack[0]) if out is None else out
    call("ed_mean_c128", stack.shape[0], n, n, ptr(stack), ptr(out), stream_handle())
    return out


#: elemental arithmetic modes (ED_MODE_* in include/easydist_gb300.h)
MODES = {"fp64": 0, "f16x3": 1, "bf16x3": 2, "tf32x3": 3, "ozaki_i8": 4}
_FLAG_NO_FACTOR, _FLAG_FORCE_FACTOR, _FLAG_LEFT_FACTOR = 0x100, 0x200, 0x800
_FLAG_GAUSS = 0x400  # ED_MODE_FLAG_GAUSS
#: plan launch settings (ED_TUNE_* keys)
TUNING_KEYS = {"f64_tile": 1, "tc_slab_kb": 2, "tc_grid": 3, "tc_stages": 4, "tc_pair": 5, "tc_kpb": 6,
               "tc_stack": 7, "f64_df": 8}
#: FP64 pair GEMM tile shapes (rows, cols) by ED_TUNE_F64_TILE value
F64_TILES = {0: (64, 64), 1: (32, 64), 2: (64, 32), 3: (32, 32)}


class ElementalPlan:
    """Owner of an ``ed_elemental_plan`` and its device workspace."""

    def __init__(self, latt_size, Ne: int, num_nabla: int, momentum_list, mode: str = "fp64", device=None,
                 batch: int = 1, factorise=True, tuning=None, gauss: bool = False):
        """``factorise=False`` keeps the tensor-core GEMM that forms the
        phase-weighted operand inside the kernel even when the momentum list
        factorises (ED_MODE_FLAG_NO_FACTOR); ``factorise="force"`` factorises
        however many (px,py) x pz combinations the list leaves unused
        (ED_MODE_FLAG_FORCE_FACTOR); ``factorise="left"`` factorises with every
        momentum's whole phase on the left operand and none on the right
        (ED_MODE_FLAG_LEFT_FACTOR: Nmom left variants per left chain, no
        unused combinations, for any list of at most 127 distinct momenta).
        ``gauss=True`` runs the factorised split
        GEMM in the Gauss three-multiplication form (ED_MODE_FLAG_GAUSS).
        ``tuning``: launch settings (``TUNING_KEYS``, see ``set_tuning``).
        ``mode="df64"``: the FP64 mode with its pair GEMM in double-float
        arithmetic on the FP32 pipe (``ED_TUNE_F64_DF``; FP64-class results)."""
        if mode == "df64":
            tuning = {**(tuning or {}), "f64_df": 1}
        elif mode not in MODES:
            raise ValueError(f"unknown elemental mode {mode!r}; available: {sorted(MODES) + ['df64']}")
        if factorise not in (True, False, "force", "left"):
            raise ValueError(f"factorise must be True, False, 'force' or 'left', not {factorise!r}")
        cmode = MODES["fp64" if mode == "df64" else mode] | {True: 0, False: _FLAG_NO_FACTOR, "force": _FLAG_FORCE_FACTOR,
                               "left": _FLAG_LEFT_FACTOR}[factorise]
        if gauss:
            cmode |= _FLAG_GAUSS
        self.factorise = factorise
        self.gauss = bool(gauss)
        Lx, Ly, Lz = latt_size[0], latt_size[1], latt_size[2]
        self.latt_size = list(latt_size)
        self.Ne = Ne
        self.mode = mode
        self.num_nabla = num_nabla
        self.batch = int(batch)
        self.momentum_list = [tuple(int(v) for v in p) for p in momentum_list]
        moms = [v for p in self.momentum_list for v in p]
        arr = (ctypes.c_int * len(moms))(*moms)
        handle = ctypes.c_void_p()
        if self.batch == 1:
            rc = _lib.lib().ed_elemental_plan_create(
                ctypes.byref(handle), Lx, Ly, Lz, Ne, num_nabla, arr, len(self.momentum_list), cmode
            )
        else:
            rc = _lib.lib().ed_elemental_plan_create_batched(
                ctypes.byref(handle), Lx, Ly, Lz, Ne, num_nabla, arr, len(self.momentum_list), cmode,
                self.batch
            )
        _lib.check(rc, "ed_elemental_plan_create")
        self._h = handle
        nbytes = ctypes.c_size_t()
        call("ed_elemental_workspace_size", self._h, ctypes.byref(nbytes))
        npairs = ctypes.c_int()
        call("ed_elemental_num_pairs", self._h, ctypes.byref(npairs))
        self.workspace_bytes = nbytes.value
        self.num_pairs = npairs.value
        fac, pxy, pz = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        call("ed_elemental_factorised", self._h, ctypes.byref(fac), ctypes.byref(pxy), ctypes.byref(pz))
        #: (Pxy, Pz) when the factorised-phase GEMM serves this plan, else None
        self.factorised = (pxy.value, pz.value) if fac.value else None
        self.device = torch.device(device or "cuda")
        self._ws = None
        if tuning:
            self.set_tuning(**tuning)

    def set_tuning(self, **settings):
        """Launch settings of later runs: ``f64_tile`` (0..3, see ``F64_TILES``),
        ``tc_slab_kb`` (0 or a power of two <= 256), ``tc_grid`` (0 or a CTA
        bound), ``tc_stages`` (0, 2 or 3).  0 restores the built-in default."""
        for name, value in settings.items():
            if name not in TUNING_KEYS:
                raise ValueError(f"unknown tuning setting {name!r}; available: {sorted(TUNING_KEYS)}")
            call("ed_elemental_set_tuning", self._h, TUNING_KEYS[name], int(value))
        # some settings change the workspace the plan needs (the stacked SM-pair GEMM's second result plane)
        nbytes = ctypes.c_size_t()
        call("ed_elemental_workspace_size", self._h, ctypes.byref(nbytes))
        if nbytes.value != self.workspace_bytes:
            self.workspace_bytes = nbytes.value
            self._ws = None

    def tuning(self) -> dict:
        out = {}
        for name, key in TUNING_KEYS.items():
            v = ctypes.c_int()
            call("ed_elemental_get_tuning", self._h, key, ctypes.byref(v))
            out[name] = v.value
        return out

    def workspace(self):
        if self._ws is None:
            self._ws = torch.empty(self.workspace_bytes, dtype=torch.uint8, device=self.device)
        return self._ws

    def run(self, links: torch.Tensor, dir_stride: int, site_stride: int, evecs: torch.Tensor, out: torch.Tensor,
            blend: torch.Tensor = None):
        """``links``: complex128 device view of the timeslice's spatial links
        (element (mu, site, a, b) at mu*dir_stride + site*site_stride + 3a+b);
        ``evecs``: ``[Ne, V3*3]``-contiguous c128/c64; ``out``: ``[Nderiv, Nmom, Ne, Ne]`` c128."""
        ws = self.workspace()
        require_cuda(evecs, "evecs")
        require_cuda(out, "out")
        if out.dtype != torch.complex128:
            raise ValueError("out must be complex128")
        bptr = None
        if blend is not None:
            require_cuda(blend, "blend")
            bptr = ptr(blend)
        call(
            "ed_elemental_run",
            self._h,
            ptr(links),
            dir_stride,
            site_stride,
            prec_of(evecs),
            ptr(evecs),
            bptr,
            ptr(out),
            ptr(ws),
            ws.numel(),
            stream_handle(),
        )
        return out

    def run_batch(self, links, dir_stride: int, site_stride: int, evecs, outs, blend: torch.Tensor = None):
        """Several timeslices in one pass (one pair-contraction launch).
        ``links``/``evecs``/``outs``: equal-length lists of device tensors, each
        as in :meth:`run`; at most ``batch`` of them."""
        nb, prec = self._check_batch(links, evecs, outs)
        ws = self.workspace()
        P = ctypes.c_void_p * nb
        call("ed_elemental_run_batch", self._h, nb, P(*[ptr(t) for t in links]), dir_stride, site_stride, prec,
             P(*[ptr(t) for t in evecs]), None if blend is None else ptr(blend), P(*[ptr(t) for t in outs]),
             ptr(ws), ws.numel(), stream_handle())
        return outs

    def _check_batch(self, links, evecs, outs):
        nb = len(links)
        if not (0 < nb <= self.batch) or len(evecs) != nb or len(outs) != nb:
            raise ValueError(f"need 1..{self.batch} timeslices with matching links, evecs and outs")
        prec = prec_of(evecs[0])
        for v in evecs:
            require_cuda(v, "evecs")
            if prec_of(v) != prec:
                raise ValueError("all eigenvector blocks must share a precision")
        for o in outs:
            require_cuda(o, "out")
        return nb, prec

    def run_batch_begin(self, links, dir_stride: int, site_stride: int, evecs):
        """First part of :meth:`run_batch` (``ed_elemental_run_batch_begin``):
        the phases and chains of ``len(links)`` timeslices.  The pair
        contraction follows in :func:`gemm_multi`, the combine in
        :meth:`run_batch_end`."""
        nb, prec = self._check_batch(links, evecs, evecs)
        ws = self.workspace()
        P = ctypes.c_void_p * nb
        call("ed_elemental_run_batch_begin", self._h, nb, P(*[ptr(t) for t in links]), dir_stride, site_stride, prec,
             P(*[ptr(t) for t in evecs]), ptr(ws), ws.numel(), stream_handle())

    def run_batch_end(self, outs, blend: torch.Tensor = None):
        """Last part of :meth:`run_batch` (``ed_elemental_run_batch_end``): the
        combine of the contracted pairs into ``outs``."""
        nb = len(outs)
        if not (0 < nb <= self.batch):
            raise ValueError(f"need 1..{self.batch} outputs")
        for o in outs:
            require_cuda(o, "out")
        ws = self.workspace()
        P = ctypes.c_void_p * nb
        call("ed_elemental_run_batch_end", self._h, nb, None if blend is None else ptr(blend),
             P(*[ptr(t) for t in outs]), ptr(ws), ws.numel(), stream_handle())
        return outs

    def describe(self):
        """Pair groups of the plan: left chain and number of right chains of
        each, and whether hermiticity (p -> -p) is used."""
        n, herm = ctypes.c_int(), ctypes.c_int()
        left = (ctypes.c_int * 64)()  # kMaxJobs
        nright = (ctypes.c_int * 64)()
        call("ed_elemental_describe", self._h, ctypes.byref(n), left, nright, ctypes.byref(herm))
        return {"left": list(left[: n.value]), "nright": list(nright[: n.value]), "herm": bool(herm.value)}

    def set_profile_events(self, start=None, stop=None):
        """Have every later run record the torch CUDA events ``start``/``stop``
        around the pair-contraction kernel (``None`` disables).  The events
        must already hold a CUDA handle (record them once beforehand)."""
        h0 = ctypes.c_void_p(start.cuda_event) if start is not None else None
        h1 = ctypes.c_void_p(stop.cuda_event) if stop is not None else None
        call("ed_elemental_set_profile_events", self._h, h0, h1)

    def check_status(self):
        """Synchronise and raise if a bounded device wait of the last run gave up."""
        code = ctypes.c_int()
        call("ed_elemental_status", self._h, ptr(self.workspace()), ctypes.byref(code), stream_handle())
        return code.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().ed_elemental_plan_destroy(h)
            except Exception:
                pass
            self._h = None


def gemm_multi(plans, nbatch) -> int:
    """The pair contraction of several batched plans (each after its
    :meth:`ElementalPlan.run_batch_begin`, ``nbatch[v]`` timeslices) in one
    launch when all take the on-chip-phase tensor-core path with the same
    split mode, else one launch per plan (``ed_elemental_gemm_multi``).
    Returns the number of GEMM launches."""
    n = len(plans)
    if n == 0 or len(nbatch) != n:
        raise ValueError("need one batch size per plan")
    wss = [p.workspace() for p in plans]
    launches = ctypes.c_int()
    call("ed_elemental_gemm_multi", n, (ctypes.c_void_p * n)(*[p._h for p in plans]), (ctypes.c_int * n)(*nbatch),
         (ctypes.c_void_p * n)(*[ptr(w) for w in wss]), (ctypes.c_size_t * n)(*[w.numel() for w in wss]),
         ctypes.byref(launches), stream_handle())
    return launches.value


class PairPlan:
    """Generic pair contraction on caller-built colour-plane chains
    (``ed_pair_plan_create`` / ``ed_pair_run``):
    ``G[p, i, r*Ne + j] = sum_k conj(X_i[k]) phase_p(k) Y_{right0+r, j}[k]``."""

    def __init__(self, latt_size, Ne: int, nchain: int, momentum_list, left: int, right0: int, nright: int,
                 mode: str = "fp64", device=None):
        if mode not in MODES:
            raise ValueError(f"unknown mode {mode!r}")
        Lx, Ly, Lz = latt_size[0], latt_size[1], latt_size[2]
        self.Ne, self.nright, self.mode = Ne, nright, mode
        self.momentum_list = [tuple(int(v) for v in p) for p in momentum_list]
        moms = [v for p in self.momentum_list for v in p]
        arr = (ctypes.c_int * len(moms))(*moms)
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().ed_pair_plan_create(ctypes.byref(h), Lx, Ly, Lz, Ne, nchain, arr,
                                                   len(self.momentum_list), MODES[mode], left, right0, nright),
                   "ed_pair_plan_create")
        self._h = h
        nbytes = ctypes.c_size_t()
        call("ed_elemental_workspace_size", self._h, ctypes.byref(nbytes))
        self.workspace_bytes = nbytes.value
        self.device = torch.device(device or "cuda")
        self._ws = None

    def run(self, chains: torch.Tensor, G: torch.Tensor = None):
        require_cuda(chains, "chains")
        if G is None:
            G = torch.empty((len(self.momentum_list), self.Ne, self.nright * self.Ne), dtype=torch.complex128,
                            device=chains.device)
        if self._ws is None:
            self._ws = torch.empty(self.workspace_bytes, dtype=torch.uint8, device=self.device)
        call("ed_pair_run", self._h, ptr(chains), ptr(G), ptr(self._ws), self._ws.numel(), stream_handle())
        return G

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().ed_elemental_plan_destroy(h)
            except Exception:
                pass
            self._h = None
