"""GB300 drop-in for ``lattice.generator.EigenvectorGenerator``.

Same constructor, ``load``, ``project_SU3``, ``stout_smear`` and ``calc``
signatures as ``lattice/generator/eigenvector.py:30-53,356-370``.  ``calc(t)``
computes the ``Ne`` lowest eigenpairs of the 3D covariant Laplacian on
timeslice ``t`` with the library's stencil kernel inside a GPU thick-restart
Lanczos (FP64 basis, reorthogonalisation and Rayleigh-Ritz), sorts them
ascending and applies the reference's renormalisation phase
(``eigenvector.py:249-257``).  It returns device tensors
``(evecs [Ne, Lz, Ly, Lx, 3] complex128, evals [Ne] float64)`` (host numpy
arrays after ``easydistillation_gb300.set_backend("numpy")``).

``stencil_precision="fp32"`` (native driver) runs the mixed solve of
``ed_lanczos_tr_ex``: the complex64 stencil inside the thick-restart
iteration (FP64 basis, Gram-Schmidt, Rayleigh-Ritz and convergence test) to a
loose tolerance, then an FP64 Chebyshev-filtered refinement of every pair to
``tol`` whose cut the first phase supplies; with ``driver="python"`` the
same idea runs as an FP32-stencil Lanczos followed by an FP64 Lanczos started
from its Ritz vectors.  ``"fp64"`` (default) uses the FP64 stencil
throughout.
"""

from __future__ import annotations

from typing import List, Sequence

import torch

from .. import lanczos as LZ
from ..backend import to_backend
from ..ops import lanczos_tr, links_to_soa, laplacian, vectors_from_planes
from .elemental import gauge_to_device

NC = 3


def project_su3_(U: torch.Tensor, tol: float = 1e-15, max_iter: int = 100):
    """In-place projection of links ``[..., 3, 3]`` (contiguous complex128 on
    the device) onto U(3) by the averaged inverse iteration of
    ``eigenvector.py:55-65`` (``U <- (U + U^-dag)/2``), in the library's
    ``ed_project_su3`` kernel (one thread per link)."""
    from .. import _lib

    if U.dtype != torch.complex128 or not U.is_cuda or not U.is_contiguous() or U.shape[-2:] != (3, 3):
        raise ValueError("links must be a contiguous complex128 CUDA tensor [..., 3, 3]")
    _lib.call("ed_project_su3", U.numel() // 9, _lib.ptr(U), float(tol), int(max_iter), _lib.stream_handle())
    return U


def stout_smear_links_(U: torch.Tensor, latt_size, nstep: int, rho: float):
    from ..stout import stout_smear_

    stout_smear_(U, latt_size, nstep, rho)


class EigenvectorGenerator:
    def __init__(self, latt_size: List[int], gauge_field, Ne: int, tol: float, *, stencil_precision: str = "fp64",
                 device=None, ncv: int = None, driver: str = "native", gs_precision: str = "fp64") -> None:
        """``ncv``: Krylov dimension of the thick-restart Lanczos (default
        max(9 Ne / 4, Ne + 32), 2 Ne with Chebyshev acceleration, capped by
        the problem size).  ``driver``: ``"native"`` runs the FP64-stencil
        eigensolve in the library (``ed_lanczos_tr``); ``"python"`` drives the
        same kernels from ``lanczos.trlanczos`` (the FP32-stencil mode always
        does).  ``gs_precision="df"`` (native driver): Gram-Schmidt in
        double-float arithmetic on the FP32 pipe (``ED_LANCZOS_GS_DF``)."""
        if stencil_precision not in ("fp64", "fp32"):
            raise ValueError("stencil_precision must be 'fp64' or 'fp32'")
        if gs_precision not in ("fp64", "df"):
            raise ValueError("gs_precision must be 'fp64' or 'df'")
        if gs_precision == "df" and driver != "native":
            raise ValueError("gs_precision='df' needs the native driver")
        self.gs_precision = gs_precision
        if driver not in ("native", "python"):
            raise ValueError("driver must be 'native' or 'python'")
        self.driver = driver
        self.ncv = ncv
        self.device = torch.device(device or "cuda")
        self.latt_size = latt_size
        self.gauge_field = gauge_field
        self.Ne = Ne
        self.tol = tol
        self.stencil_precision = stencil_precision
        self._U = None
        self._soa = {}
        self.last_stats = None

    def load(self, key: str):
        self._U = gauge_to_device(self.gauge_field.load(key), self.latt_size, self.device)
        self._soa = {}

    def project_SU3(self):
        project_su3_(self._U)
        self._soa = {}

    def stout_smear(self, nstep: int, rho: float):
        stout_smear_links_(self._U, self.latt_size, nstep, rho)
        self._soa = {}

    def _links(self, dtype):
        if dtype not in self._soa:
            self._soa[dtype] = links_to_soa(self._U, self.latt_size, dtype=dtype)
        return self._soa[dtype]

    def _matvec(self, ts: Sequence[int], dtype):
        Lx, Ly, Lz, Lt = self.latt_size
        V3 = Lx * Ly * Lz
        links = self._links(dtype)
        idx = torch.as_tensor(list(ts), device=self.device)
        sel = links if list(ts) == list(range(Lt)) else links.index_select(0, idx)

        def mv(X: torch.Tensor) -> torch.Tensor:
            B = X.shape[0]
            if dtype == torch.complex128:
                F = X.view(B, 1, NC, V3)
            else:
                F = X.to(dtype).view(B, 1, NC, V3)
            out = laplacian(sel, F, self.latt_size)
            return out.view(B, NC * V3).to(torch.complex128)

        return mv

    def calc_batch(self, ts: Sequence[int], apply_renorm_phase: bool = True, polynomial_degree: int = 0,
                   lambda_cut: float = 0.0):
        """Eigenpairs of several timeslices solved in lock step.

        With ``polynomial_degree > 0`` and ``lambda_cut > 0`` (the reference's
        Chebyshev acceleration, ``eigenvector.py:295-299``), the Lanczos
        iteration runs on ``-T_deg((2L - (12 + cut)) / (12 - cut))``, which
        maps the unwanted part of the spectrum [cut, 12] into [-1, 1] and
        makes the wanted low modes dominant; the eigenpairs of ``L`` then
        come from an FP64 Rayleigh-Ritz step on the converged vectors."""
        if self._U is None:
            raise RuntimeError("call load(key) before calc(t)")
        Lx, Ly, Lz, Lt = self.latt_size
        V3 = Lx * Ly * Lz
        n = NC * V3
        ts = list(ts)
        B = len(ts)
        if self.driver == "native":
            idx = None if ts == list(range(Lt)) else torch.as_tensor(ts, device=self.device)
            links = self._links(torch.complex128)
            sel = links if idx is None else links.index_select(0, idx)
            if self.stencil_precision == "fp32":
                # mixed solve: complex64 stencil in a loose FP64 iteration, then the FP64 Chebyshev refinement
                l32 = self._links(torch.complex64)
                l32 = l32 if idx is None else l32.index_select(0, idx)
                evals, planes, stats = lanczos_tr(sel, self.latt_size, self.Ne, self.tol, ncv=self.ncv,
                                                  poly_deg=polynomial_degree if polynomial_degree > 0 else 0,
                                                  lambda_cut=lambda_cut if lambda_cut > 0 else 0.0,
                                                  stencil_precision="fp32", links_c64=l32,
                                                  gs_precision=self.gs_precision)
            else:
                poly = polynomial_degree if (polynomial_degree > 0 and lambda_cut > 0) else 0
                evals, planes, stats = lanczos_tr(sel, self.latt_size, self.Ne,
                                                  max(self.tol, 1e-12) if poly else self.tol, ncv=self.ncv,
                                                  poly_deg=poly, lambda_cut=lambda_cut if poly else 0.0,
                                                  gs_precision=self.gs_precision)
            self.last_stats = {k: v for k, v in stats.items() if k not in ("ncv", "gs_precision")}
            evecs = planes.reshape(B, self.Ne, n)
            if apply_renorm_phase:
                LZ.renorm_phase_(evecs)
            out = vectors_from_planes(evecs.reshape(B, self.Ne, NC, V3), V3)
            return out.reshape(B, self.Ne, Lz, Ly, Lx, NC), evals
        if polynomial_degree > 0 and lambda_cut > 0:
            mv = self._matvec(ts, torch.complex64 if self.stencil_precision == "fp32" else torch.complex128)
            # below the cut T_deg has the sign (-1)^deg: negate so the wanted modes are the smallest
            cheb = LZ.chebyshev_operator(mv, polynomial_degree, lambda_cut, 12.0, negate=polynomial_degree % 2 == 0)
            # the filter separates the wanted modes: a smaller Krylov space than the plain
            # iteration's suffices (24^3, Ne = 100, degree 16: 2 Ne -> 1.13 s, 3 Ne -> 3.2 s per 8 timeslices)
            ncv = self.ncv or min(max(2 * self.Ne, self.Ne + 32), n - 1)
            res = LZ.trlanczos(cheb, B, n, self.Ne, max(self.tol, 1e-12), ncv=ncv, device=self.device)
            lam, X, resid = LZ.rayleigh_ritz(self._matvec(ts, torch.complex128), res.evecs)
            res.evals, res.evecs, res.residuals = lam, X, resid
            res.matvecs = res.matvecs * polynomial_degree + self.Ne
        elif self.stencil_precision == "fp32":
            r32 = LZ.trlanczos(self._matvec(ts, torch.complex64), B, n, self.Ne, max(self.tol, 1e-6),
                               ncv=self.ncv, device=self.device)
            v0 = r32.evecs.sum(dim=1)
            res = LZ.trlanczos(self._matvec(ts, torch.complex128), B, n, self.Ne, self.tol, v0=v0,
                               ncv=self.ncv, device=self.device)
            res.matvecs += r32.matvecs
        else:
            res = LZ.trlanczos(self._matvec(ts, torch.complex128), B, n, self.Ne, self.tol, ncv=self.ncv,
                               device=self.device)
        self.last_stats = {"restarts": res.restarts, "matvecs": res.matvecs, "converged": res.converged}
        evals, evecs = LZ.sort_ascending(res.evals, res.evecs)
        if apply_renorm_phase:
            LZ.renorm_phase_(evecs)
        out = vectors_from_planes(evecs.reshape(B, self.Ne, NC, V3), V3)
        return out.reshape(B, self.Ne, Lz, Ly, Lx, NC), evals

    def calc(self, t: int, apply_renorm_phase: bool = True, polynomial_degree: int = 0, lambda_cut: float = 0.0):
        evecs, evals = self.calc_batch([t], apply_renorm_phase, polynomial_degree, lambda_cut)
        return to_backend(evecs[0]), to_backend(evals[0])

    # The reference's per-backend solvers (scipy/cupyx eigsh on its numpy
    # stencil, ``eigenvector.py:234-257``; QUDA's eigensolver with Chebyshev
    # acceleration, ``:259-312``; eigsh on QUDA's stencil, ``:314-354``) return
    # the same eigenpairs on the same scale as ``calc``; here each runs this
    # library's eigensolve, with the Chebyshev acceleration where the QUDA
    # solver takes a degree and a cut.
    def laplacian_cupy_numpy(self, t: int, apply_renorm_phase: bool):
        return self.calc(t, apply_renorm_phase)

    def laplacian_quda(self, t: int, apply_renorm_phase: bool, polynomial_degree: int, lambda_cut: float):
        return self.calc(t, apply_renorm_phase, polynomial_degree, lambda_cut)

    def laplacian_quda_scipy(self, t: int, apply_renorm_phase: bool):
        return self.calc(t, apply_renorm_phase)
