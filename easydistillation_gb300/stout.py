"""3D stout smearing of the spatial links on the GPU.

Replaces ``EigenvectorGenerator.stout_smear`` / ``ElementalGenerator.stout_smear``
(``lattice/generator/eigenvector.py:215-232``; kernel
``lattice/generator/stout_smear.cu:159-245``; numpy form ``:123-190``): each
of the ``nstep`` steps replaces every spatial link by ``exp(iQ) U`` computed
from its 3D staples, in FP64, out of place.
"""

from __future__ import annotations

import torch

from ._lib import call, ptr, require_cuda, stream_handle


def stout_smear_(U: torch.Tensor, latt_size, nstep: int, rho: float) -> torch.Tensor:
    """In-place ``nstep`` smearing steps of ``U`` = ``[3, Lt, Lz, Ly, Lx, 3, 3]``
    complex128 (the generators' spatial links)."""
    require_cuda(U, "U")
    if U.dtype != torch.complex128 or U.shape[0] != 3:
        raise ValueError("U must be complex128 spatial links [3, Lt, Lz, Ly, Lx, 3, 3]")
    Lx, Ly, Lz = latt_size[0], latt_size[1], latt_size[2]
    nt = U.shape[1]
    if nstep <= 0:
        return U
    tmp = torch.empty_like(U)
    src, dst = U, tmp
    for _ in range(nstep):
        call("ed_stout_smear_step", Lx, Ly, Lz, nt, float(rho), ptr(src), ptr(dst), stream_handle())
        src, dst = dst, src
    if src.data_ptr() != U.data_ptr():
        U.copy_(src)
    return U
