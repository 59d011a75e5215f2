"""3D stout smearing of the spatial links (reference
``lattice/generator/stout_smear.cu:159-245``, numpy form
``lattice/generator/eigenvector.py:123-190``)."""

from __future__ import annotations


def stout_smear_(U, latt_size, nstep: int, rho: float):
    raise NotImplementedError("stout smearing on the GPU is not built yet")
