"""Seeded synthetic inputs for benchmarks and examples (no files needed).

``gauge_field`` draws SU(3) links ``U = exp(i*eps*A)`` with ``A`` a Gaussian
su(3) matrix per link (``A = sum_a w_a lambda_a / 2``, ``w_a ~ N(0, 1)``, the
Gell-Mann basis), the construction the reference's test lattices use.  The
exponential is taken through the eigendecomposition of the Hermitian ``A``, so
the links are unitary to rounding.  The result is in the on-disk ILDG order
``[Lt, Lz, Ly, Lx, 4, 3, 3]`` complex128 that ``lattice.preset`` readers return.
"""

from __future__ import annotations

from typing import Sequence

import numpy as np


def _su3_generators() -> np.ndarray:
    """The eight Gell-Mann matrices ``[8, 3, 3]``."""
    g = np.zeros((8, 3, 3), dtype=np.complex128)
    # lambda_1, 2 / 4, 5 / 6, 7: symmetric and antisymmetric off-diagonal pairs
    for n, (a, b) in zip((0, 3, 5), ((0, 1), (0, 2), (1, 2))):
        g[n, a, b] = g[n, b, a] = 1.0
        g[n + 1, a, b], g[n + 1, b, a] = -1j, 1j
    g[2] = np.diag([1.0, -1.0, 0.0])  # lambda_3
    g[7] = np.diag([1.0, 1.0, -2.0]) / np.sqrt(3.0)  # lambda_8
    return g


def gauge_field(latt_size: Sequence[int], eps: float, seed: int, ndir: int = 4) -> np.ndarray:
    """Seeded links ``[Lt, Lz, Ly, Lx, ndir, 3, 3]`` complex128, ``U = exp(i eps A)``."""
    Lx, Ly, Lz, Lt = latt_size
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((Lt, Lz, Ly, Lx, ndir, 8))
    A = np.tensordot(w, _su3_generators() / 2, axes=([-1], [0]))
    lam, Q = np.linalg.eigh(A)
    return np.einsum("...ik,...k,...jk->...ij", Q, np.exp(1j * eps * lam), Q.conj())


def colour_vectors(Ne: int, latt_size: Sequence[int], seed: int) -> np.ndarray:
    """Seeded complex Gaussian colour vectors ``[Ne, 3*Lx*Ly*Lz]`` of unit
    expected norm, standing in for eigenvectors where only the elemental
    arithmetic is exercised."""
    n = latt_size[0] * latt_size[1] * latt_size[2] * 3
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((Ne, n)) + 1j * rng.standard_normal((Ne, n))) / np.sqrt(2 * n)
