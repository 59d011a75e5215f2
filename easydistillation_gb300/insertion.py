"""Operator metadata used by the hot path: derivative index scheme, momentum
lists and momentum phases.

Mirrors ``lattice/insertion/derivative.py:23-33`` (``derivative``),
``lattice/insertion/mom_dict.py:5-175`` (``mom_dict_to_list`` for
|p|^2 <= 1, 3 and 9) and ``lattice/insertion/phase.py:6-53``
(``MomentumPhase``), whose tables are computed on the GPU in FP64.
"""

from __future__ import annotations

from typing import List, Sequence, Tuple

import torch

_MOM3 = (
    "0 0 0", "0 0 1", "0 0 -1", "0 1 0", "0 -1 0", "1 0 0", "-1 0 0", "0 1 1", "0 1 -1",
    "0 -1 1", "0 -1 -1", "1 0 1", "1 0 -1", "-1 0 1", "-1 0 -1", "1 1 0", "1 -1 0", "-1 1 0",
    "-1 -1 0", "1 1 1", "1 1 -1", "1 -1 1", "1 -1 -1", "-1 1 1", "-1 1 -1", "-1 -1 1", "-1 -1 -1",
)


def derivative(n: int) -> Tuple[int, ...]:
    """Operator index -> tuple of directions: 0 -> (), 1..3 -> (0,),(1,),(2,),
    4 + 3a + b -> (a, b), and so on in base 3."""
    if n < 0:
        raise ValueError("derivative index must be non-negative")
    length, block = 0, 1
    while n >= block:
        n -= block
        length += 1
        block *= 3
    out = [0] * length
    for k in range(length - 1, -1, -1):
        out[k] = n % 3
        n //= 3
    return tuple(out)


def num_derivative(num_nabla: int) -> int:
    return (3 ** (num_nabla + 1) - 1) // 2


def _sphere_momenta(pmax2: int) -> List[Tuple[int, int, int]]:
    """Every integer momentum with |p|^2 <= pmax2, ordered by (pz, py, px)
    ascending: the order of the reference's |p|^2 <= 9 table (123 entries,
    ``mom_dict.py:35-159``), which is this lexicographic walk."""
    r = int(pmax2 ** 0.5) + 1
    pts = [(x, y, z) for z in range(-r, r + 1) for y in range(-r, r + 1) for x in range(-r, r + 1)
           if x * x + y * y + z * z <= pmax2]
    return sorted(pts, key=lambda p: (p[2], p[1], p[0]))


def mom_dict_to_list(mom: int = 9) -> List[Tuple[int, int, int]]:
    """Momentum list of the reference (``mom_dict.py:162-175``, same default
    ``mom=9``): ``mom=1`` the zero momentum, ``mom=3`` the 27 momenta with
    |p|^2 <= 3 in the reference's table order (its first 7 are |p|^2 <= 1),
    ``mom=9`` the 123 momenta with |p|^2 <= 9; ValueError otherwise."""
    if mom == 1:
        return [(0, 0, 0)]
    if mom == 3:
        return [tuple(int(v) for v in s.split(" ")) for s in _MOM3]
    if mom == 9:
        return _sphere_momenta(9)
    raise ValueError(f"Unknown mom max = {mom}")


def _mom_dict(mom: int):
    return {i: f"{x} {y} {z}" for i, (x, y, z) in enumerate(mom_dict_to_list(mom))}


# The reference's index -> "px py pz" tables (``mom_dict.py:1-159``), the
# ``momentum_dict`` its insertion rows look momenta up in.
momDict_mom1 = _mom_dict(1)
momDict_mom3 = _mom_dict(3)
momDict_mom9 = _mom_dict(9)


class MomentumPhase:
    """Per-site phases ``exp(+2*pi*i*(px*x/Lx + py*y/Ly + pz*z/Lz))`` as FP64
    device tensors ``[Lz, Ly, Lx]``, cached per momentum."""

    def __init__(self, latt_size: Sequence[int], device=None) -> None:
        self.latt_size = list(latt_size)
        self.device = device
        self.cache = {}

    def get(self, np: Sequence[int]) -> torch.Tensor:
        from .ops import momentum_phases

        key = tuple(int(v) for v in np)
        if key not in self.cache:
            self.cache[key] = momentum_phases(self.latt_size, [key], self.device)[0]
        return self.cache[key]
