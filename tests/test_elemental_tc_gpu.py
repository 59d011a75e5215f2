"""Split-precision tensor-core elementals (tcgen05) and the Ozaki int8-slice
variant against the FP64 oracle.

Tolerances (relative Frobenius error over the whole [Nderiv, Nmom, Ne, Ne]
block): f16x3, tf32x3 and ozaki_i8 <= 1e-6 (the bar for the split-precision
path), bf16x3 <= 1e-4 (two 8-bit-mantissa slices)."""

import numpy as np
import pytest

from oracle import restatement as R
from tests.helpers import MemEigen, MemGauge, rel_err

pytestmark = pytest.mark.gpu

TOL = {"f16x3": 1e-6, "tf32x3": 1e-6, "bf16x3": 1e-4}
TOL_OZAKI = 1e-6  # four signed 6-bit slices of the complex64 operands, products with s + t <= 3


def _run(latt, Ne, num_nabla, moms, mode, t=0, seed=5):
    from easydistillation_gb300 import ElementalGenerator

    gauge = R.synthetic_gauge(latt, 0.3, seed)
    evec = np.stack([R.random_colour_vectors(Ne, latt, seed * 10 + tt) for tt in range(latt[3])])
    gen = ElementalGenerator(latt, MemGauge(gauge), MemEigen(evec, Ne), num_nabla, moms, precision=mode)
    gen.load("k")
    E = gen.calc(t).cpu().numpy()
    U = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, t]
    return E, R.elemental(evec[t], U, latt, num_nabla, moms)


@pytest.mark.parametrize("mode", ["f16x3", "tf32x3", "bf16x3"])
def test_tc_small_all_operators(mode):
    E, ref = _run([4, 4, 4, 2], 6, 2, R.mom_dict_to_list(3)[:7], mode, t=1)
    assert rel_err(E, ref) < TOL[mode]


@pytest.mark.parametrize("mode", ["f16x3", "tf32x3"])
def test_tc_open_momentum_list(mode):
    """momenta not closed under p -> -p: every (left, right) pair is computed directly"""
    moms = [(0, 0, 0), (0, 0, 1), (0, 1, 1), (1, 1, 1), (0, 0, 2), (0, 1, 2), (1, 1, 2)]
    E, ref = _run([4, 4, 4, 1], 5, 2, moms, mode)
    assert rel_err(E, ref) < TOL[mode]


@pytest.mark.parametrize("mode", ["f16x3", "tf32x3", "bf16x3"])
def test_tc_many_tiles(mode):
    """Ne and momentum count that give several ragged M and N tiles."""
    E, ref = _run([8, 8, 4, 1], 150, 1, R.mom_dict_to_list(3), mode)
    assert rel_err(E, ref) < TOL[mode]


@pytest.mark.parametrize("mode", ["f16x3", "tf32x3"])
def test_tc_long_k(mode):
    """K = 3 * 16^3 = 12288 accumulated in TMEM."""
    E, ref = _run([16, 16, 16, 1], 24, 1, R.mom_dict_to_list(3)[:7], mode)
    assert rel_err(E, ref) < TOL[mode]


def test_tc_rejects_volume_not_divisible_by_32():
    from easydistillation_gb300.ops import ElementalPlan

    with pytest.raises(Exception):
        ElementalPlan([6, 2, 2, 1], 4, 0, [(0, 0, 0)], "f16x3", device="cpu")


# ---------------------------------------------------------------- factorised phases
def _run_fac(latt, Ne, num_nabla, moms, mode, factorise, t=0, seed=5):
    from easydistillation_gb300 import ElementalGenerator

    gauge = R.synthetic_gauge(latt, 0.3, seed)
    evec = np.stack([R.random_colour_vectors(Ne, latt, seed * 10 + tt) for tt in range(latt[3])])
    gen = ElementalGenerator(latt, MemGauge(gauge), MemEigen(evec, Ne), num_nabla, moms, precision=mode,
                             factorise=factorise)
    gen.load("k")
    E = gen.calc(t).cpu().numpy()
    U = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, t]
    return gen, E, R.elemental(evec[t], U, latt, num_nabla, moms)


@pytest.mark.parametrize("mode", ["f16x3", "tf32x3", "bf16x3"])
def test_fac_all_27_momenta(mode):
    """|p|^2 <= 3: the 27 momenta are {(px,py)} x {pz} = 9 x 3, every operator"""
    gen, E, ref = _run_fac([4, 4, 4, 2], 6, 2, R.mom_dict_to_list(3), mode, True, t=1)
    assert gen._plan.factorised == (9, 3)
    assert rel_err(E, ref) < TOL[mode]


@pytest.mark.parametrize("mode", ["f16x3", "tf32x3"])
def test_fac_matches_on_chip_phase_kernel(mode):
    """the factorised and the on-chip-phase GEMMs agree with each other and the oracle"""
    moms = R.mom_dict_to_list(3)
    g1, E1, ref = _run_fac([8, 4, 4, 1], 40, 2, moms, mode, True)
    g2, E2, _ = _run_fac([8, 4, 4, 1], 40, 2, moms, mode, False)
    assert g1._plan.factorised == (9, 3) and g2._plan.factorised is None
    assert rel_err(E1, ref) < TOL[mode] and rel_err(E2, ref) < TOL[mode]
    assert rel_err(E1, E2) < 2 * TOL[mode]


def test_fac_open_product_list():
    """a product list not closed under p -> -p (no hermiticity): 4 x 3 momenta"""
    moms = [(px, py, pz) for px in (0, 1) for py in (0, 2) for pz in (0, 1, 3)]
    gen, E, ref = _run_fac([4, 4, 4, 1], 5, 2, moms, "f16x3", True)
    assert gen._plan.factorised == (4, 3)
    assert rel_err(E, ref) < TOL["f16x3"]


def test_fac_with_unrequested_combinations():
    """25 of the 27 product momenta (two combinations formed but not stored)"""
    moms = [p for p in R.mom_dict_to_list(3) if p not in ((1, 1, 1), (-1, -1, -1))]
    gen, E, ref = _run_fac([4, 4, 4, 1], 7, 1, moms, "f16x3", True)
    assert gen._plan.factorised == (9, 3)
    assert rel_err(E, ref) < TOL["f16x3"]


@pytest.mark.parametrize("mode", ["f16x3", "tf32x3"])
def test_fac_many_ragged_tiles(mode):
    """Ne = 150: 9*150 B rows and 3*150 A rows per chain, ragged in both tile directions"""
    gen, E, ref = _run_fac([8, 8, 4, 1], 150, 1, R.mom_dict_to_list(3), mode, True)
    assert gen._plan.factorised == (9, 3)
    assert rel_err(E, ref) < TOL[mode]


@pytest.mark.parametrize("Ne", [12, 14, 128, 113])
def test_fac_last_column_tile_widths(Ne):
    """9*Ne left-variant columns: 108 (one narrow tile, N = 112), 126 (one tile, rounded to 128: not
    narrow), 1152 (nine full tiles), 1017 (seven full tiles and a last one of 121 valid columns, not narrow)"""
    gen, E, ref = _run_fac([4, 4, 4, 1], Ne, 1, R.mom_dict_to_list(3), "f16x3", True)
    assert gen._plan.factorised == (9, 3)
    assert rel_err(E, ref) < TOL["f16x3"]


def test_fac_long_k():
    """K = 3 * 16^3 = 12288"""
    gen, E, ref = _run_fac([16, 16, 16, 1], 24, 1, R.mom_dict_to_list(3), "f16x3", True)
    assert gen._plan.factorised == (9, 3)
    assert rel_err(E, ref) < TOL["f16x3"]


@pytest.mark.parametrize("mode", ["f16x3", "tf32x3"])
@pytest.mark.parametrize("moms", ["first7", "open", "all27"])
def test_fac_every_phase_on_the_left(mode, moms):
    """factorise="left" (ED_MODE_FLAG_LEFT_FACTOR): each momentum's whole phase
    on the left variants and one right factor: the 7 momenta with |p|^2 <= 1
    (hermitian list, 5 x 3 as a product set), a list not closed under p -> -p,
    and the 27 momenta (27 left variants); every operator up to num_nabla = 2"""
    m = {"first7": R.mom_dict_to_list(3)[:7], "all27": R.mom_dict_to_list(3),
         "open": [(0, 0, 0), (0, 0, 1), (0, 1, 1), (1, 1, 1), (0, 0, 2), (0, 1, 2), (1, 1, 2)]}[moms]
    gen, E, ref = _run_fac([8, 4, 4, 2], 20, 2, m, mode, "left", t=1)
    assert gen._plan.factorised == (len(m), 1)
    assert rel_err(E, ref) < TOL[mode]


def test_fac_left_many_tiles_long_k():
    """7 left variants x Ne = 150 columns, ragged tiles; K = 3 * 16^3 = 12288"""
    gen, E, ref = _run_fac([16, 16, 16, 1], 150, 1, R.mom_dict_to_list(3)[:7], "f16x3", "left")
    assert gen._plan.factorised == (7, 1)
    assert rel_err(E, ref) < TOL["f16x3"]


def test_ozaki_every_phase_on_the_left():
    gen, E, ref = _run_fac([4, 4, 4, 2], 6, 1, R.mom_dict_to_list(3)[:7], "ozaki_i8", "left", t=1)
    assert gen._plan.factorised == (7, 1)
    assert rel_err(E, ref) < TOL_OZAKI


# ---------------------------------------------------------------- Ozaki int8 slices
@pytest.mark.parametrize("num_nabla, moms", [(2, "all27"), (1, "first7")])
def test_ozaki_small(num_nabla, moms):
    """int8 slice products with exact int32 sums: 27 momenta (9 x 3 variants) and the
    7 momenta with |p|^2 <= 1 (5 x 3 variants, 8 of the 15 combinations unused)"""
    m = R.mom_dict_to_list(3) if moms == "all27" else R.mom_dict_to_list(3)[:7]
    gen, E, ref = _run_fac([4, 4, 4, 2], 6, num_nabla, m, "ozaki_i8", True, t=1)
    assert gen._plan.factorised is not None
    assert rel_err(E, ref) < TOL_OZAKI


def test_ozaki_many_ragged_tiles():
    """Ne = 150: 64 x 64 tiles ragged in both directions"""
    gen, E, ref = _run_fac([8, 8, 4, 1], 150, 1, R.mom_dict_to_list(3), "ozaki_i8", True)
    assert rel_err(E, ref) < TOL_OZAKI


def test_ozaki_long_k():
    """K = 3 * 16^3 = 12288 exact int32 accumulation"""
    gen, E, ref = _run_fac([16, 16, 16, 1], 24, 1, R.mom_dict_to_list(3), "ozaki_i8", True)
    assert rel_err(E, ref) < TOL_OZAKI
