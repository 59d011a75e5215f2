"""ElementalGenerator on the GPU against golden vectors from the reference's
numpy path and against the oracle.  The plain FP64 mode must agree to 1e-12
relative (Frobenius over the whole [Nderiv, Nmom, Ne, Ne] block)."""

import numpy as np
import pytest
import torch

from oracle import restatement as R
from tests.conftest import golden
from tests.helpers import MemEigen, MemGauge, rel_err

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


@pytest.mark.parametrize("precision", ["fp64", "df64"])
@pytest.mark.parametrize("tag", ["n2_test7", "n1_mom27", "n0_mom7", "n2_blend"])
def test_elemental_fp64_golden(tag, precision):
    """The reference's own elementals: FP64, and its double-float form (df64), to 1e-12."""
    from easydistillation_gb300 import ElementalGenerator

    g = golden(f"elemental_{tag}.npz")
    latt = [int(v) for v in g["latt"]]
    Ne = g["evec"].shape[1]
    dil = None
    if g["dil_tot"].size:
        dil = ([int(v) for v in g["dil_tot"]], int(g["dil_used"]))
    gen = ElementalGenerator(latt, MemGauge(g["gauge"]), MemEigen(g["evec"], Ne), int(g["num_nabla"]),
                             [tuple(int(v) for v in p) for p in g["moms"]], dilution=dil, is_blending=dil is not None,
                             precision=precision)
    gen.load("mem")
    E = gen.calc(int(g["t"])).cpu().numpy()
    assert E.shape == g["E"].shape
    assert rel_err(E, g["E"]) < FP64_TOL


@pytest.mark.parametrize("num_nabla", [0, 1, 2])
@pytest.mark.parametrize("moms", [R.mom_dict_to_list(3)[:7], [(0, 0, 0), (1, 2, 0), (0, 1, 1)]])
def test_elemental_fp64_vs_oracle_every_timeslice(num_nabla, moms):
    """Non-cubic lattice, all timeslices, hermitian-closed and open momentum lists."""
    from easydistillation_gb300 import ElementalGenerator

    latt = [6, 4, 4, 3]
    Ne = 7
    gauge = R.synthetic_gauge(latt, 0.3, 77)
    evec = np.stack([R.random_colour_vectors(Ne, latt, 900 + t) for t in range(latt[3])])
    gen = ElementalGenerator(latt, MemGauge(gauge), MemEigen(evec, Ne), num_nabla, moms)
    gen.load("k")
    U = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3]
    for t in range(latt[3]):
        E = gen.calc(t).cpu().numpy()
        ref = R.elemental(evec[t], U[:, t], latt, num_nabla, moms)
        assert rel_err(E, ref) < FP64_TOL


def test_elemental_returns_internal_buffer_like_reference():
    from easydistillation_gb300 import ElementalGenerator

    g = golden("elemental_n0_mom7.npz")
    latt = [int(v) for v in g["latt"]]
    Ne = g["evec"].shape[1]
    gen = ElementalGenerator(latt, MemGauge(g["gauge"]), MemEigen(g["evec"], Ne), 0,
                             [tuple(int(v) for v in p) for p in g["moms"]])
    gen.load("mem")
    a = gen.calc(0)
    b = gen.calc(0)
    assert a.data_ptr() == b.data_ptr()
    assert a.dtype == torch.complex128 and a.is_cuda


def test_blending_without_dilution_raises():
    from easydistillation_gb300 import ElementalGenerator

    g = golden("elemental_n0_mom7.npz")
    latt = [int(v) for v in g["latt"]]
    with pytest.raises(ValueError):
        ElementalGenerator(latt, MemGauge(g["gauge"]), MemEigen(g["evec"], 5), 0, [(0, 0, 0)], is_blending=True)


@pytest.mark.parametrize("tile", [0, 3])
def test_elemental_df64_matches_fp64_with_k_split(tile):
    """df64 against the FP64 GPU path on a shape whose few output tiles make
    the FP64 GEMM split K (partials summed in a fixed order), for the largest
    and the smallest tile: FP64-class agreement (1e-13)."""
    from easydistillation_gb300.ops import ElementalPlan

    latt, Ne = [16, 16, 8, 1], 6
    V3 = 16 * 16 * 8
    gauge = R.synthetic_gauge(latt, 0.3, 91)
    evec = R.random_colour_vectors(Ne, latt, 92)
    U = torch.from_numpy(np.ascontiguousarray(gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3])).cuda()
    V = torch.from_numpy(evec.reshape(Ne, -1)).cuda()
    moms = R.mom_dict_to_list(3)
    outs = []
    for mode in ("fp64", "df64"):
        plan = ElementalPlan(latt, Ne, 2, moms, mode, tuning={"f64_tile": tile})
        assert plan.tuning()["f64_df"] == (1 if mode == "df64" else 0)
        o = torch.empty((13, 27, Ne, Ne), dtype=torch.complex128, device="cuda")
        plan.run(U[:, 0], V3 * 9, 9, V, o)
        outs.append(o)
    err = float(torch.linalg.vector_norm(outs[1] - outs[0]) / torch.linalg.vector_norm(outs[0]))
    assert err < 1e-13, err
    ref = R.elemental(evec, gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0], latt, 2, moms)
    assert rel_err(outs[1].cpu().numpy(), ref) < FP64_TOL
