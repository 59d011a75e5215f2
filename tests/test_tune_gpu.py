"""Plan launch settings and the autotuner on the GPU: every setting keeps the
result (bit-identical for the FP64 tile shapes, within the mode's tolerance
against the oracle for the tensor-core slab / grid settings and the forced
factorisation), and the tuned plans and generators agree with the oracle."""

import numpy as np
import pytest
import torch

from oracle import restatement as R
from tests.helpers import MemEigen, MemGauge, rel_err

pytestmark = pytest.mark.gpu


def _case(latt, Ne, seed=5, t=0):
    gauge = R.synthetic_gauge(latt, 0.3, seed)
    evec = R.random_colour_vectors(Ne, latt, seed * 10 + t)
    U = np.ascontiguousarray(gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, t])  # [3, Lz, Ly, Lx, 3, 3]
    return U, evec


def _run_plan(plan, U, evec, latt, num_nabla, moms):
    from easydistillation_gb300.insertion import num_derivative

    V3 = latt[0] * latt[1] * latt[2]
    Ud = torch.from_numpy(U).cuda()
    Vd = torch.from_numpy(np.ascontiguousarray(evec.reshape(evec.shape[0], -1))).cuda()
    out = torch.empty((num_derivative(num_nabla), len(moms), evec.shape[0], evec.shape[0]), dtype=torch.complex128,
                      device="cuda")
    plan.run(Ud, V3 * 9, 9, Vd, out)
    if plan.mode != "fp64":
        plan.check_status()
    return out.cpu().numpy()


def test_f64_tile_shapes_are_bit_identical():
    from easydistillation_gb300.ops import F64_TILES, ElementalPlan

    latt, Ne, moms = [8, 8, 4, 2], 10, R.mom_dict_to_list(3)[:7]
    U, evec = _case(latt, Ne)
    outs = []
    for shape in sorted(F64_TILES):
        p = ElementalPlan(latt, Ne, 2, moms, "fp64", tuning={"f64_tile": shape})
        outs.append(_run_plan(p, U, evec, latt, 2, moms))
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])  # every output element is the same sum in the same order
    assert rel_err(outs[0], R.elemental(evec, U, latt, 2, moms)) < 1e-12


@pytest.mark.parametrize("mode", ["f16x3", "tf32x3"])
def test_tc_slab_and_grid_settings(mode):
    """Lock-step slabs of 64 / 128 k-blocks (several slabs over K = 3*16^3), a
    grid of 2 CTAs (several tiles per CTA) and 2 / 3 operand stages against
    the oracle."""
    from easydistillation_gb300.ops import ElementalPlan

    latt, Ne, moms = [16, 16, 16, 1], 8, R.mom_dict_to_list(3)
    U, evec = _case(latt, Ne, seed=7)
    ref = R.elemental(evec, U, latt, 1, moms)
    for tuning in ({}, {"tc_slab_kb": 64}, {"tc_slab_kb": 128}, {"tc_grid": 2}, {"tc_grid": 3, "tc_slab_kb": 32},
                   {"tc_stages": 3}, {"tc_stages": 2, "tc_slab_kb": 64}):
        p = ElementalPlan(latt, Ne, 1, moms, mode, tuning=tuning)
        assert p.factorised == (9, 3)
        assert rel_err(_run_plan(p, U, evec, latt, 1, moms), ref) < 1e-6, tuning


@pytest.mark.parametrize("moms", [R.mom_dict_to_list(3)[:7], [(0, 0, 0), (1, 0, 0), (0, 1, 1), (-1, 0, 1)]])
def test_forced_factorisation_matches_oracle(moms):
    """Momentum lists that leave most (px,py) x pz combinations unused (the
    unused ones are computed and dropped)."""
    from easydistillation_gb300.ops import ElementalPlan

    latt, Ne = [8, 8, 4, 2], 12
    U, evec = _case(latt, Ne, seed=9)
    p = ElementalPlan(latt, Ne, 1, moms, "f16x3", factorise="force")
    assert p.factorised is not None
    assert rel_err(_run_plan(p, U, evec, latt, 1, moms), R.elemental(evec, U, latt, 1, moms)) < 1e-6


@pytest.mark.parametrize("mode", ["f16x3", "fp64"])
def test_autotuner_small_shape(mode, tmp_path):
    from easydistillation_gb300 import tune

    latt, Ne, moms = [8, 8, 8, 2], 16, R.mom_dict_to_list(3)[:7]
    cache = tune.TuningCache(str(tmp_path / "tuning.json"))
    res = tune.tune_elemental(latt, Ne, 1, moms, mode, batch=2, cache=cache, reps=2)
    assert not res.cached and res.ms > 0
    assert len(res.trials) >= (4 if mode == "fp64" else 2)
    assert all(t["ms"] is not None for t in res.trials)  # every candidate within the tolerance
    if mode == "fp64":
        assert all(t["rel_err"] == 0.0 for t in res.trials)
    again = tune.tune_elemental(latt, Ne, 1, moms, mode, batch=2, cache=cache)
    assert again.cached and again.best == res.best
    p = tune.tuned_plan(latt, Ne, 1, moms, mode, batch=1, cache=cache)
    U, evec = _case(latt, Ne, seed=3)
    tol = 1e-12 if mode == "fp64" else 1e-6
    assert rel_err(_run_plan(p, U, evec, latt, 1, moms), R.elemental(evec, U, latt, 1, moms)) < tol


def test_autotuned_generator_matches_oracle(tmp_path, monkeypatch):
    from easydistillation_gb300 import ElementalGenerator

    monkeypatch.setenv("ED_TUNE_CACHE", str(tmp_path / "tuning.json"))
    latt, Ne, moms = [8, 8, 4, 3], 10, R.mom_dict_to_list(3)
    gauge = R.synthetic_gauge(latt, 0.3, 21)
    evec = np.stack([R.random_colour_vectors(Ne, latt, 210 + t) for t in range(latt[3])])
    gen = ElementalGenerator(latt, MemGauge(gauge), MemEigen(evec, Ne), 2, moms, precision="f16x3", autotune=True)
    gen.load("k")
    Uh = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3]
    out = gen.calc_batch([0, 1, 2]).cpu().numpy()
    for t in range(latt[3]):
        ref = R.elemental(evec[t], Uh[:, t], latt, 2, moms)
        assert rel_err(gen.calc(t).cpu().numpy(), ref) < 1e-6
        assert rel_err(out[t], ref) < 1e-6
    assert (tmp_path / "tuning.json").exists()


def test_laplacian_tuner(tmp_path):
    from easydistillation_gb300 import ops, tune

    cache = tune.TuningCache(str(tmp_path / "tuning.json"))
    try:
        res = tune.tune_laplacian([16, 16, 16], nt=2, nvec=1, cache=cache)
        assert {t["tuning"]["use_tma"] for t in res.trials} == {0, 1, 2}
        assert all(t["ms"] is not None for t in res.trials)
        assert tune.tune_laplacian([16, 16, 16], nt=2, nvec=1, cache=cache, apply=False).cached
    finally:
        ops.laplacian_config()
