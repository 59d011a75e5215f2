"""Autotuner host logic and the plan launch settings, without a GPU: the
settings' validation through the C ABI, the GEMM forms a momentum list
admits, the coordinate search with a fake timer, and the tuning cache."""

import ctypes
import json

import pytest

from tests.conftest import ROOT  # noqa: F401  (puts the repository on sys.path)


def _plan(moms="all27", mode="f16x3", **kw):
    from easydistillation_gb300.insertion import mom_dict_to_list
    from easydistillation_gb300.ops import ElementalPlan

    lists = {"all27": mom_dict_to_list(3), "first7": mom_dict_to_list(3)[:7]}
    moms = lists[moms] if isinstance(moms, str) else moms
    return ElementalPlan([8, 8, 4, 2], 10, 2, moms, mode, device="cpu", **kw)


def test_tuning_settings_round_trip_and_validation():
    from easydistillation_gb300 import _lib

    p = _plan()
    assert p.tuning() == {"f64_tile": 0, "tc_slab_kb": 0, "tc_grid": 0, "tc_stages": 0, "tc_pair": 0, "tc_kpb": 0,
                          "tc_stack": 0, "f64_df": 0}
    p.set_tuning(f64_tile=3, tc_slab_kb=64, tc_grid=100, tc_stages=3, tc_pair=2, tc_kpb=4, tc_stack=1, f64_df=1)
    assert p.tuning() == {"f64_tile": 3, "tc_slab_kb": 64, "tc_grid": 100, "tc_stages": 3, "tc_pair": 2,
                          "tc_kpb": 4, "tc_stack": 1, "f64_df": 1}
    p.set_tuning(tc_slab_kb=0)
    assert p.tuning()["tc_slab_kb"] == 0
    for bad in ({"f64_tile": 4}, {"f64_tile": -1}, {"tc_slab_kb": 96}, {"tc_slab_kb": 512}, {"tc_grid": -2},
                {"tc_stages": 1}, {"tc_stages": 5}, {"tc_pair": 4}, {"tc_pair": -1}, {"tc_kpb": 3},
                {"tc_kpb": 8}, {"tc_stack": 3}, {"tc_stack": -1}, {"f64_df": 2}, {"f64_df": -1}):
        with pytest.raises(ValueError):
            p.set_tuning(**bad)
    with pytest.raises(ValueError):
        p.set_tuning(tile=1)
    L = _lib.lib()
    assert L.ed_elemental_set_tuning(p._h, 99, 0) == _lib.ED_ERR_ARG
    assert "unknown key" in _lib.last_error()
    v = ctypes.c_int()
    assert L.ed_elemental_get_tuning(p._h, 99, ctypes.byref(v)) == _lib.ED_ERR_ARG
    # tuning given at construction
    q = _plan(tuning={"tc_slab_kb": 128})
    assert q.tuning()["tc_slab_kb"] == 128


def test_force_factor_flag():
    from easydistillation_gb300 import _lib
    from easydistillation_gb300.insertion import mom_dict_to_list

    # the first 7 momenta leave 8 of the 5 x 3 combinations unused: on-chip by default
    assert _plan("first7").factorised is None
    assert _plan("first7", factorise="force").factorised == (5, 3)
    assert _plan("all27", factorise="force").factorised == (9, 3)
    assert _plan("all27", factorise=False).factorised is None
    with pytest.raises(ValueError):
        _plan("all27", factorise="always")
    # a repeated momentum never factorises, forced or not
    assert _plan([(0, 0, 0), (0, 0, 0)], factorise="force").factorised is None
    # the two flags together are rejected by the library
    moms = [v for p in mom_dict_to_list(3)[:7] for v in p]
    arr = (ctypes.c_int * len(moms))(*moms)
    h = ctypes.c_void_p()
    rc = _lib.lib().ed_elemental_plan_create(ctypes.byref(h), 8, 8, 4, 10, 1, arr, 7, 1 | 0x100 | 0x200)
    assert rc == _lib.ED_ERR_ARG and "unknown mode" in _lib.last_error()
    rc = _lib.lib().ed_elemental_plan_create_batched(ctypes.byref(h), 8, 8, 4, 10, 1, arr, 7, 1 | 0x300, 2)
    assert rc == _lib.ED_ERR_ARG


def test_factorise_options():
    from easydistillation_gb300.insertion import mom_dict_to_list
    from easydistillation_gb300.tune import factorise_options

    m27, m7 = mom_dict_to_list(3), mom_dict_to_list(3)[:7]
    assert factorise_options([8, 8, 4, 2], 10, 2, m27, "f16x3") == [True, False]
    assert factorise_options([8, 8, 4, 2], 10, 2, m7, "f16x3") == [True, "force", "left"]
    assert factorise_options([8, 8, 4, 2], 10, 2, [(0, 0, 0), (1, 2, 3)], "tf32x3") == [True, "force", "left"]
    assert factorise_options([8, 8, 4, 2], 10, 2, m27, "fp64") == [True]
    assert factorise_options([8, 8, 4, 2], 10, 2, m7, "ozaki_i8") == [True]
    assert factorise_options([8, 8, 4, 2], 10, 2, mom_dict_to_list(9), "f16x3") == [True]  # 123 momenta: too long


def test_left_factorisation_plans():
    """ED_MODE_FLAG_LEFT_FACTOR: every momentum a left factor, one right factor;
    the flags that choose the GEMM form exclude one another."""
    from easydistillation_gb300.insertion import mom_dict_to_list
    from easydistillation_gb300.ops import ElementalPlan

    m7 = mom_dict_to_list(3)[:7]
    assert ElementalPlan([8, 8, 4, 2], 10, 1, m7, "f16x3", device="cpu", factorise="left").factorised == (7, 1)
    assert ElementalPlan([8, 8, 4, 2], 10, 1, m7, "f16x3", device="cpu").factorised is None
    assert ElementalPlan([8, 8, 4, 2], 10, 1, m7, "f16x3", device="cpu", factorise="force").factorised == (5, 3)
    assert ElementalPlan([8, 8, 4, 2], 10, 1, m7, "fp64", device="cpu", factorise="left").factorised is None
    from easydistillation_gb300 import _lib

    h = ctypes.c_void_p()
    arr = (ctypes.c_int * 21)(*[c for p in m7 for c in p])
    for flags in (0x100 | 0x800, 0x200 | 0x800):
        rc = _lib.lib().ed_elemental_plan_create(ctypes.byref(h), 8, 8, 4, 10, 1, arr, 7, 1 | flags)
        assert rc == _lib.ED_ERR_ARG


def test_coordinate_search_picks_fastest_accurate_candidate():
    from easydistillation_gb300.tune import Candidate, _run_search

    times = {(True, ()): 10.0, (False, ()): 8.0, ("force", ()): 3.0,
             (False, (("tc_slab_kb", 128),)): 6.0, (False, (("tc_slab_kb", 64),)): 7.0}
    errors = {"force": 1e-3}  # too inaccurate: rejected however fast
    calls = []

    def measure(c):
        k = (c.factorise, tuple(sorted(c.tuning.items())))
        calls.append(k)
        return times[k], errors.get(c.factorise, 0.0)

    stages = [lambda best: [Candidate(True), Candidate(False), Candidate("force")],
              lambda best: [best, Candidate(best.factorise, {"tc_slab_kb": 128}),
                            Candidate(best.factorise, {"tc_slab_kb": 64})]]
    res = _run_search(stages, Candidate(True), measure, lambda out, ref: abs(out - ref), 1e-6)
    assert res.best.factorise is False and res.best.tuning == {"tc_slab_kb": 128}
    assert res.ms == 6.0
    assert len(calls) == 5  # the stage-2 'best' was not measured twice
    rejected = [t for t in res.trials if t["ms"] is None]
    assert len(rejected) == 1 and rejected[0]["factorise"] == "force"
    assert res.trials[0]["rel_err"] == 0.0  # the first candidate is the accuracy reference


def test_tuning_cache_round_trip(tmp_path, monkeypatch):
    from easydistillation_gb300 import tune

    path = tmp_path / "sub" / "tuning.json"
    monkeypatch.setenv("ED_TUNE_CACHE", str(path))
    assert tune.cache_path() == str(path)
    c = tune.TuningCache()
    assert c.get("dev", "k") is None
    c.put("dev", "k", {"best": {"factorise": "force", "tuning": {"tc_slab_kb": 64}}, "ms": 1.5})
    c.put("dev", "k2", {"best": {"factorise": True, "tuning": {}}, "ms": 2.0})
    c.put("dev2", "k", {"best": {"factorise": False, "tuning": {}}, "ms": 3.0})
    data = json.loads(path.read_text())
    assert set(data) == {"dev", "dev2"} and set(data["dev"]) == {"k", "k2"}
    hit = tune.TuningCache(str(path)).get("dev", "k")
    assert tune.Candidate.from_dict(hit["best"]) == tune.Candidate("force", {"tc_slab_kb": 64})
    path.write_text("not json")
    assert tune.TuningCache(str(path)).get("dev", "k") is None  # a damaged cache reads as empty


def test_tune_elemental_uses_cache_without_measuring(tmp_path, monkeypatch):
    from easydistillation_gb300 import tune
    from easydistillation_gb300.insertion import mom_dict_to_list

    monkeypatch.setattr(tune, "device_key", lambda device=None: "fake-gpu")
    cache = tune.TuningCache(str(tmp_path / "t.json"))
    moms = mom_dict_to_list(3)
    key = tune.elemental_key([32, 32, 32, 64], 200, 2, moms, "f16x3", 4)
    assert key == tune.elemental_key((32, 32, 32), 200, 2, [list(p) for p in moms], "f16x3", 4)
    assert key != tune.elemental_key([32, 32, 32, 64], 200, 2, moms, "f16x3", 2)
    cache.put("fake-gpu", key, {"best": {"factorise": True, "tuning": {"tc_slab_kb": 128}}, "ms": 150.0})
    res = tune.tune_elemental([32, 32, 32, 64], 200, 2, moms, "f16x3", batch=4, device="cpu", cache=cache)
    assert res.cached and res.best.tuning == {"tc_slab_kb": 128} and res.ms == 150.0
    with pytest.raises(ValueError):
        tune.tune_elemental([32, 32, 32, 64], 200, 2, moms, "f8", cache=cache)


def test_gauss_flag_needs_a_factorised_split_plan():
    """ED_MODE_FLAG_GAUSS: accepted for f16x3 / bf16x3 / tf32x3 plans that
    factorise (the split-plane workspace grows by half); rejected for FP64,
    Ozaki and on-chip-phase plans."""
    from easydistillation_gb300 import _lib

    base = _plan("all27", "f16x3")
    g = _plan("all27", "f16x3", gauss=True)
    assert g.factorised == (9, 3) and g.gauss
    assert g.workspace_bytes > base.workspace_bytes
    for mode in ("bf16x3", "tf32x3"):
        assert _plan("all27", mode, gauss=True).factorised == (9, 3)
    assert _plan("first7", "f16x3", factorise="force", gauss=True).factorised == (5, 3)
    for kw in ({"moms": "all27", "mode": "fp64"}, {"moms": "all27", "mode": "ozaki_i8"},
               {"moms": "first7", "mode": "f16x3"}, {"moms": "all27", "mode": "f16x3", "factorise": False}):
        with pytest.raises(RuntimeError):
            _plan(gauss=True, **kw)
        assert "Gauss form" in _lib.last_error()
