"""Two-point correlators on the reference's interface (Operator, elemental
and perambulator file data) against the reference's own outputs
(tests/golden/correlator.npz, from lattice/correlator/one_particle.py)."""

import numpy as np
import pytest

from tests.conftest import golden

pytestmark = pytest.mark.gpu

TOL = 1e-12  # FP64 throughout; relative to the largest value of each result


def _setup():
    from easydistillation_gb300.correlator import InsertionRowMom, Operator

    z = golden("correlator.npz")
    spec = eval(str(z["ops_spec"]))  # a repr of plain lists, tuples and numbers
    ops = [Operator(n, [InsertionRowMom(r, m) for r, m in rows], cs) for n, rows, cs in spec]
    return z, ops


def _close(out, ref, what):
    out = out.cpu().numpy() if hasattr(out, "cpu") else np.asarray(out)
    assert out.shape == ref.shape, what
    np.testing.assert_allclose(out, ref, rtol=TOL, atol=TOL * np.abs(ref).max(), err_msg=what)


def test_twopoint_matches_reference():
    from easydistillation_gb300.correlator import twopoint

    z, ops = _setup()
    E, P, PB = z["elem"], z["peram"], z["peram_bw"]
    ts, Lt, u = list(z["ts"]), int(z["Lt"]), int(z["usedNe"])
    _close(twopoint(ops, E, P, ts, Lt, u), z["tp"], "twopoint")
    _close(twopoint(ops, E, P, ts, Lt, u, is_sum_over_source_t=False), z["tp_all_src"], "per source")
    _close(twopoint(ops, E, P, ts, Lt, u, perambulator_bw=PB), z["tp_bw"], "perambulator_bw")
    _close(twopoint(ops, E, P, ts, Lt, int(z["Ne"])), z["tp_fullne"], "all Ne")


def test_twopoint_profile_matches_reference():
    from easydistillation_gb300.correlator import twopoint_profile

    z, ops = _setup()
    E, P, PB = z["elem"], z["peram"], z["peram_bw"]
    ts, dts, Lt, u = list(z["ts"]), list(z["dts"]), int(z["Lt"]), int(z["usedNe"])
    _close(twopoint_profile(ops, E, P, ts, dts, u), z["prof"], "profile")
    _close(twopoint_profile(ops, E, P, ts, dts, u, is_diagonal=True), z["prof_diag"], "diagonal")
    _close(twopoint_profile(ops, E, P, ts, dts, u, is_sum_over_source_t=False), z["prof_all_src"], "per source")
    _close(twopoint_profile(ops, E, P, ts, list(range(Lt)), u, perambulator_bw=PB), z["prof_bw_fullt"], "bw")


def test_twopoint_device_inputs_and_numpy_backend():
    """Perambulators already on the device give the same result; with the
    numpy backend the result is a host array, as the reference's."""
    import torch

    import easydistillation_gb300 as ed
    from easydistillation_gb300.correlator import twopoint

    z, ops = _setup()
    E = torch.from_numpy(z["elem"]).cuda()
    P = torch.from_numpy(z["peram"]).cuda()
    ts, Lt, u = list(z["ts"]), int(z["Lt"]), int(z["usedNe"])
    _close(twopoint(ops, E, P, ts, Lt, u), z["tp"], "device inputs")
    try:
        ed.set_backend("numpy")
        out = twopoint(ops, z["elem"], z["peram"], ts, Lt, u)
        assert isinstance(out, np.ndarray)
        _close(out, z["tp"], "numpy backend")
    finally:
        ed.set_backend("torch")
