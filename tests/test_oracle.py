"""The CPU oracle against golden vectors produced by the reference's own
numpy path (``tests/golden/make_golden.py``).  CPU only."""

import numpy as np
import pytest

from oracle import restatement as R
from tests.conftest import golden


def test_derivative_and_momentum_lists():
    g = golden("metadata.npz")
    for n in range(13):
        ref = tuple(int(v) for v in g["derivative"][n] if v >= 0)
        assert R.derivative(n) == ref
    assert [tuple(p) for p in g["mom3"]] == R.mom_dict_to_list(3)
    assert [R.num_derivative(k) for k in range(3)] == [1, 4, 13]


def test_correlators_on_operator_interface():
    """twopoint / twopoint_profile restated on the reference's Operator + file
    data interface, against the reference's own outputs."""
    z = golden("correlator.npz")
    spec = eval(str(z["ops_spec"]))  # a repr of plain lists, tuples and numbers
    parts = [R.operator_parts(rows, cs) for _n, rows, cs in spec]
    assert parts == eval(str(z["parts"]))
    E, P, PB = z["elem"], z["peram"], z["peram_bw"]
    ts, dts, Lt, u = list(z["ts"]), list(z["dts"]), int(z["Lt"]), int(z["usedNe"])
    cases = {
        "tp": R.twopoint_operators(parts, E, P, ts, Lt, u),
        "tp_all_src": R.twopoint_operators(parts, E, P, ts, Lt, u, is_sum_over_source_t=False),
        "tp_bw": R.twopoint_operators(parts, E, P, ts, Lt, u, perambulator_bw=PB),
        "tp_fullne": R.twopoint_operators(parts, E, P, ts, Lt, int(z["Ne"])),
        "prof": R.twopoint_profile_operators(parts, E, P, ts, dts, u),
        "prof_diag": R.twopoint_profile_operators(parts, E, P, ts, dts, u, is_diagonal=True),
        "prof_all_src": R.twopoint_profile_operators(parts, E, P, ts, dts, u, is_sum_over_source_t=False),
        "prof_bw_fullt": R.twopoint_profile_operators(parts, E, P, ts, list(range(Lt)), u, perambulator_bw=PB),
    }
    for k, v in cases.items():
        np.testing.assert_allclose(v, z[k], rtol=1e-12, atol=1e-12 * np.abs(z[k]).max(), err_msg=k)


def test_momentum_phase_sign_and_values():
    g = golden("phase_462.npz")
    latt = list(g["latt"])
    for p, ref in zip(g["moms"], g["phase"]):
        np.testing.assert_allclose(R.momentum_phase(latt, tuple(p)), ref, rtol=0, atol=1e-15)
    # e^{+i 2 pi p.x / L}: the reference sign
    ph = R.momentum_phase([4, 4, 4], (1, 0, 0))
    assert abs(ph[0, 0, 1] - 1j) < 1e-15


@pytest.mark.parametrize("tag", ["443", "642"])
def test_laplacian(tag):
    g = golden(f"laplacian_{tag}.npz")
    latt = list(g["latt"])
    U = g["gauge"].transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0]
    out = R.laplacian(g["F"], U, latt)
    np.testing.assert_allclose(out, g["LF"], rtol=0, atol=1e-13)


def test_synthetic_gauge_reproducible_and_unitary():
    g = golden("laplacian_443.npz")
    U = R.synthetic_gauge(list(g["latt"]), 0.3, 11)
    np.testing.assert_array_equal(U, g["gauge"])
    I = np.einsum("...ab,...cb->...ac", U, U.conj())
    assert np.abs(I - np.eye(3)).max() < 1e-14
    assert np.abs(np.linalg.det(U) - 1).max() < 1e-14


@pytest.mark.parametrize("tag", ["n2_test7", "n1_mom27", "n0_mom7", "n2_blend"])
def test_elemental(tag):
    g = golden(f"elemental_{tag}.npz")
    latt = list(g["latt"])
    t = int(g["t"])
    U = g["gauge"].transpose(4, 0, 1, 2, 3, 5, 6)[:3, t]
    coeff = None
    if g["dil_tot"].size:
        coeff = R.blending_coeff(g["evec"].shape[1], (list(g["dil_tot"]), int(g["dil_used"])))
    E = R.elemental(g["evec"][t], U, latt, int(g["num_nabla"]), [tuple(p) for p in g["moms"]], coeff)
    scale = np.abs(g["E"]).max()
    np.testing.assert_allclose(E, g["E"], rtol=0, atol=1e-13 * scale)


def test_displacement_elemental():
    g = golden("displacement_d2.npz")
    U = g["gauge"].transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0]
    E = R.displacement_elemental(g["evec"][0], U, list(g["latt"]), 2, [tuple(p) for p in g["moms"]])
    np.testing.assert_allclose(E, g["E"], rtol=0, atol=1e-13)


def test_eigensolve_and_stout():
    g = golden("eigen_443.npz")
    latt = list(g["latt"])
    Ne = int(g["Ne"])
    U = g["gauge"].transpose(4, 0, 1, 2, 3, 5, 6)[:3]
    evecs, evals = R.eigensolve(U[:, 0], latt, Ne, 1e-10)
    np.testing.assert_allclose(evals, g["evals0"], rtol=1e-10, atol=1e-12)
    # projectors agree (phases/degenerate rotations are arbitrary)
    P = lambda v: v.reshape(Ne, -1).T @ v.reshape(Ne, -1).conj()
    assert np.abs(P(evecs) - P(g["evecs0"])).max() < 1e-8
    sm = R.stout_smear(U, 2, 0.12)
    np.testing.assert_allclose(sm, g["smeared"], rtol=0, atol=1e-13)
    evecs1, evals1 = R.eigensolve(sm[:, 1], latt, Ne, 1e-10)
    np.testing.assert_allclose(evals1, g["evals1"], rtol=1e-10, atol=1e-12)


def test_project_su3_matches_reference():
    z = golden("project_su3.npz")
    U = z["gauge"].transpose(4, 0, 1, 2, 3, 5, 6)[:3]
    np.testing.assert_allclose(R.project_su3(U), z["projected"], rtol=0, atol=1e-14)
