"""C-ABI library checks that need no GPU: it loads, exports every symbol the
header declares, validates arguments on the host, and plans elementals."""

import ctypes
import os
import re

import pytest

from tests.conftest import ROOT


def _declared():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            names |= set(re.findall(r"^\s*int\s+(ed_\w+)\s*\(", src, re.M))
    return names


def test_library_exports_every_declared_symbol():
    from easydistillation_gb300 import _lib

    L = _lib.lib()
    declared = _declared()
    assert declared, "no declarations found"
    for name in declared:
        assert hasattr(L, name), f"{name} declared in include/ but not exported"
    assert declared <= set(_lib.exported_symbols()) | declared
    assert set(_lib.exported_symbols()) <= declared, "binding names an undeclared symbol"
    assert L.ed_version() >= 100


def test_integration_notes_name_every_entry_point():
    """The binding notes list each declared entry point with the reference
    interface it replaces (or 'no counterpart')."""
    notes = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    named = set(re.findall(r"\bed_\w+", notes))
    missing = sorted(_declared() - named)
    assert not missing, f"entry points without a line in the binding notes: {missing}"


def test_argument_validation_is_host_side():
    from easydistillation_gb300 import _lib

    L = _lib.lib()
    # bad precision / sizes / null pointers are rejected before any CUDA call
    assert L.ed_laplacian(7, 4, 4, 4, 1, 1, None, None, 0, None, 0, None) == _lib.ED_ERR_ARG
    assert "prec" in _lib.last_error()
    assert L.ed_laplacian(_lib.ED_C64, 3, 4, 4, 1, 1, 16, 32, 0, 64, 0, None) == _lib.ED_ERR_ARG
    assert "even Lx" in _lib.last_error()
    assert L.ed_covariant_derivative(0, 0, 4, 4, 4, 3, 1, 16, 32, 64, None) == _lib.ED_ERR_ARG
    assert L.ed_vectors_to_planes(0, 0, 0, 0, 64, 16, 32, None) == _lib.ED_ERR_ARG
    with pytest.raises(ValueError):
        _lib.check(_lib.ED_ERR_ARG, "x")
    # the arrow eigensolver checks its sizes on the host
    nb = ctypes.c_size_t()
    assert L.ed_arrow_eigh_workspace(2, 10, 4, ctypes.byref(nb)) == _lib.ED_OK and nb.value == 2 * 10 * 4 * 6 * 8
    assert L.ed_arrow_eigh_workspace(2, 10, 11, ctypes.byref(nb)) == _lib.ED_ERR_ARG
    assert L.ed_arrow_eigh(2, 10, 10, 4, 8, 8, 8, 8, 8, 8, 1 << 20, None) == _lib.ED_ERR_ARG  # ka >= m
    assert L.ed_arrow_eigh(2, 10, 3, 4, 8, None, 8, 8, 8, 8, 1 << 20, None) == _lib.ED_ERR_ARG  # no border
    assert L.ed_arrow_eigh(2, 10, 0, 4, 8, None, 8, 8, 8, 8, 100, None) == _lib.ED_ERR_WORKSPACE
    assert L.ed_cgs_pass(2, 5, 100, 16, 400, 16, 16, 5, None, None) == _lib.ED_ERR_ARG  # batch stride < r*n
    assert L.ed_cgs_pass(2, 5, 100, 8, 500, 16, 16, 5, None, None) == _lib.ED_ERR_ARG  # misaligned V
    assert L.ed_cgs_pass(2, 5, 100, 16, 500, 16, 16, 4, None, None) == _lib.ED_ERR_ARG  # ldh < r
    nb = ctypes.c_size_t()
    assert L.ed_lanczos_workspace(6, 6, 6, 2, 16, 40, ctypes.byref(nb)) == _lib.ED_OK and nb.value > 2 * 41 * 648 * 16
    assert L.ed_lanczos_workspace(6, 6, 6, 2, 16, 16, ctypes.byref(nb)) == _lib.ED_ERR_ARG  # ncv <= Ne
    st = (ctypes.c_int * 3)()
    assert L.ed_lanczos_tr(6, 6, 6, 2, None, 16, ctypes.c_double(1e-10), 40, 10, 0, ctypes.c_double(0.0), 256, 256, st,
                           256, 1 << 30, None) == _lib.ED_ERR_ARG  # null links
    assert L.ed_lanczos_tr(6, 6, 6, 2, 256, 16, ctypes.c_double(1e-10), 40, 10, 4, ctypes.c_double(0.0), 256, 256, st,
                           256, 1 << 30, None) == _lib.ED_ERR_ARG  # Chebyshev without a cut
    assert L.ed_lanczos_tr(6, 6, 6, 2, 256, 16, ctypes.c_double(1e-10), 40, 10, 0, ctypes.c_double(0.0), 256, 256, st,
                           256, 1024, None) == _lib.ED_ERR_WORKSPACE
    # on-disk decoding: precision codes, null / misaligned / overlapping pointers
    BE = _lib.ED_BIG_ENDIAN
    assert L.ed_decode_complex(_lib.ED_C128 | BE, 0, None, _lib.ED_C128, None, None) == _lib.ED_OK  # empty
    assert L.ed_decode_complex(2, 4, 256, _lib.ED_C128, 4096, None) == _lib.ED_ERR_ARG
    assert L.ed_decode_complex(_lib.ED_C64 | 0x20, 4, 256, _lib.ED_C128, 4096, None) == _lib.ED_ERR_ARG
    assert L.ed_decode_complex(_lib.ED_C128, 4, 256, 5, 4096, None) == _lib.ED_ERR_ARG
    assert L.ed_decode_complex(_lib.ED_C128 | BE, 4, None, _lib.ED_C128, 4096, None) == _lib.ED_ERR_ARG
    assert L.ed_decode_complex(_lib.ED_C128 | BE, 4, 264, _lib.ED_C128, 4096, None) == _lib.ED_ERR_ARG  # src % 16
    assert "misaligned" in _lib.last_error()
    assert L.ed_decode_complex(_lib.ED_C64 | BE, 4, 264, _lib.ED_C128, 4104, None) == _lib.ED_ERR_ARG  # dst % 16
    assert L.ed_decode_complex(_lib.ED_C128 | BE, 4, 256, _lib.ED_C128, 288, None) == _lib.ED_ERR_ARG  # overlap
    assert "overlap" in _lib.last_error()
    assert L.ed_decode_links(_lib.ED_C128 | BE, 0, 256, 4096, None) == _lib.ED_ERR_ARG
    assert L.ed_decode_links(_lib.ED_C128 | BE, 2, 256, 1000, None) == _lib.ED_ERR_ARG  # overlap (2 sites: 1152 B)
    assert L.ed_decode_links(_lib.ED_C64 | BE, 2, 256, 4104, None) == _lib.ED_ERR_ARG  # dst % 16
    # double-float Laplacian and split: precision code accepted (then rejected on the null pointers), bad sizes
    assert L.ed_laplacian(_lib.ED_DF, 3, 4, 4, 1, 1, None, None, 0, None, 0, None) == _lib.ED_ERR_ARG
    assert "null" in _lib.last_error()  # an odd Lx is fine for ED_DF: the check that failed is the pointers'
    assert L.ed_split_c128(-1, 256, 512, None) == _lib.ED_ERR_ARG
    assert L.ed_split_c128(4, 264, 512, None) == _lib.ED_ERR_ARG  # misaligned source
    assert L.ed_split_c128(0, None, None, None) == _lib.ED_OK  # nothing to split
    # two-point profile: sizes, source timeslice, null pointers
    assert L.ed_twopoint_profile(0, 10, 8, 0, 1, *([256] * 9), None, None) == _lib.ED_ERR_ARG
    assert L.ed_twopoint_profile(4, 10, 8, 8, 1, *([256] * 9), None, None) == _lib.ED_ERR_ARG  # t_src >= Lt
    assert L.ed_twopoint_profile(4, 10, 8, 0, 1, *([256] * 8), None, 256, None) == _lib.ED_ERR_ARG  # null work
    assert L.ed_twopoint_profile_diag(4, 10, 8, 0, 1, -1, *([256] * 7), None) == _lib.ED_ERR_ARG  # nterm < 0
    # the tensor-core wait settings (process-wide; restored)
    assert L.ed_elemental_wait_limit(-1) == _lib.ED_ERR_ARG
    assert L.ed_elemental_wait_limit(0) == _lib.ED_OK and L.ed_elemental_wait_probe(0) == _lib.ED_OK


@pytest.mark.parametrize(
    "num_nabla,moms,herm_pairs,plain_pairs",
    [
        (0, [(0, 0, 0)], 1, 1),
        (1, [(0, 0, 0), (0, 0, 1), (0, 0, -1)], 4, 4 + 3),
        (2, [(0, 0, 0), (1, 0, 0), (-1, 0, 0)], 13 + 3 + 2 + 1, 13 + 3 * 4 + 9),
        (2, [(0, 0, 0), (0, 0, 1)], None, 13 + 3 * 4 + 9),
    ],
)
def test_elemental_plan_pairs(num_nabla, moms, herm_pairs, plain_pairs):
    """Distinct (left, right) chain contractions per momentum: 34 for
    num_nabla=2 instead of the reference's 43 subsets, 19 when the momentum
    list is closed under p -> -p (hermiticity)."""
    from easydistillation_gb300.ops import ElementalPlan

    plan = ElementalPlan([4, 4, 4, 8], 6, num_nabla, moms, "fp64", device="cpu")
    expect = herm_pairs if herm_pairs is not None else plain_pairs
    assert plan.num_pairs == expect
    V3 = 64
    assert plan.workspace_bytes >= (3 ** (num_nabla + 1) - 1) // 2 * 6 * 3 * V3 * 16


def test_lattice_volume_bound():
    """Every entry point that takes Lx, Ly, Lz rejects V3 above 2^28 on the
    host (kernels number sites with 32-bit integers); 2^27 still plans."""
    from easydistillation_gb300 import _lib

    L = _lib.lib()
    big = (1024, 1024, 1024)  # V3 = 2^30
    p = 1 << 20  # a non-null, 16-byte aligned stand-in address: nothing is dereferenced
    calls = {
        "ed_laplacian": lambda: L.ed_laplacian(_lib.ED_C128, *big, 1, 1, p, p, 0, p + 4096, 0, None),
        "ed_covariant_derivative": lambda: L.ed_covariant_derivative(0, 0, *big, 0, 1, p, p, p + 4096, None),
        "ed_parallel_transport": lambda: L.ed_parallel_transport(*big, 0, 1, 1, p, p + 4096, p + 8192, None),
        "ed_stout_smear_step": lambda: L.ed_stout_smear_step(*big, 1, ctypes.c_double(0.1), p, p + 4096, None),
        "ed_link_grad": lambda: L.ed_link_grad(*big, 0, 1, ctypes.c_double(1.0), ctypes.c_double(0.0), p, p, p,
                                               None),
        "ed_links_to_soa": lambda: L.ed_links_to_soa(_lib.ED_C128, *big, 1, p, 0, 9, 36, p + 4096, None),
    }
    for name, call in calls.items():
        assert call() == _lib.ED_ERR_ARG, name
        assert "2^28" in _lib.last_error(), (name, _lib.last_error())
    nb = ctypes.c_size_t()
    assert L.ed_lanczos_workspace(*big, 1, 16, 40, ctypes.byref(nb)) == _lib.ED_ERR_ARG
    assert "2^28" in _lib.last_error()
    assert L.ed_lanczos_workspace(512, 512, 512, 1, 16, 40, ctypes.byref(nb)) == _lib.ED_OK
    assert nb.value >= 41 * 3 * (1 << 27) * 16


def test_plan_rejects_bad_arguments():
    from easydistillation_gb300.ops import ElementalPlan

    with pytest.raises(ValueError):
        ElementalPlan([4, 4, 4, 8], 6, 3, [(0, 0, 0)], "fp64", device="cpu")
    with pytest.raises(ValueError):
        ElementalPlan([4, 4, 4, 8], 0, 1, [(0, 0, 0)], "fp64", device="cpu")
    with pytest.raises(ValueError):
        ElementalPlan([4, 4, 4, 8], 4, 1, [(0, 0, 0)], "no-such-mode", device="cpu")


def test_generator_metadata_matches_reference_scheme():
    from easydistillation_gb300 import derivative, mom_dict_to_list, num_derivative
    from oracle import restatement as R

    assert [derivative(n) for n in range(40)] == [R.derivative(n) for n in range(40)]
    assert mom_dict_to_list(3) == R.mom_dict_to_list(3)
    assert [num_derivative(k) for k in range(3)] == [1, 4, 13]


def test_momentum_lists_match_reference_tables():
    """mom_dict_to_list for 1, 3, 9 and the reference's default (9) against the
    reference's own tables; other values raise like the reference."""
    from easydistillation_gb300 import mom_dict_to_list
    from tests.conftest import golden

    g = golden("metadata.npz")
    assert mom_dict_to_list(3) == [tuple(int(v) for v in p) for p in g["mom3"]]
    assert mom_dict_to_list(9) == [tuple(int(v) for v in p) for p in g["mom9"]]
    assert mom_dict_to_list() == [tuple(int(v) for v in p) for p in g["mom_default"]]
    assert len(mom_dict_to_list()) == 123 and mom_dict_to_list(1) == [(0, 0, 0)]
    assert mom_dict_to_list(3)[:7] == [p for p in mom_dict_to_list(3) if sum(v * v for v in p) <= 1]
    with pytest.raises(ValueError):
        mom_dict_to_list(5)
    # the index -> "px py pz" dictionaries insertion rows look momenta up in
    from easydistillation_gb300.insertion import momDict_mom1, momDict_mom3, momDict_mom9

    assert momDict_mom1 == {0: "0 0 0"}
    assert momDict_mom3[1] == "0 0 1" and momDict_mom3[26] == "-1 -1 -1" and len(momDict_mom3) == 27
    assert momDict_mom9[0] == "0 0 -3" and momDict_mom9[122] == "0 0 3"
    assert [tuple(int(v) for v in s.split(" ")) for s in momDict_mom9.values()] == mom_dict_to_list(9)


def test_backend_switch():
    """set_backend / get_backend mirror lattice/backend.py: numpy, torch and a
    module object are accepted, unknown names raise ValueError."""
    import numpy as np
    import torch

    import easydistillation_gb300 as ed
    from easydistillation_gb300 import backend as B

    try:
        ed.set_backend("numpy")
        assert ed.get_backend() is np
        out = B.to_backend(torch.zeros(3, dtype=torch.complex128))
        assert isinstance(out, np.ndarray) and out.dtype == np.complex128
        ed.set_backend(np)  # a module, as the reference also accepts
        assert B.backend_name() == "numpy"
        with pytest.raises(ValueError):
            ed.set_backend("jax")
    finally:
        ed.set_backend("torch")
    assert ed.get_backend() is torch
    # the reference's top-level constants and QUDA probe (lattice/constant.py, lattice/backend.py:36)
    assert (ed.Nc, ed.Ns, ed.Nd) == (3, 4, 4)
    assert ed.check_QUDA() is False and ed.check_QUDA([1, 1, 1, 2], "torch") is False


def test_operator_parts_match_reference():
    """Operator(name, [InsertionRowMom(row, mom)], coefficients).parts as the
    reference builds them (incl. the gamma 5 / 13 sign convention)."""
    from easydistillation_gb300.correlator import InsertionRowMom, Operator
    from tests.conftest import golden

    z = golden("correlator.npz")
    spec = eval(str(z["ops_spec"]))
    ops = [Operator(n, [InsertionRowMom(r, m) for r, m in rows], cs) for n, rows, cs in spec]
    assert [op.parts for op in ops] == eval(str(z["parts"]))
    with pytest.raises(AssertionError):
        Operator("bad", [InsertionRowMom([15, [(1.0, 0)]], 0)], [1.0, 2.0])


@pytest.mark.parametrize(
    "moms, mode, factorise, expect",
    [
        ("all27", "f16x3", True, (9, 3)),
        ("all27", "tf32x3", True, (9, 3)),
        ("all27", "f16x3", False, None),
        ("all27", "fp64", True, None),
        ("first7", "f16x3", True, None),  # 5 x 3 combinations for 7 momenta: too many unused
        ([(px, py, pz) for px in (0, 1) for py in (0, 2) for pz in (0, 1, 3)], "bf16x3", True, (4, 3)),
        ([(0, 0, 0), (0, 0, 1), (0, 0, 0)], "f16x3", True, None),  # a repeated momentum
    ],
)
def test_factorised_phase_selection(moms, mode, factorise, expect):
    """Plans pick the factorised-phase GEMM exactly for product momentum sets."""
    from easydistillation_gb300.insertion import mom_dict_to_list
    from easydistillation_gb300.ops import ElementalPlan

    lists = {"all27": mom_dict_to_list(3), "first7": mom_dict_to_list(3)[:7]}
    moms = lists.get(moms, moms) if isinstance(moms, str) else moms
    p = ElementalPlan([8, 8, 4, 2], 10, 2, moms, mode, device="cpu", factorise=factorise)
    assert p.factorised == expect
    if expect:
        # the factorised workspace holds both variant operands: larger than the on-chip-phase one
        q = ElementalPlan([8, 8, 4, 2], 10, 2, moms, mode, device="cpu", factorise=False)
        assert q.factorised is None and p.workspace_bytes > q.workspace_bytes


def test_ozaki_plan_limits():
    """The Ozaki int8 mode needs factorising momenta (any unused share) and K <= 163840."""
    from easydistillation_gb300.insertion import mom_dict_to_list
    from easydistillation_gb300.ops import ElementalPlan

    p = ElementalPlan([8, 8, 4, 2], 10, 1, mom_dict_to_list(3)[:7], "ozaki_i8", device="cpu")
    assert p.factorised == (5, 3)
    with pytest.raises(Exception):
        ElementalPlan([40, 40, 36, 2], 10, 1, [(0, 0, 0)], "ozaki_i8", device="cpu")


def test_eigenvector_backend_solver_names_route_to_calc():
    """EigenvectorGenerator.laplacian_cupy_numpy / laplacian_quda /
    laplacian_quda_scipy (lattice/generator/eigenvector.py:234-354) keep the
    reference's signatures and run calc with the same arguments."""
    from easydistillation_gb300 import EigenvectorGenerator

    gen = EigenvectorGenerator.__new__(EigenvectorGenerator)
    seen = []
    gen.calc = lambda *a: seen.append(a) or ("evecs", "evals")
    assert gen.laplacian_cupy_numpy(3, False) == ("evecs", "evals")
    gen.laplacian_quda(4, True, 16, 0.5)
    gen.laplacian_quda_scipy(5, True)
    assert seen == [(3, False), (4, True, 16, 0.5), (5, True)]


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """Without the built library every call raises (there is no CPU path)."""
    from easydistillation_gb300 import _lib

    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "libeasydist_gb300.so"))
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.lib()
