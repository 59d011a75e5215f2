"""ed_elemental_run_noalloc: the elemental entry point for callers that
cannot allocate device memory (their GPU memory belongs to another allocator,
or they run where allocation is not allowed).  It must give the same
elementals as ed_elemental_run with a caller workspace, call after call,
although every call reuses the library's built-in scratch array.

Collected last on purpose (file name), so that a run stopping at the first
failure has already run every other test.  Works alone in a fresh process and
after the other tests."""

import ctypes

import numpy as np
import pytest
import torch

from oracle import restatement as R

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12  # the relative tolerance of the FP64 elemental tests
# the tolerance of the split-precision tests against FP64; the no-allocation run
# and the workspace run use the same kernels, so they must agree far closer
TC_TOL = 1e-6


def _inputs(latt, Ne, seed):
    gauge = R.synthetic_gauge(latt, 0.3, seed)
    U = torch.from_numpy(np.ascontiguousarray(gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3])).cuda()
    V = torch.from_numpy(R.random_colour_vectors(Ne, latt, seed + 1).reshape(Ne, -1)).cuda()
    return U, V


def _rel(a, b):
    return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))


def test_noalloc_matches_workspace_entry_point_twice():
    from easydistillation_gb300 import _lib
    from easydistillation_gb300.ops import ElementalPlan

    latt = [4, 4, 4, 2]
    Lx, Ly, Lz, Lt = latt
    V3 = Lx * Ly * Lz
    Ne, moms = 6, R.mom_dict_to_list(3)[:7]
    plan = ElementalPlan(latt, Ne, 2, moms, "fp64")
    assert plan.workspace_bytes <= (32 << 20)
    stream = _lib.stream_handle()
    outs = []
    for seed in (3, 4):  # two calls in a row on different inputs
        U, V = _inputs(latt, Ne, seed)
        links = U[:, 1]
        ref = torch.empty((13, 7, Ne, Ne), dtype=torch.complex128, device="cuda")
        plan.run(links, Lt * V3 * 9, 9, V, ref)
        out = torch.full_like(ref, float("nan"))
        rc = _lib.lib().ed_elemental_run_noalloc(plan._h, links.data_ptr(), Lt * V3 * 9, 9, _lib.ED_C128,
                                                 V.data_ptr(), None, out.data_ptr(), stream)
        _lib.check(rc, "ed_elemental_run_noalloc")
        torch.cuda.synchronize()
        assert _rel(out, ref) < FP64_TOL
        outs.append(out)
    assert _rel(outs[0], outs[1]) > 1e-3  # the second call did not return the first call's result


def test_noalloc_rejects_plans_larger_than_its_scratch():
    from easydistillation_gb300 import _lib
    from easydistillation_gb300.ops import ElementalPlan

    plan = ElementalPlan([16, 16, 16, 1], 64, 2, R.mom_dict_to_list(3), "fp64")
    assert plan.workspace_bytes > (32 << 20)
    dummy = torch.zeros(16, dtype=torch.complex128, device="cuda")
    rc = _lib.lib().ed_elemental_run_noalloc(plan._h, dummy.data_ptr(), 0, 9, _lib.ED_C128, dummy.data_ptr(),
                                             None, dummy.data_ptr(), _lib.stream_handle())
    assert rc == _lib.ED_ERR_WORKSPACE
    assert "scratch" in _lib.last_error()


@pytest.mark.parametrize("nmom", [7, 27])
def test_noalloc_tensor_core_modes_on_a_dirty_array(nmom):
    """f16x3 through the built-in array, twice in a row on different inputs, after
    the FP64 calls above left their own bytes in it: the tensor-core modes clear
    their accumulators and status word themselves, so each call must agree with
    ed_elemental_run on a fresh caller workspace, and the status word read back
    by ed_elemental_status_noalloc must be clean.  Seven momenta run the GEMM that
    forms the phase-weighted operand on chip, 27 the factorised-phase GEMM."""
    from easydistillation_gb300 import _lib
    from easydistillation_gb300.ops import ElementalPlan

    latt = [4, 4, 4, 2]
    Lx, Ly, Lz, Lt = latt
    V3 = Lx * Ly * Lz
    Ne, moms = 6, R.mom_dict_to_list(3)[:nmom]
    plan = ElementalPlan(latt, Ne, 2, moms, "f16x3")
    assert plan.workspace_bytes <= (32 << 20)
    assert (plan.factorised is not None) == (nmom == 27)
    stream = _lib.stream_handle()
    outs = []
    for seed in (7, 8):
        U, V = _inputs(latt, Ne, seed)
        links = U[:, 0]
        ref = torch.empty((13, nmom, Ne, Ne), dtype=torch.complex128, device="cuda")
        plan.run(links, Lt * V3 * 9, 9, V, ref)
        assert plan.check_status() == 0
        out = torch.full_like(ref, float("nan"))
        rc = _lib.lib().ed_elemental_run_noalloc(plan._h, links.data_ptr(), Lt * V3 * 9, 9, _lib.ED_C128,
                                                 V.data_ptr(), None, out.data_ptr(), stream)
        _lib.check(rc, "ed_elemental_run_noalloc")
        code = ctypes.c_int(-1)
        rc = _lib.lib().ed_elemental_status_noalloc(plan._h, ctypes.byref(code), stream)
        _lib.check(rc, "ed_elemental_status_noalloc")
        assert code.value == 0
        assert _rel(out, ref) < TC_TOL
        outs.append(out)
    assert _rel(outs[0], outs[1]) > 1e-3
