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
