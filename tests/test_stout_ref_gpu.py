"""The library's stout smearing step against the reference's own CUDA kernel
(``lattice/generator/stout_smear.cu``, compiled unmodified from the
reference's source tree into ``oracle/_ref`` by ``oracle.ref_kernels``) on
the same GPU and the same links.  Both compute in FP64; they differ only in
the order of some sums, so they agree to rounding (1e-13)."""

import os

import numpy as np
import pytest
import torch

from oracle import ref_kernels
from oracle import restatement as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref_stout():
    if not os.path.exists(ref_kernels.STOUT_CUBIN):
        pytest.skip("the reference stout kernel was not built (oracle/_ref/stout_smear_ref.cubin)")
    torch.cuda.init()
    torch.zeros(1, device="cuda")  # the primary context is current on this thread
    return ref_kernels.RefStout()


@pytest.mark.parametrize("latt, eps", [([8, 6, 4, 4], 0.5), ([4, 4, 4, 2], 0.1), ([16, 16, 16, 3], 0.3)])
def test_stout_step_matches_reference_cuda_kernel(ref_stout, latt, eps):
    from easydistillation_gb300 import _lib
    from easydistillation_gb300.stout import stout_smear_

    gauge = R.synthetic_gauge(latt, eps, 23)
    U = torch.from_numpy(np.ascontiguousarray(gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3])).cuda()
    ref = torch.empty_like(U)
    ref_stout.step(ref, U, 0.1, latt, _lib.stream_handle())
    ours = U.clone()
    stout_smear_(ours, latt, 1, 0.1)
    torch.cuda.synchronize()
    assert float((ours - ref).abs().max()) < 1e-13
    # two steps: the reference's driver loop (copy, then step) against the library's ping-pong
    ref2 = torch.empty_like(U)
    ref_stout.step(ref2, ref.clone(), 0.1, latt, _lib.stream_handle())
    stout_smear_(ours, latt, 1, 0.1)
    torch.cuda.synchronize()
    assert float((ours - ref2).abs().max()) < 1e-13
