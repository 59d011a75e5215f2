"""Checks at the full benchmark sizes (32^3, Ne = 200), where the CPU oracle
is too slow, through properties that do not depend on the size:

* every split-precision elemental mode (13 operators x 27 momenta) against
  the plain FP64 GPU path on the same timeslice: relative Frobenius error
  <= 1e-6 for f16x3, tf32x3 and the Ozaki int8 slices, <= 1e-5 for bf16x3
  (two 8-bit-mantissa slices: ~2^-16 per product);
* E[no derivative, p = 0] = V^H V = identity for orthonormal eigenvectors (up
  to the complex64 rounding of V the reference applies as well);
* the plain and the Chebyshev-accelerated eigensolve of the 200 lowest modes:
  residuals ||L x - lambda x|| < 1e-9, orthonormal vectors, ascending
  eigenvalues, and the same eigenvalues to 1e-10 relative."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

LATT = [32, 32, 32, 1]
NE = 200


def _inputs(seed=9):
    from easydistillation_gb300.ops import links_to_soa  # noqa: F401  (loads the library)
    from easydistillation_gb300.synthetic import gauge_field

    g = gauge_field(LATT, 0.3, seed)  # [1, Lz, Ly, Lx, 4, 3, 3]
    U = torch.from_numpy(np.ascontiguousarray(g.transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0])).cuda()  # [3, Lz, Ly, Lx, 3, 3]
    gen = torch.Generator(device="cuda").manual_seed(seed)
    n = 3 * LATT[0] * LATT[1] * LATT[2]
    Z = torch.complex(torch.randn((n, NE), dtype=torch.float64, device="cuda", generator=gen),
                      torch.randn((n, NE), dtype=torch.float64, device="cuda", generator=gen))
    V = torch.linalg.qr(Z)[0].T.contiguous()  # [Ne, 3*V3] orthonormal rows
    return g, U, V


SPLIT_TOL = {"f16x3": 1e-6, "tf32x3": 1e-6, "ozaki_i8": 1e-6, "bf16x3": 1e-5}


@pytest.fixture(scope="module")
def fp64_full():
    """The plain FP64 GPU elementals of one 32^3, Ne = 200 timeslice (13 x 27)."""
    from easydistillation_gb300.insertion import mom_dict_to_list
    from easydistillation_gb300.ops import ElementalPlan

    _, U, V = _inputs()
    V3 = LATT[0] * LATT[1] * LATT[2]
    plan = ElementalPlan(LATT, NE, 2, mom_dict_to_list(3), "fp64", tuning={"f64_tile": 3})
    o = torch.empty((13, 27, NE, NE), dtype=torch.complex128, device="cuda")
    plan.run(U, V3 * 9, 9, V, o)
    torch.cuda.synchronize()
    del plan
    torch.cuda.empty_cache()
    return U, V, o


@pytest.mark.parametrize("mode", ["f16x3", "tf32x3", "bf16x3", "ozaki_i8"])
def test_elemental_split_modes_vs_fp64_full_size(fp64_full, mode):
    from easydistillation_gb300.insertion import mom_dict_to_list
    from easydistillation_gb300.ops import ElementalPlan

    U, V, ref = fp64_full
    V3 = LATT[0] * LATT[1] * LATT[2]
    moms = mom_dict_to_list(3)
    plan = ElementalPlan(LATT, NE, 2, moms, mode)
    o = torch.empty((13, 27, NE, NE), dtype=torch.complex128, device="cuda")
    plan.run(U, V3 * 9, 9, V, o)
    assert plan.factorised == (9, 3)
    plan.check_status()
    err = float(torch.linalg.vector_norm(o - ref) / torch.linalg.vector_norm(ref))
    assert err <= SPLIT_TOL[mode], (mode, err)
    # no derivative, zero momentum: V^H V = I up to the complex64 rounding of V
    p0 = moms.index((0, 0, 0))
    eye = torch.eye(NE, dtype=torch.complex128, device="cuda")
    assert float((o[0, p0] - eye).abs().max()) < 1e-5
    if mode == "f16x3":
        assert float((ref[0, p0] - eye).abs().max()) < 1e-6
    del plan
    torch.cuda.empty_cache()


@pytest.mark.parametrize("tuning", [{"tc_kpb": 4}, {"tc_stack": 2}, {"tc_stack": 2, "tc_kpb": 2},
                                    {"tc_pair": 2}, {"tc_pair": 2, "tc_kpb": 2}, {"tc_pair": 3},
                                    {"tc_pair": 3, "tc_kpb": 4}, {"gauss": True},
                                    {"gauss": True, "tc_kpb": 1}])
def test_f16x3_gemm_forms_vs_fp64_full_size(fp64_full, tuning):
    """The other forms of the factorised GEMM the autotuner may pick (stacked
    operands with 4 k-blocks per accumulator group; the four-product form
    with 1 or 2; SM pairs in the four-product and the stacked form) and the
    Gauss three-multiplication form at full
    size: within 1e-6 of FP64."""
    from easydistillation_gb300.insertion import mom_dict_to_list
    from easydistillation_gb300.ops import ElementalPlan

    U, V, ref = fp64_full
    V3 = LATT[0] * LATT[1] * LATT[2]
    tuning = dict(tuning)
    gauss = tuning.pop("gauss", False)
    plan = ElementalPlan(LATT, NE, 2, mom_dict_to_list(3), "f16x3", tuning=tuning, gauss=gauss)
    o = torch.empty((13, 27, NE, NE), dtype=torch.complex128, device="cuda")
    plan.run(U, V3 * 9, 9, V, o)
    plan.check_status()
    err = float(torch.linalg.vector_norm(o - ref) / torch.linalg.vector_norm(ref))
    assert err <= 1e-6, (tuning, err)
    del plan
    torch.cuda.empty_cache()


def test_chebyshev_eigensolve_full_size():
    from easydistillation_gb300.ops import lanczos_tr, laplacian, links_to_soa

    g, _, _ = _inputs(seed=10)
    U = torch.from_numpy(np.ascontiguousarray(g.transpose(4, 0, 1, 2, 3, 5, 6))).cuda()
    L = links_to_soa(U, LATT)
    ev0, X0, st0 = lanczos_tr(L, LATT, NE, 1e-10)  # plain thick-restart
    assert st0["converged"]
    ev, X, st = lanczos_tr(L, LATT, NE, 1e-12, poly_deg=16, lambda_cut=1.15 * float(ev0[0, -1]))
    assert st["converged"]
    assert torch.allclose(ev, ev0, rtol=1e-10, atol=0)
    for lam, Y in ((ev0, X0), (ev, X)):
        assert bool((lam[:, 1:] >= lam[:, :-1]).all())
        LY = laplacian(L, Y, LATT)
        res = torch.linalg.vector_norm((LY - lam[:, :, None, None].to(Y.dtype) * Y).reshape(1, NE, -1), dim=2)
        assert float(res.max()) < 1e-9
        Yf = Y.reshape(NE, -1)
        G = Yf.conj() @ Yf.T
        assert float((G - torch.eye(NE, dtype=G.dtype, device=G.device)).abs().max()) < 1e-12


def test_mixed_precision_eigensolve_full_size():
    """32^3, Ne = 200: the mixed solve (complex64 stencil in the loose FP64
    iteration, FP64 Chebyshev refinement) against the plain FP64 solve:
    eigenvalues to 1e-10 relative, residuals < 1e-9, orthonormal vectors."""
    from easydistillation_gb300.ops import lanczos_tr, laplacian, links_to_soa

    g, _, _ = _inputs(seed=10)
    U = torch.from_numpy(np.ascontiguousarray(g.transpose(4, 0, 1, 2, 3, 5, 6))).cuda()
    L = links_to_soa(U, LATT)
    L32 = links_to_soa(U, LATT, dtype=torch.complex64)
    ev0, _, st0 = lanczos_tr(L, LATT, NE, 1e-10)
    ev, X, st = lanczos_tr(L, LATT, NE, 1e-10, stencil_precision="fp32", links_c64=L32)
    assert st0["converged"] and st["converged"]
    assert torch.allclose(ev, ev0, rtol=1e-10, atol=0)
    LY = laplacian(L, X, LATT)
    res = torch.linalg.vector_norm((LY - ev[:, :, None, None].to(X.dtype) * X).reshape(1, NE, -1), dim=2)
    assert float(res.max()) < 1e-9
    Yf = X.reshape(NE, -1)
    G = Yf.conj() @ Yf.T
    assert float((G - torch.eye(NE, dtype=G.dtype, device=G.device)).abs().max()) < 1e-12
