"""Laplacian, covariant-derivative hop, layout conversion and phase kernels
against the oracle / golden vectors (GPU).  Tolerances: FP64 paths 1e-13
absolute on O(1) data; the FP32 Laplacian 2e-6 relative (Frobenius)."""

import numpy as np
import pytest
import torch

from oracle import restatement as R
from tests.conftest import golden
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu


def _planes(F, latt):
    """reference [V3*3, nvec] -> planes [nvec, 3, V3] (numpy)"""
    Lx, Ly, Lz = latt[:3]
    V3 = Lx * Ly * Lz
    return np.ascontiguousarray(F.reshape(V3, 3, -1).transpose(2, 1, 0))


def _soa(g, latt, t=0):
    from easydistillation_gb300.ops import links_to_soa

    U = torch.from_numpy(np.ascontiguousarray(g)).cuda()
    return links_to_soa(U, latt, layout="ildg")


@pytest.mark.parametrize("tag", ["443", "642"])
def test_laplacian_fp64_golden(tag):
    from easydistillation_gb300.ops import laplacian

    g = golden(f"laplacian_{tag}.npz")
    latt = list(g["latt"])
    links = _soa(g["gauge"], latt)[:1]
    F = torch.from_numpy(_planes(g["F"], latt)).cuda().unsqueeze(0)
    out = laplacian(links, F, latt)[0].cpu().numpy()  # [nvec, 3, V3]
    ref = _planes(g["LF"], latt)
    assert np.abs(out - ref).max() < 1e-13


@pytest.mark.parametrize("tag", ["443", "642"])
def test_laplacian_fp32_golden(tag):
    from easydistillation_gb300.ops import laplacian, links_to_soa

    g = golden(f"laplacian_{tag}.npz")
    latt = list(g["latt"])
    U = torch.from_numpy(np.ascontiguousarray(g["gauge"])).cuda()
    links = links_to_soa(U, latt, dtype=torch.complex64, layout="ildg")[:1]
    F = torch.from_numpy(_planes(g["F"], latt)).cuda().to(torch.complex64).unsqueeze(0)
    out = laplacian(links, F, latt)[0].cpu().numpy()
    assert rel_err(out, _planes(g["LF"], latt)) < 2e-6


@pytest.mark.parametrize("latt", [[8, 6, 4, 3], [2, 2, 2, 2], [16, 8, 6, 2]])
@pytest.mark.parametrize("dtype", [torch.complex128, torch.complex64])
def test_laplacian_batched_timeslices_and_vectors(latt, dtype):
    """nt timeslices x nvec vectors in one launch, strided timeslice views."""
    from easydistillation_gb300.ops import laplacian, links_to_soa

    Lx, Ly, Lz, Lt = latt
    V3 = Lx * Ly * Lz
    gauge = R.synthetic_gauge(latt, 0.3, 5)
    U = torch.from_numpy(gauge).cuda()
    links = links_to_soa(U, latt, dtype=dtype, layout="ildg")
    rng = np.random.default_rng(1)
    nvec = 3
    F = rng.standard_normal((Lt, nvec, V3 * 3)) + 1j * rng.standard_normal((Lt, nvec, V3 * 3))
    # timeslice stride larger than the packed size: view into a bigger buffer
    big = torch.zeros((Lt, nvec + 1, 3, V3), dtype=dtype, device="cuda")
    Fp = np.stack([_planes(F[t].T, latt) for t in range(Lt)])
    big[:, :nvec] = torch.from_numpy(Fp).to(dtype)
    out = laplacian(links, big[:, :nvec], latt).cpu().numpy()
    tol = 1e-13 if dtype == torch.complex128 else 3e-6
    for t in range(Lt):
        Ut = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, t]
        ref = _planes(R.laplacian(F[t].T, Ut, latt), latt)
        assert rel_err(out[t], ref) < tol


@pytest.mark.parametrize("d", [0, 1, 2])
@pytest.mark.parametrize("prec", [(torch.complex128, torch.complex128), (torch.complex64, torch.complex64),
                                  (torch.complex64, torch.complex128)])
def test_covariant_derivative(d, prec):
    from easydistillation_gb300.ops import covariant_derivative, links_to_soa, vectors_to_planes

    latt = [6, 4, 8, 1]
    Lx, Ly, Lz, _ = latt
    V3 = Lx * Ly * Lz
    gauge = R.synthetic_gauge(latt, 0.3, 8)
    Ut = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0]
    V = R.random_colour_vectors(11, latt, 9)  # [Ne, Lz, Ly, Lx, 3]
    links = links_to_soa(torch.from_numpy(gauge).cuda(), latt, layout="ildg")[0]
    Vin = torch.from_numpy(V.reshape(11, V3 * 3)).cuda()
    Vp = vectors_to_planes(Vin.reshape(11, V3, 3), V3, dtype=prec[0])
    out = covariant_derivative(links, Vp, latt, d, out_dtype=prec[1])
    ref = R.covariant_derivative(V.astype(np.complex64).astype(np.complex128) if prec[0] == torch.complex64 else V,
                                 Ut, d)
    refp = np.ascontiguousarray(ref.reshape(11, V3, 3).transpose(0, 2, 1))
    tol = 1e-14 if prec[1] == torch.complex128 else 1e-6
    assert rel_err(out.cpu().numpy(), refp) < tol


def test_vector_layout_roundtrip_and_c64_rounding():
    from easydistillation_gb300.ops import vectors_from_planes, vectors_to_planes

    rng = np.random.default_rng(3)
    V3 = 60
    A = rng.standard_normal((5, V3, 3)) + 1j * rng.standard_normal((5, V3, 3))
    t = torch.from_numpy(A).cuda()
    P = vectors_to_planes(t, V3)
    back = vectors_from_planes(P, V3).cpu().numpy()
    np.testing.assert_array_equal(back, A)
    P64 = vectors_to_planes(t, V3, dtype=torch.complex128, round_c64=True)
    np.testing.assert_array_equal(vectors_from_planes(P64, V3).cpu().numpy(), A.astype(np.complex64).astype(np.complex128))


def test_momentum_phases_golden():
    from easydistillation_gb300.ops import momentum_phases

    g = golden("phase_462.npz")
    latt = list(g["latt"])
    out = momentum_phases(latt, [tuple(p) for p in g["moms"]]).cpu().numpy()
    assert np.abs(out - g["phase"]).max() < 1e-15 * 8


@pytest.mark.parametrize("staged", [1, 2])
@pytest.mark.parametrize("latt, nvec", [([8, 8, 6, 3], 2), ([16, 16, 16, 2], 1), ([32, 32, 32, 2], 1),
                                        ([24, 24, 24, 1], 3), ([4, 4, 3, 2], 2), ([12, 10, 5, 2], 2)])
def test_laplacian_tma_matches_plain_and_oracle(latt, nvec, staged):
    """complex64: the TMA-staged kernel (input planes z-1, z, z+1 in shared
    memory, several z slabs per (timeslice, vector)) against the plain kernel
    and the FP64 oracle, with a padded timeslice stride."""
    from easydistillation_gb300.ops import laplacian, laplacian_config, laplacian_status, links_to_soa

    Lx, Ly, Lz, Lt = latt
    V3 = Lx * Ly * Lz
    gauge = R.synthetic_gauge(latt, 0.3, 8)
    links = links_to_soa(torch.from_numpy(gauge).cuda(), latt, dtype=torch.complex64, layout="ildg")
    rng = np.random.default_rng(3)
    F = rng.standard_normal((Lt, nvec, V3 * 3)) + 1j * rng.standard_normal((Lt, nvec, V3 * 3))
    big = torch.zeros((Lt, nvec + 1, 3, V3), dtype=torch.complex64, device="cuda")
    big[:, :nvec] = torch.from_numpy(np.stack([_planes(F[t].T, latt) for t in range(Lt)])).to(torch.complex64)
    try:
        laplacian_config(staged)
        o_tma = laplacian(links, big[:, :nvec], latt).cpu().numpy()
        assert laplacian_status() == 0
        laplacian_config(0)
        o_plain = laplacian(links, big[:, :nvec], latt).cpu().numpy()
    finally:
        laplacian_config()
    assert rel_err(o_tma, o_plain) < 1e-6
    for t in range(Lt):
        Ut = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, t]
        ref = _planes(R.laplacian(F[t].T, Ut, latt), latt)
        assert rel_err(o_tma[t], ref) < 3e-6


@pytest.mark.parametrize("tag", ["443", "642"])
def test_laplacian_double_float_golden(tag):
    """ED_DF (the double-float Laplacian of the df eigensolve mode) against the
    reference's own Laplacian output, to 1e-13 relative to the largest output
    (measured 2.6e-14: ~2^-47 per product where FP64 gives 2^-53)."""
    from easydistillation_gb300.ops import laplacian_df, split_c128

    g = golden(f"laplacian_{tag}.npz")
    latt = list(g["latt"])
    links = split_c128(_soa(g["gauge"], latt)[:1].contiguous())
    F = torch.from_numpy(_planes(g["F"], latt)).cuda().unsqueeze(0)
    out = laplacian_df(links, F, latt)[0].cpu().numpy()
    ref = _planes(g["LF"], latt)
    assert np.abs(out - ref).max() < 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("latt", [[6, 4, 8, 3], [16, 16, 16, 2], [24, 24, 24, 1]])
def test_laplacian_double_float_matches_fp64(latt):
    """Several timeslices and vectors, odd and even extents, values spanning
    several orders of magnitude (the split works on the bits of every input):
    the double-float result is the FP64 kernel's to 1e-13 relative."""
    from easydistillation_gb300.ops import laplacian, laplacian_df, links_to_soa, split_c128

    Lx, Ly, Lz, Lt = latt
    V3 = Lx * Ly * Lz
    gauge = R.synthetic_gauge(latt, 0.3, 31)
    U = torch.from_numpy(np.ascontiguousarray(gauge.transpose(4, 0, 1, 2, 3, 5, 6))).cuda()
    links = links_to_soa(U, latt)
    g = torch.Generator(device="cuda").manual_seed(5)
    F = torch.complex(torch.randn((Lt, 2, 3, V3), generator=g, device="cuda", dtype=torch.float64),
                      torch.randn((Lt, 2, 3, V3), generator=g, device="cuda", dtype=torch.float64))
    F = F * torch.exp(8 * torch.randn((Lt, 2, 3, V3), generator=g, device="cuda", dtype=torch.float64))
    ref = laplacian(links, F, latt)
    out = laplacian_df(split_c128(links), F, latt)
    err = float((out - ref).abs().max() / ref.abs().max())
    assert err < 1e-13, err
