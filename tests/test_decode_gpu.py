"""On-disk byte images converted on the device (``ed_decode_complex``,
``ed_decode_links``) against the readers' host conversion: bit-identical
results for every stored byte order and precision, special values included,
and generators fed from ILDG / QDP / npy files give the same elementals as
from the host-converted arrays."""

import numpy as np
import pytest
import torch

from oracle import restatement as R
from tests.helpers import MemEigen, MemGauge
from tests.test_preset_cpu import _write_qdp

pytestmark = pytest.mark.gpu


def _values(n, seed):
    """Complex128 values over a wide exponent range, led by signed zeros,
    infinities, subnormals (of both precisions), values at and beyond the
    float32 range and a tie-breaking case; real and imaginary parts set
    separately so that no NaN arises."""
    rng = np.random.default_rng(seed)
    z = np.empty(n, dtype=np.complex128)
    z.real = rng.standard_normal(n) * 10.0 ** rng.integers(-30, 30, n)
    z.imag = rng.standard_normal(n) * 10.0 ** rng.integers(-30, 30, n)
    special = np.array([0.0, -0.0, np.inf, -np.inf, 5e-324, -2.2250738585072014e-308, 1e-40, 3.4028235e38,
                        3.4028236e38, 1.0 + 2.0 ** -24 + 2.0 ** -50])
    k = min(n, special.size)
    z.real[:k] = special[:k]
    z.imag[:k] = special[::-1][:k]
    return z


def _bits_equal(a, b):
    return a.shape == b.shape and a.dtype == b.dtype and np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("file_dtype", [">c16", "<c16", ">c8", "<c8"])
@pytest.mark.parametrize("n", [1, 7, 100_003])
def test_decode_complex_matches_astype(file_dtype, n):
    from easydistillation_gb300.ops import decode_complex
    from easydistillation_gb300.preset import pinned_bytes

    with np.errstate(over="ignore"):
        stored = _values(n, n).astype(file_dtype)
    raw = pinned_bytes(stored).cuda()
    for dtype, np_dtype in ((torch.complex128, "<c16"), (torch.complex64, "<c8")):
        with np.errstate(over="ignore"):
            ref = stored.astype(np_dtype)
        out = decode_complex(raw, file_dtype, dtype).cpu().numpy()
        assert _bits_equal(out, ref), (file_dtype, n, np_dtype)
    # NaNs survive as NaNs (their payload is not compared)
    nan = np.full(3, np.nan + 1j * np.nan).astype(file_dtype)
    assert np.isnan(decode_complex(pinned_bytes(nan).cuda(), file_dtype).cpu().numpy()).all()


@pytest.mark.parametrize("file_dtype", [">c16", ">c8", "<c16"])
def test_decode_links_matches_host_transpose(file_dtype):
    from easydistillation_gb300.generator.elemental import links_to_device
    from easydistillation_gb300.ops import decode_links
    from easydistillation_gb300.preset import pinned_bytes

    latt = [6, 4, 2, 3]
    g = R.synthetic_gauge(latt, 0.3, 5).astype(file_dtype)  # [Lt, Lz, Ly, Lx, 4, 3, 3]
    ref = links_to_device(g.astype("<c16"), latt, "cuda")
    out = decode_links(pinned_bytes(g).cuda(), file_dtype, latt)
    assert out.shape == ref.shape and torch.equal(out, ref)


def test_ildg_file_to_device(tmp_path):
    from easydistillation_gb300.generator.elemental import links_to_device
    from easydistillation_gb300.preset import GaugeFieldIldg, write_ildg

    latt = [4, 4, 2, 3]
    Lx, Ly, Lz, Lt = latt
    g = R.synthetic_gauge(latt, 0.3, 8)
    write_ildg(str(tmp_path / "cfg.lime"), g, latt)
    d = GaugeFieldIldg(str(tmp_path) + "/", ".lime", [Lt, Lz * Ly * Lx, 4, 3, 3]).load("cfg")
    host = d[:]
    assert torch.equal(d.to_device(slice(None)).cpu(), torch.from_numpy(host))
    assert torch.equal(d.to_device((1, slice(0, 5))).cpu(), torch.from_numpy(host[1, 0:5]))
    assert d.to_device(0, dtype=torch.complex64).dtype == torch.complex64
    assert torch.equal(d.links_to_device(latt), links_to_device(host, latt, "cuda"))


def test_generators_from_files_match_host_arrays(tmp_path):
    """ElementalGenerator on an ILDG gauge file with QDP (big-endian
    complex64) and npy (complex128) eigenvector files against the same data
    given as host arrays: identical elementals; EigenvectorGenerator's links
    identical too."""
    from easydistillation_gb300 import ElementalGenerator, EigenvectorGenerator
    from easydistillation_gb300.preset import EigenvectorNpy, EigenvectorTimeSlice, GaugeFieldIldg, write_ildg

    latt, Ne, moms = [8, 8, 4, 3], 10, R.mom_dict_to_list(3)[:7]
    Lx, Ly, Lz, Lt = latt
    V3 = Lx * Ly * Lz
    gauge = R.synthetic_gauge(latt, 0.3, 31)
    evec = np.stack([R.random_colour_vectors(Ne, latt, 310 + t) for t in range(Lt)]).reshape(Lt, Ne, V3, 3)
    write_ildg(str(tmp_path / "cfg.lime"), gauge, latt)
    G = GaugeFieldIldg(str(tmp_path) + "/", ".lime", [Lt, V3, 4, 3, 3])

    ev64 = evec.astype(">c8")
    _write_qdp(tmp_path / "cfg.mod", {(t, e): ev64[t, e] for t in range(Lt) for e in range(Ne)})
    EQ = EigenvectorTimeSlice(str(tmp_path) + "/", ".mod", [Lt, Ne, V3, 3], Ne)
    np.save(tmp_path / "cfg.ev.npy", evec)
    EN = EigenvectorNpy(str(tmp_path) + "/", ".ev.npy", list(evec.shape), Ne)

    cases = [(EQ, ev64.astype("<c16")), (EN, evec)]
    for E, host_ev in cases:
        ref = ElementalGenerator(latt, MemGauge(G.load("cfg")[:]), MemEigen(host_ev, Ne), 1, moms)
        ref.load("cfg")
        gen = ElementalGenerator(latt, G, E, 1, moms)
        gen.load("cfg")
        assert torch.equal(gen._U, ref._U)
        assert torch.equal(gen.calc_batch(range(Lt)).cpu(), ref.calc_batch(range(Lt)).cpu())
        for t in range(Lt):
            assert torch.equal(gen.calc(t).cpu(), ref.calc(t).cpu())

    eg = EigenvectorGenerator(latt, G, Ne, 1e-10)
    eg.load("cfg")
    eh = EigenvectorGenerator(latt, MemGauge(G.load("cfg")[:]), Ne, 1e-10)
    eh.load("cfg")
    assert torch.equal(eg._U, eh._U)
