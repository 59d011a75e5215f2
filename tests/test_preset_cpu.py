"""File readers with the reference's preset classes (CPU): an ILDG file read
exactly as the reference's own reader read it (fixture), and .npy / raw
binary / QDP lazy-disk-map round trips."""

import os
import struct

import numpy as np

from tests.conftest import GOLDEN, golden


def test_ildg_matches_reference_reader():
    from easydistillation_gb300.preset import GaugeFieldIldg

    g = golden("ildg_small.npz")
    Lx, Ly, Lz, Lt = [int(v) for v in g["latt"]]
    data = GaugeFieldIldg(os.path.join(GOLDEN, "small"), ".lime", [Lt, Lz, Ly, Lx, 4, 3, 3]).load("")
    np.testing.assert_array_equal(data[:], g["ref_read"])
    np.testing.assert_array_equal(data[1, :, 0], g["ref_slice"])
    assert data[:].dtype == np.complex128 and data.latt_size == [Lx, Ly, Lz, Lt]


def test_npy_and_binary_presets(tmp_path):
    from easydistillation_gb300.preset import ElementalBinary, EigenvectorNpy, GaugeFieldBinary, PerambulatorNpy

    rng = np.random.default_rng(0)
    ev = (rng.standard_normal((3, 5, 8, 3)) + 1j * rng.standard_normal((3, 5, 8, 3))).astype(np.complex128)
    np.save(tmp_path / "cfgA.ev.npy", ev)
    E = EigenvectorNpy(str(tmp_path) + "/", ".ev.npy", list(ev.shape), 5)
    d = E.load("cfgA")
    np.testing.assert_array_equal(d[1, 2], ev[1, 2])
    np.testing.assert_array_equal(d[2, 0:4], ev[2, 0:4])
    assert E.Ne == 5
    gb = rng.standard_normal((2, 8, 4, 3, 3)) + 0j
    gb.astype("<c16").tofile(tmp_path / "cfgB.dat")
    G = GaugeFieldBinary(str(tmp_path) + "/", ".dat", list(gb.shape), "<c16")
    np.testing.assert_array_equal(G.load("cfgB")[:], gb)
    el = rng.standard_normal((2, 3, 4, 5, 5)).astype(np.complex128)
    el.astype("<c16").tofile(tmp_path / "cfgC.meson")
    np.testing.assert_array_equal(ElementalBinary(str(tmp_path) + "/", ".meson", list(el.shape), 5).load("cfgC")[1, 2],
                                  el[1, 2])
    pe = rng.standard_normal((2, 2, 4, 4, 3, 3)).astype(np.complex64)
    np.save(tmp_path / "cfgD.peram.npy", pe)
    np.testing.assert_array_equal(PerambulatorNpy(str(tmp_path) + "/", ".peram.npy", list(pe.shape), 3).load("cfgD")[1],
                                  pe[1])


def _write_qdp(path, blocks, xml="<foo><lattSize>4 4 4 8</lattSize><decay_dir>3</decay_dir></foo>"):
    """Minimal QDP LazyDiskMapObjFile writer (layout of lattice/filedata/timeslice.py:110-121)."""
    def s(x):
        b = x.encode()
        return struct.pack(">i", len(b)) + b

    head = s("XXXXQDPLazyDiskMapObjFileXXXX") + struct.pack(">i", 1) + s(xml)
    data_off = len(head) + 16
    body, offsets = b"", {}
    for key, arr in blocks.items():
        offsets[key] = data_off + len(body)
        body += arr.tobytes()
    trailer_pos = data_off + len(body)
    trailer = struct.pack(">I", len(blocks))
    for key, off in offsets.items():
        trailer += struct.pack(">i", 4 * len(key)) + struct.pack(">" + "i" * len(key), *key) + struct.pack(">qq", 0, off)
    with open(path, "wb") as f:
        f.write(head + struct.pack(">qq", 0, trailer_pos) + body + trailer)


def test_qdp_lazy_disk_map(tmp_path):
    from easydistillation_gb300.preset import EigenvectorTimeSlice

    rng = np.random.default_rng(1)
    blocks = {(t, e): (rng.standard_normal((6, 3)) + 1j * rng.standard_normal((6, 3))).astype(">c8")
              for t in range(2) for e in range(3)}
    _write_qdp(tmp_path / "cfg.mod", blocks)
    E = EigenvectorTimeSlice(str(tmp_path) + "/", ".mod", [2, 3, 6, 3], 3)
    d = E.load("cfg")
    for (t, e), arr in blocks.items():
        out = d[t, e]
        assert out.dtype == np.complex64
        np.testing.assert_array_equal(out, arr.astype(np.complex64))


def test_raw_gives_the_stored_values(tmp_path):
    """``raw(key)`` returns the file's own dtype (byte order and precision as
    stored), which the readers' host conversion turns into ``[key]``."""
    from easydistillation_gb300.preset import EigenvectorTimeSlice, GaugeFieldIldg

    g = golden("ildg_small.npz")
    Lx, Ly, Lz, Lt = [int(v) for v in g["latt"]]
    data = GaugeFieldIldg(os.path.join(GOLDEN, "small"), ".lime", [Lt, Lz, Ly, Lx, 4, 3, 3]).load("")
    r = data.raw(slice(None))
    assert r.dtype == np.dtype(">c16")
    np.testing.assert_array_equal(r.astype("<c16"), g["ref_read"])
    v = data.raw((1, slice(None), 0), copy=False)
    assert isinstance(v, np.memmap) and v.dtype == np.dtype(">c16")
    np.testing.assert_array_equal(np.asarray(v).astype("<c16"), g["ref_slice"])

    rng = np.random.default_rng(2)
    blocks = {(t, e): (rng.standard_normal((6, 3)) + 1j * rng.standard_normal((6, 3))).astype(">c8")
              for t in range(2) for e in range(3)}
    _write_qdp(tmp_path / "cfg.mod", blocks)
    d = EigenvectorTimeSlice(str(tmp_path) + "/", ".mod", [2, 3, 6, 3], 3).load("cfg")
    for (t, e), arr in blocks.items():
        r = d.raw((t, e))
        assert r.dtype == np.dtype(">c8")
        np.testing.assert_array_equal(r, arr)
    assert d.links_to_device([1, 1, 1, 1]) is None  # QDP records are not in the ILDG site order


def test_file_prec_codes():
    import pytest

    from easydistillation_gb300 import _lib
    from easydistillation_gb300.ops import file_prec

    assert file_prec(">c16") == _lib.ED_C128 | _lib.ED_BIG_ENDIAN
    assert file_prec("<c16") == _lib.ED_C128
    assert file_prec(">c8") == _lib.ED_C64 | _lib.ED_BIG_ENDIAN
    assert file_prec(np.complex64) == _lib.ED_C64
    with pytest.raises(ValueError):
        file_prec("<f8")


def test_pinned_bytes_split_copy(monkeypatch):
    """The byte copy behind the device-side readers: contiguous arrays above
    the per-thread chunk are split across host threads (chunk lowered here so
    a small array takes that path), other layouts copied in one pass; into a
    caller's buffer at an offset.  Runs on CPU with an ordinary tensor as
    ``out`` (page-locked memory needs a GPU)."""
    import torch

    from easydistillation_gb300 import preset

    monkeypatch.setattr(preset, "_COPY_CHUNK", 1 << 12)
    rng = np.random.default_rng(3)
    a = (rng.standard_normal((300, 37)) + 1j * rng.standard_normal((300, 37))).astype(">c16")
    for src in (a, a[:, ::3], a[7], a[:0]):
        buf = torch.zeros(src.nbytes + 24, dtype=torch.uint8)
        out = preset.pinned_bytes(src, buf[8:])
        assert out.numel() == src.nbytes
        np.testing.assert_array_equal(out.numpy().view(">c16").reshape(src.shape), src)
        assert not buf[:8].any() and not buf[8 + src.nbytes:].any()
    import pytest

    with pytest.raises(ValueError):
        preset.pinned_bytes(a, torch.zeros(a.nbytes - 1, dtype=torch.uint8))


def test_per_source_perambulator_and_correlator_data(tmp_path):
    """PerambulatorTimeslicesNpy (lattice/preset.py:114-126): one .npy per
    source timeslice, ``.t???.`` in the name replaced by the first index;
    the two-point / one-point data presets; every preset is an instance of the
    reference's base class for its kind."""
    import pytest

    from easydistillation_gb300 import preset as P

    rng = np.random.default_rng(3)
    Lt, Ne = 3, 4
    full = (rng.standard_normal((Lt, Lt, 4, 4, Ne, Ne)) + 1j * rng.standard_normal((Lt, Lt, 4, 4, Ne, Ne)))
    full = full.astype(np.complex64)
    for t in range(Lt):
        np.save(tmp_path / f"cfgE.t{t:03d}.peram.npy", full[t])
    pre = P.PerambulatorTimeslicesNpy(str(tmp_path) + "/", ".t???.peram.npy", list(full.shape), Ne)
    d = pre.load("cfgE")
    assert isinstance(pre, P.Perambulator) and pre.Ne == Ne
    assert d.source_file(2).endswith("cfgE.t002.peram.npy")
    np.testing.assert_array_equal(d[1], full[1])
    key = (2, slice(None), slice(None), slice(None), slice(None, 3), slice(None, 3))  # the correlators' key
    np.testing.assert_array_equal(d[key], full[2, :, :, :, :3, :3])
    np.testing.assert_array_equal(d[0, [2, 0]], full[0, [2, 0]])
    with pytest.raises(TypeError):
        d[0:2]
    assert d.size_in_byte > 0

    two = rng.standard_normal((2, 2, 3, 4, 5, 6))
    two.astype("<f8").tofile(tmp_path / "cfgF.2pt.bin")
    jb = P.Jpsi2gammaBinary(str(tmp_path) + "/", ".2pt.bin", list(two.shape))
    np.testing.assert_array_equal(jb.load("cfgF")[1, :, 2], two[1, :, 2])
    np.save(tmp_path / "cfgG.2pt.npy", two)
    np.testing.assert_array_equal(P.Jpsi2gammaNpy(str(tmp_path) + "/", None).load("cfgG")[:], two)
    one = rng.standard_normal((2, 7, 5))
    np.save(tmp_path / "cfgH.1pt.npy", one)
    np.testing.assert_array_equal(P.OnePointNpy(str(tmp_path) + "/", None).load("cfgH")[1], one[1])
    for obj, base in [(jb, P.TwoPoint), (P.OnePointNpy("a", None), P.OnePoint), (P.GaugeFieldIldg("a", None), P.GaugeField),
                      (P.EigenvectorNpy("a", None), P.Eigenvector), (P.ElementalNpy("a", None), P.Elemental),
                      (P.PerambulatorBinary("a", None), P.Perambulator)]:
        assert isinstance(obj, base), (obj, base)
