"""File readers with the reference's preset classes and on-disk layouts.

Mirrors ``lattice/preset.py`` and ``lattice/filedata/*.py``: each preset is
constructed as in the reference (``prefix``, ``suffix``, ``shape`` and, for
eigenvectors/elementals/perambulators, ``totNe``) and ``load(key)`` returns a
file-data object that is indexed like a numpy array (``[:]``, ``[t]``,
``[t, e]``, slices).  Reads are memory-mapped; the result is a host numpy
array with the reference's dtype conversion (ILDG data up-cast to complex128,
``lattice/filedata/ildg.py:70``; QDP lazy-disk-map data down-cast to
complex64, ``timeslice.py:96``).

Device side (no counterpart in the reference, whose readers convert on the
host): ``raw(key)`` gives the stored values without conversion;
``to_device(key)`` copies the stored bytes of complex data into pinned
memory, uploads them in one copy and converts them on the device
(``ops.decode_complex``: byte order and precision, bit-identical to the host
conversion); ``links_to_device(latt_size)`` does the same for a gauge field in
the ILDG order and transposes it to the generators' spatial-link layout in the
same pass (``ops.decode_links``).

Formats:
* ILDG / LIME (``ildg.py:82-96``): records of an 8-byte magic/version word, a
  big-endian 8-byte length, a 128-byte type string and the 8-byte padded
  payload; ``ildg-format`` holds the XML (lx, ly, lz, lt, precision) and
  ``ildg-binary-data`` the big-endian field.
* ``.npy`` (``ndarray.py:17-47``): numpy header, C order; per-source files
  (``ndarray.py:54-90``) for ``PerambulatorTimeslicesNpy``.
* raw binary (``binary.py:23-66``).
* QDP LazyDiskMapObjFile (``timeslice.py:102-129``): magic string, version,
  XML, a trailer with key tuples and offsets.
"""

from __future__ import annotations

import mmap
import os
import re
import struct
import xml.etree.ElementTree as ET
from copy import deepcopy
from time import time
from typing import Dict, List, Tuple

import numpy as np
import torch


class FileMetaData:
    def __init__(self, shape: List[int], dtype: str = "<c16", extra=None):
        self.shape = shape
        self.dtype = dtype
        self.extra = extra


class _Data:
    """Common indexing and timing of the file-data objects."""

    file = None

    def _array(self):  # pragma: no cover - implemented by subclasses
        raise NotImplementedError

    def _convert(self, a):
        return a

    # numpy dtype __getitem__ converts to (None: the stored dtype)
    _target = None

    def _account(self, start, nbytes):
        self.time_in_sec += time() - start
        self.size_in_byte += nbytes
        self.timeInSec, self.sizeInByte = self.time_in_sec, self.size_in_byte

    def _view(self, key):
        """The stored values of ``key``, memory-mapped (no copy)."""
        return self._array()[key]

    def __getitem__(self, key):
        s = time()
        ret = self._convert(np.array(self._view(key), copy=True))
        self._account(s, ret.nbytes)
        return ret

    def raw(self, key, copy: bool = True):
        """The stored values of ``key`` without conversion: a host array in
        the file's own dtype (byte order and precision as on disk); with
        ``copy=False`` the memory-mapped view."""
        s = time()
        v = self._view(key)
        ret = np.array(v, copy=True) if copy else v
        self._account(s, ret.nbytes)
        return ret

    def to_device(self, key, device=None, dtype=None):
        """``self[key]`` as a device tensor.  Complex data go up as stored and
        are converted on the device (to ``dtype``, default the reader's own
        conversion); other data are converted on the host first."""
        v = self.raw(key, copy=False)
        if np.dtype(v.dtype).kind != "c":
            t = torch.from_numpy(np.ascontiguousarray(self._convert(np.array(v, copy=True))))
            if dtype is not None:
                t = t.to(dtype)
            return t.pin_memory().to(device or "cuda", non_blocking=True)
        from . import ops

        if dtype is None:
            dtype = torch.complex128 if np.dtype(self._target or v.dtype).itemsize == 16 else torch.complex64
        raw = pinned_bytes(v).to(device or "cuda", non_blocking=True)
        return ops.decode_complex(raw, v.dtype, dtype).reshape(np.shape(v))

    def links_to_device(self, latt_size, device=None):
        """The gauge field of this file (ILDG order ``[Lt, Lz, Ly, Lx, 4, 3,
        3]``, complex) as the generators' spatial links ``[3, Lt, Lz, Ly, Lx,
        3, 3]`` complex128 on the device, converted and transposed there; None
        when the stored values are not complex numbers of that count."""
        v = self.raw(slice(None), copy=False)
        Lx, Ly, Lz, Lt = latt_size
        if np.dtype(v.dtype).kind != "c" or np.size(v) != Lt * Lz * Ly * Lx * 36:
            return None
        from . import ops

        raw = pinned_bytes(v).to(device or "cuda", non_blocking=True)
        return ops.decode_links(raw, v.dtype, latt_size)


_COPY_CHUNK = 64 << 20  # bytes per host thread above which pinned_bytes splits a contiguous copy


def pinned_bytes(a, out: torch.Tensor = None) -> torch.Tensor:
    """The bytes of array ``a`` (a memory-mapped view or any numpy array) in
    page-locked host memory, copied in one pass: a uint8 tensor of
    ``a.nbytes`` (or the first ``a.nbytes`` bytes of ``out``, a pinned uint8
    tensor, when given).  Contiguous arrays above 64 MB are copied by several
    host threads (the page-cache reads of a memory map and the copy itself
    scale with cores)."""
    a = np.asarray(a)
    if out is None:
        out = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
    elif out.dtype != torch.uint8 or out.numel() < a.nbytes:
        raise ValueError("out must be a uint8 tensor of at least a.nbytes bytes")
    dst = out[: a.nbytes].numpy()
    nthreads = min(len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else 1, 16,
                   a.nbytes // _COPY_CHUNK)
    if nthreads > 1 and a.flags.c_contiguous:
        from concurrent.futures import ThreadPoolExecutor

        src = a.reshape(-1).view(np.uint8)
        bounds = np.linspace(0, a.nbytes, nthreads + 1).astype(np.int64) // 64 * 64
        bounds[-1] = a.nbytes
        with ThreadPoolExecutor(nthreads) as ex:
            list(ex.map(lambda k: np.copyto(dst[bounds[k]: bounds[k + 1]], src[bounds[k]: bounds[k + 1]]),
                        range(nthreads)))
    else:
        np.copyto(dst.view(a.dtype).reshape(a.shape), a, casting="no")
    return out[: a.nbytes]


class NdarrayFileData(_Data):
    def __init__(self, file: str, elem: FileMetaData):
        self.file = file
        self.shape = elem.shape if elem else None
        self.dtype = elem.dtype if elem else None
        self.time_in_sec = self.timeInSec = 0.0
        self.size_in_byte = self.sizeInByte = 0

    def _array(self):
        return np.load(self.file, mmap_mode="r")


class BinaryFileData(_Data):
    def __init__(self, file: str, elem: FileMetaData):
        self.file = file
        self.shape = elem.shape
        self.dtype = elem.dtype
        self.time_in_sec = self.timeInSec = 0.0
        self.size_in_byte = self.sizeInByte = 0

    def _array(self):
        return np.memmap(self.file, dtype=self.dtype, mode="r", shape=tuple(self.shape))


class NdarrayTimeslicesFileData(_Data):
    """One ``.npy`` file per source timeslice (``ndarray.py:54-90``): the file
    name holds ``.t???.``, which the first index of every key replaces with
    ``.t{t:03d}.``; the remaining indices select within that file."""

    def __init__(self, file: str, elem: FileMetaData):
        self.file = file
        self.shape = elem.shape if elem else None
        self.dtype = elem.dtype if elem else None
        self.time_in_sec = self.timeInSec = 0.0
        self.size_in_byte = self.sizeInByte = 0

    def source_file(self, t: int) -> str:
        return re.sub(r"\.t\?\?\?\.", f".t{int(t):03d}.", self.file)

    def _view(self, key):
        head, rest = (key[0], tuple(key[1:])) if isinstance(key, tuple) else (key, ())
        if not isinstance(head, (int, np.integer)):
            raise TypeError("the first index selects the per-source file and must be an integer")
        return np.load(self.source_file(head), mmap_mode="r")[rest]

    def links_to_device(self, latt_size, device=None):
        return None  # per-source perambulator files, not a gauge field


def read_lime_records(path: str) -> Dict[str, Tuple[int, int]]:
    """type -> (payload offset, padded length) of every LIME record."""
    out = {}
    with open(path, "rb") as f:
        while True:
            head = f.read(8)
            if head == b"" or head == b"\x0A":
                break
            if not head.startswith(b"\x45\x67\x89\xAB\x00\x01"):
                raise ValueError(f"{path}: not a LIME record at offset {f.tell() - 8}")
            length = (struct.unpack(">Q", f.read(8))[0] + 7) // 8 * 8
            rtype = f.read(128).strip(b"\x00").decode("utf-8")
            out[rtype] = (f.tell(), length)
            f.seek(length, 1)
    return out


class IldgFileData(_Data):
    def __init__(self, file: str, elem: FileMetaData):
        self.file = file
        self.shape = elem.shape
        self.dtype = elem.dtype
        recs = read_lime_records(file)
        self.offset, nbytes = recs["ildg-binary-data"]
        fpos, flen = recs["ildg-format"]
        with open(file, "rb") as f:
            f.seek(fpos)
            root = ET.fromstring(f.read(flen).strip(b"\x00").decode("utf-8"))
        tag = re.match(r"\{.*\}", root.tag).group(0) if root.tag.startswith("{") else ""
        self.latt_size = [int(root.find(f"{tag}{k}").text) for k in ("lx", "ly", "lz", "lt")]
        self.bytes = int(re.match(r"^[<>=]?[iufc](?P<bytes>\d+)$", elem.dtype).group("bytes"))
        if self.bytes != int(root.find(f"{tag}precision").text) // 8 * 2:
            raise ValueError("ILDG precision does not match the preset dtype")
        if int(np.prod(self.shape)) * self.bytes != nbytes:
            raise ValueError("ILDG payload size does not match the preset shape")
        self.time_in_sec = self.timeInSec = 0.0
        self.size_in_byte = self.sizeInByte = 0

    def _array(self):
        return np.memmap(self.file, dtype=self.dtype, mode="r", offset=self.offset, shape=tuple(self.shape))

    _target = "<c16"

    def _convert(self, a):
        return a.astype("<c16")


class QDPLazyDiskMapObjFileData(_Data):
    def __init__(self, file: str, elem: FileMetaData):
        self.file = file
        self.extra = elem.extra
        self.shape = elem.shape[elem.extra :]
        self.dtype = elem.dtype
        self.extraShape = elem.shape[: elem.extra]
        with open(file, "rb") as f:
            def rstr():
                n = struct.unpack(">i", f.read(4))[0]
                return f.read(n).decode("utf-8")

            if rstr() != "XXXXQDPLazyDiskMapObjFileXXXX":
                raise ValueError(f"{file}: not a QDP LazyDiskMapObjFile")
            struct.unpack(">i", f.read(4))
            ET.fromstring(rstr())
            f.seek(struct.unpack(">qq", f.read(16))[1])
            nrec = struct.unpack(">I", f.read(4))[0]
            self.offsets = {}
            for _ in range(nrec):
                n = struct.unpack(">i", f.read(4))[0] // 4
                key = struct.unpack(">" + "i" * n, f.read(4 * n))
                self.offsets[key] = struct.unpack(">qq", f.read(16))[1]
        self.time_in_sec = self.timeInSec = 0.0
        self.size_in_byte = self.sizeInByte = 0

    _target = "<c8"

    def _convert(self, a):
        return a.astype("<c8")

    def links_to_device(self, latt_size, device=None):
        return None  # records are keyed by (t, mu), not in the ILDG site order

    def _view(self, key):
        if isinstance(key, int):
            key = (key,)
        head = tuple(key[: self.extra])
        if head not in self.offsets:
            raise IndexError(f"index {key} is out of bounds for axes")
        arr = np.memmap(self.file, dtype=self.dtype, mode="r", offset=self.offsets[head], shape=tuple(self.shape))
        return arr[tuple(key[self.extra :])]


class GaugeField:
    """Base of the gauge-field presets (``lattice/preset.py:11-13``)."""

    def __init__(self, elem: FileMetaData) -> None:
        self.elem = deepcopy(elem)


class Eigenvector:
    """Base of the eigenvector presets (``lattice/preset.py:16-19``)."""

    def __init__(self, elem: FileMetaData, eigenNum: int) -> None:
        self.elem = deepcopy(elem)
        self.Ne = eigenNum


class Elemental:
    """Base of the elemental presets (``lattice/preset.py:22-25``)."""

    def __init__(self, elem: FileMetaData, eigenNum: int) -> None:
        self.elem = deepcopy(elem)
        self.Ne = eigenNum


class Perambulator:
    """Base of the perambulator presets (``lattice/preset.py:28-31``)."""

    def __init__(self, elem: FileMetaData, eigenNum: int) -> None:
        self.elem = deepcopy(elem)
        self.Ne = eigenNum


class OnePoint:
    """Base of the one-point data presets (``lattice/preset.py:34-36``)."""

    def __init__(self, elem: FileMetaData) -> None:
        self.elem = deepcopy(elem)


class TwoPoint:
    """Base of the two-point data presets (``lattice/preset.py:39-41``)."""

    def __init__(self, elem: FileMetaData) -> None:
        self.elem = deepcopy(elem)


class _Preset:
    _data_cls = None

    def __init__(self, prefix, suffix, elem):
        self.prefix, self.suffix, self.elem = prefix, suffix, elem
        self._file, self.data = None, None

    def load(self, key: str):
        name = f"{self.prefix}{key}{self.suffix}"
        if self._file != name:
            self._file = name
            self.data = self._data_cls(name, self.elem)
        return self.data


class GaugeFieldIldg(_Preset, GaugeField):
    _data_cls = IldgFileData

    def __init__(self, prefix: str, suffix: str, shape=[128, 16**3, 4, 3, 3]):
        super().__init__(prefix, ".lime" if suffix is None else suffix, FileMetaData(shape, ">c16", 0))


class GaugeFieldBinary(_Preset, GaugeField):
    _data_cls = BinaryFileData

    def __init__(self, prefix: str, suffix: str, shape=[128, 16**3, 4, 3, 3], dtype: str = "<f8"):
        super().__init__(prefix, ".dat" if suffix is None else suffix, FileMetaData(shape, dtype, 0))


class GaugeFieldTimeSlice(_Preset, GaugeField):
    _data_cls = QDPLazyDiskMapObjFileData

    def __init__(self, prefix: str, suffix: str, shape=[128, 4, 16**3, 3, 3]):
        super().__init__(prefix, ".stout.n20.f0.12.mod" if suffix is None else suffix, FileMetaData(shape, ">c16", 2))


class EigenvectorNpy(_Preset, Eigenvector):
    _data_cls = NdarrayFileData

    def __init__(self, prefix: str, suffix: str, shape=[70, 128, 16**3, 3], totNe: int = 70):
        super().__init__(prefix, ".lime.npy" if suffix is None else suffix, FileMetaData(shape, "<c16", 2))
        self.Ne = totNe


class EigenvectorTimeSlice(_Preset, Eigenvector):
    _data_cls = QDPLazyDiskMapObjFileData

    def __init__(self, prefix: str, suffix: str, shape=[128, 70, 16**3, 3], totNe: int = 70):
        super().__init__(prefix, ".stout.n20.f0.12.laplace_eigs.3d.mod" if suffix is None else suffix,
                         FileMetaData(shape, ">c8", 2))
        self.Ne = totNe


class EigenvectorHostmem(Eigenvector):
    """Eigenvectors already in host memory (``lattice/preset.py:77-89``)."""

    def __init__(self, host_ndarray, shape=[70, 128, 16**3, 3], totNe: int = 70):
        if list(host_ndarray.shape) != list(shape):
            raise ValueError(
                f"Please check that host_ndarray shape {host_ndarray.shape} does not match expected shape "
                f"(totNe, Lt, Lz * Ly * Lx, Nc) = {shape}"
            )
        self.Ne = totNe
        self.data = host_ndarray

    def load(self, key: str = None):
        return self.data


class ElementalNpy(_Preset, Elemental):
    _data_cls = NdarrayFileData

    def __init__(self, prefix: str, suffix: str, shape=[4, 123, 128, 70, 70], totNe: int = 70):
        super().__init__(prefix, ".stout.n20.f0.12.nev70.meson.npy" if suffix is None else suffix,
                         FileMetaData(shape, "<c8", 0))
        self.Ne = totNe


class ElementalBinary(_Preset, Elemental):
    _data_cls = BinaryFileData

    def __init__(self, prefix: str, suffix: str, shape=[40, 27, 128, 70, 70], totNe: int = 70):
        super().__init__(prefix, ".stout.n20.f0.12.nev70.meson" if suffix is None else suffix,
                         FileMetaData(shape, "<c16", 0))
        self.Ne = totNe


class PerambulatorNpy(_Preset, Perambulator):
    _data_cls = NdarrayFileData

    def __init__(self, prefix: str, suffix: str, shape=[128, 128, 4, 4, 70, 70], totNe: int = 70):
        super().__init__(prefix, ".stout.n20.f0.12.nev70.peram" if suffix is None else suffix,
                         FileMetaData(shape, "<c8", 0))
        self.Ne = totNe


class PerambulatorBinary(_Preset, Perambulator):
    _data_cls = BinaryFileData

    def __init__(self, prefix: str, suffix: str, shape=[128, 128, 4, 4, 70, 70], totNe: int = 70):
        super().__init__(prefix, ".stout.n20.f0.12.nev70.peram" if suffix is None else suffix,
                         FileMetaData(shape, "<c16", 0))
        self.Ne = totNe


class PerambulatorTimeslicesNpy(_Preset, Perambulator):
    """Perambulators saved one source timeslice per ``.npy`` file
    (``lattice/preset.py:114-126``): ``prefix + key + suffix`` names the files
    with ``.t???.`` in place of the source index; ``[t_src, ...]`` reads
    ``.t{t_src:03d}.``."""

    _data_cls = NdarrayTimeslicesFileData

    def __init__(self, prefix: str, suffix: str, shape=[128, 128, 4, 4, 70, 70], totNe: int = 70):
        super().__init__(prefix, ".stout.n20.f0.12.nev70.peram" if suffix is None else suffix,
                         FileMetaData(shape, "<c8", 0))
        self.Ne = totNe


class Jpsi2gammaBinary(_Preset, TwoPoint):
    """Raw float64 two-point data (``lattice/preset.py:140-148``)."""

    _data_cls = BinaryFileData

    def __init__(self, prefix: str, suffix: str, shape=[128, 2, 3, 4, 27, 128]):
        super().__init__(prefix, ".mesonspec.2pt.bin" if suffix is None else suffix, FileMetaData(shape, "<f8", 0))


class Jpsi2gammaNpy(_Preset, TwoPoint):
    """Two-point data in ``.npy`` files (``lattice/preset.py:184-192``).  The
    reference's class passes no metadata, and its ``.npy`` reader then fails
    on ``load`` (``ndarray.py:12`` reads ``elem.shape``); here the file's own
    header gives shape and dtype."""

    _data_cls = NdarrayFileData

    def __init__(self, prefix: str, suffix: str):
        super().__init__(prefix, ".2pt.npy" if suffix is None else suffix, None)


class OnePointNpy(_Preset, OnePoint):
    """One-point data in ``.npy`` files (``lattice/preset.py:195-204``); as
    for :class:`Jpsi2gammaNpy`, shape and dtype come from the file header."""

    _data_cls = NdarrayFileData

    def __init__(self, prefix: str, suffix: str):
        super().__init__(prefix, ".1pt.npy" if suffix is None else suffix, None)


def write_ildg(path: str, gauge: np.ndarray, latt_size: List[int]):
    """Write a field ``[Lt, Lz, Ly, Lx, 4, 3, 3]`` as an ILDG/LIME file
    (``ildg-format`` XML record + big-endian complex128 ``ildg-binary-data``)."""
    Lx, Ly, Lz, Lt = latt_size
    xml = (
        '<?xml version="1.0" encoding="UTF-8"?><ildgFormat xmlns="http://www.lqcd.org/ildg">'
        f"<version>1.0</version><field>su3gauge</field><precision>64</precision>"
        f"<lx>{Lx}</lx><ly>{Ly}</ly><lz>{Lz}</lz><lt>{Lt}</lt></ildgFormat>"
    ).encode()
    payload = np.ascontiguousarray(gauge).astype(">c16").tobytes()

    def record(rtype: str, data: bytes, first: bool, last: bool) -> bytes:
        flags = (0x8000 if first else 0) | (0x4000 if last else 0)
        head = b"\x45\x67\x89\xab" + struct.pack(">H", 1) + struct.pack(">H", flags)
        head += struct.pack(">Q", len(data)) + rtype.encode().ljust(128, b"\x00")
        pad = (-len(data)) % 8
        return head + data + b"\x00" * pad

    with open(path, "wb") as f:
        f.write(record("ildg-format", xml, True, False))
        f.write(record("ildg-binary-data", payload, False, True))
