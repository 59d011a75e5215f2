"""GB300 drop-in for ``lattice.generator.ElementalGenerator``.

Same constructor, ``load(key)`` and ``calc(t)`` as the reference
(``lattice/generator/elemental.py:17-105,290-338``); the contraction runs in
the library's CUDA kernels (covariant-derivative chains, pair contractions,
operator combination).  ``calc`` returns the generator's internal
``[Nderiv, Nmom, Ne, Ne]`` complex128 device buffer, which the next call
overwrites, exactly like the reference's ``self._VPV``; after
``easydistillation_gb300.set_backend("numpy")`` it returns a host numpy copy
of it instead (the reference's numpy backend).

Extra keyword-only arguments: ``precision``, ``device``, ``factorise`` and
``autotune``.
``"fp64"`` is plain FP64 arithmetic with V rounded to complex64, as the
reference; ``"df64"`` computes the same pair contractions in double-float
arithmetic on the FP32 pipe (each complex128 operand as two complex64 parts,
~1e-14 relative), several times faster than this part's FP64 pipe.  The tensor-core modes ``"f16x3"``, ``"tf32x3"`` (relative error
~1e-7) and ``"bf16x3"`` (~1e-5) store the derivative chains in complex64 and
run the pair contractions as split-precision tcgen05 GEMMs with FP32
accumulation; they need ``Lx*Ly*Lz`` divisible by 32.  When the momentum list
is a product set {(px, py)} x {pz} (e.g. all 27 momenta with |p|^2 <= 3),
those GEMMs use the factorised phase exp(2 pi i p.x / L) = f(px, py) g(pz)
with both operands prepared in HBM; ``factorise=False`` keeps the kernel
that forms the phase-weighted operand on chip, ``factorise="force"``
factorises however many (px, py) x pz combinations go unused, and
``factorise="left"`` puts every momentum's whole phase on the left operand
(any short momentum list, none of the GEMM's work unused).
``autotune=True`` replaces ``factorise``: each plan (one per batch size) takes
the GEMM form and launch settings that the autotuner
(``easydistillation_gb300.tune``) measured fastest for its shape on this
device, cached per device and shape.
"""

from __future__ import annotations

from typing import List, Tuple

import numpy as np
import torch

from ..backend import to_backend
from ..insertion import MomentumPhase, derivative, num_derivative
from ..ops import ElementalPlan

ND = 4
NC = 3


def _blending_coeff(Ne: int, dilution) -> np.ndarray:
    """Stochastic blending coefficients, as ``elemental.py:61-95``."""
    totNe_list = dilution[0]
    if isinstance(dilution[1], int):
        usedNe_list = [dilution[1]] * len(dilution[0])
    else:
        usedNe_list = list(dilution[1])
    assert len(usedNe_list) == len(totNe_list)
    assert (np.array(usedNe_list) <= np.array(totNe_list)).all()
    assert sum(usedNe_list) == Ne
    coeff = np.zeros((Ne, Ne))
    start1 = 0
    for nv1 in range(len(usedNe_list)):
        used1, tot1 = usedNe_list[nv1], totNe_list[nv1]
        start2 = 0
        for nv2 in range(len(usedNe_list)):
            used2, tot2 = usedNe_list[nv2], totNe_list[nv2]
            if nv1 != nv2:
                coeff[start1 : start1 + used1, start2 : start2 + used2] = tot1 * tot2 / used1 / used2
            else:
                c1 = tot1 / used1
                c2 = c1 * (tot1 - 1) / (used1 - 1)
                block = np.full((used1, used2), c2)
                np.fill_diagonal(block, c1)
                coeff[start1 : start1 + used1, start2 : start2 + used2] = block
            start2 += used2
        start1 += used1
    return coeff


def _host_array(x) -> np.ndarray:
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy()
    if hasattr(x, "get") and not isinstance(x, np.ndarray):  # cupy arrays
        return x.get()
    return np.asarray(x)


def links_to_device(gauge_data, latt_size, device) -> torch.Tensor:
    """Load ``gauge_field.load(key)[:]`` (ILDG order ``[Lt, Lz, Ly, Lx, Nd, 3, 3]``)
    and return the spatial links in the generators' transposed layout
    ``[3, Lt, Lz, Ly, Lx, 3, 3]`` complex128 on the device
    (``elemental.py:103``, ``eigenvector.py:50``)."""
    Lx, Ly, Lz, Lt = latt_size
    if isinstance(gauge_data, torch.Tensor):
        U = gauge_data.to(device=device, dtype=torch.complex128)
    else:
        arr = np.ascontiguousarray(_host_array(gauge_data)).astype(np.complex128, copy=False)
        U = torch.from_numpy(arr).pin_memory().to(device, non_blocking=True)
    U = U.reshape(Lt, Lz, Ly, Lx, -1, NC, NC)
    return U.permute(4, 0, 1, 2, 3, 5, 6)[: ND - 1].contiguous()


def gauge_to_device(gauge_file_data, latt_size, device) -> torch.Tensor:
    """Spatial links ``[3, Lt, Lz, Ly, Lx, 3, 3]`` complex128 on the device
    from ``gauge_field.load(key)``.  A reader of this package that offers
    ``links_to_device`` (ILDG, npy, raw binary with complex values) uploads
    the stored bytes and converts and transposes them on the device; any other
    object is read with ``[:]`` (the reference's ``elemental.py:103``) and
    goes through :func:`links_to_device`."""
    if hasattr(gauge_file_data, "links_to_device"):
        U = gauge_file_data.links_to_device(latt_size, device)
        if U is not None:
            return U
    return links_to_device(gauge_file_data[:], latt_size, device)


def admit_batch(latt_size, Ne, num_nabla, momentum_list, precision="fp64", device=None, max_batch=8,
                reserve=0.1, factorise: bool = True) -> int:
    """Largest batch of timeslices whose plan workspace fits the free HBM of
    ``device`` (keeping a ``reserve`` fraction free), between 1 and ``max_batch``."""
    device = torch.device(device or "cuda")
    free, _total = torch.cuda.mem_get_info(device)
    budget = free * (1.0 - reserve)
    best = 1
    for b in range(1, max_batch + 1):
        need = ElementalPlan(latt_size, Ne, num_nabla, momentum_list, precision, device, batch=b,
                             factorise=factorise).workspace_bytes
        if need <= budget:
            best = b
        else:
            break
    return best


class ElementalGenerator:
    def __init__(
        self,
        latt_size: List[int],
        gauge_field,
        eigenvector,
        num_nabla: int = 0,
        momentum_list: List[Tuple[int]] = [(0, 0, 0)],
        dilution: Tuple = None,
        is_blending: bool = False,
        *,
        precision: str = "fp64",
        device=None,
        factorise=True,
        autotune: bool = False,
    ) -> None:
        Lx, Ly, Lz, Lt = latt_size
        self.device = torch.device(device or "cuda")
        self.latt_size = latt_size
        self.gauge_field = gauge_field
        self.eigenvector = eigenvector
        self.num_derivative = num_derivative(num_nabla)
        self.derivative_list = [derivative(n) for n in range(self.num_derivative)]
        self.num_momentum = len(momentum_list)
        self.momentum_list = momentum_list
        Ne = eigenvector.Ne
        self.Ne = Ne
        self.precision = precision
        self.factorise = factorise
        self.autotune = autotune
        self._U = None
        self._VPV = torch.zeros((self.num_derivative, self.num_momentum, Ne, Ne), dtype=torch.complex128,
                                device=self.device)
        self._eigenvector_data = None
        self._momentum_phase = MomentumPhase(latt_size, self.device)
        self._num_nabla = num_nabla
        self._plan = self._make_plan(1)
        self._stage = None

        if is_blending and (dilution is not None):
            self.stocastic_coeff = torch.from_numpy(_blending_coeff(Ne, dilution)).to(self.device)
        elif is_blending:
            raise ValueError("Dilution tuple is not defined.")
        else:
            self.stocastic_coeff = None

    def _make_plan(self, batch: int) -> ElementalPlan:
        """The plan for ``batch`` timeslices per run: built as ``factorise``
        says, or, with ``autotune``, in the form and with the launch settings
        the autotuner measured fastest for this shape (cached per device)."""
        if self.autotune:
            from ..tune import tuned_plan

            return tuned_plan(self.latt_size, self.Ne, self._num_nabla, self.momentum_list, self.precision,
                              self.device, batch=batch)
        return ElementalPlan(self.latt_size, self.Ne, self._num_nabla, self.momentum_list, self.precision,
                             self.device, batch=batch, factorise=self.factorise)

    def load(self, key: str):
        self._U = gauge_to_device(self.gauge_field.load(key), self.latt_size, self.device)
        self._eigenvector_data = self.eigenvector.load(key)

    def _read_vectors(self, t: int) -> torch.Tensor:
        """``V[e] = eigenvector[t, e]`` for e < Ne (``elemental.py:297-298``),
        staged through pinned host memory into a device buffer."""
        Lx, Ly, Lz, Lt = self.latt_size
        Ne = self.Ne
        data = self._eigenvector_data
        if isinstance(data, torch.Tensor):
            return data[t, :Ne].reshape(Ne, Lz * Ly * Lx * NC).to(self.device).contiguous()
        if hasattr(data, "raw"):
            dev = self._read_vectors_raw(t, data)
            if dev is not None:
                return dev
        if self._stage is None:
            self._stage = torch.empty((Ne, Lz * Ly * Lx * NC), dtype=torch.complex128).pin_memory()
        # the previous host->device copy out of the pinned stage must finish before it is refilled
        if getattr(self, "_stage_event", None) is not None:
            self._stage_event.synchronize()
        stage = self._stage.numpy()
        block = None
        try:
            block = _host_array(data[t, 0:Ne])
            if block.shape[0] != Ne or block.size != stage.size:
                block = None
        except Exception:
            block = None
        if block is not None:
            stage[...] = block.reshape(stage.shape)
        else:
            for e in range(Ne):
                stage[e] = _host_array(data[t, e]).reshape(-1)
        dev = self._stage.to(self.device, non_blocking=True)
        if getattr(self, "_stage_event", None) is None:
            self._stage_event = torch.cuda.Event()
        self._stage_event.record()
        return dev

    def _read_vectors_raw(self, t: int, data) -> torch.Tensor:
        """``eigenvector[t, 0:Ne]`` from a reader of this package: the stored
        bytes (one memory-mapped block, or one record per e for keyed files
        such as QDP lazy-disk maps) are copied into a pinned byte stage,
        uploaded in one copy and converted to complex128 on the device
        (``ops.decode_complex``).  None when the stored values are not
        complex numbers, so the caller converts on the host."""
        from .. import ops
        from ..preset import pinned_bytes

        Lx, Ly, Lz, Lt = self.latt_size
        Ne, n = self.Ne, Lz * Ly * Lx * NC
        views = None
        try:
            v = data.raw((t, slice(0, Ne)), copy=False)
            if np.size(v) == Ne * n:
                views = [v]
        except (IndexError, TypeError, ValueError, KeyError):
            views = None
        if views is None:
            views = [data.raw((t, e), copy=False) for e in range(Ne)]
            if sum(np.size(v) for v in views) != Ne * n:
                raise ValueError(f"eigenvector data of timeslice {t} do not hold {Ne} vectors of {n} components")
        dt = np.dtype(views[0].dtype)
        if dt.kind != "c" or any(np.dtype(v.dtype) != dt for v in views):
            return None
        nbytes = Ne * n * dt.itemsize
        if getattr(self, "_raw_stage", None) is None or self._raw_stage.numel() < nbytes:
            self._raw_stage = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        # the previous host->device copy out of the pinned stage must finish before it is refilled
        if getattr(self, "_stage_event", None) is not None:
            self._stage_event.synchronize()
        off = 0
        for v in views:
            pinned_bytes(v, self._raw_stage[off:])
            off += v.nbytes
        raw = self._raw_stage[:nbytes].to(self.device, non_blocking=True)
        if getattr(self, "_stage_event", None) is None:
            self._stage_event = torch.cuda.Event()
        self._stage_event.record()
        return ops.decode_complex(raw, dt, torch.complex128).reshape(Ne, n)

    def _fetch_chunk(self, chunk, slot, stream):
        """Eigenvectors of the timeslices in ``chunk`` into the device input
        buffers of ``slot``: direct asynchronous copies on ``stream`` when the
        eigenvector data is a (pinned) torch tensor, else through the pinned
        stage (:meth:`_read_vectors`)."""
        Lx, Ly, Lz, Lt = self.latt_size
        Ne, n = self.Ne, Lx * Ly * Lz * NC
        data = self._eigenvector_data
        bufs = self._in_bufs[slot]
        with torch.cuda.stream(stream):
            for k, t in enumerate(chunk):
                if isinstance(data, torch.Tensor):
                    bufs[k].copy_(data[t, :Ne].reshape(Ne, n), non_blocking=True)
                else:
                    bufs[k].copy_(self._read_vectors(t))
        return bufs[: len(chunk)]

    def calc_batch(self, ts, out: torch.Tensor = None, batch: int = None):
        """Elementals of several timeslices, ``[len(ts), Nderiv, Nmom, Ne, Ne]``.

        Timeslices go through batched plans of up to ``batch`` timeslices
        (default: as many as :func:`admit_batch` allows in free HBM, at most
        8), one pair-contraction launch per batch.  The batches are pipelined:
        the eigenvectors of batch k+1 are copied to the device on one stream
        and, when ``out`` is a host tensor (pinned for asynchronous copies),
        the elementals of batch k-1 are copied back on another while batch k
        computes."""
        if self._U is None:
            raise RuntimeError("call load(key) before calc_batch(ts)")
        Lx, Ly, Lz, Lt = self.latt_size
        V3 = Lx * Ly * Lz
        ts = list(ts)
        shape = (self.num_derivative, self.num_momentum, self.Ne, self.Ne)
        if out is None:
            out = torch.empty((len(ts),) + shape, dtype=torch.complex128, device=self.device)
        host_out = out.device.type == "cpu"
        if batch is None:
            # with autotune the GEMM form is chosen per batch size: admit what every form fits
            forms = (True, False, "force", "left") if self.autotune else (self.factorise,)
            batch = min(admit_batch(self.latt_size, self.Ne, self._num_nabla, self.momentum_list, self.precision,
                                    self.device, max_batch=min(8, len(ts)), factorise=f) for f in forms)
        plan = getattr(self, "_bplan", None)
        if plan is None or plan.batch != batch:
            plan = self._bplan = self._make_plan(batch)
        evdt = self._eigenvector_data.dtype if isinstance(self._eigenvector_data, torch.Tensor) else torch.complex128
        if getattr(self, "_in_bufs", None) is None or len(self._in_bufs[0]) != batch or \
                self._in_bufs[0][0].dtype != evdt:
            self._in_bufs = [[torch.empty((self.Ne, V3 * NC), dtype=evdt, device=self.device) for _ in range(batch)]
                             for _ in range(2)]
            self._streams = (torch.cuda.Stream(self.device), torch.cuda.Stream(self.device))
        if host_out and (getattr(self, "_out_bufs", None) is None or self._out_bufs[0].shape[0] != batch):
            self._out_bufs = [torch.empty((batch,) + shape, dtype=torch.complex128, device=self.device)
                              for _ in range(2)]
        h2d, d2h = self._streams
        compute = torch.cuda.current_stream(self.device)
        chunks = [ts[s0 : s0 + batch] for s0 in range(0, len(ts), batch)]
        in_ready = [torch.cuda.Event(), torch.cuda.Event()]
        in_free = [None, None]   # compute finished reading the input slot
        out_free = [None, None]  # the host copy of an output slot finished
        h2d.wait_stream(compute)  # links and earlier work on the compute stream come first
        vecs = self._fetch_chunk(chunks[0], 0, h2d)
        in_ready[0].record(h2d)
        for k, chunk in enumerate(chunks):
            slot = k % 2
            if k + 1 < len(chunks):  # prefetch the next batch into the other slot
                nslot = 1 - slot
                if in_free[nslot] is not None:
                    h2d.wait_event(in_free[nslot])
                nvecs = self._fetch_chunk(chunks[k + 1], nslot, h2d)
                in_ready[nslot].record(h2d)
            compute.wait_event(in_ready[slot])
            if host_out:
                if out_free[slot] is not None:
                    compute.wait_event(out_free[slot])
                outs = [self._out_bufs[slot][j] for j in range(len(chunk))]
            else:
                s0 = k * batch
                outs = [out[s0 + j] for j in range(len(chunk))]
            links = [self._U[:, t] for t in chunk]
            plan.run_batch(links, Lt * V3 * 9, 9, vecs, outs, blend=self.stocastic_coeff)
            ev = torch.cuda.Event()
            ev.record(compute)
            in_free[slot] = ev
            if host_out:
                d2h.wait_event(ev)
                with torch.cuda.stream(d2h):
                    out[k * batch : k * batch + len(chunk)].copy_(self._out_bufs[slot][: len(chunk)],
                                                                  non_blocking=True)
                e2 = torch.cuda.Event()
                e2.record(d2h)
                out_free[slot] = e2
            if k + 1 < len(chunks):
                vecs = nvecs
        compute.wait_stream(h2d)
        compute.wait_stream(d2h)
        if self.precision != "fp64":
            plan.check_status()  # synchronises the compute stream
        elif host_out:
            compute.synchronize()
        return out

    def calc(self, t: int):
        if self._U is None:
            raise RuntimeError("call load(key) before calc(t)")
        Lx, Ly, Lz, Lt = self.latt_size
        V3 = Lx * Ly * Lz
        V = self._read_vectors(t)
        links_t = self._U[:, t]
        self._plan.run(links_t, dir_stride=Lt * V3 * 9, site_stride=9, evecs=V, out=self._VPV,
                       blend=self.stocastic_coeff)
        if self.precision != "fp64":
            self._plan.check_status()
        return to_backend(self._VPV)

    def project_SU3(self):
        """Iterative projection back onto SU(3) (``elemental.py:107-118``)."""
        from .eigenvector import project_su3_

        project_su3_(self._U)

    def stout_smear(self, nstep: int, rho: float):
        from .eigenvector import stout_smear_links_

        stout_smear_links_(self._U, self.latt_size, nstep, rho)
