"""Autotuner for the launch settings of elemental plans and of the Laplacian.

The reference has nothing to tune (its contractions are opt_einsum/BLAS
calls, ``lattice/generator/elemental.py:324-329``); here the kernels expose
choices whose best value depends on the shape:

* whether a tensor-core plan uses the factorised-phase GEMM (both operands
  prepared in HBM, all ``(px,py) x pz`` combinations computed, the unused ones
  wasted) or the GEMM that forms the phase-weighted operand on chip (exactly
  the requested momenta, slower per product);
* the K-slab length of the persistent factorised GEMM's lock-step schedule
  (shorter slabs keep the CTAs closer together in K, for L2 reuse of the
  operand rows, at the cost of more result flushes), its number of operand
  stages, whether it runs on single SMs (128 x 128 tiles) or on SM pairs
  (two-CTA clusters, 256 x 128 tiles), and how many k-blocks it accumulates
  in one TMEM buffer (1, or 2: half the buffer hand-overs, a larger FP32
  accumulation error, gated by the tolerance below);
* the tile shape of the FP64 pair GEMM (an Ne that is not a multiple of 64
  wastes part of every 64-row tile);
* the complex64 Laplacian kernel: neighbours read through L1/L2, or input
  planes staged by TMA.

Candidates are timed on the device with CUDA events, on seeded synthetic
inputs of the requested shape (the kernels' speed does not depend on the
values), after a warm-up run.  A candidate whose output differs from the
default settings' output by more than the mode's tolerance is rejected.  The
winners are cached in a JSON file per device, library version and shape
(``$ED_TUNE_CACHE``, else ``~/.cache/easydist_gb300/tuning.json``).
"""

from __future__ import annotations

import json
import os
import tempfile
import threading
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import torch

from . import _lib
from .insertion import num_derivative
from .ops import F64_TILES, MODES, ElementalPlan

# the FP64 mode and its double-float form: the same plans, tiles and tolerance
F64_MODES = ("fp64", "df64")

#: relative Frobenius tolerance of a candidate against the default settings, per mode
TOLERANCE = {"fp64": 1e-12, "df64": 1e-12, "f16x3": 1e-6, "tf32x3": 1e-6, "bf16x3": 1e-5, "ozaki_i8": 1e-6}
#: lock-step slab lengths (k-blocks) of the factorised GEMM: the default first, then the candidates
SLABS = (256, 128, 64)

_cache_lock = threading.Lock()


def cache_path() -> str:
    p = os.environ.get("ED_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "easydist_gb300", "tuning.json")


def device_key(device=None) -> str:
    """Device name, compute capability, SM count and library version: tuned
    settings are valid for exactly this combination."""
    device = torch.device(device or "cuda")
    props = torch.cuda.get_device_properties(device)
    return f"{props.name}|sm_{props.major}{props.minor}|{props.multi_processor_count}sm|lib{_lib.lib().ed_version()}"


def elemental_key(latt_size, Ne, num_nabla, momentum_list, mode, batch, evec_dtype=torch.complex128) -> str:
    Lx, Ly, Lz = (int(v) for v in latt_size[:3])
    moms = ";".join(",".join(str(int(v)) for v in p) for p in momentum_list)
    ev = "c64" if evec_dtype == torch.complex64 else "c128"
    return f"elemental|{Lx}x{Ly}x{Lz}|Ne{int(Ne)}|nabla{int(num_nabla)}|{mode}|b{int(batch)}|{ev}|{moms}"


def laplacian_key(latt_size, nt, nvec) -> str:
    Lx, Ly, Lz = (int(v) for v in latt_size[:3])
    return f"laplacian|{Lx}x{Ly}x{Lz}|nt{int(nt)}|nvec{int(nvec)}|c64"


class TuningCache:
    """JSON file ``{device_key: {shape_key: entry}}``; writes are atomic."""

    def __init__(self, path: Optional[str] = None):
        self.path = path or cache_path()

    def _load(self) -> dict:
        try:
            with open(self.path) as f:
                data = json.load(f)
            return data if isinstance(data, dict) else {}
        except (OSError, ValueError):
            return {}

    def get(self, dev: str, key: str) -> Optional[dict]:
        with _cache_lock:
            return self._load().get(dev, {}).get(key)

    def put(self, dev: str, key: str, entry: dict) -> None:
        with _cache_lock:
            data = self._load()
            data.setdefault(dev, {})[key] = entry
            d = os.path.dirname(os.path.abspath(self.path))
            os.makedirs(d, exist_ok=True)
            fd, tmp = tempfile.mkstemp(dir=d, prefix=".tuning.", suffix=".json")
            with os.fdopen(fd, "w") as f:
                json.dump(data, f, indent=1, sort_keys=True)
            os.replace(tmp, self.path)


@dataclass
class Candidate:
    """One point of the search: how the plan is built (``factorise``) and its
    launch settings (``tuning``, ED_TUNE_* names)."""

    factorise: object = True
    tuning: Dict[str, int] = field(default_factory=dict)

    def as_dict(self) -> dict:
        return {"factorise": self.factorise, "tuning": dict(self.tuning)}

    @staticmethod
    def from_dict(d: dict) -> "Candidate":
        return Candidate(d.get("factorise", True), dict(d.get("tuning", {})))


@dataclass
class TuneResult:
    best: Candidate
    ms: float
    trials: List[dict]  # every candidate tried: settings, ms (None if rejected), error vs default
    cached: bool = False


# momentum lists up to this length also try the factorisation with every phase on the left operand
LEFT_FACTOR_MAX_MOM = 16


def factorise_options(latt_size, Ne, num_nabla, momentum_list, mode) -> List[object]:
    """The distinct GEMM forms a tensor-core plan can take for this momentum
    list: ``True`` (factorised when at most a quarter of the combinations go
    unused, else on chip), ``"force"`` when it differs from ``True``,
    ``"left"`` (every phase on the left operand) for lists that are not close
    to a product set and have at most ``LEFT_FACTOR_MAX_MOM`` momenta (its
    left operand grows with the momentum count), and ``False`` (on chip) when
    ``True`` factorises.  Host-side plans only."""
    if mode in F64_MODES:
        return [True]
    if mode == "ozaki_i8":
        return [True]  # runs on factorised operands only

    def fac(f):
        try:
            return ElementalPlan(latt_size, Ne, num_nabla, momentum_list, mode, device="cpu", factorise=f).factorised
        except Exception:
            return None

    opts: List[object] = [True]
    default = fac(True)
    if default is None:
        if fac("force") is not None:
            opts.append("force")
        if len(momentum_list) <= LEFT_FACTOR_MAX_MOM and fac("left") is not None:
            opts.append("left")
    else:
        opts.append(False)
    return opts


def _run_search(stages: Sequence[Callable[[Candidate], List[Candidate]]], start: Candidate,
                measure: Callable[[Candidate], Tuple[float, object]],
                error: Callable[[object, object], float], tol: float) -> TuneResult:
    """Coordinate search: each stage proposes candidates around the current
    best; the first measured candidate (the defaults) is the accuracy
    reference.  ``measure(c) -> (ms, output)``; ``error(out, ref) -> rel``."""
    trials: List[dict] = []
    seen: Dict[str, float] = {}
    ref_out = None
    best, best_ms = start, None
    for stage in stages:
        stage_best, stage_ms = best, best_ms
        for c in stage(best):
            k = json.dumps(c.as_dict(), sort_keys=True)
            if k in seen:
                continue
            ms, out = measure(c)
            if ref_out is None:
                ref_out, err = out, 0.0
            else:
                err = float(error(out, ref_out))
            ok = err <= tol
            seen[k] = ms
            trials.append({**c.as_dict(), "ms": ms if ok else None, "rel_err": err})
            if ok and (stage_ms is None or ms < stage_ms):
                stage_best, stage_ms = c, ms
            del out
        best, best_ms = stage_best, stage_ms
    return TuneResult(best, best_ms, trials)


def _rel_err(a: torch.Tensor, b: torch.Tensor) -> float:
    return float(torch.linalg.vector_norm(a - b) / torch.clamp(torch.linalg.vector_norm(b), min=1e-300))


def _synthetic_inputs(latt_size, Ne, device, evec_dtype, seed=7):
    """Random unitary links ``[3, V3, 3, 3]`` and random vectors ``[Ne, 3 V3]``
    on the device (the timing does not depend on the values)."""
    Lx, Ly, Lz = latt_size[:3]
    V3 = Lx * Ly * Lz
    g = torch.Generator(device=device).manual_seed(seed)
    z = torch.randn((3, V3, 3, 3), dtype=torch.complex128, device=device, generator=g)
    links = torch.linalg.qr(z)[0].contiguous()
    v = torch.randn((Ne, 3 * V3), dtype=torch.complex128, device=device, generator=g)
    v = (v / torch.linalg.vector_norm(v, dim=1, keepdim=True)).to(evec_dtype)
    return links, v


#: the FP64 tile shapes are timed on a lattice of at most this extent per
#: direction (the tile choice depends on Ne and the pair groups; the time of
#: every shape grows in proportion to K = 3 V3)
FP64_PROXY_EXTENT = 12


def tune_elemental(latt_size, Ne: int, num_nabla: int, momentum_list, mode: str = "f16x3", batch: int = 1,
                   device=None, evec_dtype=torch.complex128, reps: int = 3, cache: Optional[TuningCache] = None,
                   retune: bool = False, forms: Optional[Sequence[object]] = None) -> TuneResult:
    """Best ``Candidate`` (plan form and launch settings) for this elemental
    shape, from the cache or by measurement.  ``batch`` timeslices per run, as
    the caller's plan will have; ``reps`` timed runs per candidate (median).
    ``forms`` restricts the GEMM forms tried (``factorise`` values, e.g.
    ``[True]``: the library's default form for the momentum list).
    The FP64 mode is timed on a proxy lattice (``FP64_PROXY_EXTENT``)."""
    if mode not in MODES and mode not in F64_MODES:
        raise ValueError(f"unknown elemental mode {mode!r}")
    device = torch.device(device or "cuda")
    cache = cache or TuningCache()
    dev = device_key(device)
    key = elemental_key(latt_size, Ne, num_nabla, momentum_list, mode, batch, evec_dtype)
    if forms is not None:
        key += "|forms=" + ",".join(str(f) for f in forms)
    if not retune:
        hit = cache.get(dev, key)
        if hit is not None:
            return TuneResult(Candidate.from_dict(hit["best"]), hit["ms"], hit.get("trials", []), cached=True)

    moms = [tuple(int(v) for v in p) for p in momentum_list]
    nd, nm = num_derivative(num_nabla), len(moms)
    meas_latt = list(latt_size[:3]) + list(latt_size[3:])
    if mode in F64_MODES:
        meas_latt[:3] = [min(FP64_PROXY_EXTENT, int(L)) for L in latt_size[:3]]
        reps = min(reps, 2)  # the tile shapes differ by tens of percent
    links, vecs = _synthetic_inputs(meas_latt, Ne, device, evec_dtype)
    V3 = meas_latt[0] * meas_latt[1] * meas_latt[2]
    outs = [torch.empty((nd, nm, Ne, Ne), dtype=torch.complex128, device=device) for _ in range(batch)]

    def measure(c: Candidate):
        plan = ElementalPlan(meas_latt, Ne, num_nabla, moms, mode, device, batch=batch, factorise=c.factorise,
                             tuning=c.tuning)
        try:
            run = lambda: plan.run_batch([links] * batch, V3 * 9, 9, [vecs] * batch, outs)
            run()  # warm-up: first-use setup, function attributes
            if mode not in F64_MODES:
                plan.check_status()
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
            torch.cuda.synchronize(device)
            for a, b in ev:
                a.record()
                run()
                b.record()
            torch.cuda.synchronize(device)
            if mode not in F64_MODES:
                plan.check_status()
            times = sorted(a.elapsed_time(b) for a, b in ev)
            return times[len(times) // 2], outs[0].clone()
        finally:
            del plan
            torch.cuda.empty_cache()

    stages: List[Callable[[Candidate], List[Candidate]]] = []
    if mode in F64_MODES:
        stages.append(lambda best: [Candidate(True, {"f64_tile": t}) for t in sorted(F64_TILES)])
    else:
        tried = list(forms) if forms is not None else factorise_options(latt_size, Ne, num_nabla, moms, mode)
        stages.append(lambda best: [Candidate(f, {}) for f in tried])

        def factorised(best: Candidate) -> bool:
            probe = ElementalPlan(latt_size, Ne, num_nabla, moms, mode, device="cpu", batch=batch,
                                  factorise=best.factorise)
            return probe.factorised is not None and mode != "ozaki_i8"

        def forms_on_sms(best: Candidate) -> List[Candidate]:
            # the factorised GEMM on single SMs (stacked operands with 2 or 4 k-blocks per accumulator group,
            # or the four-product form) or on SM pairs (four-product form, or the stacked operands spread over
            # the pair with 4 k-blocks per TMEM buffer)
            if not factorised(best):
                return []
            return [Candidate(best.factorise, dict(t)) for t in
                    ({}, {"tc_kpb": 4}, {"tc_stack": 2, "tc_kpb": 2}, {"tc_pair": 2, "tc_kpb": 2},
                     {"tc_pair": 3, "tc_kpb": 4})]

        def slabs(best: Candidate) -> List[Candidate]:
            if not factorised(best):
                return []
            base = dict(best.tuning)
            # the other stage count: 4 (of 48 KB) for the four-product SM pairs, 3 otherwise (single SMs: 2 by
            # default; stacked SM pairs: 4 of 32 KB by default)
            more_stages = 4 if base.get("tc_pair") == 2 else 3
            return ([best] + [Candidate(best.factorise, {**base, "tc_slab_kb": s}) for s in SLABS[1:]] +
                    [Candidate(best.factorise, {**base, "tc_stages": more_stages}),
                     Candidate(best.factorise, {**base, "tc_stages": more_stages, "tc_slab_kb": SLABS[1]})])

        def onchip_forms(best: Candidate) -> List[Candidate]:
            # the on-chip-phase GEMM: stacked operands with 2 or 4 k-blocks per group, or the four-product form
            if factorised(best) or mode == "ozaki_i8":
                return []
            return [Candidate(best.factorise, dict(t)) for t in ({}, {"tc_kpb": 4}, {"tc_stack": 2})]

        stages.append(forms_on_sms)
        stages.append(onchip_forms)
        stages.append(slabs)
    start = Candidate(True if forms is None else list(forms)[0], {})
    res = _run_search(stages, start, measure, _rel_err, TOLERANCE[mode])
    cache.put(dev, key, {"best": res.best.as_dict(), "ms": res.ms, "trials": res.trials,
                         "measured_lattice": meas_latt[:3]})
    return res


def tuned_plan(latt_size, Ne, num_nabla, momentum_list, mode="f16x3", device=None, batch=1,
               evec_dtype=torch.complex128, **kw) -> ElementalPlan:
    """An ``ElementalPlan`` built with the autotuner's choice for its shape."""
    res = tune_elemental(latt_size, Ne, num_nabla, momentum_list, mode, batch, device, evec_dtype, **kw)
    return ElementalPlan(latt_size, Ne, num_nabla, momentum_list, mode, device, batch=batch,
                         factorise=res.best.factorise, tuning=res.best.tuning)


def tune_laplacian(latt_size, nt: int = 1, nvec: int = 1, device=None, reps: int = 5,
                   cache: Optional[TuningCache] = None, retune: bool = False, apply: bool = True) -> TuneResult:
    """Choose the complex64 Laplacian kernel (``use_tma`` 0 = L1/L2, 1 = input
    planes staged by TMA, 2 = strips staged by TMA) for this shape by timing them; ``apply`` sets the winner process-wide
    (``ops.laplacian_config``)."""
    from .ops import laplacian, laplacian_config, laplacian_status

    device = torch.device(device or "cuda")
    cache = cache or TuningCache()
    dev = device_key(device)
    key = laplacian_key(latt_size, nt, nvec)
    res = None
    if not retune:
        hit = cache.get(dev, key)
        if hit is not None:
            res = TuneResult(Candidate.from_dict(hit["best"]), hit["ms"], hit.get("trials", []), cached=True)
    if res is None:
        Lx, Ly, Lz = latt_size[:3]
        V3 = Lx * Ly * Lz
        g = torch.Generator(device=device).manual_seed(11)
        U = torch.linalg.qr(torch.randn((nt, V3, 3, 3, 3), dtype=torch.complex128, device=device,
                                        generator=g))[0]
        links = U.permute(0, 2, 3, 4, 1).reshape(nt, 27, V3).to(torch.complex64).contiguous()
        F = torch.randn((nt, nvec, 3, V3), dtype=torch.complex64, device=device, generator=g)
        out = torch.empty_like(F)

        def measure(c: Candidate):
            laplacian_config(int(c.tuning.get("use_tma", 0)))
            try:
                laplacian(links, F, latt_size, out)
                ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                      for _ in range(reps)]
                for a, b in ev:
                    a.record()
                    laplacian(links, F, latt_size, out)
                    b.record()
                torch.cuda.synchronize(device)
                if laplacian_status() != 0:
                    raise RuntimeError("the TMA-staged Laplacian reported a wait timeout")
                times = sorted(a.elapsed_time(b) for a, b in ev)
                return times[len(times) // 2], out.clone()
            finally:
                laplacian_config()  # the library default

        stages = [lambda best: [Candidate(True, {"use_tma": m}) for m in (0, 1, 2)]]
        res = _run_search(stages, Candidate(True, {"use_tma": 0}), measure, _rel_err, 1e-5)
        cache.put(dev, key, {"best": res.best.as_dict(), "ms": res.ms, "trials": res.trials})
    if apply:
        laplacian_config(int(res.best.tuning.get("use_tma", 0)))
    return res
