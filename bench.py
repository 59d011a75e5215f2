"""Benchmark: elemental timeslices/s at 32^3 x 64, Ne = 200, 13 operators x 27 momenta.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--mode MODE] [--impl ours|reference]

One step = one timeslice of ``ElementalGenerator.calc``: covariant-derivative
chains, all pair contractions and the operator combination, with the links
of all 64 timeslices and the eigenvectors of several timeslices resident in
HBM (the step rotates over timeslices, so every step's inputs exceed the
129 MB L2).  ``value`` is timeslices/s over all ranks (replicas: each rank
computes its own timeslices, no collective on the data path).  ``e2e`` is
the same metric through the public generator with host eigenvectors
(host->device copy of the c128 eigenvectors and device->host copy of the
elementals inside the timed region).

``--impl reference`` times the CPU restatement of the reference numpy path
(the oracle) on the host cores on a bounded sample of the same workload.
Synthetic inputs: SU(3) links exp(i*0.3*A), random orthonormal eigenvectors.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "elemental timeslices/s 32³×64 Ne=200: split-prec vs FP64 GPU at rel err ≤1e-6"
LATT = [32, 32, 32, 64]
NE = 200
NUM_NABLA = 2
NMOM = 27
RESIDENT_T = 4  # timeslices of eigenvectors kept resident (315 MB each in c128)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="f16x3",
                    help="elemental mode: f16x3 (headline), tf32x3, bf16x3, ozaki_i8, fp64, df64")
    ap.add_argument("--lattice", default=None, help="Lx,Ly,Lz,Lt override (parity runs only)")
    ap.add_argument("--ne", type=int, default=NE)
    ap.add_argument("--batch", type=int, default=4, help="timeslices per step (one pair-contraction launch)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 GPU comparison run")
    ap.add_argument("--no-factor", action="store_true",
                    help="keep the on-chip phase GEMM although the 27 momenta factorise")
    ap.add_argument("--no-stencil", action="store_true", help="skip the Laplacian bandwidth measurement")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the measurements of the other configurations that the default line carries (other "
                         "split modes, eigensolve, mixed volumes, gradient)")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="build the plans with the built-in defaults instead of the autotuner's choice (which is "
                         "measured before the timed region and cached per device and shape)")
    ap.add_argument("--gauss", action="store_true",
                    help="headline plan in the Gauss three-multiplication form (ED_MODE_FLAG_GAUSS; --no-autotune runs)")
    ap.add_argument("--tuning", default="",
                    help="explicit plan launch settings for --no-autotune runs, e.g. tc_kpb=2,tc_pair=1 (profiling)")
    ap.add_argument("--eigen", action="store_true", help="measure the batched GPU eigensolve instead")
    ap.add_argument("--stencil", action="store_true",
                    help="measure only the Laplacian kernels (c64, c64 TMA-staged, c128) at --lattice")
    ap.add_argument("--stout", action="store_true",
                    help="measure only one stout smearing step at --lattice (default 32^3 x 64), the library's kernel "
                         "beside the reference's own CUDA kernel")
    ap.add_argument("--secondary", action="store_true",
                    help="measure the components beside the hot path: stout smearing, displacement elementals, "
                         "two-point correlators, ILDG gauge-file loading")
    ap.add_argument("--gauge-load", action="store_true",
                    help="measure only loading a 32^3 x 64 ILDG gauge file into device links (host conversion "
                         "vs device decode)")
    ap.add_argument("--eigen-batch", type=int, default=8)
    ap.add_argument("--eigen-precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--eigen-gs", default="fp64", choices=["fp64", "df"],
                    help="Gram-Schmidt arithmetic of the eigensolve (df: double-float on the FP32 pipe)")
    ap.add_argument("--eigen-cpu", action="store_true", help="also time the oracle's scipy eigensolve (slow)")
    ap.add_argument("--eigen-poly", type=int, default=0, help="Chebyshev degree for --eigen (0: plain Lanczos)")
    ap.add_argument("--eigen-ncv", type=int, default=None, help="Krylov dimension for --eigen")
    ap.add_argument("--mixed", action="store_true",
                    help="measure graphed batches over mixed volumes (16^3 Ne=64, 24^3 Ne=128, 32^3 Ne=256)")
    ap.add_argument("--grad", action="store_true",
                    help="measure the correlator-loss gradient (24^3x48, Ne=100) with a finite-difference check")
    return ap.parse_args()


def parse_tuning(text):
    """``key=value,...`` plan settings (``ElementalPlan.set_tuning`` names) -> dict."""
    out = {}
    for item in filter(None, (t.strip() for t in text.split(","))):
        k, v = item.split("=")
        out[k.strip()] = int(v)
    return out


def launches_per_step(mode, B=1, factorised=False):
    """Kernels of one batched step of B timeslices: per timeslice the links
    to SoA, vectors to planes, 12 hops and the combine; once per batch the
    phases and the pair GEMM; tensor-core modes add absmax, scale, split,
    phase scaling and the double-float to complex128 conversion (the FP64
    mode packs complex128 links, the split modes complex64 ones); the
    factorised-phase GEMM splits two operands and builds two factor tables
    (absmax, scale, 2 factor phases, 2 scalings, 2 splits, conversion)."""
    if mode == "ozaki_i8":  # 2 factor phases, 2 scalings, 2 row maxima, 2 digit splits; no absmax/conversion
        return B * (1 + 1 + 12 + 1) + 1 + 1 + 8
    extra = 0 if mode in ("fp64", "df64") else (9 if factorised else 5)
    return B * (1 + 1 + 12 + 1) + 1 + 1 + extra


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def max_over_ranks(value, device=None):
    from easydistillation_gb300.replicas import max_over_ranks as _m

    return _m(value, device)


def plan_group_rights(plan):
    return plan.describe()["nright"]


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        def run():
            while not self._stop.is_set():
                try:
                    out = subprocess.run(
                        ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                         "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                    if out.returncode == 0 and out.stdout.strip():
                        self.rows.append([v.strip() for v in out.stdout.strip().split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)

        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if len(r) > 3 + k and r[3 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ---------------------------------------------------------------- inputs
def make_inputs(latt, Ne, seed=2, distinct_t=RESIDENT_T):
    """Seeded synthetic links exp(i*0.3*A) for `distinct_t` timeslices, tiled
    to Lt (timeslices are independent, so the timed steps see distinct data
    as long as they rotate over fewer than `distinct_t` of them), and
    RESIDENT_T sets of random c128 vectors of norm 1."""
    import numpy as np

    from easydistillation_gb300.synthetic import colour_vectors, gauge_field

    Lx, Ly, Lz, Lt = latt
    nt = min(Lt, distinct_t)
    g = gauge_field([Lx, Ly, Lz, nt], 0.3, 1000 + seed)
    gauge = np.ascontiguousarray(np.tile(g, (Lt // nt + 1, 1, 1, 1, 1, 1, 1))[:Lt])
    evecs = [colour_vectors(Ne, latt, seed * 100 + t) for t in range(RESIDENT_T)]
    return gauge, evecs


# Work units of one reference timeslice (lattice/generator/elemental.py:299-329)
# at num_nabla = 2: 43 subsets, each rebuilding its two chains (78 hops in
# total), and one phase-weighted zgemm per subset and momentum.
REF_HOPS = 78
REF_SUBSETS = 43
# DRAM bytes (read + write) of one tc_fac_gemm_kernel<f16x3> launch in the stacked form on the default workload
# (32^3, Ne = 200, 4 timeslices), from one single-pass ncu capture (profiles/tc_fac_gemm_f16x3_32cube_dram.md)
FAC_TRAFFIC_BYTES = 190.38e9 + 15.77e9
# FP64 FMA throughput of this part (register-resident DFMA loop on all SMs)
FP64_PEAK_TFLOPS = 1.25
FP64_PEAK_SOURCE = "nominal GB300 FP64"


def cpu_model() -> str:
    """The host CPU's model name (lscpu), for the baseline lines."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def _oracle_inputs(latt, Ne, seed=2):
    """Seeded synthetic inputs for the CPU legs, built with the oracle alone
    (nothing of the GPU package is imported on the reference arm): one
    timeslice of links exp(i 0.3 A) and Ne orthonormal vectors."""
    from oracle import restatement as R

    g = R.synthetic_gauge(list(latt[:3]) + [1], 0.3, 1000 + seed)
    U = g.transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0]
    V = R.random_colour_vectors(Ne, list(latt[:3]) + [1], seed * 100)
    return U, V


def cpu_reference_sample(latt, Ne, threads, reps=2):
    """Bounded CPU sample for the ``cpu_baseline`` key of the GPU line (10-30 s
    of host work): the oracle's restatement of the reference numpy path at full
    size, one covariant-derivative hop of all Ne vectors and one phase-weighted
    zgemm, each the median of ``reps`` runs, scaled by the reference's counts
    per timeslice (78 hops, 43 x 27 zgemm).  ``--impl reference`` times whole
    timeslices instead."""
    os.environ.setdefault("OPENBLAS_NUM_THREADS", str(threads))
    import numpy as np

    from oracle import restatement as R

    U, V = _oracle_inputs(latt, Ne)
    V = V.astype(np.complex64).astype(np.complex128)
    ph = R.momentum_phase(latt, (0, 0, 1))
    th, tg = [], []
    for _ in range(reps):
        t0 = time.perf_counter()
        W = R.covariant_derivative(V, U, 1)
        t1 = time.perf_counter()
        lp = (-1 * ph[None, :, :, :, None] * W.conj()).reshape(Ne, -1)
        _ = lp @ V.reshape(Ne, -1).T
        t2 = time.perf_counter()
        th.append(t1 - t0)
        tg.append(t2 - t1)
    hop, gemm = statistics.median(th), statistics.median(tg)
    per_ts = REF_HOPS * hop + REF_SUBSETS * NMOM * gemm
    return per_ts, (f"oracle at {latt[0]}^3, Ne={Ne}: one hop ({hop:.2f} s) and one phase-weighted zgemm "
                    f"({gemm:.2f} s) timed, scaled by {REF_HOPS} hops + {REF_SUBSETS}x{NMOM} zgemm per timeslice "
                    f"(an estimate; --impl reference times whole timeslices)")


def run_reference(args, rank, world):
    """The reference arm: the reference's CPU algorithm for this path, as the
    oracle restates it (``ElementalGenerator.calc``: per derivative operator and
    left/right subset, both chains rebuilt and one phase-weighted zgemm per
    momentum), on the host cores, on the GPU arm's workload (32^3, Ne = 200,
    13 operators x 27 momenta).  The K timed steps together compute WHOLE
    timeslices: the 43 (operator, subset) work items of a timeslice, in the
    reference's loop order, are split into K consecutive groups, step i runs
    group i (with K > 43 the items continue into further timeslices), and
    ``value`` = timeslices computed / total time.  Warm-up steps run one
    momentum's zgemm each.  On the default workload (or with ``--eigen-cpu``)
    it also times scipy/ARPACK, the reference's eigensolver, on one 24^3,
    Ne = 100 timeslice.  Rank 0 only."""
    if rank != 0:
        return
    threads = len(os.sched_getaffinity(0))
    import numpy as np

    from oracle import restatement as R

    latt = [int(v) for v in args.lattice.split(",")] if args.lattice else LATT
    Ne = args.ne
    moms = R.mom_dict_to_list(3)[:NMOM]
    U, V = _oracle_inputs(latt, Ne)
    Vc = V.astype(np.complex64).astype(np.complex128)  # the reference's complex64 buffer
    phases = [R.momentum_phase(latt, p) for p in moms]
    items = R.elemental_items(NUM_NABLA)
    out = np.zeros((R.num_derivative(NUM_NABLA), NMOM, Ne, Ne), np.complex128)
    for _ in range(args.warmup):
        lp = (phases[0][None, :, :, :, None] * Vc.conj()).reshape(Ne, -1)
        _ = lp @ Vc.reshape(Ne, -1).T
    K = max(1, args.steps)
    n_items = -(-K // len(items)) * len(items)  # whole timeslices, at least one item per step
    bounds = [round(i * n_items / K) for i in range(K + 1)]
    step_s = []
    for i in range(K):
        t0 = time.perf_counter()
        for q in range(bounds[i], bounds[i + 1]):
            if q % len(items) == 0:
                out[...] = 0
            R.elemental_item_into(out, Vc, U, items[q % len(items)], phases)
        step_s.append(time.perf_counter() - t0)
    total = sum(step_s)
    timeslices = n_items / len(items)
    val = timeslices / total
    est, est_sample = cpu_reference_sample(latt, Ne, threads)
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "timeslices/s", "n_gpus": args.gpus,
        "steps": K, "warmup": args.warmup, "ms_per_step": total / K * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": f"elemental {latt[0]}^3x{latt[3]}, Ne={Ne}, 13 ops x {NMOM} momenta (CPU, "
                               f"{timeslices:g} whole timeslice(s) over the timed steps)"},
        "cpu_baseline": {"value": val, "unit": "timeslices/s", "cores": threads, "kind": "port",
                         "cpu_model": cpu_model(),
                         "sample": f"{timeslices:g} whole timeslice(s) of the oracle's restatement of "
                                   f"ElementalGenerator.calc ({len(items)} operator/subset items, each rebuilding "
                                   f"its chains and running {NMOM} phase-weighted zgemms), split over {K} steps; "
                                   f"OpenBLAS on {threads} threads",
                         "seconds_per_timeslice": total / timeslices,
                         "estimate_from_one_hop_one_zgemm": {"value": 1.0 / est, "sample": est_sample}},
        "e2e": {"value": val, "unit": "timeslices/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if args.eigen_cpu or not args.lattice:
        ulatt = [24, 24, 24, 1]
        Ue, _ = _oracle_inputs(ulatt, 1, seed=1)
        t0 = time.perf_counter()
        R.eigensolve(Ue, ulatt, 100, 1e-10)
        dt = time.perf_counter() - t0
        line["eigensolve_cpu"] = {"value": 1.0 / dt, "unit": "timeslices/s", "seconds": dt,
                                  "workload": "24^3, Ne=100, tol 1e-10, scipy eigsh (ARPACK), one timeslice"}
    print(json.dumps(line), flush=True)


def bench_stencil(U, latt, dev, reps=20):
    """HBM roofline of the 3D Laplacian kernel as the batched Lanczos uses it:
    one application = every timeslice x one vector.  Algorithmic bytes per
    site: 27 link + 3 input + 3 output complex numbers (264 B at c64, 528 B at
    c128); the 64 timeslices of links exceed L2, so every application streams
    them from HBM."""
    import torch

    from easydistillation_gb300.ops import (laplacian, laplacian_config, laplacian_df, laplacian_status, links_to_soa,
                                            split_c128)

    Lx, Ly, Lz, Lt = latt
    V3 = Lx * Ly * Lz
    peaks = load_peaks()
    pk, src = (peaks["hbm_gbs"], "measured") if "hbm_gbs" in peaks else (6800.0, "fallback")
    out = {}
    variants = (("c64", torch.complex64, 8, 2, "laplacian_strip_kernel (default: links and input staged by TMA)"),
                ("c64_l1", torch.complex64, 8, 0, "laplacian_kernel<float,2> (neighbours through L1/L2)"),
                ("c64_tma_planes", torch.complex64, 8, 1, "laplacian_tma_kernel (input planes staged by TMA)"),
                ("c128", torch.complex128, 16, 0, "laplacian_kernel<double,1>"),
                ("c128_df", torch.complex128, 16, -1, "laplacian_df_kernel (double-float on the FP32 pipe)"))
    for name, dt, s, tma, kname in variants:
        laplacian_config(max(tma, 0))
        links = links_to_soa(U, latt, dtype=dt)
        if tma < 0:  # the double-float kernel: links split once, complex128 vectors
            links = split_c128(links)
            lap = lambda L_, X_, latt_, out: laplacian_df(L_, X_, latt_, out=out)  # noqa: E731
        else:
            lap = laplacian
        F = torch.randn((Lt, 1, 3, V3), dtype=dt, device=dev)
        G = torch.empty_like(F)
        for _ in range(3):
            lap(links, F, latt, out=G)
        torch.cuda.synchronize()
        # the reps launches replayed from a CUDA graph, so that host-side launch time cannot leave gaps between
        # these ~0.1 ms kernels (a Python loop of launches measured 0.57 of HBM instead of 0.86 in a busy process)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            for r in range(reps):
                if r % 2 == 0:
                    lap(links, F, latt, out=G)
                else:
                    lap(links, G, latt, out=F)
        graph.replay()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        graph.replay()
        b.record()
        torch.cuda.synchronize()
        laplacian_status()
        del graph
        ms = a.elapsed_time(b) / reps
        nbytes = V3 * Lt * (27 * s + 6 * s)
        gbs = nbytes / ms / 1e6
        out[name] = {"bound": "hbm", "achieved": gbs, "peak": pk, "unit": "GB/s", "frac": gbs / pk,
                     "peak_source": src, "traffic": None, "bytes_per_launch": nbytes, "kernel_ms": ms,
                     "kernel": kname, "workload": f"{Lx}^3 x {Lt} timeslices x 1 vector"}
        if s == 16 and tma >= 0:
            # FP64 arithmetic, not HBM, bounds the complex128 stencil on this part: 444 flops per site
            fl = 444.0 * V3 * Lt / ms / 1e9
            out[name].update({"bound": "fp64", "fp64_tflops": fl, "fp64_peak_tflops": FP64_PEAK_TFLOPS,
                              "fp64_frac": fl / FP64_PEAK_TFLOPS, "fp64_peak_source": FP64_PEAK_SOURCE})
        del links, F, G
    laplacian_config()  # the library default
    return out


# ---------------------------------------------------------------- ours
def run_ours(args, rank, world):
    import numpy as np
    import torch

    from easydistillation_gb300 import ElementalGenerator
    from easydistillation_gb300.generator.elemental import links_to_device
    from easydistillation_gb300.ops import ElementalPlan

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    latt = [int(v) for v in args.lattice.split(",")] if args.lattice else LATT
    Lx, Ly, Lz, Lt = latt
    V3 = Lx * Ly * Lz
    Ne = args.ne
    from easydistillation_gb300.insertion import mom_dict_to_list

    moms = mom_dict_to_list(3)[:NMOM]
    gauge, evecs_host = make_inputs(latt, Ne, seed=2 + rank)
    U = links_to_device(gauge, latt, dev)  # [3, Lt, Lz, Ly, Lx, 3, 3] c128 resident
    V = [torch.from_numpy(x).to(dev) for x in evecs_host]  # resident c128 eigenvectors
    B = args.batch
    tuned = None
    if args.no_factor:
        args.autotune = False  # an explicit GEMM form
    if args.autotune:
        from easydistillation_gb300.tune import tune_elemental

        t0 = time.perf_counter()
        res = tune_elemental(latt, Ne, NUM_NABLA, moms, args.mode, B, dev)
        tuned = {"cached": res.cached, "seconds": time.perf_counter() - t0, "trials": res.trials}
        plan = ElementalPlan(latt, Ne, NUM_NABLA, moms, args.mode, dev, batch=B, factorise=res.best.factorise,
                             tuning=res.best.tuning)
    else:
        plan = ElementalPlan(latt, Ne, NUM_NABLA, moms, args.mode, dev, batch=B, factorise=not args.no_factor,
                             tuning=parse_tuning(args.tuning), gauss=args.gauss)
    outs = [torch.empty((13, NMOM, Ne, Ne), dtype=torch.complex128, device=dev) for _ in range(B)]
    out = outs[0]
    stream = torch.cuda.current_stream()

    def step(i):
        # one batch of B timeslices: one pass, one pair-contraction launch
        ts = [((i * B + k) * 7 + rank) % Lt for k in range(B)]
        plan.run_batch([U[:, t] for t in ts], Lt * V3 * 9, 9, [V[(i * B + k) % RESIDENT_T] for k in range(B)],
                       outs)

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    # per-step events around the pair-contraction kernel (the dominant kernel)
    kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for a, b in kev:
        a.record(stream)
        b.record(stream)
    sampler = ClockSampler(dev.index)
    sampler.start()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    start.record(stream)
    for i in range(args.steps):
        plan.set_profile_events(*kev[i])
        step(args.warmup + i)
    end.record(stream)
    torch.cuda.synchronize()
    plan.set_profile_events(None, None)
    clocks = sampler.stop()
    if args.mode != "fp64" and plan.check_status() != 0:
        raise RuntimeError("tensor-core kernel reported a timeout")
    ms = start.elapsed_time(end)
    ms = max_over_ranks(ms, dev if world > 1 else None)
    ms_per_step = ms / args.steps
    value = world * args.steps * B / (ms / 1e3)

    # roofline of the pair-contraction kernel
    kms = statistics.mean(a.elapsed_time(b) for a, b in kev)
    # algorithmic work: the reference's 43 chain-pair subsets (num_nabla = 2) per
    # momentum, 8*Ne^2*3V3 real flops each; this implementation evaluates only
    # plan.num_pairs distinct pair products per momentum and combines them.
    units = REF_SUBSETS * NMOM * B
    alg_flop = units * 8.0 * Ne * Ne * 3 * V3
    peaks = load_peaks()
    if args.mode == "ozaki_i8":
        pxy, pz = plan.factorised
        rights = plan_group_rights(plan)[: len(plan_group_rights(plan)) // B]
        tiles = sum(-(-(j * pz * Ne) // 64) for j in rights) * (-(-(pxy * Ne) // 64))
        iops = B * tiles * 64 * 64 * 3 * V3 * 40 * 2.0  # 10 slice pairs x 4 real products, 2 ops per MAC
        roofline = {"bound": "int8 tensor (mma.sync)", "achieved": alg_flop / kms / 1e9, "peak": None,
                    "unit": "TFLOP/s", "frac": None, "traffic": None, "kernel": "tc_ozaki_gemm_kernel",
                    "kernel_ms": kms, "int8_tops_executed": iops / kms / 1e9,
                    "note": "achieved in the 43-subset flop count; the kernel issues 40 int8 products per complex "
                            "multiply-add (10 slice pairs x 4); mma.sync int8 measured at 158 TOPS on this part "
                            "by a register-only probe (tcgen05 has no kind::i8 on sm_103a)"}
    elif args.mode in ("fp64", "df64"):
        roofline = {"bound": "fp64" if args.mode == "fp64" else "fp32 (double-float)",
                    "achieved": alg_flop / kms / 1e9, "peak": None, "unit": "TFLOP/s", "frac": None,
                    "traffic": None, "kernel": "pair_gemm_f64_kernel" if args.mode == "fp64" else "pair_gemm_df_kernel",
                    "kernel_ms": kms}
    else:
        pk, pk_src = peaks.get("bf16_tflops_sustained"), "measured bf16 sustained"
        if pk is None:
            pk, pk_src = 1700.0, "fallback"
        # 128 x 128 tiles; 12 MMAs of 128x128x(K) per complex multiply-add
        rights = plan_group_rights(plan)[: len(plan_group_rights(plan)) // B]
        if plan.factorised:
            pxy, pz = plan.factorised
            tiles = sum(-(-(j * pz * Ne) // 128) for j in rights) * (-(-(pxy * Ne) // 128))
            pair_form = plan.tuning().get("tc_pair", 0)
            kname = {2: "tc_fac2_gemm_kernel", 3: "tc_fac2s_gemm_kernel"}.get(pair_form, "tc_fac_gemm_kernel")
            kname = f"{kname}<{args.mode}>"
        else:
            tiles = sum(-(-(j * Ne) // 128) for j in rights) * (-(-(Ne * NMOM) // 128))
            kname = f"tc_pair_gemm_kernel<{args.mode}>"
        per_mac = 9 if getattr(plan, "gauss", False) else 12  # real MMAs per complex multiply-add (3 split products)
        mma_flop = B * tiles * 128 * 128 * 3 * V3 * per_mac * 2.0
        tun = plan.tuning()
        default_workload = (plan.factorised is not None and args.mode == "f16x3" and B == 4 and Ne == NE
                            and list(latt[:3]) == LATT[:3] and not getattr(plan, "gauss", False)
                            and tun.get("tc_stack", 0) != 2 and tun.get("tc_pair", 0) < 2)
        roofline = {"bound": "tensor", "achieved": alg_flop / kms / 1e9, "peak": pk, "unit": "TFLOP/s",
                    "frac": alg_flop / kms / 1e9 / pk,
                    "traffic": FAC_TRAFFIC_BYTES if default_workload else None,
                    "traffic_unit": "bytes per launch (DRAM read + write, ncu)", "peak_source": pk_src,
                    "kernel": kname, "kernel_ms": kms,
                    "mma_tflops_executed": mma_flop / kms / 1e9, "mma_frac": mma_flop / kms / 1e9 / pk,
                    "pairs_evaluated_per_momentum": plan.num_pairs, "ref_subsets_per_momentum": REF_SUBSETS,
                    "note": "achieved = algorithmic flops 8*Ne^2*3V3*Nmom*43 per timeslice (the reference's subset "
                            "count); the kernel evaluates 19 distinct chain pairs per momentum and issues 12 "
                            "fp16/tf32 MMA products per complex multiply-add (9 in the Gauss form; 3 split "
                            "products each) plus tile padding (mma_*)"}

    # the Laplacian's HBM roofline (kernel launches replayed from a CUDA graph)
    stencil = None if args.no_stencil else bench_stencil(U, latt, dev)

    # the plain FP64 GPU path on the same timeslice: speed and the split-precision error against it
    fp64 = None
    split_modes = None
    if args.mode not in ("fp64", "df64") and not args.no_fp64:
        t_tune = None
        if args.autotune:
            from easydistillation_gb300.tune import tuned_plan

            t_tune = time.perf_counter()
            plan64 = tuned_plan(latt, Ne, NUM_NABLA, moms, "fp64", dev)
            t_tune = time.perf_counter() - t_tune
        else:
            plan64 = ElementalPlan(latt, Ne, NUM_NABLA, moms, "fp64", dev)
        out64 = torch.empty_like(out)
        t_ref = (args.warmup * 7 + rank) % Lt
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        plan64.run(U[:, t_ref], Lt * V3 * 9, 9, V[args.warmup % RESIDENT_T], out64)
        b.record(stream)
        plan.run(U[:, t_ref], Lt * V3 * 9, 9, V[args.warmup % RESIDENT_T], out)
        torch.cuda.synchronize()
        ms64 = a.elapsed_time(b)
        rel = float(torch.linalg.vector_norm(out - out64) / torch.linalg.vector_norm(out64))
        fp64 = {"value": 1e3 / ms64, "unit": "timeslices/s", "rel_err_vs_fp64": rel,
                "speedup_split_over_fp64": (value / world) / (1e3 / ms64), "plan_settings": plan64.tuning(),
                "autotune_seconds": t_tune}
        # the same FP64 contraction in double-float arithmetic on the FP32 pipe (precision "df64"), same tiles
        plan_df = ElementalPlan(latt, Ne, NUM_NABLA, moms, "df64", dev,
                                tuning={"f64_tile": plan64.tuning()["f64_tile"]})
        out_df = torch.empty_like(out)
        plan_df.run(U[:, t_ref], Lt * V3 * 9, 9, V[args.warmup % RESIDENT_T], out_df)  # warm-up
        torch.cuda.synchronize()
        a.record(stream)
        plan_df.run(U[:, t_ref], Lt * V3 * 9, 9, V[args.warmup % RESIDENT_T], out_df)
        b.record(stream)
        torch.cuda.synchronize()
        ms_df = a.elapsed_time(b)
        fp64["df64"] = {"value": 1e3 / ms_df, "unit": "timeslices/s",
                        "rel_err_vs_fp64": float(torch.linalg.vector_norm(out_df - out64) /
                                                 torch.linalg.vector_norm(out64)),
                        "speedup_over_fp64": ms64 / ms_df,
                        "note": "the FP64 mode's pair GEMM in double-float arithmetic on the FP32 pipe"}
        del plan64, plan_df, out_df
        torch.cuda.empty_cache()
        if not args.no_extra and rank == 0:
            # the other split-precision modes on the same workload, each with its error against FP64
            split_modes = bench_split_modes(args, latt, Ne, moms, U, V, out64, t_ref, dev, stream,
                                            exclude=args.mode)
        del out64
        torch.cuda.empty_cache()

    # end to end through the public generator: host eigenvectors in, host elementals out
    e2e = None
    if not args.no_e2e:
        class _D:
            def __init__(self, a):
                self.a = a
                self.file = "mem"

            def __getitem__(self, k):
                return self.a[k]

        class _Src:
            def __init__(self, a, Ne=None):
                self.d = _D(a)
                self.Ne = Ne

            def load(self, key):
                return self.d

        # eigenvectors in pinned host memory ([RESIDENT_T, Ne, Lz, Ly, Lx, 3] c128), elementals back into
        # pinned host memory; one calc_batch call over all timed steps, whose batches pipeline the copies
        ev = torch.from_numpy(np.stack([x.reshape(Ne, Lz, Ly, Lx, 3) for x in evecs_host])).pin_memory()
        class _TSrc:  # eigenvector source whose load() returns the pinned tensor itself
            def __init__(self, t, Ne):
                self.t, self.Ne = t, Ne

            def load(self, key):
                return self.t

        gen = ElementalGenerator(latt, _Src(gauge), _TSrc(ev, Ne), NUM_NABLA, moms, precision=args.mode, device=dev,
                                 factorise=not args.no_factor, autotune=args.autotune)
        gen.load("bench")
        # at least 8 batches, so that the pipeline's fill (first upload) and drain (last download) are amortised
        nts = max(args.steps, 8) * B
        host_out = torch.empty((nts, 13, NMOM, Ne, Ne), dtype=torch.complex128).pin_memory()
        ts_all = [k % RESIDENT_T for k in range(nts)]
        gen.calc_batch(ts_all[:B], out=host_out[:B], batch=B)  # warm-up: plans, buffers, streams
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        gen.calc_batch(ts_all, out=host_out, batch=B)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        e2e = {"value": world * nts / dt, "unit": "timeslices/s",
               "h2d_bytes_per_step": B * Ne * V3 * 3 * 16, "d2h_bytes_per_step": int(host_out[:B].numel() * 16),
               "steps": nts // B,
               "api": "ElementalGenerator.calc_batch over all timed steps (pinned host eigenvectors in, pinned host "
                      "elementals out; host<->device copies of batch k+-1 overlap the compute of batch k)"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = len(os.sched_getaffinity(0))
        per_ts, sample = cpu_reference_sample(latt, Ne, threads)
        cpu = {"value": 1.0 / per_ts, "unit": "timeslices/s", "cores": threads, "kind": "port", "sample": sample,
               "cpu_model": cpu_model()}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "timeslices/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128" if args.mode in ("fp64", "df64") else args.mode, "data": "synthetic",
            "config": {"workload": f"elemental {Lx}^3x{Lt}, Ne={Ne}, 13 ops x {NMOM} momenta, mode={args.mode}, "
                                   f"{B} timeslices per step",
                       "timeslices_per_step": B,
                       "factorised_phases": plan.factorised,
                       "plan_settings": {"factorise": plan.factorise, **plan.tuning()},
                       "pairs_per_momentum": plan.num_pairs, "l2": "inputs larger than L2 (rotating timeslices)",
                       "parallelism": f"replicas x{world}"},
            "gpu_launches": args.steps * launches_per_step(args.mode, B, plan.factorised is not None),
            "clocks": clocks, "roofline": roofline, "e2e": e2e, "cpu_baseline": cpu, "fp64_gpu": fp64,
            "split_modes": split_modes, "stencil_roofline": stencil,
        }
        if not args.no_extra:
            # the other configurations' measurements, each timed by itself after the headline measurement
            del plan, outs, out, V
            torch.cuda.empty_cache()
            line["stout"] = bench_stout(latt, dev, event_seconds, True, U=U)
            del U
            torch.cuda.empty_cache()
            line["correlators"] = bench_correlators(dev, event_seconds)
            torch.cuda.empty_cache()
            line["eigensolve"] = bench_eigen_default(dev)
            torch.cuda.empty_cache()
            line["eigensolve_32cube"] = bench_eigen_32(dev)
            torch.cuda.empty_cache()
            line["elementals_24cube"] = bench_elemental_24(dev)
            torch.cuda.empty_cache()
            line["mixed_volumes"] = measure_mixed(args, dev)
            torch.cuda.empty_cache()
            line["gradient"] = measure_grad(args, dev)
        if tuned is not None:
            line["autotune"] = tuned
        print(json.dumps(line), flush=True)


def bench_split_modes(args, latt, Ne, moms, U, V, out64, t_ref, dev, stream, exclude=None, reps=2):
    """Every split-precision mode other than the headline one on the headline
    workload: timeslices/s over ``reps`` batched steps (after one warm-up
    step, CUDA events; batch 2 for the tensor-core modes, 1 for the Ozaki
    int8 mode), the pair-GEMM kernel time, and the relative Frobenius error
    against the FP64 GPU elementals of timeslice ``t_ref``."""
    import torch

    from easydistillation_gb300.ops import ElementalPlan

    Lx, Ly, Lz, Lt = latt
    V3 = Lx * Ly * Lz
    out = {}
    for name in ("f16x3", "tf32x3", "bf16x3", "ozaki_i8", "f16x3_gauss3m"):
        mode, gauss = name.split("_gauss")[0], name.endswith("gauss3m")
        if name == exclude:
            continue
        B = 1 if mode == "ozaki_i8" else 2
        plan = ElementalPlan(latt, Ne, NUM_NABLA, moms, mode, dev, batch=B, gauss=gauss)
        outs = [torch.empty((13, NMOM, Ne, Ne), dtype=torch.complex128, device=dev) for _ in range(B)]

        def step(i):
            ts = [((i * B + k) * 7) % Lt for k in range(B)]
            plan.run_batch([U[:, t] for t in ts], Lt * V3 * 9, 9, [V[(i * B + k) % RESIDENT_T] for k in range(B)],
                           outs)

        step(0)
        kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for a, b in kev:
            a.record(stream)
            b.record(stream)
        a0, b0 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a0.record(stream)
        for i in range(reps):
            plan.set_profile_events(*kev[i])
            step(1 + i)
        b0.record(stream)
        torch.cuda.synchronize()
        plan.set_profile_events(None, None)
        ms = a0.elapsed_time(b0)
        kms = statistics.mean(a.elapsed_time(b) for a, b in kev)
        plan.run(U[:, t_ref], Lt * V3 * 9, 9, V[args.warmup % RESIDENT_T], outs[0])
        plan.check_status()
        err = float(torch.linalg.vector_norm(outs[0] - out64) / torch.linalg.vector_norm(out64))
        out[name] = {"value": reps * B / (ms / 1e3), "unit": "timeslices/s", "kernel_ms_per_step": kms,
                     "timeslices_per_step": B, "rel_err_vs_fp64": err, "factorised_phases": plan.factorised}
        if gauss:
            out[name]["form"] = "Gauss three multiplications (ED_MODE_FLAG_GAUSS), 2 k-blocks per group"
        del plan, outs
        torch.cuda.empty_cache()
    return out


def bench_eigen_default(dev, batch=8):
    """The FP64 eigensolve configuration, 24^3, Ne = 100, tol 1e-10, on a batch
    of ``batch`` timeslices (links exp(i 0.3 A)): the plain native
    thick-restart Lanczos, the Chebyshev-accelerated one (degree 16, cut 15 %
    above the largest eigenvalue of the plain solve), and the mixed solve
    (complex64 stencil in a loose FP64 iteration, then the FP64 Chebyshev
    refinement with the cut found automatically).  Each: timeslices/s of one
    solve after an untimed one, the largest residual ||L x - lambda x|| (FP64
    stencil), the largest deviation of the Gram matrix from identity and the
    largest eigenvalue difference to the plain solve."""
    import torch

    from easydistillation_gb300.ops import lanczos_tr, laplacian, links_to_soa
    from easydistillation_gb300.generator.elemental import links_to_device

    latt = [24, 24, 24, batch]
    Ne = 100
    gauge, _ = make_inputs(latt, 1, distinct_t=batch)
    U = links_to_device(gauge, latt, dev)
    L64 = links_to_soa(U, latt)
    L32 = links_to_soa(U, latt, dtype=torch.complex64)

    def quality(ev, X, ref_ev=None):
        LY = laplacian(L64, X, latt)
        res = torch.linalg.vector_norm((LY - ev[:, :, None, None].to(X.dtype) * X).reshape(batch, Ne, -1), dim=2)
        Xf = X.reshape(batch, Ne, -1)
        G = Xf.conj() @ Xf.transpose(1, 2)
        eye = torch.eye(Ne, dtype=G.dtype, device=G.device)
        q = {"max_residual": float(res.max()), "max_gram_dev": float((G - eye).abs().max())}
        if ref_ev is not None:
            q["max_rel_eval_diff_vs_plain"] = float(((ev - ref_ev).abs() / ref_ev.abs()).max())
        return q

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    out = {"workload": f"24^3, Ne={Ne}, tol 1e-10, {batch} timeslices per solve"}
    (ev0, X0, st0), dt0 = timed(lambda: lanczos_tr(L64, latt, Ne, 1e-10))
    out["plain_fp64"] = {"value": batch / dt0, "unit": "timeslices/s", "converged": st0["converged"],
                         "restarts": st0["restarts"], **quality(ev0, X0)}
    cut = 1.15 * float(ev0[:, -1].max())
    (ev1, X1, st1), dt1 = timed(lambda: lanczos_tr(L64, latt, Ne, 1e-12, poly_deg=16, lambda_cut=cut))
    out["chebyshev_fp64"] = {"value": batch / dt1, "unit": "timeslices/s", "converged": st1["converged"],
                             "degree": 16, "lambda_cut": cut, "note": "cut taken from the plain solve",
                             **quality(ev1, X1, ev0)}
    (ev2, X2, st2), dt2 = timed(lambda: lanczos_tr(L64, latt, Ne, 1e-10, stencil_precision="fp32", links_c64=L32))
    out["mixed_fp32_stencil"] = {"value": batch / dt2, "unit": "timeslices/s", "converged": st2["converged"],
                                 "matvecs_fp32": st2["matvecs_fp32"], "matvecs_fp64": st2["matvecs_fp64"],
                                 "restarts_fp32_phase": st2["restarts_fp32"],
                                 "note": "complex64 stencil in a loose FP64 iteration, then FP64 Chebyshev "
                                         "refinement (cut found automatically)", **quality(ev2, X2, ev0)}
    # the same three solves in the double-float mode (Gram-Schmidt, rotation and FP64-class stencil on the FP32 pipe)
    df = {}
    (ev3, X3, st3), dt3 = timed(lambda: lanczos_tr(L64, latt, Ne, 1e-10, gs_precision="df"))
    df["plain"] = {"value": batch / dt3, "converged": st3["converged"], "restarts": st3["restarts"],
                   **quality(ev3, X3, ev0)}
    (ev4, X4, st4), dt4 = timed(lambda: lanczos_tr(L64, latt, Ne, 1e-12, poly_deg=16, lambda_cut=cut,
                                                   gs_precision="df"))
    df["chebyshev"] = {"value": batch / dt4, "converged": st4["converged"], **quality(ev4, X4, ev0)}
    (ev5, X5, st5), dt5 = timed(lambda: lanczos_tr(L64, latt, Ne, 1e-10, stencil_precision="fp32", links_c64=L32,
                                                   gs_precision="df"))
    df["mixed_fp32_stencil"] = {"value": batch / dt5, "converged": st5["converged"], **quality(ev5, X5, ev0)}
    out["double_float_gram_schmidt"] = {"unit": "timeslices/s", **df,
                                        "note": "gs_precision='df': Gram-Schmidt passes, restart rotations and the "
                                                "FP64-class stencil on the FP32 pipe in double-float arithmetic "
                                                "(~2^-47 products); recurrence, projected eigenproblem, "
                                                "convergence test and final Rayleigh quotients FP64"}
    return out


def bench_elemental_24(dev):
    """The plain-FP64 configuration's elementals: 24^3, Ne = 100, 13 operators
    x 27 momenta, one timeslice per run (CUDA events, after a warm-up run):
    FP64, its double-float form (df64) and f16x3, each with its relative
    Frobenius error against the FP64 result."""
    import torch

    from easydistillation_gb300.generator.elemental import links_to_device
    from easydistillation_gb300.insertion import mom_dict_to_list
    from easydistillation_gb300.ops import ElementalPlan

    latt, Ne = [24, 24, 24, 2], 100
    V3 = 24 ** 3
    moms = mom_dict_to_list(3)
    gauge, evecs = make_inputs(latt, Ne, distinct_t=2)
    U = links_to_device(gauge, latt, dev)
    V = torch.from_numpy(evecs[0].reshape(Ne, -1)).to(dev)
    out = {"workload": "24^3, Ne=100, 13 ops x 27 momenta, one timeslice per run"}
    ref = None
    for mode in ("fp64", "df64", "f16x3"):
        plan = ElementalPlan(latt, Ne, NUM_NABLA, moms, mode, dev,
                             tuning={"f64_tile": 3} if mode in ("fp64", "df64") else None)
        o = torch.empty((13, 27, Ne, Ne), dtype=torch.complex128, device=dev)
        plan.run(U[:, 0], 2 * V3 * 9, 9, V, o)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        plan.run(U[:, 0], 2 * V3 * 9, 9, V, o)
        b.record()
        torch.cuda.synchronize()
        if mode != "fp64":
            plan.check_status()
        if ref is None:
            ref = o
        out[mode] = {"value": 1e3 / a.elapsed_time(b), "unit": "timeslices/s",
                     "rel_err_vs_fp64": float(torch.linalg.vector_norm(o - ref) / torch.linalg.vector_norm(ref))}
        del plan
    return out


def bench_eigen_32(dev, batch=2):
    """The mixed-precision configuration's eigensolve, 32^3, Ne = 200, tol
    1e-10, ``batch`` timeslices per solve: the plain FP64 solve, the mixed
    solve (complex64 stencil inside the loose FP64 iteration, then the FP64
    Chebyshev refinement; FP64 Gram-Schmidt and Rayleigh-Ritz) and the same in
    the double-float mode; timeslices/s of one solve after an untimed one, the
    largest residual (FP64 stencil) and eigenvalue difference to the plain
    solve."""
    import torch

    from easydistillation_gb300.generator.elemental import links_to_device
    from easydistillation_gb300.ops import lanczos_tr, laplacian, links_to_soa

    latt = [32, 32, 32, batch]
    Ne = 200
    gauge, _ = make_inputs(latt, 1, distinct_t=batch)
    U = links_to_device(gauge, latt, dev)
    L64 = links_to_soa(U, latt)
    L32 = links_to_soa(U, latt, dtype=torch.complex64)
    del U

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    def max_res(ev, X):
        LY = laplacian(L64, X, latt)
        return float(torch.linalg.vector_norm((LY - ev[:, :, None, None].to(X.dtype) * X).reshape(batch, Ne, -1),
                                              dim=2).max())

    out = {"workload": f"32^3, Ne={Ne}, tol 1e-10, {batch} timeslices per solve"}
    (ev0, X0, st0), dt0 = timed(lambda: lanczos_tr(L64, latt, Ne, 1e-10))
    out["plain_fp64"] = {"value": batch / dt0, "unit": "timeslices/s", "converged": st0["converged"],
                         "max_residual": max_res(ev0, X0)}
    del X0
    for name, gs in (("mixed_fp32_stencil", "fp64"), ("mixed_fp32_stencil_df", "df")):
        (ev, X, st), dt = timed(lambda: lanczos_tr(L64, latt, Ne, 1e-10, stencil_precision="fp32", links_c64=L32,
                                                   gs_precision=gs))
        out[name] = {"value": batch / dt, "unit": "timeslices/s", "converged": st["converged"],
                     "max_residual": max_res(ev, X),
                     "max_rel_eval_diff_vs_plain": float(((ev - ev0).abs() / ev0.abs()).max()),
                     "matvecs_fp32": st["matvecs_fp32"], "matvecs_fp64": st["matvecs_fp64"]}
        del X
    out["note"] = ("mixed: complex64 stencil inside the loose FP64 iteration, then the FP64 Chebyshev refinement "
                   "(cut found automatically); _df: Gram-Schmidt, rotations and FP64-class stencil in double-float")
    return out


def measure_mixed(args, dev):
    """The mixed-volume configuration as a dict (see ``run_mixed``)."""
    return run_mixed(args, emit=False)


def measure_grad(args, dev):
    """The differentiation configuration as a dict (see ``run_grad``)."""
    return run_grad(args, emit=False)


def run_mixed(args, emit=True):
    """Secondary measurement (``--mixed``): 96 timeslices, 32 each of 16^3
    (Ne=64), 24^3 (Ne=128) and 32^3 (Ne=256), links exp(i eps A) with eps
    alternating 0.1 / 0.3 over timeslices, 4 operators x 7 momenta, split
    precision.  All 96 timeslices are one CUDA-graph replay: per volume a
    batched plan (batch admitted by HBM footprint) reads the resident inputs
    in place; the plans take the autotuner's choice (``--no-autotune``: defaults)."""
    import torch

    from easydistillation_gb300.batch import MixedVolumeGraph, VolumeBinding
    from easydistillation_gb300.generator.elemental import links_to_device
    from easydistillation_gb300.insertion import mom_dict_to_list
    from easydistillation_gb300.synthetic import gauge_field

    dev = torch.device("cuda", 0)
    mode = args.mode
    moms = mom_dict_to_list(3)[:7]
    vols = [([16, 16, 16, 32], 64), ([24, 24, 24, 32], 128), ([32, 32, 32, 32], 256)]
    gen = torch.Generator(device=dev).manual_seed(3003)
    bindings = []
    for latt, Ne in vols:
        Lx, Ly, Lz, Lt = latt
        V3 = Lx * Ly * Lz
        # 2 distinct timeslices per eps, tiled (timeslices are independent)
        g = [gauge_field([Lx, Ly, Lz, 2], eps, 1000 + 3 + k) for k, eps in enumerate((0.1, 0.3))]
        U = torch.stack([links_to_device(x, [Lx, Ly, Lz, 2], dev) for x in g], dim=2)  # [3, 2, eps, ...]
        U = U.reshape(3, 4, Lz, Ly, Lx, 3, 3)  # t' = 2*t + eps index: eps alternates
        V = torch.complex(torch.randn((4, Ne, V3 * 3), generator=gen, device=dev, dtype=torch.float64),
                          torch.randn((4, Ne, V3 * 3), generator=gen, device=dev, dtype=torch.float64))
        V /= (2 * V3 * 3) ** 0.5
        bindings.append(VolumeBinding(latt, Ne, U, V, [t % 4 for t in range(Lt)]))
    reps = max(1, args.steps)
    n_per = sum(len(b.timeslices) for b in bindings)

    def sweep(single_launch):
        t0 = time.perf_counter()
        mv = MixedVolumeGraph(bindings, 1, moms, mode, max_batch=8, device=dev, autotune=args.autotune,
                              single_launch=single_launch)
        setup_s = time.perf_counter() - t0
        mv.capture()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            mv.run()
        b.record()
        torch.cuda.synchronize()
        mv.check_status()
        return mv, a.elapsed_time(b) / 1e3, setup_s

    mv1, dt1, _ = sweep(False)  # one GEMM launch per volume chunk, for comparison
    launches1 = mv1.gemm_launches
    del mv1
    torch.cuda.empty_cache()
    mv, dt, setup_s = sweep(True)
    line = {"metric": "mixed-volume elemental timeslices/s (96 timeslices: 16^3 Ne=64, 24^3 Ne=128, 32^3 Ne=256; "
                      "4 ops x 7 momenta)", "value": reps * n_per / dt, "unit": "timeslices/s",
            "seconds_per_sweep": dt / reps, "mode": mode,
            "batches": {f"{v[0][0]}^3": p.batch for v, p in zip(vols, mv.plans)},
            "plan_settings": {f"{v[0][0]}^3": {"factorise": p.factorise, "factorised": p.factorised, **p.tuning()}
                              for v, p in zip(vols, mv.plans)},
            "autotune": args.autotune, "plan_setup_seconds": setup_s,
            "graph_replays_per_sweep": 1, "gemm_launches_per_sweep": mv.gemm_launches,
            "per_volume_gemm_launches": {"value": reps * n_per / dt1, "seconds_per_sweep": dt1 / reps,
                                         "gemm_launches_per_sweep": launches1},
            "data": "synthetic, resident in HBM"}
    del mv, bindings
    if emit:
        print(json.dumps(line), flush=True)
    return line


def run_grad(args, emit=True):
    """Secondary measurement (``--grad``): gradient of the correlator
    log-ratio loss (t = 6, 12; operator nabla_x, p = 0; gamma_5) with respect
    to the profile weights w_k and the links at 24^3 x 48, Ne = 100, through
    the hand-written adjoints; a central finite difference (h = 1e-6) along a
    random link direction and a random weight direction checks it."""
    import numpy as np
    import torch

    from easydistillation_gb300.autograd import correlator_log_ratio
    from easydistillation_gb300.correlator import gamma
    from easydistillation_gb300.generator.elemental import links_to_device
    from easydistillation_gb300.synthetic import gauge_field

    dev = torch.device("cuda", 0)
    latt = [24, 24, 24, 48]
    Lx, Ly, Lz, Lt = latt
    V3 = Lx * Ly * Lz
    Ne = 100
    g = gauge_field([Lx, Ly, Lz, 4], 0.3, 1004)
    U4 = links_to_device(g, [Lx, Ly, Lz, 4], dev)
    U = U4[:, torch.arange(Lt, device=dev) % 4].contiguous()
    gen = torch.Generator(device=dev).manual_seed(4006)
    V = torch.complex(torch.randn((Lt, Ne, V3 * 3), generator=gen, device=dev, dtype=torch.float64),
                      torch.randn((Lt, Ne, V3 * 3), generator=gen, device=dev, dtype=torch.float64)) / (2 * V3 * 3) ** 0.5
    rng = np.random.default_rng(4004)
    w = torch.from_numpy(rng.uniform(0.5, 1.5, Ne)).to(dev)
    evals = torch.from_numpy(np.sort(rng.uniform(0.2, 0.6, (Lt, Ne)), axis=1)).to(dev)
    rng5 = np.random.default_rng(4005)
    tau = torch.from_numpy(rng5.standard_normal((Lt, 4, 4, Ne, Ne)) + 1j * rng5.standard_normal((Lt, 4, 4, Ne, Ne))).to(dev)
    g5 = gamma(15, dev)

    def loss(U_, w_):
        return correlator_log_ratio(U_, V, evals, w_, tau, latt, g5, d=1, t1=6, t2=12)

    times = []
    for _ in range(max(2, args.steps + 1)):
        U1 = U.clone().requires_grad_(True)
        w1 = w.clone().requires_grad_(True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        L = loss(U1, w1)
        L.backward()
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    h = 1e-6
    dU = torch.randn(U.shape, generator=gen, device=dev, dtype=torch.complex128)
    dw = torch.randn(w.shape, generator=gen, device=dev, dtype=torch.float64)
    with torch.no_grad():
        fdU = float((loss(U + h * dU, w) - loss(U - h * dU, w)) / (2 * h))
        fdw = float((loss(U, w + h * dw) - loss(U, w - h * dw)) / (2 * h))
    anU = float((U1.grad.conj() * dU).real.sum())
    anw = float((w1.grad * dw).sum())
    line = {"metric": "correlator-loss gradient (dL/dw, dL/dU) 24^3x48 Ne=100", "value": 1.0 / min(times[1:]),
            "unit": "loss+gradient evaluations/s", "seconds": min(times[1:]), "loss": float(L.detach()),
            "fd_check": {"h": h, "dU_directional": [anU, fdU], "dw_directional": [anw, fdw],
                         "rel_err_U": abs(anU - fdU) / max(abs(fdU), 1e-30),
                         "rel_err_w": abs(anw - fdw) / max(abs(fdw), 1e-30)},
            "data": "synthetic: links exp(i 0.3 A), Gaussian vectors and perambulator [48,4,4,100,100], "
                    "w ~ U(0.5, 1.5), sigma = 1"}
    if emit:
        print(json.dumps(line), flush=True)
    return line


# FP64 flops of one stout link update (a complex multiply-add = 8 flops, a 3x3 complex product 216):
# four staples of two products (1728) and their sum (72), rho C U^dag (234), the anti-Hermitian
# traceless projection (~36), Q^2 (216), Re tr Q^3 (72), f0 + f1 Q + f2 Q^2 (132), exp(iQ) U (216):
# about 2.7e3, not counting the scalar sqrt / acos / sincos of the Cayley-Hamilton coefficients
STOUT_FLOP_PER_LINK = 2.7e3


def bench_stout(latt, dev, timed, no_cpu, U=None):
    """One stout smearing step (rho = 0.1) of the spatial links of ``latt``: the
    library's kernel, the reference's own CUDA kernel on the same links (when
    ``oracle/_ref`` holds it), and the oracle's numpy form on one timeslice.
    ``U``: device links [3, Lt, Lz, Ly, Lx, 3, 3] to smear (a copy is taken;
    synthetic ones otherwise)."""
    import numpy as np
    import torch

    from easydistillation_gb300.generator.elemental import links_to_device
    from easydistillation_gb300.stout import stout_smear_

    if U is None:
        gauge, _ = make_inputs(latt, 1, distinct_t=4)
        U = links_to_device(gauge, latt, dev)
    else:
        gauge = None
        U = U[:3].clone()
    Lx, Ly, Lz, Lt = latt
    nlinks = 3 * Lx * Ly * Lz * Lt
    sec = timed(lambda: stout_smear_(U, latt, 1, 0.1), 5)
    stout = {"links_per_s": nlinks / sec, "seconds_per_step": sec,
             "fp64_tflops_est": nlinks * STOUT_FLOP_PER_LINK / sec / 1e12, "fp64_peak_tflops": FP64_PEAK_TFLOPS,
             "workload": f"{Lx}x{Ly}x{Lz} x {Lt} spatial links, one step, rho 0.1"}
    from oracle import ref_kernels

    if os.path.exists(ref_kernels.STOUT_CUBIN):
        # the reference's kernel with its driver loop (lattice/generator/eigenvector.py:197-199):
        # U_in = U.copy(); kernel(U, U_in, ...)
        rk = ref_kernels.RefStout()
        U_in = torch.empty_like(U)
        stream = torch.cuda.current_stream().cuda_stream

        def ref_step():
            U_in.copy_(U)
            rk.step(U, U_in, 0.1, latt, stream)

        rsec = timed(ref_step, 5)
        stout["reference_cuda_kernel"] = {
            "links_per_s": nlinks / rsec, "seconds_per_step": rsec, "speedup_of_library": rsec / sec,
            "what": "lattice/generator/stout_smear.cu compiled unmodified for sm_103a, grid (V3, 3) x block (Lt), "
                    "with the reference's copy of the field before each step"}
        del U_in
    else:
        stout["reference_cuda_kernel"] = {"unavailable": "oracle/_ref/stout_smear_ref.cubin was not built"}
    if not no_cpu and gauge is not None:
        from oracle import restatement as R

        U1 = np.ascontiguousarray(gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, :1])
        t0 = time.perf_counter()
        R.stout_smear(U1, 1, 0.1)
        cdt = time.perf_counter() - t0
        stout["cpu_baseline"] = {"links_per_s": 3 * Lx * Ly * Lz / cdt, "kind": "port", "cores": 1,
                                 "sample": "oracle numpy stout step on one timeslice"}
    del U
    return stout


def bench_correlators(dev, timed):
    """The two-point correlator of ``lattice/correlator/one_particle.py:12-77``
    at 48 timeslices, Ne = 100, gamma_5 (every source), and its
    eigenvector-resolved profile (``:80-135``, one source, every sink time)
    with its diagonal, on the library's kernels; synthetic complex Gaussian
    perambulator and elementals."""
    import torch

    from easydistillation_gb300.correlator import _source_terms, gamma, twopoint_assembled

    out = {}
    Lt, Ne = 48, 100
    g = torch.Generator(device=dev).manual_seed(4005)
    peram = torch.complex(torch.randn((Lt, Lt, 4, 4, Ne, Ne), generator=g, device=dev, dtype=torch.float64),
                          torch.randn((Lt, Lt, 4, 4, Ne, Ne), generator=g, device=dev, dtype=torch.float64))
    el = torch.complex(torch.randn((1, Lt, Ne, Ne), generator=g, device=dev, dtype=torch.float64),
                       torch.randn((1, Lt, Ne, Ne), generator=g, device=dev, dtype=torch.float64))
    ops = [(gamma(15, dev)[None], el)]
    sec = timed(lambda: twopoint_assembled(ops, peram, range(Lt), Lt), 2)
    out["twopoint"] = {"correlators_per_s": 1.0 / sec, "seconds": sec,
                       "workload": "48 timeslices, Ne=100, gamma_5, all 48 sources"}
    # the eigenvector-resolved profile of one source at every sink time (ed_twopoint_profile) and its diagonal
    tau0 = peram[0].contiguous()
    psec = timed(lambda: _source_terms(tau0, tau0, ops, 0, list(range(Lt)), "profile"), 3)
    dsec = timed(lambda: _source_terms(tau0, tau0, ops, 0, list(range(Lt)), "diagonal"), 3)
    # gamma_5: 16 left blocks and 4 right blocks of 4 Ne^3 complex multiply-adds per sink time
    pflop = Lt * (16 + 16) * Ne ** 3 * 8.0
    out["twopoint_profile"] = {"seconds_per_source": psec, "fp64_tflops": pflop / psec / 1e12,
                               "diagonal_seconds_per_source": dsec,
                               "workload": "one source, 48 sink times, Ne=100, gamma_5, [48, Ne, Ne] out"}
    del peram, el
    torch.cuda.empty_cache()
    return out


def run_secondary(args):
    """Secondary measurement (``--secondary``) of the components beside the
    hot path, each timed with CUDA events after a warm-up run:

    * stout smearing (``lattice/generator/stout_smear.cu:159-245``), 32^3 x 64
      spatial links, rho = 0.1: links/s and the FP64 rate from the 2.7 kflop
      per link counted above, beside the reference's own CUDA kernel
      (compiled unmodified into ``oracle/_ref`` where the reference's sources
      were present) on the same links and GPU, each with the reference's
      driver loop around it (copy the field, one out-of-place step); the
      oracle's numpy form on one timeslice as the CPU baseline;
    * DisplacementElementalGenerator.calc, 24^3, Ne = 100, distance 2, 7
      momenta, FP64 and f16x3: timeslices/s;
    * the two-point correlator of ``lattice/correlator/one_particle.py:12-77``
      at 48 timeslices, Ne = 100, gamma_5, summed over all 48 sources:
      correlators/s;
    * loading a 32^3 x 64 ILDG gauge file (big-endian complex128, 1.2 GB) into
      the generators' device links: the host conversion (memory map, astype,
      pinned copy, upload, transpose; ``lattice/filedata/ildg.py:70``) against
      the stored bytes uploaded and converted on the device
      (``IldgFileData.links_to_device``), wall-clock from the page cache, and
      the decode kernel alone against the HBM roofline (27 complex128 read and
      written per site)."""
    import numpy as np
    import torch

    from easydistillation_gb300 import DisplacementElementalGenerator
    from easydistillation_gb300.correlator import gamma, twopoint_assembled
    from easydistillation_gb300.generator.elemental import links_to_device
    from easydistillation_gb300.insertion import mom_dict_to_list
    from easydistillation_gb300.stout import stout_smear_

    dev = torch.device("cuda", 0)
    timed = event_seconds
    out = {}
    # stout smearing
    out["stout"] = bench_stout([32, 32, 32, 64], dev, timed, args.no_cpu)
    # displacement elementals
    latt = [24, 24, 24, 8]
    V3 = 24 ** 3
    gauge, evecs = make_inputs(latt, 100, distinct_t=4)

    class _D:
        def __init__(self, a):
            self.a, self.file = a, "mem"

        def __getitem__(self, k):
            return self.a[k]

    class _Src:
        def __init__(self, a, Ne=None):
            self.d, self.Ne = _D(a), Ne

        def load(self, key):
            return self.d

    ev = np.stack([evecs[t % len(evecs)].reshape(100, 24, 24, 24, 3) for t in range(latt[3])])
    disp = {}
    for prec in ("fp64", "f16x3"):
        gen = DisplacementElementalGenerator(latt, _Src(gauge), _Src(ev, 100), 2, mom_dict_to_list(3)[:7],
                                             precision=prec, device=dev)
        gen.load("bench")
        sec = timed(lambda: [gen.calc(t) for t in range(4)], 2) / 4
        disp[prec] = {"timeslices_per_s": 1.0 / sec}
    out["displacement_elemental"] = dict(disp, workload="24^3, Ne=100, distance 2, 7 momenta")
    out.update(bench_correlators(dev, timed))
    # ILDG gauge file -> device links
    out["gauge_load"] = bench_gauge_load(dev, timed)
    print(json.dumps({"metric": "secondary components", **out}), flush=True)


def event_seconds(fn, reps):
    """Seconds per call of ``fn`` by CUDA events on the current stream, after
    one untimed call, with a synchronize on both sides."""
    import torch

    fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / 1e3 / reps


def run_gauge_load(args):
    """Secondary measurement (``--gauge-load``): only the ILDG gauge-file line
    of ``--secondary``."""
    import torch

    dev = torch.device("cuda", 0)
    print(json.dumps({"metric": "ILDG gauge file -> device links",
                      "gauge_load": bench_gauge_load(dev, event_seconds)}), flush=True)


def bench_gauge_load(dev, timed):
    import shutil
    import tempfile

    import torch

    from easydistillation_gb300.generator.elemental import links_to_device
    from easydistillation_gb300.ops import decode_links
    from easydistillation_gb300.preset import GaugeFieldIldg, pinned_bytes, write_ildg

    latt = [32, 32, 32, 64]
    Lx, Ly, Lz, Lt = latt
    sites = Lx * Ly * Lz * Lt
    tmp = tempfile.mkdtemp(prefix="ed_gauge_")
    try:
        if shutil.disk_usage(tmp).free < 4 * sites * 36 * 16:
            return {"skipped": "not enough free disk space for a 1.2 GB file"}
        gauge, _ = make_inputs(latt, 1, distinct_t=4)
        write_ildg(os.path.join(tmp, "cfg.lime"), gauge, latt)
        del gauge
        data = GaugeFieldIldg(tmp + "/", ".lime", [Lt, Lz * Ly * Lx, 4, 3, 3]).load("cfg")

        def wall(fn, reps=2):
            best = None
            for _ in range(reps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                r = fn()
                torch.cuda.synchronize()
                dt = time.perf_counter() - t0
                best = dt if best is None else min(best, dt)
                del r
            return best

        host = wall(lambda: links_to_device(data[:], latt, dev))
        device = wall(lambda: data.links_to_device(latt, dev))
        ref, got = links_to_device(data[:], latt, dev), data.links_to_device(latt, dev)
        same = bool(torch.equal(ref, got))
        del ref, got
        raw = pinned_bytes(data.raw(slice(None), copy=False)).to(dev)
        sec = timed(lambda: decode_links(raw, ">c16", latt), 5)
        nbytes = sites * 27 * 16 * 2
        peaks = load_peaks()
        pk, src = (peaks["hbm_gbs"], "measured") if "hbm_gbs" in peaks else (6800.0, "fallback")
        return {"host_convert_s": host, "device_decode_s": device, "speedup": host / device,
                "identical": same, "decode_kernel_ms": sec * 1e3, "decode_kernel_gbs": nbytes / sec / 1e9,
                "decode_kernel_hbm_frac": nbytes / sec / 1e9 / pk, "hbm_peak_gbs": pk, "hbm_peak_source": src,
                "workload": "32^3 x 64 ILDG file (1.2 GB, big-endian complex128) -> [3, Lt, Lz, Ly, Lx, 3, 3] "
                            "complex128 device links; wall-clock best of 2, file in the page cache"}
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def run_stencil(args):
    """Secondary measurement (``--stencil``): the HBM roofline of the Laplacian
    kernels alone (the lines ``bench_stencil`` adds to the main JSON line), at
    ``--lattice`` (default 32^3 x 64) on 4 distinct timeslices of links tiled
    over Lt."""
    import torch

    from easydistillation_gb300.generator.elemental import links_to_device

    latt = [int(v) for v in args.lattice.split(",")] if args.lattice else LATT
    dev = torch.device("cuda", 0)
    gauge, _ = make_inputs(latt, 1, distinct_t=4)
    U = links_to_device(gauge, latt, dev)
    print(json.dumps({"metric": "laplacian HBM roofline", "stencil_roofline": bench_stencil(U, latt, dev)}),
          flush=True)


def run_eigen(args):
    """Secondary measurement (``--eigen``): EigenvectorGenerator.calc_batch on
    ``--eigen-batch`` timeslices at ``--lattice`` (default 24^3 x 64, Ne from
    ``--ne``, tol 1e-10), FP64 or FP32 stencil, after one untimed solve of the
    same batch (``--warmup 0`` skips it); the oracle's scipy/ARPACK eigensolve
    of one timeslice on the host cores with ``--eigen-cpu``."""
    import torch

    from easydistillation_gb300 import EigenvectorGenerator

    latt = [int(v) for v in args.lattice.split(",")] if args.lattice else [24, 24, 24, 64]
    Ne = args.ne
    gauge, _ = make_inputs(latt, 1, distinct_t=max(args.eigen_batch, 1))

    class _G:
        def __init__(self, a):
            self.a = a
            self.file = "mem"

        def __getitem__(self, k):
            return self.a[k]

    class _Src:
        def load(self, key):
            return _G(gauge)

    gen = EigenvectorGenerator(latt, _Src(), Ne, 1e-10, stencil_precision=args.eigen_precision, ncv=args.eigen_ncv,
                               gs_precision=args.eigen_gs)
    gen.load("bench")
    ts = list(range(args.eigen_batch))
    kw = {}
    if args.eigen_poly > 0:
        # lambda_cut: 15 % above the largest wanted eigenvalue, from a first plain solve of one timeslice
        _, ev0 = gen.calc_batch(ts[:1])
        kw = {"polynomial_degree": args.eigen_poly, "lambda_cut": 1.15 * float(ev0[0, -1])}
    if args.warmup > 0:
        gen.calc_batch(ts, **kw)  # one untimed solve of the same call: first-use setup of kernels and libraries
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    evecs, evals = gen.calc_batch(ts, **kw)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    line = {"metric": f"eigensolve timeslices/s {latt[0]}^3 Ne={Ne} tol 1e-10", "value": len(ts) / dt,
            "unit": "timeslices/s", "seconds": dt, "batch": len(ts), "stencil_precision": args.eigen_precision,
            "gs_precision": args.eigen_gs,
            "polynomial_degree": args.eigen_poly, "ncv": gen.ncv,
            "stats": gen.last_stats, "lowest_evals_t0": [float(v) for v in evals[0, :3].cpu()]}
    if args.eigen_cpu:
        from oracle import restatement as R

        U = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0]
        t1 = time.perf_counter()
        _, ev = R.eigensolve(U, latt, Ne, 1e-10)
        cdt = time.perf_counter() - t1
        line["cpu_baseline"] = {"value": 1.0 / cdt, "unit": "timeslices/s", "kind": "port",
                                "cores": len(os.sched_getaffinity(0)), "sample": "one timeslice, scipy eigsh",
                                "max_eval_diff": float(abs(ev - evals[0].cpu().numpy()).max())}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.eigen:
        run_eigen(args)
        return
    if args.mixed:
        run_mixed(args)
        return
    if args.grad:
        run_grad(args)
        return
    if args.stencil:
        run_stencil(args)
        return
    if args.secondary:
        run_secondary(args)
        return
    if args.stout:
        import torch

        latt = [int(v) for v in args.lattice.split(",")] if args.lattice else LATT
        line = {"metric": "stout smearing links/s",
                **bench_stout(latt, torch.device("cuda", 0), event_seconds, args.no_cpu)}
        print(json.dumps(line), flush=True)
        return
    if args.gauge_load:
        run_gauge_load(args)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        n = str(len(os.sched_getaffinity(0)))
        for var in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS"):
            os.environ.setdefault(var, n)
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        torch.distributed.init_process_group("nccl")
    run_ours(args, rank, world)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
