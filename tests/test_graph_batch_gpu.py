"""CUDA-graph-captured batched elementals and mixed lattice volumes
(different Ne per volume) against per-timeslice generator runs / the oracle."""

import numpy as np
import pytest
import torch

from oracle import restatement as R
from tests.helpers import MemEigen, MemGauge, rel_err

pytestmark = pytest.mark.gpu


def _inputs(latt, Ne, eps, seed):
    gauge = R.synthetic_gauge(latt, eps, seed)
    evec = np.stack([R.random_colour_vectors(Ne, latt, seed * 3 + t) for t in range(latt[3])])
    return gauge, evec


def test_graphed_batch_replays_match_generator():
    from easydistillation_gb300 import ElementalGenerator
    from easydistillation_gb300.batch import GraphedElementalBatch

    latt = [4, 4, 4, 4]
    Ne, moms = 6, R.mom_dict_to_list(3)[:7]
    gauge, evec = _inputs(latt, Ne, 0.3, 5)
    gen = ElementalGenerator(latt, MemGauge(gauge), MemEigen(evec, Ne), 2, moms)
    gen.load("k")
    U = gen._U  # [3, Lt, ...] device
    V = torch.from_numpy(evec.reshape(latt[3], Ne, -1)).cuda()
    runner = GraphedElementalBatch(latt, Ne, 2, moms, "fp64", batch=2)
    for chunk in ([0, 1], [2, 3], [3, 1]):  # several replays of the same graph
        out = runner.run([U[:, t] for t in chunk], [V[t] for t in chunk]).cpu().numpy()
        for k, t in enumerate(chunk):
            assert rel_err(out[k], gen.calc(t).cpu().numpy()) < 1e-14
    assert runner.graph is not None


def test_mixed_volumes_f16x3_vs_oracle():
    from easydistillation_gb300.batch import VolumeGroup, run_mixed_volumes
    from easydistillation_gb300.generator.elemental import links_to_device

    moms = R.mom_dict_to_list(3)[:7]
    specs = {"small": ([4, 4, 4, 3], 8, 0.1, 11), "large": ([8, 4, 4, 2], 12, 0.3, 12)}
    groups, links, evecs, ref_in = {}, {}, {}, {}
    for name, (latt, Ne, eps, seed) in specs.items():
        gauge, evec = _inputs(latt, Ne, eps, seed)
        groups[name] = VolumeGroup(latt, Ne, list(range(latt[3])))
        links[name] = links_to_device(gauge, latt, "cuda")
        evecs[name] = torch.from_numpy(evec.reshape(latt[3], Ne, -1)).cuda()
        ref_in[name] = (gauge, evec)
    out = run_mixed_volumes(groups, links, evecs, 1, moms, "f16x3", max_batch=2)
    for name, (latt, Ne, eps, seed) in specs.items():
        gauge, evec = ref_in[name]
        U = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3]
        for t in range(latt[3]):
            ref = R.elemental(evec[t], U[:, t], latt, 1, moms)
            assert rel_err(out[name][t].cpu().numpy(), ref) < 1e-6


@pytest.mark.parametrize("mode", ["f16x3", "ozaki_i8"])
def test_graphed_factorised_modes(mode):
    """CUDA graph capture and replay of the factorised-phase GEMM (a persistent
    cooperative launch) and of the Ozaki int8 GEMM, against the oracle."""
    from easydistillation_gb300.batch import GraphedElementalBatch

    latt = [8, 4, 4, 3]
    Ne, moms = 9, R.mom_dict_to_list(3)
    gauge, evec = _inputs(latt, Ne, 0.3, 11)
    U = torch.from_numpy(gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3].copy()).cuda()
    V = torch.from_numpy(evec.reshape(latt[3], Ne, -1)).cuda()
    runner = GraphedElementalBatch(latt, Ne, 2, moms, mode, batch=2)
    assert runner.plan.factorised == (9, 3)
    Uh = gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3]
    for chunk in ([0, 1], [2, 0], [1, 2]):
        out = runner.run([U[:, t] for t in chunk], [V[t] for t in chunk]).cpu().numpy()
        for k, t in enumerate(chunk):
            ref = R.elemental(evec[t], Uh[:, t], latt, 2, moms)
            assert rel_err(out[k], ref) < 1e-6
    runner.plan.check_status()
    assert runner.graph is not None


def test_mixed_volume_graph_one_replay():
    """Two volumes with their own Ne in ONE captured graph, bound to the input
    tensors in place (repeated timeslices allowed); a second replay after the
    inputs change recomputes everything."""
    from easydistillation_gb300.batch import MixedVolumeGraph, VolumeBinding
    from easydistillation_gb300.generator.elemental import links_to_device

    moms = R.mom_dict_to_list(3)
    specs = [([8, 4, 4, 2], 10, 0.3, 31, [0, 1, 1, 0, 1]), ([4, 4, 4, 3], 6, 0.1, 32, [2, 0, 1])]
    vols, host = [], []
    for latt, Ne, eps, seed, ts in specs:
        gauge, evec = _inputs(latt, Ne, eps, seed)
        vols.append(VolumeBinding(latt, Ne, links_to_device(gauge, latt, "cuda"),
                                  torch.from_numpy(evec.reshape(latt[3], Ne, -1)).cuda(), ts))
        host.append((gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3], evec))
    mv = MixedVolumeGraph(vols, 2, moms, "f16x3", max_batch=2)
    assert mv.passes() == 3 + 2

    def check():
        outs = [o.cpu().numpy() for o in mv.run()]
        mv.check_status()
        for (latt, Ne, eps, seed, ts), (Uh, evec), out in zip(specs, host, outs):
            for k, t in enumerate(ts):
                assert rel_err(out[k], R.elemental(evec[t], Uh[:, t], latt, 2, moms)) < 1e-6

    check()
    assert mv.graph is not None
    rng = np.random.default_rng(5)
    for v, (Uh, evec) in zip(vols, host):
        evec *= np.exp(1j * rng.uniform(0, 2 * np.pi, evec.shape[:2]))[..., None, None, None, None]
        v.evecs.copy_(torch.from_numpy(evec.reshape(evec.shape[0], evec.shape[1], -1)))
    check()


@pytest.mark.parametrize("mode", ["f16x3", "tf32x3"])
def test_mixed_volumes_one_gemm_launch_per_round(mode):
    """Three volumes with their own Ne on the on-chip-phase tensor-core path
    (4 operators x 7 momenta): every round of admitted chunks contracts all
    volumes with ONE pair-GEMM launch (ed_elemental_gemm_multi).  With batches
    of 2 and 5, 3 and 4 timeslices the three rounds hold 3, 3 and 1 volumes.  Results agree
    with the oracle and are bit-identical to one GEMM launch per volume chunk
    (every tile runs the same MMA and flush sequence in either launch)."""
    from easydistillation_gb300.batch import MixedVolumeGraph, VolumeBinding
    from easydistillation_gb300.generator.elemental import links_to_device

    moms = R.mom_dict_to_list(3)[:7]
    specs = [([8, 4, 4, 3], 10, 0.3, 61, [0, 1, 2, 2, 0]), ([4, 4, 4, 2], 6, 0.1, 62, [1, 0, 1]),
             ([8, 8, 4, 2], 12, 0.3, 63, [0, 1, 1, 0])]
    vols, host = [], []
    for latt, Ne, eps, seed, ts in specs:
        gauge, evec = _inputs(latt, Ne, eps, seed)
        vols.append(VolumeBinding(latt, Ne, links_to_device(gauge, latt, "cuda"),
                                  torch.from_numpy(evec.reshape(latt[3], Ne, -1)).cuda(), ts))
        host.append((gauge.transpose(4, 0, 1, 2, 3, 5, 6)[:3], evec))
    mv = MixedVolumeGraph(vols, 1, moms, mode, max_batch=2)
    outs = [o.clone() for o in mv.run()]
    mv.check_status()
    assert mv.graph is not None and mv.gemm_launches == 3  # one launch per round
    for (latt, Ne, eps, seed, ts), (Uh, evec), out in zip(specs, host, outs):
        for k, t in enumerate(ts):
            assert rel_err(out[k].cpu().numpy(), R.elemental(evec[t], Uh[:, t], latt, 1, moms)) < 1e-6
    per_volume = MixedVolumeGraph(vols, 1, moms, mode, max_batch=2, single_launch=False)
    ref = per_volume.run()
    per_volume.check_status()
    assert per_volume.gemm_launches == 3 + 2 + 2
    for a, b in zip(outs, ref):
        assert torch.equal(a, b)


def test_gemm_multi_groups_onchip_plans_and_runs_factorised_alone():
    """ed_elemental_gemm_multi over two on-chip-phase plans and one plan on the
    left-only factorised GEMM (4 operators x 7 momenta): the two on-chip plans
    share one launch, the factorised one runs alone (2 launches), and every
    result is bit-identical to the plan's own run_batch."""
    from easydistillation_gb300.generator.elemental import links_to_device
    from easydistillation_gb300.ops import ElementalPlan, gemm_multi

    moms = R.mom_dict_to_list(3)[:7]
    specs = [([8, 4, 4, 2], 10, True), ([4, 4, 4, 2], 6, True), ([8, 8, 4, 2], 12, "left")]
    plans, ins, outs, refs = [], [], [], []
    for k, (latt, Ne, fac) in enumerate(specs):
        gauge, evec = _inputs(latt, Ne, 0.3, 70 + k)
        U = links_to_device(gauge, latt, "cuda")
        V = torch.from_numpy(evec.reshape(latt[3], Ne, -1)).cuda()
        plan = ElementalPlan(latt, Ne, 1, moms, "f16x3", batch=2, factorise=fac)
        assert (plan.factorised is not None) == (fac == "left")
        Lt, V3 = latt[3], latt[0] * latt[1] * latt[2]
        links, evs = [U[:, t] for t in range(2)], [V[t] for t in range(2)]
        ref = [torch.empty((4, 7, Ne, Ne), dtype=torch.complex128, device="cuda") for _ in range(2)]
        plan.run_batch(links, Lt * V3 * 9, 9, evs, ref)
        plans.append(plan)
        ins.append((links, Lt * V3 * 9, evs))
        outs.append([torch.full_like(r, float("nan")) for r in ref])
        refs.append(ref)
    for plan, (links, ds, evs) in zip(plans, ins):
        plan.run_batch_begin(links, ds, 9, evs)
    assert gemm_multi(plans, [2, 2, 2]) == 2
    for plan, out in zip(plans, outs):
        plan.run_batch_end(out)
    for plan, out, ref in zip(plans, outs, refs):
        assert plan.check_status() == 0
        for a, b in zip(out, ref):
            assert torch.equal(a, b)
