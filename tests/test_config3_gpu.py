"""Mixed volumes at their real sizes in ONE captured graph with ONE pair-GEMM
launch: one timeslice each of 16^3 (Ne = 64), 24^3 (Ne = 128) and 32^3
(Ne = 256), links exp(i eps A) with eps 0.1 / 0.3, 4 operators x 7 momenta,
f16x3, against the plain FP64 GPU path of each volume: relative Frobenius
error <= 1e-6."""

import pytest
import torch

from oracle import restatement as R

pytestmark = pytest.mark.gpu

TOL = 1e-6


def test_mixed_real_volumes_one_graph_vs_fp64():
    from easydistillation_gb300.batch import MixedVolumeGraph, VolumeBinding
    from easydistillation_gb300.generator.elemental import links_to_device
    from easydistillation_gb300.ops import ElementalPlan

    moms = R.mom_dict_to_list(3)[:7]
    specs = [([16, 16, 16, 1], 64, 0.1, 3001), ([24, 24, 24, 1], 128, 0.3, 3002), ([32, 32, 32, 1], 256, 0.1, 3003)]
    vols = []
    for latt, Ne, eps, seed in specs:
        gauge = R.synthetic_gauge(latt, eps, seed)
        V3 = latt[0] * latt[1] * latt[2]
        gen = torch.Generator(device="cuda").manual_seed(seed)
        V = torch.complex(torch.randn((1, Ne, V3 * 3), generator=gen, device="cuda", dtype=torch.float64),
                          torch.randn((1, Ne, V3 * 3), generator=gen, device="cuda", dtype=torch.float64))
        V /= (2 * V3 * 3) ** 0.5
        vols.append(VolumeBinding(latt, Ne, links_to_device(gauge, latt, "cuda"), V, [0]))
    mv = MixedVolumeGraph(vols, 1, moms, "f16x3", max_batch=1)
    outs = [o.clone() for o in mv.run()]
    mv.check_status()
    assert mv.graph is not None
    assert mv.gemm_launches == 1  # the three volumes' pair contractions share one launch
    for (latt, Ne, eps, seed), v, out in zip(specs, vols, outs):
        V3 = latt[0] * latt[1] * latt[2]
        plan = ElementalPlan(latt, Ne, 1, moms, "fp64", tuning={"f64_tile": 3})
        ref = torch.empty((4, 7, Ne, Ne), dtype=torch.complex128, device="cuda")
        plan.run(v.links[:, 0], latt[3] * V3 * 9, 9, v.evecs[0], ref)
        err = float(torch.linalg.vector_norm(out[0] - ref) / torch.linalg.vector_norm(ref))
        assert err <= TOL, (latt, Ne, err)
        del plan
    torch.cuda.empty_cache()
