"""Generate the golden fixtures by running the reference's own numpy path.

Run in a container that has the EasyDistillation sources (read-only is fine):

    python tests/golden/make_golden.py [path/to/EasyDistillation]

The reference package imports ``mpi4py`` through its work-queue module
(``lattice/dispatch.py:6``); that module is off the hot path, so a stub is
placed in ``sys.modules`` before the import.  The reference numpy backend is
selected (``lattice/backend.py:14-33``) and the public generator classes are
driven through small in-memory ``GaugeField``/``Eigenvector`` adaptors that
expose the ``load(key)[...]`` protocol of ``lattice.preset``.

Every fixture stores its inputs next to the reference outputs, so the tests
need neither the reference sources nor this script at run time.
"""

from __future__ import annotations

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from oracle.restatement import synthetic_gauge, random_colour_vectors  # noqa: E402


def import_reference(ref_root: str):
    stub = types.ModuleType("mpi4py")
    stub.MPI = types.SimpleNamespace(COMM_WORLD=None)
    sys.modules.setdefault("mpi4py", stub)
    sys.path.insert(0, ref_root)
    import lattice  # noqa: F401

    lattice.set_backend("numpy")
    return lattice


class _Data:
    def __init__(self, arr, name):
        self.arr = arr
        self.file = name
        self.sizeInByte = arr.nbytes
        self.timeInSec = 1e-3

    def __getitem__(self, key):
        return np.asarray(self.arr[key]).copy()


class MemGauge:
    """In-memory stand-in for a ``lattice.preset.GaugeField``."""

    def __init__(self, arr):
        self.data = _Data(arr, "memory-gauge")

    def load(self, key):
        return self.data


class MemEigen:
    """In-memory stand-in for a ``lattice.preset.Eigenvector``."""

    def __init__(self, arr, Ne):
        self.Ne = Ne
        self.data = _Data(arr, "memory-eigenvector")

    def load(self, key):
        return self.data


def main(ref_root: str):
    lattice = import_reference(ref_root)
    from lattice.generator.eigenvector import _Laplacian
    from lattice.insertion.derivative import derivative
    from lattice.insertion.mom_dict import mom_dict_to_list
    from lattice.insertion.phase import MomentumPhase

    out = {}

    # --- metadata -------------------------------------------------------
    np.savez_compressed(
        os.path.join(HERE, "metadata.npz"),
        derivative=np.array([list(derivative(n)) + [-1] * (2 - len(derivative(n))) for n in range(13)]),
        mom3=np.array(mom_dict_to_list(3)),
        mom9=np.array(mom_dict_to_list(9)),
        mom_default=np.array(mom_dict_to_list()),
    )

    # --- Laplacian on random vectors (two lattices, incl. an L=2 axis) --
    for tag, latt, eps, seed in (("443", [4, 4, 4, 2], 0.3, 11), ("642", [6, 4, 2, 1], 0.1, 12)):
        Lx, Ly, Lz, Lt = latt
        g = synthetic_gauge(latt, eps, seed)
        U = g.transpose(4, 0, 1, 2, 3, 5, 6)[:3, 0].copy()
        U_dag = U.transpose(0, 1, 2, 3, 5, 4).conj()
        rng = np.random.default_rng(seed + 100)
        n = Lz * Ly * Lx * 3
        F = rng.standard_normal((n, 3)) + 1j * rng.standard_normal((n, 3))
        LF = _Laplacian(F, U, U_dag, latt)
        np.savez_compressed(os.path.join(HERE, f"laplacian_{tag}.npz"), latt=latt, gauge=g, F=F, LF=LF)

    # --- momentum phases -------------------------------------------------
    latt = [4, 6, 2, 1]
    mp = MomentumPhase(latt)
    moms = mom_dict_to_list(3)[:7] + [(0, 1, 2), (1, 1, 2)]
    np.savez_compressed(
        os.path.join(HERE, "phase_462.npz"),
        latt=latt,
        moms=np.array(moms),
        phase=np.stack([mp.get(tuple(p)) for p in moms]),
    )

    # --- elementals through the public generator -------------------------
    cases = [
        # tag, latt, eps, seed, Ne, num_nabla, momenta, t, dilution
        ("n2_test7", [4, 4, 4, 2], 0.3, 21, 6, 2,
         [(0, 0, 0), (0, 0, 1), (0, 1, 1), (1, 1, 1), (0, 0, 2), (0, 1, 2), (1, 1, 2)], 1, None),
        ("n1_mom27", [4, 4, 4, 1], 0.3, 22, 4, 1, mom_dict_to_list(3), 0, None),
        ("n0_mom7", [4, 4, 2, 1], 0.1, 23, 5, 0, mom_dict_to_list(3)[:7], 0, None),
        ("n2_blend", [4, 4, 4, 1], 0.3, 24, 6, 2, mom_dict_to_list(3)[:3], 0, ([4, 5], 3)),
    ]
    for tag, latt, eps, seed, Ne, nn, moms, t, dil in cases:
        Lx, Ly, Lz, Lt = latt
        g = synthetic_gauge(latt, eps, seed)
        evec = np.stack([random_colour_vectors(Ne, latt, seed + 1000 + tt) for tt in range(Lt)])
        gen = lattice.ElementalGenerator(
            latt, MemGauge(g), MemEigen(evec, Ne), nn, moms, dilution=dil, is_blending=dil is not None
        )
        gen.load("mem")
        E = gen.calc(t).copy()
        np.savez_compressed(
            os.path.join(HERE, f"elemental_{tag}.npz"),
            latt=latt, gauge=g, evec=evec, num_nabla=nn, moms=np.array(moms), t=t, E=E,
            dil_tot=np.array(dil[0] if dil else []), dil_used=np.array(dil[1] if dil else 0),
        )

    # --- displacement elemental -------------------------------------------
    latt = [4, 4, 4, 1]
    g = synthetic_gauge(latt, 0.3, 31)
    evec = random_colour_vectors(4, latt, 1031)[None]
    moms = mom_dict_to_list(3)[:3]
    gen = lattice.DisplacementElementalGenerator(latt, MemGauge(g), MemEigen(evec, 4), 2, moms)
    gen.load("mem")
    E = gen.calc(0).copy()
    np.savez_compressed(os.path.join(HERE, "displacement_d2.npz"), latt=latt, gauge=g, evec=evec, moms=np.array(moms), E=E)

    # --- eigensolve + stout smearing through EigenvectorGenerator --------
    latt = [4, 4, 4, 2]
    g = synthetic_gauge(latt, 0.3, 41)
    gen = lattice.EigenvectorGenerator(latt, MemGauge(g), 8, 1e-10)
    gen.load("mem")
    evecs0, evals0 = gen.calc(0)
    gen.stout_smear(2, 0.12)
    smeared = gen._U[:3].copy()
    evecs1, evals1 = gen.calc(1)
    np.savez_compressed(
        os.path.join(HERE, "eigen_443.npz"),
        latt=latt, gauge=g, Ne=8, tol=1e-10,
        evecs0=evecs0, evals0=np.asarray(evals0), smeared=smeared, evecs1=evecs1, evals1=np.asarray(evals1),
    )
    print("golden fixtures written to", HERE)


def make_ildg_fixture(ref_root: str):
    """A small ILDG file written by this package's writer and read back by the
    reference's own reader (lattice/filedata/ildg.py), pinning the format."""
    lattice = import_reference(ref_root)
    from easydistillation_gb300.preset import write_ildg

    latt = [2, 4, 2, 2]
    g = synthetic_gauge(latt, 0.3, 51)
    path = os.path.join(HERE, "small.lime")
    write_ildg(path, g, latt)
    Lx, Ly, Lz, Lt = latt
    ref = lattice.GaugeFieldIldg(os.path.join(HERE, "small"), ".lime", [Lt, Lz, Ly, Lx, 4, 3, 3]).load("")
    np.savez_compressed(os.path.join(HERE, "ildg_small.npz"), latt=latt, gauge=g, ref_read=ref[:],
                        ref_slice=ref[1, :, 0])


def make_config0_chain(ref_root: str):
    """The reference's own chain at the plain-FP64 CPU configuration: 4^3 x 8,
    links exp(i 0.1 A) (seed 1000), EigenvectorGenerator (Ne = 20, tol 1e-10,
    ARPACK) on all 8 timeslices, and its eigenvectors fed to
    ElementalGenerator(num_nabla = 1, the 7 momenta with |p|^2 <= 1)."""
    lattice = import_reference(ref_root)
    from lattice.insertion.mom_dict import mom_dict_to_list

    latt = [4, 4, 4, 8]
    Ne, tol = 20, 1e-10
    g = synthetic_gauge(latt, 0.1, 1000)
    eig = lattice.EigenvectorGenerator(latt, MemGauge(g), Ne, tol)
    eig.load("mem")
    evecs, evals = [], []
    for t in range(latt[3]):
        v, lam = eig.calc(t)
        evecs.append(np.asarray(v))
        evals.append(np.asarray(lam))
    evecs = np.stack(evecs)
    moms = mom_dict_to_list(3)[:7]
    gen = lattice.ElementalGenerator(latt, MemGauge(g), MemEigen(evecs, Ne), 1, moms)
    gen.load("mem")
    E = np.stack([gen.calc(t).copy() for t in range(latt[3])])
    np.savez_compressed(os.path.join(HERE, "config0_chain.npz"), latt=latt, gauge=g, Ne=Ne, tol=tol,
                        evecs=evecs, evals=np.stack(evals), moms=np.array(moms), E=E)


def make_correlator_fixture(ref_root: str):
    """lattice.correlator.one_particle.twopoint / twopoint_profile on synthetic
    elementals [Nderiv, Nmom, Lt, Ne, Ne] and perambulators
    [Lt, Lt, 4, 4, Ne, Ne] (complex Gaussian), for operators built with the
    reference's own Operator class (several parts, derivative and momentum
    combinations, and the gamma 5 / 13 sign convention of its constructor)."""
    import_reference(ref_root)
    from lattice.correlator.one_particle import twopoint, twopoint_profile
    from lattice.insertion import InsertionRowMom, Operator

    Lt, Ne, usedNe, nder, nmom = 6, 4, 3, 4, 3
    rng = np.random.default_rng(61)

    def cgauss(*shape):
        return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)

    elem = cgauss(nder, nmom, Lt, Ne, Ne)
    peram = cgauss(Lt, Lt, 4, 4, Ne, Ne)
    peram_bw = cgauss(Lt, Lt, 4, 4, Ne, Ne)
    ops_spec = [
        # (name, [(row, momentum index)], coefficients); row = [gamma, [(coeff, derivative), ...], ...]
        ("g5", [([15, [(1.0, 0)]], 0)], [1.0]),
        ("nabla", [([1, [(1.0, 1), (-0.5, 2)], 8, [(0.25, 0)]], 1), ([5, [(1.0, 3)]], 2)], [1.0, 0.7]),
        ("g13_mom", [([13, [(2.0, 2)]], 1)], [-1.5]),
    ]
    ops = [Operator(n, [InsertionRowMom(r, m) for r, m in rows], cs) for n, rows, cs in ops_spec]
    ts = [0, 2, 5]
    dts = [0, 1, 3, 4]
    res = {
        "tp": twopoint(ops, elem, peram, ts, Lt, usedNe),
        "tp_all_src": twopoint(ops, elem, peram, ts, Lt, usedNe, is_sum_over_source_t=False),
        "tp_bw": twopoint(ops, elem, peram, ts, Lt, usedNe, perambulator_bw=peram_bw),
        "tp_fullne": twopoint(ops, elem, peram, ts, Lt, Ne),
        "prof": twopoint_profile(ops, elem, peram, ts, dts, usedNe),
        "prof_diag": twopoint_profile(ops, elem, peram, ts, dts, usedNe, is_diagonal=True),
        "prof_all_src": twopoint_profile(ops, elem, peram, ts, dts, usedNe, is_sum_over_source_t=False),
        "prof_bw_fullt": twopoint_profile(ops, elem, peram, ts, list(range(Lt)), usedNe, perambulator_bw=peram_bw),
    }
    spec = np.array(repr(ops_spec))
    np.savez_compressed(os.path.join(HERE, "correlator.npz"), Lt=Lt, Ne=Ne, usedNe=usedNe, elem=elem, peram=peram,
                        peram_bw=peram_bw, ts=np.array(ts), dts=np.array(dts), ops_spec=spec,
                        parts=np.array(repr([op.parts for op in ops])), **res)


def make_project_su3_fixture(ref_root: str):
    """EigenvectorGenerator.project_SU3 (lattice/generator/eigenvector.py:55-65)
    on links pushed off SU(3) by 1e-3 Gaussian noise."""
    lattice = import_reference(ref_root)
    latt = [4, 4, 2, 2]
    g = synthetic_gauge(latt, 0.3, 71)
    rng = np.random.default_rng(72)
    g = g + 1e-3 * (rng.standard_normal(g.shape) + 1j * rng.standard_normal(g.shape))
    gen = lattice.EigenvectorGenerator(latt, MemGauge(g), 4, 1e-10)
    gen.load("mem")
    gen.project_SU3()
    np.savez_compressed(os.path.join(HERE, "project_su3.npz"), latt=latt, gauge=g, projected=gen._U[:3].copy())


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    main(root)
    make_ildg_fixture(root)
    make_config0_chain(root)
    make_correlator_fixture(root)
    make_project_su3_fixture(root)
