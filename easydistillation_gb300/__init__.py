"""GB300-native (sm_103a) implementation of EasyDistillation's hot path.

Drop-in generators (same constructors, ``load(key)`` and ``calc(t)`` as
``lattice.generator``):

* :class:`EigenvectorGenerator` -- lowest eigenpairs of the 3D covariant
  Laplacian per timeslice (GPU stencil kernel inside a GPU thick-restart
  Lanczos);
* :class:`ElementalGenerator` -- displaced, momentum-projected elementals
  ``E[d, p, i, j]`` (GPU covariant-derivative chains and pair contractions).

The arithmetic runs in ``libeasydist_gb300.so`` (C ABI:
``include/easydist_gb300.h``), built in-tree by
``python -m easydistillation_gb300.build``.  There is no CPU fallback.
"""

from .backend import check_QUDA, get_backend, set_backend
from .generator import DisplacementElementalGenerator, EigenvectorGenerator, ElementalGenerator
from .insertion import MomentumPhase, derivative, mom_dict_to_list, num_derivative
from .preset import (
    EigenvectorHostmem,
    EigenvectorNpy,
    EigenvectorTimeSlice,
    ElementalBinary,
    ElementalNpy,
    GaugeFieldBinary,
    GaugeFieldIldg,
    GaugeFieldTimeSlice,
    Jpsi2gammaNpy,
    PerambulatorBinary,
    PerambulatorNpy,
)

NC, NS, ND = 3, 4, 4
Nc, Ns, Nd = NC, NS, ND  # the reference's names (lattice/constant.py)

__all__ = [
    "DisplacementElementalGenerator",
    "EigenvectorGenerator",
    "ElementalGenerator",
    "MomentumPhase",
    "derivative",
    "mom_dict_to_list",
    "get_backend",
    "set_backend",
    "check_QUDA",
    "num_derivative",
    "GaugeFieldIldg",
    "GaugeFieldBinary",
    "GaugeFieldTimeSlice",
    "Jpsi2gammaNpy",
    "EigenvectorNpy",
    "EigenvectorTimeSlice",
    "EigenvectorHostmem",
    "ElementalNpy",
    "ElementalBinary",
    "PerambulatorNpy",
    "PerambulatorBinary",
    "NC",
    "NS",
    "ND",
    "Nc",
    "Ns",
    "Nd",
]
