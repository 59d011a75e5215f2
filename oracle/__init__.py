"""CPU oracle for the EasyDistillation hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, in plain numpy/scipy, the reference algorithms that the
GPU library reproduces: the 3D covariant Laplacian, the covariant-derivative
chains, the momentum phases, the displaced momentum-projected elemental, the
per-timeslice eigensolve and the stout smearing step.  Each function cites the
reference file and lines it follows (paths relative to the EasyDistillation
source tree).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it, and only as the checker or as the timed CPU
baseline.  The product path (``easydistillation_gb300``) never imports it and
has no CPU fallback.

Parity pinning: the restatement is checked against golden vectors produced by
running the reference's own numpy code path (``tests/golden/make_golden.py``),
committed under ``tests/golden/``.
"""

from .restatement import *  # noqa: F401,F403
