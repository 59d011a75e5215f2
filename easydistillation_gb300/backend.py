"""Array type the generators return: the counterpart of ``lattice/backend.py:7-33``.

The reference keeps one process-global array module (``numpy`` or ``cupy``,
``set_backend`` / ``get_backend``) and every generator computes with it, so
its ``calc`` returns that module's arrays.  Here the arithmetic always runs
in the library's CUDA kernels; the backend only decides what ``calc`` hands
back:

* ``"torch"`` (the default): CUDA tensors, no copy;
* ``"numpy"``: host ``numpy.ndarray`` copies (the copy synchronises the
  current stream), so that a driver written against the reference's numpy
  backend, e.g. ``data = backend.zeros(...); data[t] = elemental.calc(t)``
  (``tests/test_elemental.py:37,44``), runs unchanged;
* ``"cupy"``: CuPy arrays sharing the device memory (DLPack, no copy); needs
  CuPy, like the reference's cupy backend.

``get_backend()`` returns the module itself, as the reference's does.
"""

from __future__ import annotations

_NAMES = ("torch", "numpy", "cupy")
_BACKEND = "torch"


def set_backend(backend) -> None:
    """Select the array type of the generators' results: ``"torch"``,
    ``"numpy"`` or ``"cupy"`` (a module object works too, as in the
    reference).  ValueError for anything else; ImportError when CuPy is asked
    for and missing."""
    global _BACKEND
    if not isinstance(backend, str):
        backend = getattr(backend, "__name__", str(backend))
    name = backend.lower()
    if name not in _NAMES:
        raise ValueError('backend must be "numpy", "cupy" or "torch"')
    if name == "cupy":
        import cupy  # noqa: F401  (ImportError, as the reference raises, when absent)
    _BACKEND = name


def backend_name() -> str:
    return _BACKEND


def get_backend():
    """The module of the selected backend (``torch``, ``numpy`` or ``cupy``)."""
    if _BACKEND == "numpy":
        import numpy

        return numpy
    if _BACKEND == "cupy":
        import cupy

        return cupy
    import torch

    return torch


def to_backend(x):
    """A generator result (a torch tensor) in the selected backend's array type."""
    if _BACKEND == "torch":
        return x
    if _BACKEND == "numpy":
        return x.detach().cpu().numpy()
    import cupy

    return cupy.from_dlpack(x.detach())


def check_QUDA(grid_size=None, backend="cupy", resource_path=None) -> bool:
    """Counterpart of ``lattice/backend.py:36`` (``check_QUDA``), which
    initialises PyQUDA when it is importable and reports whether it is.  The
    paths the reference sends to QUDA (the Laplacian eigensolve, stout
    smearing) run in this library's own kernels, so there is no QUDA to
    initialise: always False, and driver code written against the reference
    takes its non-QUDA branches."""
    return False
