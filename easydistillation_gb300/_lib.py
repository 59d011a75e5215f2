"""ctypes binding of ``libeasydist_gb300.so`` (the C ABI in include/easydist_gb300.h).

The library is built in-tree by :mod:`easydistillation_gb300.build`.  There is
no CPU fallback: if the shared library is missing, or a call reports a CUDA
error, the operation raises.
"""

from __future__ import annotations

import ctypes
import os
import threading

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libeasydist_gb300.so")

ED_OK = 0
ED_ERR_ARG = -1
ED_ERR_CUDA = -2
ED_ERR_UNSUPPORTED = -3
ED_ERR_WORKSPACE = -4
ED_ERR_TIMEOUT = -5

ED_C128 = 0
ED_C64 = 1
ED_DF = 2  # ed_laplacian: double-float links (ed_split_c128), complex128 vectors
ED_LANCZOS_GS_DF = 0x100  # flag OR-ed into the stencil precision of ed_lanczos_tr_ex
ED_BIG_ENDIAN = 0x10

_c = ctypes
_vp = _c.c_void_p
_ll = _c.c_longlong
_i = _c.c_int

_SIGNATURES = {
    "ed_version": ([], _i),
    "ed_last_error": ([_c.c_char_p, _c.c_size_t], _i),
    "ed_links_to_soa": ([_i, _i, _i, _i, _i, _vp, _ll, _ll, _ll, _vp, _vp], _i),
    "ed_vectors_to_planes": ([_i, _i, _i, _ll, _i, _vp, _vp, _vp], _i),
    "ed_decode_complex": ([_i, _ll, _vp, _i, _vp, _vp], _i),
    "ed_decode_links": ([_i, _ll, _vp, _vp, _vp], _i),
    "ed_vectors_from_planes": ([_i, _i, _ll, _i, _vp, _vp, _vp], _i),
    "ed_momentum_phases": ([_i, _i, _i, _c.POINTER(_i), _i, _vp, _vp], _i),
    "ed_laplacian": ([_i, _i, _i, _i, _i, _i, _vp, _vp, _ll, _vp, _ll, _vp], _i),
    "ed_split_c128": ([_ll, _vp, _vp, _vp], _i),
    "ed_stout_smear_step": ([_i, _i, _i, _i, _c.c_double, _vp, _vp, _vp], _i),
    "ed_project_su3": ([_ll, _vp, _c.c_double, _i, _vp], _i),
    "ed_covariant_derivative": ([_i, _i, _i, _i, _i, _i, _i, _vp, _vp, _vp, _vp], _i),
    "ed_elemental_plan_create": (
        [_c.POINTER(_vp), _i, _i, _i, _i, _i, _c.POINTER(_i), _i, _i],
        _i,
    ),
    "ed_elemental_plan_destroy": ([_vp], _i),
    "ed_elemental_workspace_size": ([_vp, _c.POINTER(_c.c_size_t)], _i),
    "ed_elemental_num_pairs": ([_vp, _c.POINTER(_i)], _i),
    "ed_elemental_run": ([_vp, _vp, _ll, _ll, _i, _vp, _vp, _vp, _vp, _c.c_size_t, _vp], _i),
    "ed_elemental_status": ([_vp, _vp, _c.POINTER(_i), _vp], _i),
    "ed_elemental_set_profile_events": ([_vp, _vp, _vp], _i),
    "ed_elemental_run_noalloc": ([_vp, _vp, _ll, _ll, _i, _vp, _vp, _vp, _vp], _i),
    "ed_elemental_status_noalloc": ([_vp, _c.POINTER(_i), _vp], _i),
    "ed_elemental_plan_create_batched": (
        [_c.POINTER(_vp), _i, _i, _i, _i, _i, _c.POINTER(_i), _i, _i, _i],
        _i,
    ),
    "ed_elemental_run_batch": (
        [_vp, _i, _c.POINTER(_vp), _ll, _ll, _i, _c.POINTER(_vp), _vp, _c.POINTER(_vp), _vp, _c.c_size_t, _vp],
        _i,
    ),
    "ed_elemental_run_batch_begin": (
        [_vp, _i, _c.POINTER(_vp), _ll, _ll, _i, _c.POINTER(_vp), _vp, _c.c_size_t, _vp],
        _i,
    ),
    "ed_elemental_gemm_multi": (
        [_i, _c.POINTER(_vp), _c.POINTER(_i), _c.POINTER(_vp), _c.POINTER(_c.c_size_t), _c.POINTER(_i), _vp],
        _i,
    ),
    "ed_elemental_run_batch_end": ([_vp, _i, _vp, _c.POINTER(_vp), _vp, _c.c_size_t, _vp], _i),
    "ed_link_grad": ([_i, _i, _i, _i, _i, _c.c_double, _c.c_double, _vp, _vp, _vp, _vp], _i),
    "ed_twopoint_trace": ([_i, _i, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp], _i),
    "ed_twopoint_profile": ([_i, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp], _i),
    "ed_twopoint_profile_diag": ([_i, _i, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp], _i),
    "ed_chain_adjoint": ([_i, _i, _i, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp], _i),
    "ed_parallel_transport": ([_i, _i, _i, _i, _i, _i, _vp, _vp, _vp, _vp], _i),
    "ed_mean_c128": ([_i, _ll, _ll, _vp, _vp, _vp], _i),
    "ed_pair_plan_create": (
        [_c.POINTER(_vp), _i, _i, _i, _i, _i, _c.POINTER(_i), _i, _i, _i, _i, _i],
        _i,
    ),
    "ed_pair_run": ([_vp, _vp, _vp, _vp, _c.c_size_t, _vp], _i),
    "ed_elemental_describe": ([_vp, _c.POINTER(_i), _c.POINTER(_i), _c.POINTER(_i), _c.POINTER(_i)], _i),
    "ed_laplacian_config": ([_i], _i),
    "ed_laplacian_status": ([_c.POINTER(_i), _vp], _i),
    "ed_laplacian_wait_limit": ([_c.c_longlong], _i),
    "ed_laplacian_wait_probe": ([_c.c_int], _i),
    "ed_elemental_wait_limit": ([_c.c_longlong], _i),
    "ed_elemental_wait_probe": ([_c.c_int], _i),
    "ed_elemental_factorised": ([_vp, _c.POINTER(_i), _c.POINTER(_i), _c.POINTER(_i)], _i),
    "ed_elemental_set_tuning": ([_vp, _i, _i], _i),
    "ed_arrow_eigh_workspace": ([_i, _i, _i, _c.POINTER(_c.c_size_t)], _i),
    "ed_cgs_pass": ([_i, _i, _ll, _vp, _ll, _vp, _vp, _i, _vp, _vp], _i),
    "ed_cgs_pass_df": ([_i, _i, _ll, _vp, _ll, _vp, _vp, _i, _vp, _vp, _c.c_size_t, _vp], _i),
    "ed_lanczos_workspace": ([_i, _i, _i, _i, _i, _i, _c.POINTER(_c.c_size_t)], _i),
    "ed_lanczos_tr": ([_i, _i, _i, _i, _vp, _i, _c.c_double, _i, _i, _i, _c.c_double, _vp, _vp, _c.POINTER(_i), _vp,
                       _c.c_size_t, _vp], _i),
    "ed_lanczos_workspace_ex": ([_i, _i, _i, _i, _i, _i, _i, _c.POINTER(_c.c_size_t)], _i),
    "ed_lanczos_tr_ex": ([_i, _i, _i, _i, _vp, _vp, _i, _i, _c.c_double, _i, _i, _i, _c.c_double, _vp, _vp,
                          _c.POINTER(_i), _vp, _c.c_size_t, _vp], _i),
    "ed_arrow_eigh": ([_i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _c.c_size_t, _vp], _i),
    "ed_elemental_get_tuning": ([_vp, _i, _c.POINTER(_i)], _i),
}

_lock = threading.Lock()
_lib = None


class EDError(RuntimeError):
    """A library call returned a non-zero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[ed status {code}] {msg}")
        self.code = code


def exported_symbols():
    """Names the binding expects the library to export."""
    return list(_SIGNATURES)


def lib():
    """Load the shared library (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m easydistillation_gb300.build` "
                "(there is no CPU fallback)"
            )
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(2048)
    lib().ed_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int, what: str = ""):
    if rc == ED_OK:
        return
    msg = last_error()
    if rc == ED_ERR_ARG:
        raise ValueError(f"{what}: {msg}" if what else msg)
    raise EDError(rc, f"{what}: {msg}" if what else msg)


def call(name: str, *args):
    check(getattr(lib(), name)(*args), name)


def ptr(t: torch.Tensor) -> int:
    return t.data_ptr()


def stream_handle(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def require_cuda(t: torch.Tensor, name: str):
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
