"""The reference's own CUDA kernels, compiled from its source tree and launched
through the CUDA driver API (test infrastructure, like the rest of ``oracle/``).

``lattice/generator/stout_smear.cu`` is the only CUDA code in the reference
(CuPy compiles and launches it in ``EigenvectorGenerator._stout_smear_cuda_kernel``,
``lattice/generator/eigenvector.py:192-201``).  ``build_ref()`` compiles it here,
unmodified, through ``oracle/ref_kernel/stout_launcher.cu`` into
``oracle/_ref/stout_smear_ref.cubin`` (sm_103a device code, so the prebuilt
file also runs on machines without the reference sources); ``RefStout`` loads
that cubin into the current CUDA context and runs one smearing step with the
reference's launch geometry.  Used by the tests and by ``bench.py --secondary``
to compare the library's stout kernel with the reference's on the same GPU.
"""

from __future__ import annotations

import ctypes
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
STOUT_CUBIN = os.path.join(REF_DIR, "stout_smear_ref.cubin")
REFERENCE_ROOT = os.environ.get("ED_REFERENCE_ROOT", "/root/reference")
STOUT_SRC = os.path.join(REFERENCE_ROOT, "lattice", "generator", "stout_smear.cu")


def build_ref(force: bool = False) -> bool:
    """Compile the reference stout kernel into ``oracle/_ref`` when its source
    tree is present; returns whether the cubin exists afterwards."""
    if not os.path.exists(STOUT_SRC):
        return os.path.exists(STOUT_CUBIN)
    if not force and os.path.exists(STOUT_CUBIN) and os.path.getmtime(STOUT_CUBIN) >= max(
            os.path.getmtime(STOUT_SRC), os.path.getmtime(os.path.join(HERE, "ref_kernel", "stout_launcher.cu")),
            os.path.getmtime(os.path.join(HERE, "ref_kernel", "cupy", "complex.cuh"))):
        return True
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    os.makedirs(REF_DIR, exist_ok=True)
    cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
           "-I", os.path.join(HERE, "ref_kernel"), f'-DED_REF_STOUT_CU="{STOUT_SRC}"',
           os.path.join(HERE, "ref_kernel", "stout_launcher.cu"), "-o", STOUT_CUBIN]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on the reference stout kernel:\n{r.stdout}\n{r.stderr}")
    return True


class RefStout:
    """One step of the reference's stout smearing kernel on device buffers
    ``[3, Lt, Lz, Ly, Lx, 3, 3]`` complex128 (out of place)."""

    def __init__(self):
        if not os.path.exists(STOUT_CUBIN):
            raise FileNotFoundError(STOUT_CUBIN)
        self._cuda = ctypes.CDLL("libcuda.so.1")
        self._mod = ctypes.c_void_p()
        self._check(self._cuda.cuModuleLoad(ctypes.byref(self._mod), STOUT_CUBIN.encode()), "cuModuleLoad")
        self._fn = ctypes.c_void_p()
        self._check(self._cuda.cuModuleGetFunction(ctypes.byref(self._fn), self._mod, b"ed_ref_stout_smear_f64"),
                    "cuModuleGetFunction")

    def __del__(self):
        mod = getattr(self, "_mod", None)
        if mod is not None and mod.value:
            try:
                self._cuda.cuModuleUnload(mod)
            except Exception:
                pass
            self._mod = None

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUDA driver error {rc}")

    def step(self, U_out, U_in, rho: float, latt, stream: int = 0) -> None:
        Lx, Ly, Lz, Lt = (int(v) for v in latt)
        assert U_out.dtype == U_in.dtype and U_in.numel() == 3 * Lt * Lz * Ly * Lx * 9
        assert U_out.is_contiguous() and U_in.is_contiguous() and U_out.data_ptr() != U_in.data_ptr()
        vals = [ctypes.c_void_p(U_out.data_ptr()), ctypes.c_void_p(U_in.data_ptr()), ctypes.c_double(rho),
                ctypes.c_int(Lx), ctypes.c_int(Ly), ctypes.c_int(Lz), ctypes.c_int(Lt)]
        params = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in vals])
        # grid (Lx*Ly*Lz, 3), block (Lt): lattice/generator/eigenvector.py:199
        self._check(self._cuda.cuLaunchKernel(self._fn, ctypes.c_uint(Lx * Ly * Lz), ctypes.c_uint(3),
                                              ctypes.c_uint(1), ctypes.c_uint(Lt), ctypes.c_uint(1),
                                              ctypes.c_uint(1), ctypes.c_uint(0), ctypes.c_void_p(stream), params,
                                              None), "cuLaunchKernel")
