"""Measurement aids for bench.py and the ncu captures under profiles/ (not part of the library).

* ``fma_probe.cu`` -- the FMA issue-rate probe that gives the FP64 roofline beside HBM;
  ``build()`` compiles it into ``_build/libgsa_probe.so`` and ``fma_rate()`` runs it.
* ``profile_cases.py`` -- runs one benchmark workload a few times for a profiler to capture.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(HERE, "fma_probe.cu")
_SO = os.path.join(HERE, "_build", "libgsa_probe.so")
_lib = None


def build() -> str:
    """Compile the probe for sm_103a (incremental on modification time)."""
    os.makedirs(os.path.dirname(_SO), exist_ok=True)
    if os.path.exists(_SO) and os.path.getmtime(_SO) >= os.path.getmtime(_SRC):
        return _SO
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    tmp = _SO + f".tmp{os.getpid()}"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-shared",
                    "-Xcompiler", "-fPIC", "--cudart", "static", "-o", tmp, _SRC], check=True)
    os.replace(tmp, _SO)
    return _SO


def fma_rate(stream_ptr: int, dtype: str = "f64", iters: int = 1 << 14) -> float:
    """FMAs per second the GPU retires (8 independent chains per thread, 2048 threads per SM)."""
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        _lib.probe_fma_rate.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int64,
                                        ctypes.POINTER(ctypes.c_double)]
        _lib.probe_fma_rate.restype = ctypes.c_int
    out = ctypes.c_double(0.0)
    rc = _lib.probe_fma_rate(ctypes.c_void_p(stream_ptr), 0 if dtype == "f32" else 1, iters, ctypes.byref(out))
    if rc:
        raise RuntimeError(f"probe_fma_rate failed ({rc})")
    return out.value
