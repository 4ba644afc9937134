"""Builds the benchmark's integer-issue probe (int_issue.cu) in-tree into
bench_probe/_build/libintissue.so for sm_103a, and loads it.  The probe
measures the roofline denominator of the integer-pipe-bound sweeps; it is
measurement code, not part of the engine library."""
from __future__ import annotations

import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "int_issue.cu")
LIB = os.path.join(HERE, "_build", "libintissue.so")


def build() -> str:
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    nvcc = "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-shared",
                    "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden", "-o", LIB, SRC,
                    "-lcudart_static", "-lrt", "-ldl", "-lpthread"], check=True)
    return LIB


def probe_int_issue(device: int = 0) -> tuple[float, float, float]:
    """Measured integer lane-ops/s: (LOP3 only, IMAD only, interleaved)."""
    lib = ctypes.CDLL(build())
    lib.probe_int_issue.argtypes = [ctypes.c_int, ctypes.c_void_p]
    lib.probe_int_issue.restype = ctypes.c_int
    out = (ctypes.c_double * 3)()
    st = lib.probe_int_issue(int(device), out)
    if st != 0:
        raise RuntimeError(f"integer issue probe failed (status {st})")
    return out[0], out[1], out[2]
