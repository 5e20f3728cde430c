"""Build recipe of libangelo_tcprobe.so, the test-only tensor-core probe
library (tc_probe.cu): nvcc for sm_103a with the product's flags and
headers, linked next to this file.  It is not part of libangelo_gb.so.

``build()`` rebuilds when the probe or a header it includes is newer than
the library; ``load()`` binds the C ABI declared in tc_probe.h."""
from __future__ import annotations

import ctypes
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libangelo_tcprobe.so")
SRC = os.path.join(HERE, "tc_probe.cu")

c_i32, c_vp = ctypes.c_int32, ctypes.c_void_p
SIGNATURES = {
    "angelo_probe_last_error_string": (ctypes.c_char_p, []),
    "angelo_tc_gemm_x3": (c_i32, [c_vp, c_vp, c_vp, c_i32, c_i32, c_i32, c_i32, c_i32, c_i32, c_vp,
                                  c_vp]),
    "angelo_tc_mma_rate": (c_i32, [c_i32, c_i32, c_i32, c_vp, c_vp, c_vp]),
}


def build(force: bool = False) -> str:
    from angelo_gb import build as B
    deps = [SRC, os.path.join(HERE, "tc_probe.h")] + glob.glob(os.path.join(B.CSRC, "*.cuh")) + \
        glob.glob(os.path.join(B.INCLUDE, "*.h"))
    if not force and os.path.exists(LIB) and \
            all(os.path.getmtime(p) <= os.path.getmtime(LIB) for p in deps):
        return LIB
    tmp = LIB + ".tmp"
    cmd = [B._nvcc(), *B.NVCC_FLAGS, "-I", B.INCLUDE, "-I", B.CSRC, "-I", HERE, "-shared", SRC,
           "-o", tmp, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {SRC}:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def call(name, *args):
    L = load()
    rc = getattr(L, name)(*args)
    if rc != 0:
        raise RuntimeError(f"{name}: status {rc}: {L.angelo_probe_last_error_string().decode()}")
    return rc
