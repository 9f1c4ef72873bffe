"""Measures the accumulation bias of the tcgen05 TF32 GEMM (forge_gpu_selftest_tc_gemm).

    python -m forge_gb300.tcbias

Operands are TF32-exact (the products are exact in FP32), 256 x 256 outputs, K from 8 to 8192, once with
all-positive entries (every partial sum grows, so a truncating accumulator shows as a negative mean
error) and once with random signs.  Prints one JSON line per case: the mean, RMS and max of
(D - exact) / max|exact|.
"""
from __future__ import annotations

import ctypes as C
import json

import numpy as np

from .api import load_library


def tf32(x: np.ndarray) -> np.ndarray:
    """Rounds toward zero to the 10-bit TF32 mantissa (the values are then exact in TF32)."""
    b = np.asarray(x, np.float32).view(np.uint32) & np.uint32(0xFFFFE000)
    return b.view(np.float32)


def measure(K: int, positive: bool, M: int = 256, N: int = 256, seed: int = 0) -> dict:
    lib = load_library()
    rng = np.random.default_rng(seed)
    A = tf32(rng.uniform(0.5, 1.0, (M, K)))
    B = tf32(rng.uniform(0.5, 1.0, (N, K)))
    if not positive:
        A = tf32(A * rng.choice([-1.0, 1.0], (M, K)))
    D = np.zeros((M, N), np.float32)
    rc = lib.forge_gpu_selftest_tc_gemm(M, N, K, 1, A.ctypes.data_as(C.c_void_p), B.ctypes.data_as(C.c_void_p),
                                        D.ctypes.data_as(C.c_void_p))
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    rel = (D - ref) / np.abs(ref).max()
    return dict(K=K, sign="positive" if positive else "mixed", rc=rc, mean_rel=float(rel.mean()),
                rms_rel=float(np.sqrt((rel ** 2).mean())), max_rel=float(np.abs(rel).max()))


def main():
    for positive in (True, False):
        for K in (8, 32, 128, 512, 2048, 8192):
            print(json.dumps(measure(K, positive)), flush=True)


if __name__ == "__main__":
    main()
