"""Times the batched partial Hermitian eigen-solver (zdiagRed, LapackRoutines.f90:381-433) alone.

    python -m forge_gb300.eigbench --m 20 --precision mixed --batch 1

The matrix is a seeded random Hermitian matrix (entries ~0.1) of the size of the commensurate
twisted bilayer (m, m+1), N = 4 (3m^2 + 3m + 1); eigenpairs 1..N/2+10 are computed, as in the SCF.
Prints one JSON line: N, wall seconds, info and per-stage milliseconds from the library's CUDA-event
profiler.  Used for the eigen-solver's ncu captures.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import forge_gb300 as fg  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--m", type=int, default=20)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--batch", type=int, default=1)
    ap.add_argument("--repeat", type=int, default=1)
    args = ap.parse_args()
    hf = fg.HartreeFock(fg.Setup(ntheta=args.m, numk=1))
    N = hf.N
    rng = np.random.default_rng(0)
    A = rng.standard_normal((N, N)) * 0.1 + 1j * rng.standard_normal((N, N)) * 0.1
    A = np.tril((A + A.conj().T) / 2)
    As = np.asfortranarray(np.repeat(A[:, :, None], args.batch, axis=2))
    hf.set_precision(args.precision)
    for _ in range(args.repeat):
        hf.profile(True)
        t = time.time()
        w, Z, info = hf.zheevr_batch(As, N // 2 + 10, vectors=False)
        dt = time.time() - t
        prof = {k: round(v["ms"], 2) for k, v in hf.profile_read().items() if v["launches"]}
        print(json.dumps(dict(N=N, batch=args.batch, precision=args.precision, s=dt, info=info, prof=prof)),
              flush=True)
    hf.close()


if __name__ == "__main__":
    main()
