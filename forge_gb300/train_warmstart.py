"""Trains the warm-start networks on converged fields that the SCF itself produces.

Training systems are an uneven-size set: twisted bilayers
(m, m+1) for m = 8, 12, 16, and the alternating-twist trilayer at m = 12, at several fillings
and dielectric constants.  They are converged together with the mixed-precision SCF: every
iteration solves the H(k) of all systems still above the tolerance in ONE batched eigen-solve
(forge_gpu_scf_iteration_group, the uneven-size batch) to a mean-field residual of 1e-5 eV
(training targets need no more).  Then site and bond samples are drawn and both MLPs are trained
on the GPU by the library's kernels.

    python -m forge_gb300.train_warmstart [--quick] [--out path.npz]
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
from forge_gb300 import warmstart as wsm  # noqa: E402

SYSTEMS = [
    # (m, nlayers, numk, nu, eps)
    (8, 2, 6, 2.0, 10.0), (8, 2, 6, 0.0, 10.0), (8, 2, 6, -2.0, 10.0), (8, 2, 6, 2.0, 6.0), (8, 2, 6, 2.0, 15.0),
    (12, 2, 6, 2.0, 10.0), (12, 2, 6, -2.0, 10.0), (12, 2, 6, 1.0, 10.0), (12, 2, 6, 3.0, 10.0),
    (16, 2, 4, 2.0, 10.0), (16, 2, 4, 0.0, 10.0),
    (12, 3, 4, 2.0, 10.0),
    # the (10, 11) bilayer at the fillings other than +2 (the warm start's target workload there)
    (10, 2, 6, 0.0, 10.0), (10, 2, 6, 1.0, 10.0), (10, 2, 6, 3.0, 10.0), (10, 2, 6, -2.0, 10.0),
]
QUICK = [(8, 2, 6, 2.0, 10.0), (8, 2, 6, 0.0, 10.0), (12, 2, 4, 2.0, 10.0)]


def converge_group(systems, tol=1e-5, itmax=60, degfactor="corrected"):
    """All systems to the residual tolerance with one batched eigen-solve per iteration over the
    systems not yet converged; returns [(Setup, HartreeFock, iterations, residual)]."""
    runs = []
    for (m, L, numk, nu, eps) in systems:
        S = fg.Setup(ntheta=m, nlayers=L, RotateLayers=(-1, 1, -1)[:L], numk=numk, nfilling=nu, epsilon=eps,
                     degfactor_mode=degfactor, precision="mixed")
        hf = fg.HartreeFock(S)
        hf.LongRangeInteraction(copy_out=False)
        E, _ = hf.PlainGuess()
        runs.append(dict(S=S, hf=hf, E=np.asarray(E, float), n=0, res=1.0))
    while True:
        active = [r for r in runs if r["res"] > tol and r["n"] < itmax]
        if not active:
            break
        reps, E, _ = fg.ScfIterationGroup([r["hf"] for r in active], np.stack([r["E"] for r in active]))
        for r, rep, e in zip(active, reps, E):
            r["E"], r["n"], r["res"] = e, r["n"] + 1, rep["residual"]
    return [(r["S"], r["hf"], r["n"], r["res"]) for r in runs]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--out", default=wsm.WEIGHTS)
    ap.add_argument("--epochs", type=int, default=80)
    ap.add_argument("--degfactor", default="corrected", choices=["corrected", "reference"],
                    help="occupation weight of the partially filled states used for the training SCFs")
    args = ap.parse_args()
    samples, log = [], []
    systems = QUICK if args.quick else SYSTEMS
    t = time.time()
    for (m, L, numk, nu, eps), (S, hf, n, res) in zip(systems, converge_group(systems, degfactor=args.degfactor)):
        P, dens, V = hf.GetState()
        samples.append(wsm.training_samples(S, hf.geometry, P, dens))
        hf.close()
        log.append(dict(m=m, nlayers=L, numk=numk, nu=nu, eps=eps, iters=n, residual=res))
        print(json.dumps(log[-1]), flush=True)
    print(json.dumps(dict(converge_s=time.time() - t)), flush=True)
    ws = wsm.WarmStart(seed=0)
    t = time.time()
    ls, lb = ws.fit(samples, epochs=args.epochs, lr=2e-3)
    print(json.dumps(dict(train_s=time.time() - t, site_loss=ls, bond_loss=lb,
                          n_site=int(sum(len(s[0]) for s in samples)),
                          n_bond=int(sum(len(s[2]) for s in samples)))), flush=True)
    ws.save(args.out)
    print(args.out)


if __name__ == "__main__":
    main()
