"""Trains the warm-start networks on converged fields that the SCF itself produces.

Training systems are an uneven-size set: twisted bilayers
(m, m+1) for m = 8, 12, 16, and the alternating-twist trilayer at m = 12, at several fillings
and dielectric constants.  They are converged together with the mixed-precision SCF: every
iteration solves the H(k) of all systems still above the tolerance in ONE batched eigen-solve
(forge_gpu_scf_iteration_group, the uneven-size batch) to a mean-field residual of 1e-5 eV
(training targets need no more).  Then site and bond samples are drawn and both MLPs are trained
on the GPU by the library's kernels.

The convergence can be split over several runs: with --cache DIR the samples of every converged
system are written there as soon as its group finishes, and a later run converges only the systems
not yet cached; --group-size bounds how many systems share one batched solve, and --budget-s stops
starting groups (and iterating the current one) once the wall-clock budget is spent.  Training uses
every cached and newly converged system.

    python -m forge_gb300.train_warmstart [--quick] [--out path.npz] [--cache DIR] [--budget-s S]
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


def system_setup(system, degfactor="corrected"):
    m, L, numk, nu, eps = system
    return fg.Setup(ntheta=m, nlayers=L, RotateLayers=(-1, 1, -1)[:L], numk=numk, nfilling=nu, epsilon=eps,
                    degfactor_mode=degfactor, precision="mixed")


def _open_context(S):
    hf = fg.HartreeFock(S)
    hf.LongRangeInteraction(copy_out=False)
    E, _ = hf.PlainGuess()
    return hf, E


def converge_group(systems, tol=1e-5, itmax=60, degfactor="corrected", deadline=None, open_context=_open_context,
                   group_iteration=None, clock=time.time):
    """All systems to the residual tolerance with one batched eigen-solve per iteration over the
    systems not yet converged (forge_gpu_scf_iteration_group); returns [(Setup, context, iterations,
    residual)].  With ``deadline`` (a clock value) no iteration starts after it, and the systems above
    the tolerance then are returned as they are."""
    if group_iteration is None:
        group_iteration = fg.ScfIterationGroup
    runs = []
    for system in systems:
        S = system_setup(system, degfactor)
        hf, E = open_context(S)
        runs.append(dict(S=S, hf=hf, E=np.asarray(E, float), n=0, res=float("inf")))
    while deadline is None or clock() < deadline:
        active = [r for r in runs if r["res"] > tol and r["n"] < itmax]
        if not active:
            break
        reps, E, _ = group_iteration([r["hf"] for r in active], np.stack([r["E"] for r in active]))
        for r, rep, e in zip(active, reps, E):
            r["E"], r["n"], r["res"] = e, r["n"] + 1, rep["residual"]
    return [(r["S"], r["hf"], r["n"], r["res"]) for r in runs]


def cache_name(system, degfactor="corrected") -> str:
    m, L, numk, nu, eps = system
    return f"samples-m{m}-L{L}-k{numk}-nu{nu:+.1f}-eps{eps:.1f}-{degfactor}.npz"


def collect_samples(systems, tol=1e-5, degfactor="corrected", cache=None, group_size=0, budget_s=None,
                    converge=converge_group, sample=None, clock=time.time, log=print):
    """Training samples of every system that is cached or converges within the budget, in the order of
    ``systems``; systems still above ``tol`` when the budget ends are left out (and not cached)."""
    if sample is None:
        def sample(S, hf):
            P, dens, _ = hf.GetState()
            return wsm.training_samples(S, hf.geometry, P, dens)
    got = {}
    todo = []
    for system in systems:
        path = os.path.join(cache, cache_name(system, degfactor)) if cache else None
        if path and os.path.exists(path):
            d = np.load(path)
            got[system] = (d["xs"], d["ys"], d["xb"], d["yb"])
        else:
            todo.append(system)
    deadline = None if budget_s is None else clock() + budget_s
    size = group_size if group_size > 0 else max(1, len(todo))
    for g0 in range(0, len(todo), size):
        if deadline is not None and clock() >= deadline:
            break
        group = todo[g0:g0 + size]
        for system, (S, hf, n, res) in zip(group, converge(group, tol=tol, degfactor=degfactor, deadline=deadline)):
            ok = res <= tol
            if ok:
                xs, ys, xb, yb = sample(S, hf)
                got[system] = (xs, ys, xb, yb)
                if cache:
                    os.makedirs(cache, exist_ok=True)
                    np.savez_compressed(os.path.join(cache, cache_name(system, degfactor)), xs=xs, ys=ys, xb=xb,
                                        yb=yb)
            if hasattr(hf, "close"):
                hf.close()
            m, L, numk, nu, eps = system
            log(json.dumps(dict(m=m, nlayers=L, numk=numk, nu=nu, eps=eps, iters=n, residual=res, used=ok)))
    return [got[s] for s in systems if s in got]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--out", default=wsm.WEIGHTS)
    ap.add_argument("--epochs", type=int, default=80)
    ap.add_argument("--degfactor", default="corrected", choices=["corrected", "reference"],
                    help="occupation weight of the partially filled states used for the training SCFs")
    ap.add_argument("--cache", default="", help="directory of per-system training samples (resumable runs)")
    ap.add_argument("--group-size", type=int, default=0, help="systems per batched solve (0: all at once)")
    ap.add_argument("--budget-s", type=float, default=None, help="wall-clock budget of the convergence stage")
    args = ap.parse_args()
    systems = QUICK if args.quick else SYSTEMS
    t = time.time()
    samples = collect_samples(systems, degfactor=args.degfactor, cache=args.cache or None,
                              group_size=args.group_size, budget_s=args.budget_s,
                              log=lambda line: print(line, flush=True))
    print(json.dumps(dict(converge_s=time.time() - t, systems_used=len(samples), systems=len(systems))), flush=True)
    if not samples:
        raise SystemExit("no converged system to train on")
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
