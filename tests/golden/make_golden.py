"""Generates the golden fixtures in this folder from the CPU oracle.

The reference (Fortran, Intel MKL) cannot be compiled in this environment and ships
no test vectors, so these fixtures pin the oracle's own outputs (regression pins),
checked in tests/test_oracle.py and used as known answers by the GPU tests.
Run from the repository root:  python tests/golden/make_golden.py [fixture ...]
(no argument: every fixture; otherwise only the named ones, e.g. oracle_variants_m1_k3).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import forge_oracle as fo  # noqa: E402


def variant_runs():
    """The switches outside the configured path on the m = 1, 3x3 k cell, three iterations each:
    (name, oracle result).  numS = 2 starts from spin-split guesses at fillings +-1."""
    base = dict(ntheta=1, numk=3, nfilling=2.0, degfactor_mode="corrected")
    s1 = fo.Setup(**base)
    g = fo.build_geometry(s1)
    T = fo.pair_tables(s1, g)
    LR = fo.long_range_interaction(s1, g)
    out = []
    for name, flags in (("c3", dict(nenforceC3=1)), ("sym", dict(nenforceT=1, nenforceC2=1, nenforceC2T=1)),
                        ("valley", dict(nenforceValley=1))):
        out.append((name, fo.run_scf(fo.Setup(**base, **flags), g, T, LR, itmax=3)))
    P0 = np.stack([fo.plain_guess(fo.Setup(**{**base, "nfilling": base["nfilling"] + d}), g, T)[0]
                   for d in (1.0, -1.0)])
    out.append(("spin2", fo.run_scf_2spins(fo.Setup(numS=2, **base), g, T, LR, P_init=P0, itmax=3)))
    return out


def write_variants():
    arrays = {}
    for name, r in variant_runs():
        arrays[name + "_E_in"] = np.array([l.E_in for l in r["logs"]])
        arrays[name + "_step"] = np.array([l.step for l in r["logs"]])
        arrays[name + "_P"] = r["P"]
    np.savez_compressed(os.path.join(HERE, "oracle_variants_m1_k3.npz"), **arrays)


def main(names=None):
    if names is None or "oracle_variants_m1_k3" in names:
        write_variants()
    if names is not None and not {"oracle_m1_k3", "oracle_cfg0"} & set(names):
        return
    s = fo.Setup(ntheta=1, numk=3, itmax=3)
    r = fo.run_scf(s)
    np.savez_compressed(os.path.join(HERE, "oracle_m1_k3.npz"), coords=r["geometry"].coords, LR=r["LR"], P=r["P"],
                        V=r["V"], E_in=np.array([l.E_in for l in r["logs"]]),
                        step=np.array([l.step for l in r["logs"]]), bands=r["bands"])
    # the (5, 6) bilayer (m=5, 6x6 k grid, charge neutrality): small derived quantities only
    s = fo.Setup(ntheta=5, numk=6, itmax=3)
    r = fo.run_scf(s)
    rng = np.random.default_rng(0)
    idx = rng.integers(0, s.ndim, size=(256, 2))
    np.savez_compressed(os.path.join(HERE, "oracle_cfg0.npz"), E_in=np.array([l.E_in for l in r["logs"]]),
                        step=np.array([l.step for l in r["logs"]]), dn=np.array([l.dn_max for l in r["logs"]]),
                        nocc=np.array([l.nocc for l in r["logs"]]), npart=np.array([l.npart for l in r["logs"]]),
                        EF=np.array([l.EF for l in r["logs"]]), bands=r["bands"], idx=idx,
                        P_sample=r["P"][:, idx[:, 0], idx[:, 1]], V=r["V"], trace=np.trace(r["P"][0]))


if __name__ == "__main__":
    main(sys.argv[1:] or None)
