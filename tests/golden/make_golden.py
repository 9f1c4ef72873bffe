"""Generates the golden fixtures in this folder from the CPU oracle.

The reference (Fortran, Intel MKL) cannot be compiled in this environment and ships
no test vectors, so these fixtures pin the oracle's own outputs (regression pins),
checked in tests/test_oracle.py and used as known answers by the GPU tests.
Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import forge_oracle as fo  # noqa: E402


def main():
    s = fo.Setup(ntheta=1, numk=3, itmax=3)
    r = fo.run_scf(s)
    np.savez_compressed(os.path.join(HERE, "oracle_m1_k3.npz"), coords=r["geometry"].coords, LR=r["LR"], P=r["P"],
                        V=r["V"], E_in=np.array([l.E_in for l in r["logs"]]),
                        step=np.array([l.step for l in r["logs"]]), bands=r["bands"])
    # config 0 (m=5, 6x6 k grid, charge neutrality): small derived quantities only
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
    main()
