"""Generates tests/golden/relaxation_uq.npz: the in-plane displacement tables (uqx, uqy) that the
reference's LatticeRelaxation hard-codes per twist (Geometry.f90:305-1056), for the twists the
tests use: ntheta = 2, 5, 10, 31 and 35 (the smallest, configs 0 and 1, the 1.05 deg headline, the
largest table).

The reference's literals carry no kind parameter (for example ``uqx(2,1)=-0.0007312154977677281``),
so by the Fortran standard they are default REAL constants, rounded to single precision before the
assignment widens them (the reference builds with ifort and no -fpconstant / -r8); only ``0.0_dp``
is double.  The stored tables are those effective values.  Entries the reference leaves unset are 0.

This script reads the reference source where it lies; run it from the repository root:

    python tests/golden/make_relaxation_tables.py [path/to/Geometry.f90]
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
THETAS = (2, 5, 10, 31, 35)


def fortran_literal(text: str) -> float:
    t = text.strip().lower()
    if t.endswith("_dp"):
        return float(t[:-3])
    if "d" in t:
        return float(t.replace("d", "e"))
    return float(np.float32(float(t)))


def parse(src: str, ntheta: int):
    block = re.search(r"if\(ntheta\.EQ\.%d\)then(.*?)endif" % ntheta, src, re.S)
    if block is None:
        raise KeyError(f"no displacement table for ntheta = {ntheta}")
    uq = {"x": np.zeros((5, 5)), "y": np.zeros((5, 5))}
    for comp, n, m, val in re.findall(r"uq([xy])\((\d),(\d)\)\s*=\s*([-+0-9.eEdD_p]+)", block.group(1)):
        uq[comp][int(n) - 1, int(m) - 1] = fortran_literal(val)
    return uq["x"], uq["y"]


def main():
    path = sys.argv[1] if len(sys.argv) > 1 else "/root/reference/Geometry.f90"
    with open(path) as f:
        src = f.read()
    out = {}
    for m in THETAS:
        ux, uy = parse(src, m)
        out[f"uqx_{m}"], out[f"uqy_{m}"] = ux, uy
    np.savez_compressed(os.path.join(HERE, "relaxation_uq.npz"), ntheta=np.array(THETAS), **out)
    print("wrote", {m: (int(np.count_nonzero(out[f"uqx_{m}"])), float(np.abs(out[f"uqx_{m}"]).max())) for m in THETAS})


if __name__ == "__main__":
    main()
