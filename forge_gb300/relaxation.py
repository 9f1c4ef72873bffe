"""In-plane displacement tables of FORGE's LatticeRelaxation (Geometry.f90:279-1135).

The reference hard-codes one table of Fourier components, uqx(n, m) and uqy(n, m) for
n = 2..5, m = 1..n-1, per twist ntheta = 2..35 (Geometry.f90:305-1056), and relaxes bilayers with
it when nrelax = 1 (Main.f90:156-160).  This module ships no table: ``read_displacement_table``
reads the one for a given ntheta out of a FORGE Geometry.f90 source file, with the Fortran kind
rules of its literals, and ``Setup(nrelax=1, relaxation=...)`` takes the result.
"""
from __future__ import annotations

import re
from typing import Tuple

import numpy as np


def fortran_real_literal(text: str) -> float:
    """The value a Fortran real literal constant gives when assigned to a real(dp) variable.

    A literal with a ``_dp`` kind parameter or a ``d`` exponent is double precision; any other
    (``-0.00073``, ``7.4e-07``) is default REAL, i.e. rounded to single precision before the
    assignment widens it (no -r8 / -fpconstant, as the reference is built)."""
    t = text.strip().lower()
    if t.endswith("_dp"):
        return float(t[:-3])
    if "_" in t:
        raise ValueError(f"unsupported kind parameter in {text!r}")
    if "d" in t:
        return float(t.replace("d", "e"))
    return float(np.float32(float(t)))


_ASSIGN = re.compile(r"^\s*uq([xy])\(\s*(\d)\s*,\s*(\d)\s*\)\s*=\s*([-+0-9.eEdD_pP]+)\s*$")
_OPEN = re.compile(r"^\s*if\s*\(\s*ntheta\s*\.eq\.\s*(\d+)\s*\)\s*then\s*$", re.I)
_CLOSE = re.compile(r"^\s*end\s*if\s*$", re.I)


def read_displacement_table(path: str, ntheta: int) -> Tuple[np.ndarray, np.ndarray]:
    """(uqx, uqy), each 5 x 5 with [n-1, m-1] = uqx(n, m), for ``ntheta`` from a FORGE Geometry.f90.

    A twist without a table block gives zeros, as the reference's initialisation does
    (Geometry.f90:305-306)."""
    uq = {"x": np.zeros((5, 5)), "y": np.zeros((5, 5))}
    inside = False
    with open(path) as f:
        for line in f:
            code = line.split("!", 1)[0]
            if not inside:
                mo = _OPEN.match(code)
                inside = bool(mo) and int(mo.group(1)) == ntheta
                continue
            if _CLOSE.match(code):
                inside = False
                continue
            ma = _ASSIGN.match(code)
            if ma:
                comp, n, m, val = ma.groups()
                n, m = int(n), int(m)
                if not (1 <= m < n <= 5):
                    raise ValueError(f"uq{comp}({n},{m}) outside the table n = 2..5, m = 1..n-1")
                uq[comp][n - 1, m - 1] = fortran_real_literal(val)
    return uq["x"], uq["y"]
