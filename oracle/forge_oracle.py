"""CPU oracle for FORGE's real-space Hartree-Fock SCF (TEST INFRASTRUCTURE ONLY).

This module restates, in numpy + scipy LAPACK, the reference algorithm of
forge-team/forge (Fortran 90 / OpenMP / MKL).  It is the checker for the CUDA
path in ``forge_gb300``: only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it.  It
is never the thing measured on the GPU path and never a fallback for it.

Parity status: **parity unpinned by the reference itself.**  The reference
ships no tests, golden vectors or fixtures, and it cannot be compiled here (no
Fortran compiler in this image or on the GPU host; its sources do not travel
to the GPU host).  The restatement is pinned instead by (1) a second,
independent restatement of the pair tables and energies in C
(``oracle/forge_oracle_c.c``) that must agree to rounding, (2) algebraic
invariants of the reference (Tr P(0), Hermiticity of H(k), the P(-R)=P(R)^H
storage convention, the exactly quadratic ODA energy), and (3) integer index
maps (neighbour cells, k grid, site maps) that are fixed by the reference's
loops.

Every function cites the reference file:line it follows.  Arrays follow the
reference's Fortran layout where it matters (0-based in Python):
``P[c, i, j]`` is ``zFock(i+1, j+1, c+1)``; ``coords[i, :]`` is
``Coords(i+1, :)``.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np

F32_1EM6 = float(np.float32(1e-6))  # the default-real literal ``1e-6`` of Geometry.f90:154


# ---------------------------------------------------------------------------
# Setup (Setup.f90:6-74)
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class Setup:
    """Runtime mirror of the compile-time parameters of Setup.f90:6-74.

    Only the parameters that the Hartree-Fock path reads are kept; names
    follow the reference.  ``degfactor_mode`` selects how partially occupied
    degenerate states are weighted in GetFock: ``"reference"`` reproduces
    ``zdeg = cmplx(DegFactor, dp)`` (HartreeFock.f90:529) literally, i.e. the
    single-precision real part and an imaginary part equal to ``dp`` = 8;
    ``"corrected"`` uses the real weight DegFactor.  ``nenforceC3 = 1`` (Setup.f90:27) selects
    Solve_C3 / GetFock_C3 in the SCF drivers; ``nenforceC2``, ``nenforceT``, ``nenforceC2T``
    (Setup.f90:28-30) symmetrise every new density matrix of the SCF loop (``enforce_symmetries``);
    ``nenforceValley`` (Setup.f90:31) averages the window part with its valley transform (``window_fock``).
    """

    ntheta: int = 5
    nlayers: int = 2
    RotateLayers: tuple = (-1, 1)
    numk: int = 6
    nfilling: float = 0.0
    U: float = 4.0
    epsilon: float = 10.0
    Delta: float = 0.0
    numI: int = 1
    numC: int = 3
    nscreen: int = 2
    xi: float = 10.0 / 0.246
    fphase: int = 0
    itmax: int = 2
    EnergyTolerance: float = 0.0001
    StepAlternative: float = 1.0
    pressure: float = 1.0
    numS: int = 1
    nenforceC3: int = 0
    nenforceC2: int = 0
    nenforceT: int = 0
    nenforceC2T: int = 0
    nenforceValley: int = 0
    degfactor_mode: str = "reference"
    # Setup.f90:12 nrelax: 1 applies LatticeRelaxation to bilayers (Main.f90:156-160) with the in-plane
    # displacement table relax_uq = (uqx, uqy), 5 x 5 each, [n-1, m-1] holding uqx(n, m) of
    # Geometry.f90:305-1056 for this ntheta (the reference hard-codes one table per ntheta = 2..35)
    nrelax: int = 0
    relax_uq: Optional[tuple] = None

    # derived (Setup.f90:10, 23-24, 58-69)
    @property
    def ndim(self) -> int:
        m = self.ntheta
        return self.nlayers * 2 * (m * m + (m + 1) ** 2 + (m + 1) * m)

    @property
    def numb(self) -> int:
        return min(20, self.ndim)

    @property
    def ncb(self) -> int:
        return self.numb // 2

    @property
    def nLower(self) -> int:
        return (self.ndim - 2 * self.numb + 2 * self.ncb) // 2 + 1

    @property
    def nUpper(self) -> int:
        return (self.ndim + 2 * self.ncb) // 2

    @property
    def NeutralityPoint(self) -> int:
        return (self.ndim // 2 - self.nLower) + 1

    @property
    def Nk(self) -> int:
        return self.numk * self.numk

    @property
    def alpha(self) -> float:
        return 5.853 / self.epsilon * 1.0

    @property
    def alphaH(self) -> float:
        return 5.853 / self.epsilon * 1.0

    @property
    def a0(self) -> float:
        return 1.0 / math.sqrt(3.0)

    @property
    def r0(self) -> float:
        return 0.184

    @property
    def d0(self) -> float:
        return 1.35772 / self.pressure

    @property
    def tz(self) -> float:
        return 1.35772 / self.pressure


A1 = (0.5, math.sqrt(3.0) * 0.5)   # Setup.f90:71
A2 = (-0.5, math.sqrt(3.0) * 0.5)  # Setup.f90:72
PI = 4.0 * math.atan(1.0)          # Setup.f90:74


# ---------------------------------------------------------------------------
# Geometry (Geometry.f90, Main.f90:123-163)
# ---------------------------------------------------------------------------
def number_neighbor_cells(numI: int) -> int:
    """Geometry.f90:14-35."""
    cnt = 0
    for n1 in range(-numI, numI + 1):
        for n2 in range(-numI, numI + 1):
            if -numI <= n1 + n2 <= numI and (n1 != 0 or n2 != 0):
                cnt += 1
    return cnt // 2 + 1


def order_neighbor_cells(numI: int, nnc: int):
    """Geometry.f90:40-91: R list (0,0),(-1,0),(-1,1),(0,-1),... ."""
    u1 = [0] * nnc
    u2 = [0] * nnc
    icount = 0
    if numI > 0:
        for a, b in ((-1, 0), (-1, 1), (0, -1)):
            icount += 1
            u1[icount], u2[icount] = a, b
    if numI > 1:
        for n1 in range(-numI, numI + 1):
            for n2 in range(-numI, numI + 1):
                if -numI <= n1 + n2 <= numI and icount < nnc - 1:
                    if n1 != 0 or n2 != 0:
                        icount += 1
                        u1[icount], u2[icount] = n1, n2
                        if (n1, n2) in ((-1, 0), (-1, 1), (0, -1)):
                            icount -= 1
    return np.array(u1, dtype=np.int64), np.array(u2, dtype=np.int64)


def sample_bz(numk: int, g1, g2):
    """Geometry.f90:96-127. Returns (nMomentaComponents[Nk,2], nMomentaFlattened, MomentaValues[numk,numk,2])."""
    comps = np.zeros((numk * numk, 2), dtype=np.int64)
    flat = np.zeros((numk, numk), dtype=np.int64)
    icount = 0
    for ivk1 in range(numk):
        for ivk2 in range(numk):
            icount += 1
            comps[icount - 1] = (ivk1, ivk2)
            flat[ivk1, ivk2] = icount
    vals = np.zeros((numk, numk, 2))
    for ivk2 in range(numk):
        for ivk1 in range(numk):
            vals[ivk1, ivk2, 0] = (ivk1 * g1[0] + ivk2 * g2[0]) / float(numk)
            vals[ivk1, ivk2, 1] = (ivk1 * g1[1] + ivk2 * g2[1]) / float(numk)
    return comps, flat, vals


def _ws_accept(x1: float, x2: float, m: int, rmax: float) -> bool:
    r1 = abs(x1 * (3.0 * m + 1) + x2 * (3.0 * m + 2)) + F32_1EM6
    r2 = abs(x1 - x2 * (3.0 * m + 1)) + F32_1EM6
    r3 = abs(x1 * (3.0 * m + 2) + x2) + F32_1EM6
    return r1 < rmax and r2 < rmax and r3 < rmax


def wigner_seitz_cell(s: Setup, t1, t2, cs: float, sn: float) -> np.ndarray:
    """Geometry.f90:132-273: site coordinates (unrotated), layer-major, A block then B block per layer."""
    m = s.ntheta
    nrad = 3 * m
    rmax = 3.0 * m ** 2 + 3.0 * m + 1.0
    sq3 = math.sqrt(3.0)
    coords = np.zeros((s.ndim, 3))
    rows = []
    for nlayer in range(1, s.nlayers + 1):
        z = (float(np.float32(nlayer - 1)) - float(np.float32(s.nlayers - 1)) / 2.0) * s.tz
        rot = s.RotateLayers[nlayer - 1]
        if rot == -1:
            for n1 in range(-nrad, nrad + 1):
                for n2 in range(-nrad, nrad + 1):
                    an1 = n1 + 1.0 / 3.0
                    an2 = n2 - 2.0 / 3.0
                    if _ws_accept(an1, an2, m, rmax):
                        rows.append(((n1 + 1.0 / 3.0) * A1[0] + (n2 - 2.0 / 3.0) * A2[0],
                                     (n1 + 1.0 / 3.0) * A1[1] + (n2 - 2.0 / 3.0) * A2[1], z))
            rows.append(((-t2[0] - t1[0]) / 3.0, (-t2[1] - t1[1]) / 3.0, z))
            for n1 in range(-nrad, nrad + 1):
                for n2 in range(-nrad, nrad + 1):
                    bn1 = n1 + 2.0 / 3.0
                    bn2 = n2 - 1.0 / 3.0
                    if _ws_accept(bn1, bn2, m, rmax):
                        rows.append((bn1 * A1[0] + bn2 * A2[0], bn1 * A1[1] + bn2 * A2[1], z))
            rows.append(((t2[0] + t1[0]) / 3.0, (t2[1] + t1[1]) / 3.0, z))
        elif rot == 1:
            for n1 in range(-nrad, nrad + 1):
                for n2 in range(-nrad, nrad + 1):
                    an1 = (n1 + 1.0 / 3.0) * (cs - sn / sq3) - 2 * (n2 - 2.0 / 3.0) * sn / sq3
                    an2 = (n2 - 2.0 / 3.0) * (cs + sn / sq3) + 2 * (n1 + 1.0 / 3.0) * sn / sq3
                    if _ws_accept(an1, an2, m, rmax):
                        rows.append((an1 * A1[0] + an2 * A2[0], an1 * A1[1] + an2 * A2[1], z))
            rows.append(((t1[0] + t2[0]) / 3.0, (t1[1] + t2[1]) / 3.0, z))
            for n1 in range(-nrad, nrad + 1):
                for n2 in range(-nrad, nrad + 1):
                    bn1 = (n1 + 2.0 / 3.0) * (cs - sn / sq3) - 2 * (n2 - 1.0 / 3.0) * sn / sq3
                    bn2 = (n2 - 1.0 / 3.0) * (cs + sn / sq3) + 2 * (n1 + 2.0 / 3.0) * sn / sq3
                    if _ws_accept(bn1, bn2, m, rmax):
                        rows.append((bn1 * A1[0] + bn2 * A2[0], bn1 * A1[1] + bn2 * A2[1], z))
            rows.append(((-t1[0] - t2[0]) / 3.0, (-t1[1] - t2[1]) / 3.0, z))
        else:
            raise ValueError("RotateLayers entries must be -1 or +1")
    if len(rows) != s.ndim:
        raise RuntimeError(f"Wigner-Seitz cell found {len(rows)} sites, expected ndim={s.ndim}")
    coords[:] = np.array(rows)
    return coords


def _rot(R, v):
    """matmul(RotMatrix, v) for a 2x2 column-major RotMatrix, no FMA (Main.f90:135)."""
    return (R[0][0] * v[0] + R[0][1] * v[1], R[1][0] * v[0] + R[1][1] * v[1])


@dataclasses.dataclass
class Geometry:
    coords: np.ndarray          # (N,3)
    t1: tuple
    t2: tuple
    t3: tuple
    g1: tuple
    g12: tuple
    ucell1: np.ndarray          # nUnitCell_1 (NNC,)
    ucell2: np.ndarray          # nUnitCell_2 (NNC,)
    kcomp: np.ndarray           # nMomentaComponents (Nk,2) int64
    kflat: np.ndarray           # nMomentaFlattened (numk,numk)
    kvals: np.ndarray           # MomentaValues (numk,numk,2)
    c2pairs: np.ndarray         # nC2pairs, 1-based like the reference
    c3pairs: np.ndarray         # nC3pairs, 1-based
    c2_count: int
    c3_count: int

    @property
    def tn(self) -> np.ndarray:
        """reshape([t1,t2,t3],[2,3]) of Main.f90:249, as a (3,2) array of vectors."""
        return np.array([self.t1, self.t2, self.t3])

    def vk(self, icount: int) -> np.ndarray:
        ivk1, ivk2 = self.kcomp[icount]
        return self.kvals[ivk1, ivk2]


def build_geometry(s: Setup) -> Geometry:
    """Main.f90:102-163: neighbour cells, reciprocal vectors, rotation, k grid, sites, C2/C3 maps."""
    nnc = number_neighbor_cells(s.numI)
    u1, u2 = order_neighbor_cells(s.numI, nnc)
    m = s.ntheta
    aMoire = 3.0 * m ** 2 + 3.0 * m + 1.0
    f = (4.0 * PI / 3.0) / aMoire
    g1 = (f * (float(3 * m + 1) * A1[0] + A2[0]), f * (float(3 * m + 1) * A1[1] + A2[1]))
    g12 = (f * (float(3 * m + 2) * A2[0] - A1[0]), f * (float(3 * m + 2) * A2[1] - A1[1]))
    cs = 1.0 - 1.0 / (2.0 * aMoire)
    sn = math.sqrt(1.0 - cs ** 2)
    th = 0.5 * math.acos(cs)
    c, sgn = math.cos(th), math.sin(th)
    # reshape([c,-s,s,c],[2,2]) column-major: R(1,1)=c, R(2,1)=-s, R(1,2)=s, R(2,2)=c
    R = ((c, sgn), (-sgn, c))
    g1 = _rot(R, g1)
    g12 = _rot(R, g12)
    kcomp, kflat, kvals = sample_bz(s.numk, g1, g12)
    t1 = (float(m) * A1[0] + float(m + 1) * A2[0], float(m) * A1[1] + float(m + 1) * A2[1])
    t2 = (float(-m - 1) * A1[0] + float(2 * m + 1) * A2[0], float(-m - 1) * A1[1] + float(2 * m + 1) * A2[1])
    coords = wigner_seitz_cell(s, t1, t2, cs, sn)
    # Main.f90:148-150 rotates (x, y); the z coordinate is kept (the reference's
    # assignment of the 2-vector to the 3-row is read as "rotate x,y in place").
    for n in range(s.ndim):
        x, y = _rot(R, (coords[n, 0], coords[n, 1]))
        coords[n, 0], coords[n, 1] = x, y
    t1 = _rot(R, t1)
    t2 = _rot(R, t2)
    t3 = (t2[0] - t1[0], t2[1] - t1[1])
    if s.nrelax == 1 and s.nlayers == 2:
        if s.relax_uq is None:
            raise ValueError("nrelax = 1 needs the displacement table relax_uq = (uqx, uqy) of this ntheta")
        coords, matched = lattice_relaxation(s, coords, g1, g12, *s.relax_uq)
        if matched != (s.ndim // 4, s.ndim // 4):
            raise ValueError(f"LatticeRelaxation matched {matched} layer-2 sites, expected {s.ndim // 4} per quarter")
    c2, c2cnt = c2_related_points(s, coords)
    c3, c3cnt = c3_related_points(s, coords)
    return Geometry(coords, t1, t2, t3, g1, g12, u1, u2, kcomp, kflat, kvals, c2, c3, c2cnt, c3cnt)


def lattice_relaxation(s: Setup, coords, g1, g12, uqx, uqy):
    """LatticeRelaxation (Geometry.f90:279-1135) of a bilayer, on the rotated sites (Main.f90:156-160).

    Layer 1 (sites 1..ndim/2): r += delta / 2 with
        delta = -sum_{nn = 1, 3, 5} sum_{n = 2..5} sum_{m = 1..n-1} 2 R((nn-1) pi/3) u(n, m) sin(q . r),
        q = (n-1) Gn(nn) + (m-1) Gn(nn+2),
    Gn = (g1, g12, g12 - g1, -g1, -g12, g1 - g12, g1, g12) (Geometry.f90:292-299) and u(n, m) =
    (uqx(n, m), uqy(n, m)) rotated by the angle (nn-1) pi/3 (Geometry.f90:1058-1085).
    Layer 2 becomes the x-mirror (-x, y) of relaxed layer 1, keeping its z (Geometry.f90:1087-1088).
    It is then re-indexed per sublattice quarter (Geometry.f90:1092-1132): for each site i of the
    quarter, in order, the first site j of the same quarter whose UNRELAXED (x, y) lies within 0.25 a
    of it takes its coordinates; the quarter's last site then takes (x, -y, z) of the mirrored site
    stored at that index.  The reference prints ERROR RELAXATION when a quarter's count (matches + 1)
    is not ndim/4, and leaves the unmatched sites undefined; here they are NaN.

    uqx, uqy: 5 x 5, [n-1, m-1] = uqx(n, m).  Returns (coords, (count quarter 3, count quarter 4)).
    """
    N = s.ndim
    c = np.array(coords, dtype=np.float64, copy=True)
    nr = c.copy()
    G = [tuple(g1), tuple(g12), (g12[0] - g1[0], g12[1] - g1[1])]
    G += [(-v[0], -v[1]) for v in G] + [tuple(g1), tuple(g12)]
    terms = []
    for nn in (1, 3, 5):
        ang = float(nn - 1) * PI / 3.0
        ca, sa = math.cos(ang), math.sin(ang)
        for n in range(2, 6):
            for m in range(1, n):
                qx = float(n - 1) * G[nn - 1][0] + float(m - 1) * G[nn + 1][0]
                qy = float(n - 1) * G[nn - 1][1] + float(m - 1) * G[nn + 1][1]
                ux = ca * uqx[n - 1][m - 1] - sa * uqy[n - 1][m - 1]
                uy = sa * uqx[n - 1][m - 1] + ca * uqy[n - 1][m - 1]
                terms.append((qx, qy, ux, uy))
    half = N // 2
    for i in range(half):
        rx, ry = float(c[i, 0]), float(c[i, 1])
        dx = dy = 0.0
        for qx, qy, ux, uy in terms:
            sq = math.sin(qx * rx + qy * ry)
            dx = dx - 2.0 * ux * sq
            dy = dy - 2.0 * uy * sq
        c[i, 0] = rx + dx / 2.0
        c[i, 1] = ry + dy / 2.0
        c[i + half, 0] = -c[i, 0]
        c[i + half, 1] = c[i, 1]
    tmp = np.full_like(c, np.nan)
    counts = []
    for lo, hi in ((half, 3 * N // 4), (3 * N // 4, N)):
        cnt = 0
        for i in range(lo, hi):
            d = np.sqrt((c[i, 0] - nr[lo:hi, 0]) ** 2 + (c[i, 1] - nr[lo:hi, 1]) ** 2)
            hit = np.flatnonzero(d < 0.25)
            if hit.size:
                cnt += 1
                tmp[lo + hit[0]] = c[i]
        cnt += 1
        tmp[hi - 1] = (c[hi - 1, 0], -c[hi - 1, 1], c[hi - 1, 2])
        counts.append(cnt)
    c[half:] = tmp[half:]
    return c, tuple(counts)


def c2_related_points(s: Setup, coords):
    """Geometry.f90:1140-1167 (1-based map, count).  The pair distances of a layer are evaluated as
    one array (the same IEEE operations as the reference's scalar loop); the matches are then applied
    in the loop's (i, j) order, so repeated matches resolve as in the reference."""
    N, L = s.ndim, s.nlayers
    X = np.asarray(coords, dtype=np.float64)
    pairs = np.zeros(N, dtype=np.int64)
    cnt = 0
    per = N // L
    for il in range(L):
        a0, b0 = per * il, per * il + per // 2
        xi, yi = X[a0:b0, 0][:, None], X[a0:b0, 1][:, None]
        xj, yj = X[b0:a0 + per, 0][None, :], X[b0:a0 + per, 1][None, :]
        r = np.sqrt((xi + xj) ** 2 + (yi + yj) ** 2)
        for i, j in zip(*np.nonzero(r < 1e-5)):
            pairs[a0 + i] = b0 + j + 1
            pairs[b0 + j] = a0 + i + 1
            cnt += 1
    return pairs, cnt


def c3_related_points(s: Setup, coords):
    """Geometry.f90:1172-1223 (1-based map, count), with the distances of a sublattice block as one
    array and the matches applied in the reference's loop order (the last match of a site wins)."""
    N, L = s.ndim, s.nlayers
    X = np.asarray(coords, dtype=np.float64)
    per = N // L
    pairs = np.zeros(N, dtype=np.int64)
    cnt = 0
    sq = math.sqrt(3.0)
    for nl in range(1, L + 1):
        base = (nl - 1) * per
        for lo, hi in ((base + 1, base + per // 2), (base + per // 2 + 1, base + per)):
            x, y = X[lo - 1:hi, 0], X[lo - 1:hi, 1]
            x3 = -.5 * x - .5 * sq * y
            y3 = .5 * sq * x - .5 * y
            r = np.sqrt((x[None, :] - x3[:, None]) ** 2 + (y[None, :] - y3[:, None]) ** 2)
            for i, j in zip(*np.nonzero(r < 1e-3)):
                pairs[lo - 1 + i] = lo + j
                cnt += 1
    for nl in range(1, L + 1):
        pairs[(nl - 1) * per + per // 2 - 1] = (nl - 1) * per + per // 2
        pairs[(nl - 1) * per + per - 1] = (nl - 1) * per + per
        cnt += 2
    return pairs, cnt


# ---------------------------------------------------------------------------
# Model functions ft / fv (TightBinding.f90:216-230, HartreeFock.f90:1232-1274)
# ---------------------------------------------------------------------------
def ft(s: Setup, ri, rj):
    """TightBinding.f90:216-230, vectorised over broadcast arrays of shape (...,3)."""
    ri = np.asarray(ri, dtype=np.float64)
    rj = np.asarray(rj, dtype=np.float64)
    d = ri - rj
    r = np.sqrt(d[..., 0] ** 2 + d[..., 1] ** 2 + d[..., 2] ** 2)
    with np.errstate(divide="ignore", invalid="ignore"):
        cs = d[..., 2] / r
        val = -2.7 * np.exp((s.a0 - r) / s.r0) * (1 - cs ** 2) + 0.48 * np.exp((s.d0 - r) / s.r0) * cs ** 2
    return np.where(r > 0.001, val, 0.0)


def fv(s: Setup, ri, rj):
    """HartreeFock.f90:1232-1274 (dual-gate image sum for nscreen=2, single gate for nscreen=1)."""
    ri = np.asarray(ri, dtype=np.float64)
    rj = np.asarray(rj, dtype=np.float64)
    xi_, yi, zi = ri[..., 0], ri[..., 1], ri[..., 2]
    xj, yj, zj = rj[..., 0], rj[..., 1], rj[..., 2]
    dx, dy, dz = xi_ - xj, yi - yj, zi - zj
    r = np.sqrt(dx * dx + dy * dy + dz * dz)
    r2 = np.sqrt(dx * dx + dy * dy)
    xi = s.xi
    shape = np.broadcast(xi_, xj).shape
    if s.nscreen == 2:
        near = (r2 < xi) | (r2 < 2 * s.nlayers * s.tz)
        rho2 = (xj - xi_) ** 2 + (yj - yi) ** 2
        acc = np.zeros(shape)
        for n in range(-20, 21):
            sgn = 1.0 if n % 2 == 0 else -1.0
            acc = acc + sgn / np.sqrt(rho2 + (zj - (n * xi + zi * sgn)) ** 2)
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
            far = 2.0 * math.sqrt(2.0) / np.sqrt(r2 / xi) * np.exp(-PI * r2 / xi) / xi
        out = np.where(near, acc, far)
        return np.where(r > 0.01, out, 0.0)
    if s.nscreen == 1:
        with np.errstate(divide="ignore", invalid="ignore"):
            val = 1.0 / r - 1.0 / np.sqrt(dx * dx + dy * dy + (zi + zj + xi) ** 2)
        return np.where(r > 0.01, val, 0.0)
    raise ValueError("nscreen must be 1 or 2")


def cell_shift(g: Geometry, c: int) -> np.ndarray:
    """n1*t1 + n2*t2 for neighbour cell c (0-based), as used in HartreeFock.f90:90-91."""
    n1, n2 = int(g.ucell1[c]), int(g.ucell2[c])
    return np.array([n1 * g.t1[0] + n2 * g.t2[0], n1 * g.t1[1] + n2 * g.t2[1]])


def _shift_coords(coords, n1, n2, g: Geometry, sign: float):
    """[Coords(:,1:2) -/+ n1*t1 -/+ n2*t2, Coords(:,3)] in the reference's evaluation order."""
    out = coords.copy()
    if sign < 0:
        out[:, 0] = coords[:, 0] - n1 * g.t1[0] - n2 * g.t2[0]
        out[:, 1] = coords[:, 1] - n1 * g.t1[1] - n2 * g.t2[1]
    else:
        out[:, 0] = coords[:, 0] + n1 * g.t1[0] + n2 * g.t2[0]
        out[:, 1] = coords[:, 1] + n1 * g.t1[1] + n2 * g.t2[1]
    return out


@dataclasses.dataclass
class PairTables:
    """ft and fv for all orbital pairs and the 1 + 2*(NNC-1) cell images.

    ``tm[c][i,j] = ft(r_i, r_j - R_c)``, ``tp[c][i,j] = ft(r_i, r_j + R_c)``;
    same for ``vm``/``vp`` with fv.  c = 0 is R = 0 (tm[0] == tp[0]).
    """

    tm: np.ndarray
    tp: np.ndarray
    vm: np.ndarray
    vp: np.ndarray


_CLIB = None


def _clib():
    """Loads oracle/libforge_oracle.so (built by oracle/Makefile), or returns None."""
    global _CLIB
    if _CLIB is None:
        import ctypes
        import os
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libforge_oracle.so")
        if not os.path.exists(path):
            return None
        lib = ctypes.CDLL(path)
        lib.fo_pair_tables.restype = None
        lib.fo_long_range.restype = None
        lib.fo_rank1_projector.restype = None
        _CLIB = lib
    return _CLIB


def _model_struct(s: Setup):
    import ctypes

    class FoModel(ctypes.Structure):
        _fields_ = [("a0", ctypes.c_double), ("r0", ctypes.c_double), ("d0", ctypes.c_double),
                    ("tz", ctypes.c_double), ("xi", ctypes.c_double), ("nlayers", ctypes.c_int64),
                    ("nscreen", ctypes.c_int64)]
    return FoModel(s.a0, s.r0, s.d0, s.tz, s.xi, s.nlayers, s.nscreen)


def _ptr(a):
    import ctypes
    return a.ctypes.data_as(ctypes.c_void_p)


def pair_tables(s: Setup, g: Geometry, use_c: Optional[bool] = None) -> PairTables:
    """Tabulates the ft/fv calls of HartreeFock.f90:81-110 and 1035-1043, 1125-1133.

    ``use_c`` selects the C restatement (default: when built) or the numpy one.
    """
    lib = _clib() if use_c in (None, True) else None
    if use_c and lib is None:
        raise RuntimeError("oracle/libforge_oracle.so is not built")
    if lib is not None:
        import ctypes
        N = s.ndim
        nnc = len(g.ucell1)
        X = np.ascontiguousarray(g.coords)
        out = [np.zeros((nnc, N, N)) for _ in range(4)]
        u1 = np.ascontiguousarray(g.ucell1, dtype=np.int64)
        u2 = np.ascontiguousarray(g.ucell2, dtype=np.int64)
        t1 = np.array(g.t1)
        t2 = np.array(g.t2)
        mdl = _model_struct(s)
        lib.fo_pair_tables(ctypes.c_int64(N), _ptr(X), ctypes.c_int64(nnc), _ptr(u1), _ptr(u2), _ptr(t1), _ptr(t2),
                           ctypes.byref(mdl), *[_ptr(o) for o in out])
        return PairTables(*out)
    N = s.ndim
    nnc = len(g.ucell1)
    X = g.coords
    tm = np.zeros((nnc, N, N))
    tp = np.zeros((nnc, N, N))
    vm = np.zeros((nnc, N, N))
    vp = np.zeros((nnc, N, N))
    ri = X[:, None, :]
    for c in range(nnc):
        n1, n2 = int(g.ucell1[c]), int(g.ucell2[c])
        Xm = _shift_coords(X, n1, n2, g, -1.0)
        Xp = _shift_coords(X, n1, n2, g, +1.0)
        tm[c] = ft(s, ri, Xm[None, :, :])
        tp[c] = ft(s, ri, Xp[None, :, :])
        vm[c] = fv(s, ri, Xm[None, :, :])
        vp[c] = fv(s, ri, Xp[None, :, :])
    return PairTables(tm, tp, vm, vp)


def long_range_interaction(s: Setup, g: Geometry, use_c: Optional[bool] = None) -> np.ndarray:
    """HartreeFock.f90:14-53: LR(n,m) = sum over |n1|,|n2|,|n1+n2|<=numC of fv(r_n - n1 t1 - n2 t2, r_m)."""
    N = s.ndim
    lib = _clib() if use_c in (None, True) else None
    if use_c and lib is None:
        raise RuntimeError("oracle/libforge_oracle.so is not built")
    if lib is not None:
        import ctypes
        LR = np.zeros((N, N))
        X = np.ascontiguousarray(g.coords)
        mdl = _model_struct(s)
        lib.fo_long_range(ctypes.c_int64(N), _ptr(X), _ptr(np.array(g.t1)), _ptr(np.array(g.t2)),
                          ctypes.c_int64(s.numC), ctypes.byref(mdl), _ptr(LR))
        return LR
    X = g.coords
    LR = np.zeros((N, N))
    nC = s.numC
    for n1 in range(-nC, nC + 1):
        for n2 in range(-nC, nC + 1):
            if -nC <= n1 + n2 <= nC:
                Xs = X.copy()
                Xs[:, 0] = X[:, 0] - n1 * g.t1[0] - n2 * g.t2[0]
                Xs[:, 1] = X[:, 1] - n1 * g.t1[1] - n2 * g.t2[1]
                LR += fv(s, Xs[:, None, :], X[None, :, :])
    # only m >= n is computed, then mirrored (HartreeFock.f90:28-51)
    iu = np.triu_indices(N, 1)
    LR.T[iu] = LR[iu]
    return LR


# ---------------------------------------------------------------------------
# Hamiltonian (HartreeFock.f90:57-127)
# ---------------------------------------------------------------------------
def hamiltonian(s: Setup, g: Geometry, T: PairTables, potential, P, vk) -> np.ndarray:
    """Full Hermitian H(k) whose lower triangle is the reference's zH (HartreeFock.f90:57-127).

    P has shape (NNC, N, N) with P[c] = zFock(:,:,c+1).  fphase=0 makes zphase=1.
    """
    N = s.ndim
    nnc = T.tm.shape[0]
    alpha = s.alpha
    H = np.zeros((N, N), dtype=np.complex128)
    H += -alpha * T.vm[0] * np.conj(P[0]) + T.tm[0]
    zs = np.zeros((N, N), dtype=np.complex128)
    for c in range(1, nnc):
        sh = cell_shift(g, c)
        th = float(vk[0] * sh[0] + vk[1] * sh[1])
        em = complex(math.cos(th), -math.sin(th))   # exp(-i k.R)
        ep = complex(math.cos(th), math.sin(th))    # exp(+i k.R)
        H += T.tm[c] * em + T.tp[c] * ep
        zs += -alpha * T.vm[c] * np.conj(P[c]) * em
        # - alpha fv(r_j, r_i - R) P(j,i) e^{+ikR}: vm[c][j,i] transposed
        zs += -alpha * T.vm[c].T * P[c].T * ep
    H += zs
    if s.fphase != 0:
        X = g.coords
        ph = np.exp(-1j * ((X[:, None, 0] - X[None, :, 0]) * vk[0] + (X[:, None, 1] - X[None, :, 1]) * vk[1]) * s.fphase)
        H *= ph
    H[np.diag_indices(N)] += potential
    if s.nlayers > 1:
        per = N // s.nlayers
        for n1 in range(s.nlayers):
            H[np.arange(per) + n1 * per, np.arange(per) + n1 * per] += (n1 - (s.nlayers - 1) / 2.0) * s.Delta / (s.nlayers - 1)
    # zH holds only the lower triangle (HartreeFock.f90:76); Hermitian completion
    L = np.tril(H)
    return L + np.conj(np.tril(H, -1)).T


def eigh_lower(H: np.ndarray, nUpper: int):
    """zdiagRed (LapackRoutines.f90:381-433): zheevr('V','I','L', il=1, iu=nUpper, abstol=dlamch('S'))."""
    from scipy.linalg import lapack
    n = H.shape[0]
    safemin = np.finfo(np.float64).tiny
    w, z, m, isuppz, info = lapack.zheevr(H, compute_v=1, range="I", lower=1, il=1, iu=nUpper,
                                          abstol=safemin, lwork=max(65 * n, 1), lrwork=max(24 * n, 1),
                                          liwork=max(10 * n, 1))
    if info != 0:
        raise RuntimeError(f"zheev failed {info}")
    return w[:m].copy(), z[:, :m].copy()


def bloch_phase_int(ivk1: int, ivk2: int, n1: int, n2: int, numk: int) -> complex:
    """exp(-2 pi i (ivk1 n1 + ivk2 n1 + ivk2 n2)/numk) of HartreeFock.f90:471 and 521."""
    th = -2.0 * PI * float(ivk1 * n1 + ivk2 * n1 + ivk2 * n2) / float(numk)
    return complex(math.cos(th), math.sin(th))


def solve(s: Setup, g: Geometry, T: PairTables, potential, P, keep_h=False):
    """Solve (HartreeFock.f90:402-483).

    Returns Bands (numb, Nk), zEigenvectors (N, numb, Nk), zFockBulk (NNC, N, N) (not divided by Nk),
    plus the full eigenvalue lists of bands 1..nUpper per k.
    """
    N, Nk, numb = s.ndim, s.Nk, s.numb
    nL, nU = s.nLower, s.nUpper
    nnc = T.tm.shape[0]
    bands = np.zeros((numb, Nk))
    evecs = np.zeros((N, numb, Nk), dtype=np.complex128)
    bulk = np.zeros((nnc, N, N), dtype=np.complex128)
    allw = np.zeros((nU, Nk))
    Hs = []
    for ic in range(Nk):
        ivk1, ivk2 = (int(x) for x in g.kcomp[ic])
        vk = g.kvals[ivk1, ivk2]
        H = hamiltonian(s, g, T, potential, P, vk)
        if keep_h:
            Hs.append(H.copy())
        w, Z = eigh_lower(H, nU)
        allw[:, ic] = w
        bands[:, ic] = w[nL - 1:nU]
        evecs[:, :, ic] = Z[:, nL - 1:nU]
        if s.fphase != 0:
            zph = np.exp(1j * (g.coords[:, 0] * vk[0] + g.coords[:, 1] * vk[1]) * s.fphase)
        else:
            zph = 1.0
        occ = np.conj(Z[:, :nL - 1] * (zph if np.ndim(zph) == 0 else zph[:, None]))
        Ck = occ @ np.conj(occ).T     # sum_n conj(psi_i) psi_j
        bulk[0] += Ck
        for c in range(1, nnc):
            bulk[c] += Ck * bloch_phase_int(ivk1, ivk2, int(g.ucell1[c]), int(g.ucell2[c]), s.numk)
    out = dict(bands=bands, evecs=evecs, bulk=bulk, eigs=allw)
    if keep_h:
        out["H"] = Hs
    return out


# ---------------------------------------------------------------------------
# Sorting and Fermi level
# ---------------------------------------------------------------------------
def dsort_lists(arr: np.ndarray) -> np.ndarray:
    """Heap sort on column 0 of arr (rows moved together), TightBinding.f90:984-1027 (not stable)."""
    a = [list(r) for r in np.asarray(arr, dtype=np.float64)]
    n = len(a)
    if n < 2:
        return np.array(a)
    # 1-based indexing as in the reference
    a = [None] + a
    l = n // 2 + 1
    ir = n
    while True:
        if l > 1:
            l -= 1
            copy = list(a[l])
        else:
            copy = list(a[ir])
            a[ir] = list(a[1])
            ir -= 1
            if ir == 1:
                a[1] = copy
                break
        i = l
        j = 2 * l
        while j <= ir:
            if j < ir and a[j][0] < a[j + 1][0]:
                j += 1
            if copy[0] < a[j][0]:
                a[i] = list(a[j])
                i = j
                j = 2 * j
            else:
                j = ir + 1
        a[i] = copy
    return np.array(a[1:])


def sort_energies_1spin(s: Setup, g: Geometry, bands, evecs=None):
    """SortEnergies_1Spin (HartreeFock.f90:885-925).

    Returns (sorted energies, sorted flat indices (1-based icount), nSortedMomenta, zSortedEigenvectors or None).
    """
    Nk, numb = s.Nk, s.numb
    n = Nk * numb
    e = np.zeros((n, 2))
    for ic in range(1, n + 1):
        indev = (ic - 1) // Nk + 1
        e[ic - 1, 0] = bands[indev - 1, ic - (indev - 1) * Nk - 1]
        e[ic - 1, 1] = float(ic)
    srt = dsort_lists(e)
    idx = np.rint(srt[:, 1]).astype(np.int64)
    indev = (idx - 1) // Nk + 1
    kidx = idx - (indev - 1) * Nk           # 1-based k
    moms = g.kcomp[kidx - 1].copy()
    sv = None
    if evecs is not None:
        sv = evecs[:, indev - 1, kidx - 1]
    return srt[:, 0].copy(), idx, moms, sv, indev - 1, kidx - 1


def fortran_nint(x: float) -> int:
    """Fortran NINT: round half away from zero."""
    return int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5))


def fermi_level(s: Setup, sorted_e, spin_factor: Optional[int] = None):
    """Main.f90:400-412: nFermiLevel, FermiEnergy, nOccStates, nPartOccStates, DegFactor.

    ``spin_factor`` replaces the numS factor of nFermiLevel; the initial guess (Main.f90:255) has none.
    """
    Nk = s.Nk
    fac = s.numS if spin_factor is None else spin_factor
    nF = fac * fortran_nint(float(Nk * s.NeutralityPoint) + float(Nk) / 2.0 * s.nfilling)
    EF = (sorted_e[nF - 1] + sorted_e[nF]) / 2.0
    tol = s.EnergyTolerance
    nocc = 0
    npart = 0
    for e in sorted_e:
        if (e - EF) < -tol:
            nocc += 1
        elif abs(e - EF) < tol:
            nocc += 1
            npart += 1
    with np.errstate(divide="ignore", invalid="ignore"):
        deg = np.float64(1.0) / np.float64(npart) * np.float64(nF + npart - nocc)
    return nF, EF, nocc, npart, float(deg)


def zdeg_weight(s: Setup, degf: float) -> complex:
    """zdeg of HartreeFock.f90:529: cmplx(DegFactor, dp) -> real(DegFactor,4) + 8i in reference mode."""
    if s.degfactor_mode == "reference":
        with np.errstate(over="ignore", invalid="ignore"):
            return complex(float(np.float32(degf)), 8.0)
    return complex(degf, 0.0)


def get_fock(s: Setup, g: Geometry, sorted_vecs, moms, nocc: int, npart: int, degf: float) -> np.ndarray:
    """GetFock (HartreeFock.f90:487-560): window projector into all NNC cells (not divided by Nk)."""
    N = s.ndim
    nnc = len(g.ucell1)
    out = np.zeros((nnc, N, N), dtype=np.complex128)
    zdeg = zdeg_weight(s, degf)
    for rng, extra in ((range(0, nocc - npart), 1.0 + 0j), (range(nocc - npart, nocc), zdeg)):
        for nb in rng:
            ivk1, ivk2 = (int(x) for x in moms[nb])
            vk = g.kvals[ivk1, ivk2]
            psi = sorted_vecs[:, nb]
            if s.fphase != 0:
                psi = psi * np.exp(1j * (g.coords[:, 0] * vk[0] + g.coords[:, 1] * vk[1]) * s.fphase)
            zp = np.conj(psi)
            outer = np.outer(zp, np.conj(zp))
            for c in range(nnc):
                out[c] += outer * (bloch_phase_int(ivk1, ivk2, int(g.ucell1[c]), int(g.ucell2[c]), s.numk) * extra)
    return out


# ---------------------------------------------------------------------------
# C3-reduced solve and projector (nenforceC3 = 1; HartreeFock.f90:131-398, 564-881)
# ---------------------------------------------------------------------------
def c3_invariant(numk: int, icount: int) -> bool:
    """The k points Solve_C3 / GetFock_C3 treat as C3-invariant (HartreeFock.f90:219, 588): icount 1,
    numk/3*(numk+1)+1 and 2*numk/3*(numk+1)+1 (1-based, integer division).  These are the invariant
    points of the grid only when numk is a multiple of 3."""
    return icount in (1, numk // 3 * (numk + 1) + 1, 2 * numk // 3 * (numk + 1) + 1)


def c3_related_momenta(s: Setup, g: Geometry) -> np.ndarray:
    """C3_RelatedMomenta (HartreeFock.f90:151-166): (Nk, 3) 1-based icounts of k, C3 k and C3^2 k,
    icount = ivk1*numk + ivk2 + 1."""
    numk = s.numk
    rel = np.zeros((s.Nk, 3), dtype=np.int64)
    for ic in range(1, s.Nk + 1):
        a, b = (int(x) for x in g.kcomp[ic - 1])
        rel[ic - 1, 0] = ic
        rel[ic - 1, 1] = ((-a - b) % numk) * numk + (a % numk) + 1
        rel[ic - 1, 2] = (b % numk) * numk + ((-a - b) % numk) + 1
    return rel


def c3_representatives(s: Setup, rel: np.ndarray) -> list:
    """MomentaMod_C3 (HartreeFock.f90:168-187): the first k of every C3 orbit, in icount order."""
    included = set()
    reps = []
    for ic in range(1, s.Nk + 1):
        if ic not in included:
            reps.append(ic)
            included.update((ic, int(rel[ic - 1, 1]), int(rel[ic - 1, 2])))
    return reps


def _corner_sites(s: Setup):
    """(0-based index of site ndim/nlayers*(l-1) + ndim/nlayers/2, of site ndim/nlayers*l, RotateLayers(l))."""
    per = s.ndim // s.nlayers
    return [(per * l + per // 2 - 1, per * (l + 1) - 1, int(s.RotateLayers[l])) for l in range(s.nlayers)]


def _c3_vector_phase(s: Setup, q: int) -> np.ndarray:
    """zphase of the C3-rotated eigenvectors for fphase = 0 (HartreeFock.f90:223-235, 249-261): 1 except
    exp(-+2 pi i q/numk) on the two corner sites of each layer (sign by RotateLayers)."""
    z = np.ones(s.ndim, dtype=np.complex128)
    th = 2 * PI * float(q) / float(s.numk)
    for ih, ie, rot in _corner_sites(s):
        if rot == -1:
            z[ih], z[ie] = np.exp(complex(0.0, -th)), np.exp(complex(0.0, th))
        elif rot == 1:
            z[ih], z[ie] = np.exp(complex(0.0, th)), np.exp(complex(0.0, -th))
    return z


def _c3_matrix_image(s: Setup, M: np.ndarray, p0: np.ndarray, q: int) -> np.ndarray:
    """M(nC3pairs, nC3pairs) with the corner phases of HartreeFock.f90:303-327: for RotateLayers -1, the
    rows of the two corner sites times exp(-i th), exp(+i th) and their columns times exp(+i th),
    exp(-i th), th = 2 pi q/numk; the opposite signs for RotateLayers 1.  The first image takes
    q = ivk1+ivk2, the second (applied to the first) q = -ivk1 (HartreeFock.f90:342-366)."""
    out = M[np.ix_(p0, p0)].copy()
    th = 2 * PI * float(abs(q)) / float(s.numk)
    sgn = 1.0 if q >= 0 else -1.0
    em, ep = np.exp(complex(0.0, -sgn * th)), np.exp(complex(0.0, sgn * th))
    for ih, ie, rot in _corner_sites(s):
        if rot == -1:
            out[ih, :] *= em
            out[ie, :] *= ep
            out[:, ih] *= ep
            out[:, ie] *= em
        elif rot == 1:
            out[ih, :] *= ep
            out[ie, :] *= em
            out[:, ih] *= em
            out[:, ie] *= ep
    return out


def _c3_orbit_sum(s: Setup, g: Geometry, B1: np.ndarray, ka, kb, kc) -> np.ndarray:
    """B1 and its two C3 images spread over the neighbour cells (HartreeFock.f90:292-372): cell c gets
    B1 with the Bloch phase of k = ka, the first image with that of kb, the second with that of kc."""
    nnc = len(g.ucell1)
    p0 = g.c3pairs - 1
    a, b = ka
    T = np.zeros((nnc, s.ndim, s.ndim), dtype=np.complex128)
    T[0] = B1
    for c in range(1, nnc):
        T[c] = B1 * bloch_phase_int(a, b, int(g.ucell1[c]), int(g.ucell2[c]), s.numk)
    M1 = _c3_matrix_image(s, B1, p0, a + b)
    T[0] += M1
    for c in range(1, nnc):
        T[c] += M1 * bloch_phase_int(kb[0], kb[1], int(g.ucell1[c]), int(g.ucell2[c]), s.numk)
    M2 = _c3_matrix_image(s, M1, p0, -a)
    T[0] += M2
    for c in range(1, nnc):
        T[c] += M2 * bloch_phase_int(kc[0], kc[1], int(g.ucell1[c]), int(g.ucell2[c]), s.numk)
    return T


def solve_c3(s: Setup, g: Geometry, T: PairTables, potential, P):
    """Solve_C3 (HartreeFock.f90:131-398), fphase = 0: one eigen-solve per C3 orbit of k points.

    The bands of the orbit's representative are copied to the two rotated k; for orbits of three
    points, the eigenvectors of C3 k and C3^2 k are the representative's permuted by nC3pairs twice
    and once, with the corner phases of _c3_vector_phase.  The bulk projector of the representative
    is added with its two C3 images (the third of the sum for the invariant points).  Returns the
    dict of ``solve``.  numk must be a multiple of 3: for other numk the reference treats k points
    that are not C3-invariant as invariant and leaves the eigenvectors of their orbit unset.
    """
    if s.numk % 3 != 0:
        raise ValueError("Solve_C3 needs numk divisible by 3")
    if s.fphase != 0:
        raise ValueError("the C3-reduced solve is restated for fphase = 0")
    N, Nk, numb, numk = s.ndim, s.Nk, s.numb, s.numk
    nL, nU = s.nLower, s.nUpper
    nnc = T.tm.shape[0]
    rel = c3_related_momenta(s, g)
    p0 = g.c3pairs - 1
    bands = np.zeros((numb, Nk))
    evecs = np.zeros((N, numb, Nk), dtype=np.complex128)
    bulk = np.zeros((nnc, N, N), dtype=np.complex128)
    allw = np.zeros((nU, Nk))
    for ic in c3_representatives(s, rel):
        a, b = (int(x) for x in g.kcomp[ic - 1])
        k2, k3 = int(rel[ic - 1, 1]), int(rel[ic - 1, 2])
        H = hamiltonian(s, g, T, potential, P, g.kvals[a, b])
        w, Z = eigh_lower(H, nU)
        for kk in (ic, k2, k3):
            bands[:, kk - 1] = w[nL - 1:nU]
            allw[:, kk - 1] = w
        evecs[:, :, ic - 1] = Z[:, nL - 1:nU]
        inv = c3_invariant(numk, ic)
        if not inv:
            c2a, c2b = (int(x) for x in g.kcomp[k2 - 1])
            c3b = int(g.kcomp[k3 - 1][1])
            evecs[:, :, k2 - 1] = Z[p0[p0], nL - 1:nU] * _c3_vector_phase(s, c2a + c2b)[:, None]
            evecs[:, :, k3 - 1] = Z[p0, nL - 1:nU] * _c3_vector_phase(s, c3b)[:, None]
        occ = np.conj(Z[:, :nL - 1])
        B1 = occ @ np.conj(occ).T
        kb = tuple(int(x) for x in g.kcomp[k3 - 1])
        kc = tuple(int(x) for x in g.kcomp[k2 - 1])
        Tk = _c3_orbit_sum(s, g, B1, (a, b), kb, kc)
        bulk += Tk / 3.0 if inv else Tk
    return dict(bands=bands, evecs=evecs, bulk=bulk, eigs=allw)


def get_fock_c3(s: Setup, g: Geometry, sorted_vecs, moms, nocc: int, npart: int, degf: float) -> np.ndarray:
    """GetFock_C3 (HartreeFock.f90:564-881), fphase = 0: GetFock for states at k points that are not
    C3-invariant; a state at an invariant k enters as the third of its projector plus its two C3
    images (with the Bloch phase of its own k in every cell)."""
    N = s.ndim
    nnc = len(g.ucell1)
    out = np.zeros((nnc, N, N), dtype=np.complex128)
    zdeg = zdeg_weight(s, degf)
    for rng, extra in ((range(0, nocc - npart), 1.0 + 0j), (range(nocc - npart, nocc), zdeg)):
        for nb in rng:
            a, b = (int(x) for x in moms[nb])
            zp = np.conj(sorted_vecs[:, nb])
            outer = np.outer(zp, np.conj(zp))
            if not c3_invariant(s.numk, a * s.numk + b + 1):
                for c in range(nnc):
                    out[c] += outer * (bloch_phase_int(a, b, int(g.ucell1[c]), int(g.ucell2[c]), s.numk) * extra)
            else:
                out += _c3_orbit_sum(s, g, outer * extra, (a, b), (a, b), (a, b)) / complex(3.0, 0.0)
    return out


def enforce_symmetries(s: Setup, g: Geometry, P) -> np.ndarray:
    """Main.f90:513-534, applied to the new zFock of each SCF iteration (not to the initial guess):
    time reversal P <- Re P, then C2 P(m) <- (P(m) + conj(P(m)(p, p))^T)/2, then C2T
    P(m) <- (P(m) + P(m)(p, p)^T)/2 for every cell m, p = nC2pairs.  The right-hand sides are
    evaluated before the assignment, as in the Fortran array expressions."""
    if not (s.nenforceT or s.nenforceC2 or s.nenforceC2T):
        return P
    P = np.array(P, dtype=np.complex128)
    if s.nenforceT == 1:
        P = P.real.astype(np.complex128)
    if s.nenforceC2 == 1 or s.nenforceC2T == 1:
        if np.any(g.c2pairs < 1):
            raise ValueError("nC2pairs does not pair every site (C2_RelatedPoints reported a mismatch)")
        p0 = g.c2pairs - 1
    if s.nenforceC2 == 1:
        for m in range(P.shape[0]):
            P[m] = 0.5 * (P[m] + np.conj(P[m][np.ix_(p0, p0)].T))
    if s.nenforceC2T == 1:
        for m in range(P.shape[0]):
            P[m] = 0.5 * (P[m] + P[m][np.ix_(p0, p0)].T)
    return P


# ---------------------------------------------------------------------------
# Valley projection (nenforceValley = 1; Main.f90:470-500, TightBinding.f90:60-270,
# LapackRoutines.f90:241-267, 865-893)
# ---------------------------------------------------------------------------
def rot_matrix(s: Setup) -> np.ndarray:
    """RotMatrix = reshape([c, -s, s, c], [2, 2]) with c, s of half the twist angle (Main.f90:133),
    as a [row, col] array."""
    m = s.ntheta
    cs = 1.0 - 1.0 / (2.0 * (3.0 * m ** 2 + 3.0 * m + 1.0))
    th = 0.5 * math.acos(cs)
    return np.array([[math.cos(th), math.sin(th)], [-math.sin(th), math.cos(th)]])


def ftvalley(dx, dy, Rm) -> np.ndarray:
    """ftvalley (TightBinding.f90:235-270) of the separations (dx, dy) = r_i - r_j (arrays): i
    sign(cos 3 phi)/sqrt(27) for 0.2 < |r_i - r_j| < 1.2, phi the angle of RotMatrix (r_i - r_j), and 0
    otherwise."""
    dx = np.asarray(dx, dtype=np.float64)
    dy = np.asarray(dy, dtype=np.float64)
    rij = np.sqrt(dx ** 2 + dy ** 2)
    x = Rm[0, 0] * dx + Rm[0, 1] * dy
    y = Rm[1, 0] * dx + Rm[1, 1] * dy
    with np.errstate(divide="ignore", invalid="ignore"):
        at = np.arctan(y / x)
    phi = np.where(x > 0, at, np.where((x < 0) & (y > 0), at + PI, -PI + at))
    phi = np.where(x == 0, np.where(y > 0, PI / 2.0, -PI / 2.0), phi)
    val = 1j * np.copysign(1.0, np.cos(3.0 * phi)) / math.sqrt(27.0)
    return np.where((rij < 1.2) & (rij > 0.2), val, 0.0 + 0.0j)


def valley_phase(s: Setup, g: Geometry, vk) -> np.ndarray:
    """ValleyPhase (TightBinding.f90:60-157), fphase = 0: the valley operator at k, nonzero only between
    sites of the same sublattice block of a layer; each pair adds its term in the home cell and in
    the neighbour cells R_c (r_j - R_c with exp(-i k.R_c), r_i - R_c with exp(+i k.R_c)), with
    RotMatrix^T for layers rotated by -1 and RotMatrix for layers rotated by +1."""
    if s.fphase != 0:
        raise ValueError("the valley operator is restated for fphase = 0")
    N = s.ndim
    per = N // s.nlayers
    R = rot_matrix(s)
    X = g.coords
    V = np.zeros((N, N), dtype=np.complex128)
    for l in range(s.nlayers):
        rl = int(s.RotateLayers[l])
        if rl not in (-1, 1):
            continue
        Rm = R.T if rl == -1 else R
        for lo, hi in ((per * l, per * l + per // 2), (per * l + per // 2, per * (l + 1))):
            xi, yi = X[lo:hi, 0][:, None], X[lo:hi, 1][:, None]
            xj, yj = X[lo:hi, 0][None, :], X[lo:hi, 1][None, :]
            blk = ftvalley(xi - xj, yi - yj, Rm)
            for c in range(1, len(g.ucell1)):
                n1, n2 = float(g.ucell1[c]), float(g.ucell2[c])
                sx, sy = n1 * g.t1[0] + n2 * g.t2[0], n1 * g.t1[1] + n2 * g.t2[1]
                kr = float(vk[0] * sx + vk[1] * sy)
                blk = blk + ftvalley(xi - ((xj - n1 * g.t1[0]) - n2 * g.t2[0]),
                                     yi - ((yj - n1 * g.t1[1]) - n2 * g.t2[1]), Rm) * np.exp(complex(0.0, -kr))
                blk = blk + ftvalley(((xi - n1 * g.t1[0]) - n2 * g.t2[0]) - xj,
                                     ((yi - n1 * g.t1[1]) - n2 * g.t2[1]) - yj, Rm) * np.exp(complex(0.0, kr))
            V[lo:hi, lo:hi] += blk
    return V


def unitarize(A: np.ndarray) -> np.ndarray:
    """z_unitarize (LapackRoutines.f90:865-893): U sign(Lambda) U^H of the Hermitian A = U Lambda U^H
    (sign(1, 0) = +1)."""
    w, U = np.linalg.eigh(A)
    return (U * np.copysign(1.0, w)[None, :]) @ U.conj().T


def valley_transform(s: Setup, g: Geometry, evecs: np.ndarray) -> np.ndarray:
    """ValleyTransform (TightBinding.f90:162-208): at every k the window eigenvectors X (N x numb)
    become X unitarize(X^H V(k) X), V(k) = valley_phase."""
    out = np.empty_like(evecs)
    for ic in range(s.Nk):
        a, b = (int(x) for x in g.kcomp[ic])
        X = evecs[:, :, ic]
        Vp = X.conj().T @ (valley_phase(s, g, g.kvals[a, b]) @ X)
        out[:, :, ic] = X @ unitarize(Vp)
    return out


def window_fock(s: Setup, g: Geometry, sol: dict, sv, moms, nocc: int, npart: int, degf: float) -> np.ndarray:
    """The window part of the new zFock (before + zFockBulk, / Nk): GetFock (or GetFock_C3), or with
    nenforceValley = 1 the average of GetFock of the sorted eigenvectors and of their valley-transformed
    copies (Main.f90:470-500: zFock = .5 (GetFock + GetFock after ValleyTransform) + zFockBulk)."""
    Pw = get_fock_any(s, g, sv, moms, nocc, npart, degf)
    if s.nenforceValley != 1:
        return Pw
    ev = valley_transform(s, g, sol["evecs"])
    _, _, moms2, sv2, _, _ = sort_energies_1spin(s, g, sol["bands"], ev)
    return 0.5 * (Pw + get_fock_any(s, g, sv2, moms2, nocc, npart, degf))


def solve_any(s: Setup, g: Geometry, T: PairTables, potential, P):
    """Solve or Solve_C3 by nenforceC3 (Main.f90:244-250, 375-381)."""
    return solve_c3(s, g, T, potential, P) if s.nenforceC3 == 1 else solve(s, g, T, potential, P)


def get_fock_any(s: Setup, g: Geometry, sorted_vecs, moms, nocc: int, npart: int, degf: float) -> np.ndarray:
    """GetFock or GetFock_C3 by nenforceC3 (Main.f90:273-279, 502-508)."""
    f = get_fock_c3 if s.nenforceC3 == 1 else get_fock
    return f(s, g, sorted_vecs, moms, nocc, npart, degf)


# ---------------------------------------------------------------------------
# Energies, ODA step, potential (HartreeFock.f90:1012-1227, Main.f90:300-342, 549-595)
# ---------------------------------------------------------------------------
def kinetic_energy(s: Setup, T: PairTables, P) -> float:
    """GetKineticEnergy (HartreeFock.f90:1012-1059)."""
    nnc = T.tm.shape[0]
    z = np.sum(T.tm[0] * P[0])
    for c in range(1, nnc):
        z += np.sum(T.tm[c] * P[c]) + np.sum(T.tp[c] * np.conj(P[c].T))
    N = P.shape[1]
    if s.nlayers > 1 and s.Delta != 0.0:
        per = N // s.nlayers
        for n1 in range(s.nlayers):
            d = np.diagonal(P[0])[n1 * per:(n1 + 1) * per]
            z += np.sum(d) * ((n1 - (s.nlayers - 1) / 2.0) * s.Delta / (s.nlayers - 1))
    return float(z.real)


def fock_energy(s: Setup, T: PairTables, P) -> float:
    """GetFockEnergy (HartreeFock.f90:1098-1145)."""
    nnc = T.vm.shape[0]
    z = -0.5 * np.sum(T.vm[0] * np.abs(P[0]) ** 2)
    for c in range(1, nnc):
        z += -0.5 * np.sum(T.vm[c] * np.abs(P[c]) ** 2) - 0.5 * np.sum(T.vp[c] * np.abs(P[c].T) ** 2)
    return float(z)


def hartree_hubbard_energy(LR, d1, d2):
    """GetHartreeHubbardEnergy (HartreeFock.f90:1066-1092)."""
    sm = d1 + d2
    eh = 0.5 * float(sm @ LR @ sm)
    eu = float(np.dot(d1, d2))
    return eh, eu


@dataclasses.dataclass
class Energies:
    kinetic: float
    fock: float
    hartree: float
    hubbard: float

    def total(self, s: Setup) -> float:
        """Main.f90:312 / 556 for numS=1."""
        return (s.alpha * self.fock * (3 - s.numS) + self.kinetic * (3 - s.numS)
                + s.U * self.hubbard + s.alphaH * self.hartree)


def energies(s: Setup, T: PairTables, LR, P, dens) -> Energies:
    d = dens - 0.5
    eh, eu = hartree_hubbard_energy(LR, d, d)
    return Energies(kinetic_energy(s, T, P), fock_energy(s, T, P), eh, eu)


def optimal_step(s: Setup, T: PairTables, LR, P_new, P_in, dens, dens_in, E_in: Energies, energy_fn=None):
    """OptimalStep (HartreeFock.f90:1148-1227): returns (Step, energies at Step, E1, E_half).

    ``energy_fn`` is ``energies`` (numS=1, the default) or ``energies_2spins`` (numS=2, spin-stacked
    P and densities); the step rule is the same for both.
    """
    energies_ = energies if energy_fn is None else energy_fn
    c0 = E_in.total(s)
    E1 = energies_(s, T, LR, P_new, dens)
    t1 = E1.total(s)
    Eh = energies_(s, T, LR, 0.5 * (P_in + P_new), .5 * (dens + dens_in))
    t2 = Eh.total(s)
    c1 = 4.0 * t2 - t1 - 3.0 * c0
    c2 = t1 - c0 - c1
    if c2 > 0 and abs(-c1 / 2.0 / c2 - .5) < 0.5:
        step = -c1 / 2.0 / c2
    elif t1 < c0:
        step = 1.0
    else:
        step = s.StepAlternative
    Es = energies_(s, T, LR, (1.0 - step) * P_in + step * P_new, (1 - step) * dens_in + step * dens)
    return step, Es, t1, t2


def potential(s: Setup, LR, dens) -> np.ndarray:
    """Main.f90:577-585 (numS=1): V_n = 2 alphaH sum_m LR(n,m)(n_m - 1/2) + U (n_n - 1/2)."""
    d = dens - 0.5
    return 2.0 * s.alphaH * (LR @ d) + s.U * d


def hf_residual(s: Setup, T: PairTables, V_new, V_old, P_new, P_old) -> float:
    """Residual of the Hartree-Fock mean field between iterations (eV).

    The reference logs max|dn| and dE only (Main.f90:616-623) and stops at
    itmax; this residual is the max over sites of |dV| and over pairs/cells of
    alpha*|fv|*|dP|, i.e. the largest change of any H_HF matrix element.
    """
    dV = float(np.max(np.abs(V_new - V_old)))
    dP = np.abs(P_new - P_old)
    nnc = T.vm.shape[0]
    r = 0.0
    for c in range(nnc):
        r = max(r, float(np.max(s.alpha * np.abs(T.vm[c]) * dP[c])))
        if c > 0:
            r = max(r, float(np.max(s.alpha * np.abs(T.vp[c]) * dP[c].T)))
    return max(dV, r)


# ---------------------------------------------------------------------------
# SCF driver (Main.f90:236-679, numS=1; symmetry switches of Main.f90:513-534 by the Setup flags)
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class IterationLog:
    it: int
    dn_max: float
    step: float
    dE: float
    E_in: float
    kin_in: float
    fock_in: float
    hartree_in: float
    hubbard_in: float
    EF: float
    nocc: int
    npart: int
    residual: float


def plain_guess(s: Setup, g: Geometry, T: PairTables):
    """Main.f90:236-288 (nRead=0): non-interacting bands, sort, Fermi, GetFock, P=(window+bulk)/Nk."""
    N = s.ndim
    nnc = len(g.ucell1)
    P0 = np.zeros((nnc, N, N), dtype=np.complex128)
    V0 = np.zeros(N)
    sol = solve_any(s, g, T, V0, P0)
    se, _, moms, sv, _, _ = sort_energies_1spin(s, g, sol["bands"], sol["evecs"])
    nF, EF, nocc, npart, degf = fermi_level(s, se, spin_factor=1)
    P = get_fock_any(s, g, sv, moms, nocc, npart, degf)
    P = (P + sol["bulk"]) / complex(float(s.Nk), 0.0)
    return P, dict(sol=sol, EF=EF, nocc=nocc, npart=npart, degf=degf)


class PulayMixer:
    """Anderson / Pulay mixing of the density matrix, the library's FORGE_MIX_PULAY option (no
    counterpart in the reference, which mixes with OptimalStep only).

    x_next = x + beta r - sum_i g_i (dX_i + beta dR_i), r = P_new - P_in, g minimising
    |r - sum_i g_i dR_i|, over the last `depth` difference pairs.  The pairs and the previous
    residual are stored in complex64, as on the device; x and r stay complex128.
    """

    def __init__(self, depth: int = 6, beta: float = 0.7):
        self.depth, self.beta = depth, beta
        self.pairs = []          # [dX (c64), dR (c64)], oldest first
        self.pending = None      # dX of the last step, waiting for its dR
        self.rprev = None

    def step(self, P_in, P_new):
        r = P_new - P_in
        if self.rprev is None:
            x = P_in + self.beta * r
        else:
            dR = (r - self.rprev.astype(np.complex128)).astype(np.complex64)
            self.pairs.append([self.pending, dR])
            if len(self.pairs) > self.depth:
                self.pairs.pop(0)
            k = len(self.pairs)
            G = np.zeros((k, k))
            b = np.zeros(k)
            for i, (_, di) in enumerate(self.pairs):
                d64 = di.astype(np.complex128)
                b[i] = float(np.real(np.vdot(d64, r)))
                for j, (_, dj) in enumerate(self.pairs):
                    G[i, j] = float(np.real(np.vdot(d64, dj.astype(np.complex128))))
            G[np.diag_indices(k)] += 1e-10 * np.max(np.diag(G))
            try:
                gam = np.linalg.solve(G, b)
            except np.linalg.LinAlgError:
                gam = np.zeros(k)
            x = P_in + self.beta * r
            for gi, (dx, dr) in zip(gam, self.pairs):
                x = x - gi * (dx.astype(np.complex128) + self.beta * dr.astype(np.complex128))
        self.pending = (x - P_in).astype(np.complex64)
        self.rprev = r.astype(np.complex64)
        return x


def run_scf(s: Setup, g: Optional[Geometry] = None, T: Optional[PairTables] = None, LR=None,
            P_init=None, itmax: Optional[int] = None, residual_tol: Optional[float] = None,
            keep_history: bool = False, mixer: Optional[PulayMixer] = None, linear_beta: Optional[float] = None):
    """Main.f90:236-679 for numS=1: initial guess, energies, potential, then the SCF loop with ODA mixing
    (or, with ``mixer``, Anderson / Pulay mixing: the state is the mixer's output, Step is 1 and the
    residual is that of (P_in, P_new); or, with ``linear_beta``, linear mixing: Main.f90:558-595 with
    the fixed Step = linear_beta in place of OptimalStep's, the library's FORGE_MIX_LINEAR).

    Stops after ``itmax`` iterations (reference behaviour) or earlier when
    ``residual_tol`` is given and the mean-field residual drops below it.
    """
    if g is None:
        g = build_geometry(s)
    if T is None:
        T = pair_tables(s, g)
    if LR is None:
        LR = long_range_interaction(s, g)
    if P_init is None:
        P, _ = plain_guess(s, g, T)
    else:
        P = np.array(P_init, dtype=np.complex128)
    dens = np.real(np.diagonal(P[0])).copy()
    E = energies(s, T, LR, P, dens)
    Etot = E.total(s)
    V = potential(s, LR, dens)
    dens_in = dens.copy()
    P_in = P.copy()
    logs = []
    history = []
    itmax = s.itmax if itmax is None else itmax
    it = 0
    last = {}
    while it < itmax:
        it += 1
        sol = solve_any(s, g, T, V, P)
        se, _, moms, sv, _, _ = sort_energies_1spin(s, g, sol["bands"], sol["evecs"])
        nF, EF, nocc, npart, degf = fermi_level(s, se)
        Pw = window_fock(s, g, sol, sv, moms, nocc, npart, degf)
        P_new = enforce_symmetries(s, g, (Pw + sol["bulk"]) / complex(float(s.Nk), 0.0))
        E_in, Etot_in = E, Etot
        dens_new = np.real(np.diagonal(P_new[0])).copy()
        if mixer is not None:
            res = hf_residual(s, T, potential(s, LR, dens_new), V, P_new, P_in)
            P = mixer.step(P_in, P_new)
            step, t1, t2 = 1.0, float("nan"), float("nan")
            dens = np.real(np.diagonal(P[0])).copy()
            E = energies(s, T, LR, P, dens)
            Etot = E.total(s)
            dn = float(np.max(np.abs(dens - dens_in)))
            V = potential(s, LR, dens)
        else:
            if linear_beta is not None:
                step, t1, t2 = float(linear_beta), float("nan"), float("nan")
            else:
                step, E, t1, t2 = optimal_step(s, T, LR, P_new, P_in, dens_new, dens_in, E_in)
            P = step * P_new + (1.0 - step) * P_in
            dens = np.real(np.diagonal(P[0])).copy()
            if linear_beta is not None:
                E = energies(s, T, LR, P, dens)
            Etot = E.total(s)
            dn = float(np.max(np.abs(dens - dens_in)))
            V_old = V
            V = potential(s, LR, dens)
            res = hf_residual(s, T, V, V_old, P, P_in)
        dens_in = dens.copy()
        P_in = P.copy()
        logs.append(IterationLog(it, dn, step, Etot_in - Etot, Etot_in, E_in.kinetic, E_in.fock,
                                 E_in.hartree, E_in.hubbard, EF, nocc, npart, res))
        last = dict(bands=sol["bands"], eigs=sol["eigs"], EF=EF, nocc=nocc, npart=npart, degf=degf,
                    P_new=P_new, step=step, E1=t1, Ehalf=t2)
        if keep_history:
            history.append(dict(P=P.copy(), V=V.copy(), **last))
        if residual_tol is not None and res < residual_tol:
            break
    return dict(P=P, V=V, dens=dens, E=E, Etot=Etot, logs=logs, geometry=g, tables=T, LR=LR,
                history=history, **last)


# ---------------------------------------------------------------------------
# Spin-polarised path (numS = 2; Main.f90:290-342, 365-595; HartreeFock.f90:929-1004)
# Spin-resolved arrays are stacked on a leading spin axis: P[sp, c, i, j] is zFock(i+1, j+1, c+1, sp+1),
# dens[sp, i] is Density(i+1, sp+1), V[sp, i] is Potential(i+1, sp+1).
# ---------------------------------------------------------------------------
def window_sort_2spins(s: Setup) -> np.ndarray:
    """nWindowSort_2Spins of Main.f90:416-419: W[i, sp] = W(i+1, sp+1) = (NP - 1, NP + 3) for both spins."""
    NP = s.NeutralityPoint
    return np.array([[NP - 1, NP - 1], [NP + 3, NP + 3]], dtype=np.int64)


def sort_energies_2spins(numk: int, numb: int, window, se1, se2):
    """SortEnergies_2Spins (HartreeFock.f90:929-1004): merges the two spin-sorted lists.

    Returns (energies, spin labels 1/2), each of length 2*numb*numk**2.  The first (W(1,1)-1)*Nk
    spin-1 states and (W(1,2)-1)*Nk spin-2 states are copied in front without merging; the states up
    to Nk*(W(2,sp)-1) are merged (runs may extend past that bound); the remaining spin-1 tail and
    then the spin-2 tail are appended unmerged.  As in the reference, the front copy of spin 2 reads
    the spin-2 list at the spin-1 counter (HartreeFock.f90:949), so every entry it writes is the
    spin-2 energy at position (W(1,1)-1)*Nk+1; only the labels of that block are per state.
    """
    W = np.asarray(window, dtype=np.int64)
    Nk = numk * numk
    n = numb * Nk
    se1 = np.asarray(se1, dtype=np.float64)
    se2 = np.asarray(se2, dtype=np.float64)
    out_e = np.zeros(2 * n)
    out_s = np.zeros(2 * n, dtype=np.int64)
    cb = 0

    def put(e, sp):
        nonlocal cb
        out_e[cb] = e
        out_s[cb] = sp
        cb += 1

    c1 = c2 = 1                                   # 1-based counters ncount1, ncount2
    for _ in range((int(W[0, 0]) - 1) * Nk):
        put(se1[c1 - 1], 1)
        c1 += 1
    for _ in range((int(W[0, 1]) - 1) * Nk):
        put(se2[c1 - 1], 2)
        c2 += 1
    lim1, lim2 = Nk * (int(W[1, 0]) - 1), Nk * (int(W[1, 1]) - 1)
    while c1 <= lim1 and c2 <= lim2:
        if se1[c1 - 1] <= se2[c2 - 1]:
            put(se1[c1 - 1], 1)
            c1 += 1
            while c1 <= n and se1[c1 - 1] <= se2[c2 - 1]:
                put(se1[c1 - 1], 1)
                c1 += 1
            put(se2[c2 - 1], 2)
            c2 += 1
        else:
            put(se2[c2 - 1], 2)
            c2 += 1
            while c2 <= n and se2[c2 - 1] <= se1[c1 - 1]:
                put(se2[c2 - 1], 2)
                c2 += 1
            put(se1[c1 - 1], 1)
            c1 += 1
    while c1 <= n:
        put(se1[c1 - 1], 1)
        c1 += 1
    while c2 <= n:
        put(se2[c2 - 1], 2)
        c2 += 1
    return out_e, out_s


def fermi_level_2spins(s: Setup, merged_e, labels):
    """Main.f90:421-453: nFermiLevel, FermiEnergy, nOccStates(2), nPartOccStates(2), DegFactor.

    Occupations are counted per spin label over the merged list; DegFactor is 0 when neither spin has
    a partially occupied state.
    """
    Nk = s.Nk
    nF = s.numS * fortran_nint(float(Nk * s.NeutralityPoint) + float(Nk) / 2.0 * s.nfilling)
    EF = (merged_e[nF - 1] + merged_e[nF]) / 2.0
    tol = s.EnergyTolerance
    nocc = [0, 0]
    npart = [0, 0]
    for e, sp in zip(merged_e, labels):
        k = 0 if sp == 1 else 1
        if (e - EF) < -tol:
            nocc[k] += 1
        elif abs(e - EF) < tol:
            nocc[k] += 1
            npart[k] += 1
    if npart[0] != 0 or npart[1] != 0:
        deg = 1.0 / float(npart[0] + npart[1]) * float(nF + npart[0] + npart[1] - nocc[0] - nocc[1])
    else:
        deg = 0.0
    return nF, EF, nocc, npart, deg


def energies_2spins(s: Setup, T: PairTables, LR, P, dens) -> Energies:
    """Main.f90:300-310 / OptimalStep for numS=2: kinetic and Fock energies summed over the spins,
    Hartree and Hubbard from (n_1 - 1/2, n_2 - 1/2)."""
    kin = sum(kinetic_energy(s, T, P[sp]) for sp in range(2))
    fock = sum(fock_energy(s, T, P[sp]) for sp in range(2))
    eh, eu = hartree_hubbard_energy(LR, dens[0] - 0.5, dens[1] - 0.5)
    return Energies(kin, fock, eh, eu)


def potential_2spins(s: Setup, LR, dens) -> np.ndarray:
    """Main.f90:331-341 / 586-594: V_1 = alphaH LR (n_1 + n_2 - 1) + U (n_2 - 1/2), V_2 likewise with
    U (n_1 - 1/2)."""
    h = s.alphaH * (LR @ (dens[0] + dens[1] - 1.0))
    return np.stack([h + s.U * (dens[1] - 0.5), h + s.U * (dens[0] - 0.5)])


def plain_guess_2spins(s: Setup, g: Geometry, T: PairTables):
    """Main.f90:236-292 with numS=2: the spin-1 guess of ``plain_guess``, copied to spin 2."""
    P1, info = plain_guess(s, g, T)
    return np.stack([P1, P1.copy()]), info


def _density_2spins(P) -> np.ndarray:
    return np.stack([np.real(np.diagonal(P[sp, 0])).copy() for sp in range(2)])


def run_scf_2spins(s: Setup, g: Optional[Geometry] = None, T: Optional[PairTables] = None, LR=None,
                   P_init=None, itmax: Optional[int] = None, residual_tol: Optional[float] = None,
                   keep_history: bool = False):
    """Main.f90:236-679 for numS=2 with ODA mixing (symmetry switches as in run_scf).

    Per iteration: both spins are solved with their own potential and density matrix, sorted, merged
    by ``sort_energies_2spins``, occupied by ``fermi_level_2spins`` (one Fermi level and DegFactor,
    per-spin counts), projected per spin, and mixed with one OptimalStep over the spin-summed energy.
    ``P_init`` (2, nnc, N, N) replaces the plain guess.  The residual is the largest of the per-spin
    mean-field residuals; ``dn`` in the logs is the largest per-spin max|dn| (DensityConvergence).
    """
    if s.numS != 2:
        raise ValueError("run_scf_2spins needs numS = 2")
    if g is None:
        g = build_geometry(s)
    if T is None:
        T = pair_tables(s, g)
    if LR is None:
        LR = long_range_interaction(s, g)
    if P_init is None:
        P, _ = plain_guess_2spins(s, g, T)
    else:
        P = np.array(P_init, dtype=np.complex128)
    dens = _density_2spins(P)
    E = energies_2spins(s, T, LR, P, dens)
    Etot = E.total(s)
    V = potential_2spins(s, LR, dens)
    dens_in = dens.copy()
    P_in = P.copy()
    W = window_sort_2spins(s)
    logs = []
    history = []
    itmax = s.itmax if itmax is None else itmax
    last = {}
    it = 0
    while it < itmax:
        it += 1
        sols, ses, movs = [], [], []
        for sp in range(2):
            sol = solve_any(s, g, T, V[sp], P[sp])
            se, _, moms, sv, _, _ = sort_energies_1spin(s, g, sol["bands"], sol["evecs"])
            sols.append(sol)
            ses.append(se)
            movs.append((moms, sv))
        me, ml = sort_energies_2spins(s.numk, s.numb, W, ses[0], ses[1])
        nF, EF, nocc, npart, degf = fermi_level_2spins(s, me, ml)
        P_new = np.stack([enforce_symmetries(s, g, (window_fock(s, g, sols[sp], movs[sp][1], movs[sp][0], nocc[sp],
                                                                 npart[sp], degf) + sols[sp]["bulk"])
                                             / complex(float(s.Nk), 0.0))
                          for sp in range(2)])
        E_in, Etot_in = E, Etot
        dens_new = _density_2spins(P_new)
        step, E, t1, t2 = optimal_step(s, T, LR, P_new, P_in, dens_new, dens_in, E_in,
                                       energy_fn=energies_2spins)
        Etot = E.total(s)
        P = step * P_new + (1.0 - step) * P_in
        dens = _density_2spins(P)
        dn = float(np.max(np.abs(dens - dens_in)))
        V_old = V
        V = potential_2spins(s, LR, dens)
        res = max(hf_residual(s, T, V[sp], V_old[sp], P[sp], P_in[sp]) for sp in range(2))
        dens_in = dens.copy()
        P_in = P.copy()
        logs.append(IterationLog(it, dn, step, Etot_in - Etot, Etot_in, E_in.kinetic, E_in.fock,
                                 E_in.hartree, E_in.hubbard, EF, nocc[0] + nocc[1], npart[0] + npart[1], res))
        last = dict(bands=np.stack([x["bands"] for x in sols]), EF=EF, nocc=nocc, npart=npart, degf=degf,
                    merged=(me, ml), P_new=P_new, step=step, E1=t1, Ehalf=t2)
        if keep_history:
            history.append(dict(P=P.copy(), V=V.copy(), **last))
        if residual_tol is not None and res < residual_tol:
            break
    return dict(P=P, V=V, dens=dens, E=E, Etot=Etot, logs=logs, geometry=g, tables=T, LR=LR,
                history=history, **last)


def order_parameters(s: Setup, g: Geometry, P) -> dict:
    """Order parameters from P(R=0) and the site maps (Geometry.f90:1140-1223).

    layer polarisation: sum over layer l of (l - (L-1)/2) * sum_i (n_i - 1/2);
    sublattice polarisation: A-block minus B-block density;
    C2T / C3 breaking norms: ||P(0) - g.P(0)||_F with g the site maps.
    """
    N = s.ndim
    L = s.nlayers
    per = N // L
    n = np.real(np.diagonal(P[0])) - 0.5
    layer = sum((l - (L - 1) / 2.0) * np.sum(n[l * per:(l + 1) * per]) for l in range(L))
    sub = sum(np.sum(n[l * per:l * per + per // 2]) - np.sum(n[l * per + per // 2:(l + 1) * per]) for l in range(L))
    c2 = g.c2pairs - 1
    c3 = g.c3pairs - 1
    P0 = P[0]
    c2t = float(np.linalg.norm(P0 - P0[np.ix_(c2, c2)].T)) if np.all(c2 >= 0) else float("nan")
    c3n = float(np.linalg.norm(P0 - P0[np.ix_(c3, c3)])) if np.all(c3 >= 0) else float("nan")
    return dict(layer_polarization=float(layer), sublattice_polarization=float(sub), c2t_breaking=c2t,
                c3_breaking=c3n)


def plot_bands_lines(s: Setup, g: Geometry, bands, EF: float):
    """PlotBands (TightBinding.f90:275-369) as a list of rows [x, Bands(1..numb) - EF] (p = 0)."""
    numk, numb, p = s.numk, s.numb, 0
    g1, g12 = g.g1, g.g12
    vK1x, vK1y = (g1[0] + g12[0]) / 3.0, (g1[1] + g12[1]) / 3.0
    vMx, vMy = (g1[0] + g12[0]) / 2.0, (g1[1] + g12[1]) / 2.0
    aKG = math.sqrt(vK1x ** 2 + vK1y ** 2)
    aGM = math.sqrt((vMx - g12[0]) ** 2 + (vMy - g12[1]) ** 2)
    aMK = math.sqrt((vK1x - vMx) ** 2 + (vK1y - vMy) ** 2)
    aT = 3 * aKG + aGM + aMK
    n3, n6, n2 = float(numk // 3), float(numk // 6), float(numk // 2)
    rows = []

    def row(x, i1, i2):
        k = g.kflat[i1, i2] - 1
        rows.append([x] + [bands[b, k] - EF for b in range(numb)])

    with np.errstate(divide="ignore", invalid="ignore"):
        for ivk in range(0, numk // 3):
            row(np.float64(ivk) * aKG / n3 / aT, (2 * numk // 3 + ivk) % numk, (2 * numk // 3 - 2 * ivk + p * numk // 2) % numk)
        row(aKG / aT, 0, p * numk // 2)
        for ivk in range(1, numk // 3 + 1):
            row(aKG / aT + aKG * ivk / n3 / aT, ivk % numk, (numk - 2 * ivk + p * numk // 2) % numk)
        for ivk in range(1, numk // 6 + 1):
            row(2 * aKG / aT + aMK * ivk / n6 / aT, (numk // 3 + ivk) % numk, (numk // 3 + ivk + p * numk // 2) % numk)
        for ivk in range(1, numk // 2):
            row((2 * aKG + aMK) / aT + aGM * ivk / n2 / aT, (numk // 2 - ivk) % numk, (numk // 2 + ivk + p * numk // 2) % numk)
        for ivk in range(0, numk // 3 + 1):
            row((2 * aKG + aMK + aGM) / aT + np.float64(ivk) * aKG / n3 / aT, ivk % numk, (ivk + p * numk // 2) % numk)
    return rows
