"""Learned SCF starting guess (no counterpart in the reference).

FORGE starts its SCF from the non-interacting bands (Main.f90:236-288) or a checkpoint
(Main.f90:202-234).  Here a small MLP, trained on GPU by the library's own kernels on
converged fields of smaller cells and other fillings, predicts the converged mean field
from local moire descriptors:

  site  i      -> density deviation n_i - 1/2          (its Hartree + Hubbard potential follows
                                                          from LR exactly, Main.f90:577-585)
  bond (i,j,R) -> Re, Im P_ij(R) for |r_i - r_j + R| < BOND_CUTOFF (the Fock hopping
                  renormalisation -alpha fv conj(P), HartreeFock.f90:81, 108-110)

Descriptors are periodic in the moire cell (cos/sin of the first-shell moire reciprocal
vectors at the site or bond centre: the local stacking registry), plus sublattice, layer,
bond vector, filling nu and 1/epsilon, so they transfer between twist angles.

The predicted field is diagonalised once (the cost of the plain guess) to give the starting
density matrix.  `start` then applies the fallback rule: the first SCF iteration runs from the
network's state and from the plain guess, and the SCF continues from the plain guess whenever
the network's first residual is worse (the price is one guess and one iteration of the loser).
`apply` alone is the cheaper form that compares the predicted field with the zero field.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from typing import Optional, Sequence

import numpy as np

from .api import ForgeError, Geometry, HartreeFock, Setup, _check, _ptr, load_library

BOND_CUTOFF = 1.6           # lattice constants a (2.46 A): up to 4th in-plane neighbours, AA-like interlayer
DENS_SCALE = 100.0          # network units of the site target
SITE_IN, BOND_IN = 12, 18
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "warmstart_weights.npz")


def _moire_g(geo: Geometry):
    g1 = np.asarray(geo.g1, float)
    g12 = np.asarray(geo.g12, float)
    g2 = g12 - g1
    return np.stack([g1, g2, -(g1 + g2)])


def _globals(setup: Setup, geo: Geometry):
    L = float(np.linalg.norm(geo.tn[:, 0]))
    return np.array([setup.nfilling / 4.0, 10.0 / setup.epsilon, 10.0 / L, setup.nlayers / 3.0])


def site_features(setup: Setup, geo: Geometry) -> np.ndarray:
    """(N, SITE_IN): registry embedding (6), sublattice, layer height, outer-layer flag, globals."""
    X = np.asarray(geo.Coords)
    N = X.shape[0]
    L = setup.nlayers
    per = N // L
    G = _moire_g(geo)
    ph = X[:, :2] @ G.T
    sub = np.where((np.arange(N) % per) < per // 2, 1.0, -1.0)
    z = X[:, 2] / (1.35772 * max(1, L - 1))
    layer = np.arange(N) // per
    outer = ((layer == 0) | (layer == L - 1)).astype(float)
    gl = np.broadcast_to(_globals(setup, geo)[:2], (N, 2))
    f = np.concatenate([np.cos(ph), np.sin(ph), sub[:, None], z[:, None], outer[:, None], gl,
                        np.full((N, 1), 10.0 / float(np.linalg.norm(geo.tn[:, 0])))], axis=1)
    assert f.shape[1] == SITE_IN
    return f.astype(np.float32)


def bond_list(setup: Setup, geo: Geometry, cutoff: float = BOND_CUTOFF):
    """All (i, j, c) with |r_i - (r_j - R_c)| < cutoff, c = 0..3 cells of nUnitCell_1/2."""
    X = np.asarray(geo.Coords)
    t1, t2 = geo.tn[:, 0], geo.tn[:, 1]
    out = []
    for c in range(4):
        R = geo.nUnitCell_1[c] * t1 + geo.nUnitCell_2[c] * t2
        Y = X[:, :2] - R[None, :]
        # cell lists would be faster; N^2 in blocks is fine up to N ~ 1.2e4
        for i0 in range(0, X.shape[0], 1024):
            d2 = ((X[i0:i0 + 1024, None, :2] - Y[None, :, :]) ** 2).sum(-1) + \
                 (X[i0:i0 + 1024, None, 2] - X[None, :, 2]) ** 2
            ii, jj = np.nonzero(d2 < cutoff * cutoff)
            out.append(np.stack([ii + i0, jj, np.full_like(ii, c)], axis=1))
    return np.concatenate(out, axis=0)


def bond_features(setup: Setup, geo: Geometry, bonds: np.ndarray) -> np.ndarray:
    X = np.asarray(geo.Coords)
    N = X.shape[0]
    L = setup.nlayers
    per = N // L
    t1, t2 = geo.tn[:, 0], geo.tn[:, 1]
    i, j, c = bonds[:, 0], bonds[:, 1], bonds[:, 2]
    R = np.asarray(geo.nUnitCell_1)[c, None] * t1[None, :] + np.asarray(geo.nUnitCell_2)[c, None] * t2[None, :]
    rj = X[j, :2] - R
    d = np.concatenate([X[i, :2] - rj, (X[i, 2] - X[j, 2])[:, None]], axis=1)
    mid = 0.5 * (X[i, :2] + rj)
    G = _moire_g(geo)
    ph = mid @ G.T
    sub_i = np.where((i % per) < per // 2, 1.0, -1.0)
    sub_j = np.where((j % per) < per // 2, 1.0, -1.0)
    zi = X[i, 2] / (1.35772 * max(1, L - 1))
    zj = X[j, 2] / (1.35772 * max(1, L - 1))
    r = np.linalg.norm(d, axis=1)
    gl = np.broadcast_to(_globals(setup, geo), (len(i), 4))
    f = np.concatenate([np.cos(ph), np.sin(ph), sub_i[:, None], sub_j[:, None], zi[:, None], zj[:, None], d,
                        r[:, None], (i == j).astype(float)[:, None], gl[:, :3]], axis=1)
    assert f.shape[1] == BOND_IN, f.shape
    return f.astype(np.float32)


def training_samples(setup: Setup, geo: Geometry, P: np.ndarray, dens: np.ndarray):
    """Site and bond samples from a converged state (P as (N, N, 4) zFock, dens = Re diag P(0))."""
    xs = site_features(setup, geo)
    ys = ((dens - 0.5) * DENS_SCALE).astype(np.float32)[:, None]
    bonds = bond_list(setup, geo)
    xb = bond_features(setup, geo, bonds)
    pv = P[bonds[:, 0], bonds[:, 1], bonds[:, 2]]
    yb = np.stack([pv.real, pv.imag], axis=1).astype(np.float32)
    return xs, ys, xb, yb


class Mlp:
    """Handle to the library's MLP (forge_gpu_mlp_*)."""

    def __init__(self, din: int, dout: int, seed: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        _check(self.lib.forge_gpu_mlp_create(din, dout, seed, C.byref(h)))
        self.h = h
        self.din, self.dout = din, dout
        self.nparam = int(self.lib.forge_gpu_mlp_num_params(h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.forge_gpu_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self, bf16: bool = False) -> np.ndarray:
        w = np.zeros(self.nparam, np.float32)
        if bf16:
            _check(self.lib.forge_gpu_mlp_get_params(self.h, None, _ptr(w)))
        else:
            _check(self.lib.forge_gpu_mlp_get_params(self.h, _ptr(w), None))
        return w

    def set_params(self, w: np.ndarray):
        w = np.ascontiguousarray(w, np.float32)
        _check(self.lib.forge_gpu_mlp_set_params(self.h, _ptr(w)))

    def set_loss_weights(self, wt: Sequence[float]):
        w = np.ascontiguousarray(wt, np.float32)
        _check(self.lib.forge_gpu_mlp_set_loss_weights(self.h, _ptr(w)))

    def forward(self, X: np.ndarray) -> np.ndarray:
        X = np.ascontiguousarray(X, np.float32)
        Y = np.zeros((X.shape[0], self.dout), np.float32)
        _check(self.lib.forge_gpu_mlp_forward(self.h, _ptr(X), X.shape[0], _ptr(Y)))
        return Y

    def gradient(self, X: np.ndarray, T: np.ndarray):
        X = np.ascontiguousarray(X, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        G = np.zeros(self.nparam, np.float32)
        loss = np.zeros(1, np.float32)
        _check(self.lib.forge_gpu_mlp_gradient(self.h, _ptr(X), _ptr(T), X.shape[0], _ptr(G), _ptr(loss)))
        return G, float(loss[0])

    def train(self, X: np.ndarray, T: np.ndarray, epochs: int, batch: int = 1024, lr: float = 1e-3, seed: int = 0):
        X = np.ascontiguousarray(X, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        loss = np.zeros(1, np.float32)
        _check(self.lib.forge_gpu_mlp_train(self.h, _ptr(X), _ptr(T), X.shape[0], epochs, batch, lr, seed,
                                            _ptr(loss)))
        return float(loss[0])


class WarmStart:
    """The two networks (site density, bond density matrix) with their input normalisation."""

    def __init__(self, seed: int = 0):
        self.site = Mlp(SITE_IN, 1, seed)
        self.bond = Mlp(BOND_IN, 2, seed + 1)
        self.norm = {}

    def _norm(self, key, X, fit=False):
        if fit or key not in self.norm:
            mu, sd = X.mean(0), X.std(0) + 1e-6
            self.norm[key] = (mu.astype(np.float32), sd.astype(np.float32))
        mu, sd = self.norm[key]
        return ((X - mu) / sd).astype(np.float32)

    def fit(self, samples, epochs: int = 40, lr: float = 2e-3, seed: int = 0):
        xs = np.concatenate([s[0] for s in samples])
        ys = np.concatenate([s[1] for s in samples])
        xb = np.concatenate([s[2] for s in samples])
        yb = np.concatenate([s[3] for s in samples])
        ls = self.site.train(self._norm("site", xs, True), ys, epochs, 256, lr, seed)
        lb = self.bond.train(self._norm("bond", xb, True), yb, epochs, 2048, lr, seed)
        return ls, lb

    def predict(self, setup: Setup, geo: Geometry):
        xs = self._norm("site", site_features(setup, geo))
        dn = self.site.forward(xs)[:, 0].astype(np.float64) / DENS_SCALE
        bonds = bond_list(setup, geo)
        pb = self.bond.forward(self._norm("bond", bond_features(setup, geo, bonds))).astype(np.float64)
        return dn, bonds, pb

    def save(self, path: str = WEIGHTS):
        os.makedirs(os.path.dirname(path), exist_ok=True)
        np.savez_compressed(path, site=self.site.params(), bond=self.bond.params(),
                            site_mu=self.norm["site"][0], site_sd=self.norm["site"][1],
                            bond_mu=self.norm["bond"][0], bond_sd=self.norm["bond"][1])

    @classmethod
    def load(cls, path: str = WEIGHTS):
        d = np.load(path)
        ws = cls()
        ws.site.set_params(d["site"])
        ws.bond.set_params(d["bond"])
        ws.norm = {"site": (d["site_mu"], d["site_sd"]), "bond": (d["bond_mu"], d["bond_sd"])}
        return ws


def predicted_state(hf: HartreeFock, ws: WarmStart) -> np.ndarray:
    """zFock-shaped (N, N, 4) field: predicted P on the short bonds, n_i - 1/2 + 1/2 on the diagonal."""
    dn, bonds, pb = ws.predict(hf.setup, hf.geometry)
    N = hf.N
    P = np.zeros((N, N, 4), dtype=np.complex128, order="F")
    P[bonds[:, 0], bonds[:, 1], bonds[:, 2]] = pb[:, 0] + 1j * pb[:, 1]
    P[np.arange(N), np.arange(N), 0] = 0.5 + dn
    return P


def start(hf: HartreeFock, setup: Setup, ws: Optional[WarmStart] = None, path: str = WEIGHTS):
    """The learned start with the fallback rule: the SCF starts from the network's field unless the
    network's first residual is worse than the plain guess's.

    Both starts run their first SCF iteration: the network's field (forge_gpu_field_guess, one
    diagonalisation) and then the plain guess (Main.f90:236-346).  The first iteration's residual of
    each is compared; the plain run continues in place when it is not worse, otherwise the network
    run's state after its first iteration is restored.  Returns (energies after the first iteration,
    that iteration's report, info).  info["first_residuals"] = (network, plain)."""
    E_w = apply(hf, setup, ws, path, fallback=False)
    used = bool(hf.warm_start_used)
    info = {"field_residuals": list(hf.warm_start_residuals)}
    if used:
        rep_w, E_w1, _ = hf.ScfIteration(E_w)
        P_w, _, _ = hf.GetState()
        r_w = rep_w["residual"]
    else:
        r_w = float("nan")
    E_p, _ = hf.PlainGuess()
    rep_p, E_p1, _ = hf.ScfIteration(E_p)
    r_p = rep_p["residual"]
    info["first_residuals"] = [r_w, r_p]
    if used and r_w < r_p:
        hf.SetState(P_w)
        E = hf.PrepareState()
        hf.warm_start_used = True
        info["warm_start_used"] = True
        return tuple(E), rep_w, info
    hf.warm_start_used = False
    info["warm_start_used"] = False
    return tuple(E_p1), rep_p, info


def apply(hf: HartreeFock, setup: Setup, ws: Optional[WarmStart] = None, path: str = WEIGHTS,
          fallback: bool = True):
    """Starting guess for `hf` from the network's field (one diagonalisation); returns the initial
    energies (4).  A non-finite prediction is never used (plain guess).  With `fallback`, the plain
    guess is also taken when the predicted field's residual (against the field of the state it
    gives) is not below the zero field's; `start` applies the first-iteration rule instead."""
    if ws is None:
        if not os.path.exists(path):
            raise ForgeError(-1, f"warm-start weights not found at {path}")
        ws = WarmStart.load(path)
    P = predicted_state(hf, ws)
    if not np.all(np.isfinite(P)):
        # a network that produced NaN / Inf (corrupt weights, out-of-range descriptors) is not used
        hf.warm_start_residuals = (float("nan"), float("nan"))
        E2, _ = hf.PlainGuess()
        hf.warm_start_used = False
        return tuple(E2)
    E = np.zeros(4)
    res = np.zeros(2)
    rc = hf.lib.forge_gpu_field_guess(hf.ctx, _ptr(np.asfortranarray(P)), _ptr(E), _ptr(res))
    _check(rc, allow_info=True)
    hf.warm_start_residuals = (float(res[0]), float(res[1]))
    if not np.isfinite(res[0]) or (fallback and not (res[0] < res[1])):
        E2, _ = hf.PlainGuess()
        hf.warm_start_used = False
        return tuple(E2)
    hf.warm_start_used = True
    return tuple(E)
