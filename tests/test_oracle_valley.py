"""CPU tests of the oracle's valley projection (nenforceValley = 1: ValleyPhase, ValleyTransform,
unitarize; Main.f90:470-500).

The valley operator is an approximate symmetry of the continuum-like bands: it must be Hermitian,
act within each sublattice block, nearly commute with the non-interacting H(k) (the Bloch-phase
convention of its neighbour-cell terms is what makes it commute: the opposite sign gives a commutator
15 times larger), and split the window at Gamma into two valleys.  The transform built from it
is a Hermitian involution on each k's window, and the valley-averaged window keeps the charge."""
import numpy as np
import pytest

from oracle import forge_oracle as fo


@pytest.fixture(scope="module")
def system():
    s = fo.Setup(ntheta=2, numk=3, nfilling=2.0, degfactor_mode="corrected")
    g = fo.build_geometry(s)
    return s, g, fo.pair_tables(s, g)


def _comm(H, V):
    return np.linalg.norm(H @ V - V @ H, 2) / (np.linalg.norm(H, 2) * np.linalg.norm(V, 2))


def test_valley_operator_structure_and_commutation(system):
    s, g, T = system
    N = s.ndim
    per = N // s.nlayers
    V0, P0 = np.zeros(N), np.zeros((4, N, N), complex)
    for ic in range(s.Nk):
        a, b = (int(x) for x in g.kcomp[ic])
        vk = g.kvals[a, b]
        V = fo.valley_phase(s, g, vk)
        assert np.max(np.abs(V - V.conj().T)) == 0.0
        blocks = np.zeros((N, N), bool)
        for l in range(s.nlayers):
            for lo, hi in ((per * l, per * l + per // 2), (per * l + per // 2, per * (l + 1))):
                blocks[lo:hi, lo:hi] = True
        assert np.all(V[~blocks] == 0)
        H = fo.hamiltonian(s, g, T, V0, P0, vk)
        assert _comm(H, V) < 0.04
        if ic > 0:      # at Gamma the two phase conventions coincide
            assert _comm(H, fo.valley_phase(s, g, -vk)) > 10 * _comm(H, V)


def test_valley_splits_the_window_at_gamma(system):
    s, g, T = system
    N = s.ndim
    H = fo.hamiltonian(s, g, T, np.zeros(N), np.zeros((4, N, N), complex), g.kvals[0, 0])
    w, Z = fo.eigh_lower(H, s.nUpper)
    X = Z[:, s.nLower - 1:]
    lam = np.linalg.eigvalsh(X.conj().T @ fo.valley_phase(s, g, g.kvals[0, 0]) @ X)
    assert (lam < -0.5).sum() == s.numb // 2 and (lam > 0.5).sum() == s.numb // 2


def test_unitarize_is_a_hermitian_involution():
    rng = np.random.default_rng(2)
    A = rng.standard_normal((20, 20)) + 1j * rng.standard_normal((20, 20))
    A = A + A.conj().T
    S = fo.unitarize(A)
    assert np.max(np.abs(S - S.conj().T)) < 1e-13
    assert np.max(np.abs(S @ S - np.eye(20))) < 1e-13
    # S commutes with A and has the signs of its eigenvalues
    assert np.max(np.abs(S @ A - A @ S)) < 1e-12
    assert np.allclose(np.linalg.eigvalsh(S), np.sort(np.sign(np.linalg.eigvalsh(A))))


def test_valley_transform_keeps_each_window(system):
    s, g, T = system
    N = s.ndim
    sol = fo.solve(s, g, T, np.zeros(N), np.zeros((4, N, N), complex))
    ev = fo.valley_transform(s, g, sol["evecs"])
    for ic in range(s.Nk):
        X, Y = sol["evecs"][:, :, ic], ev[:, :, ic]
        assert np.max(np.abs(X @ X.conj().T - Y @ Y.conj().T)) < 1e-12     # same window subspace
        assert np.max(np.abs(Y.conj().T @ Y - np.eye(s.numb))) < 1e-12


def test_valley_scf_keeps_the_charge(system):
    s, g, T = system
    sv = fo.Setup(ntheta=2, numk=3, nfilling=2.0, degfactor_mode="corrected", nenforceValley=1)
    LR = fo.long_range_interaction(sv, g)
    r = fo.run_scf(sv, g, T, LR, itmax=2)
    expect = (s.nLower - 1) + fo.fortran_nint(s.Nk * s.NeutralityPoint + s.Nk / 2 * s.nfilling) / s.Nk
    assert abs(np.trace(r["P_new"][0]).real - expect) < 1e-10
    assert np.max(np.abs(r["P_new"][0] - r["P_new"][0].conj().T)) < 1e-12
