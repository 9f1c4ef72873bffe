"""Mixed-precision eigen-solver (FP32 Householder + tcgen05 split-TF32 updates, FP64 tridiagonal
solve) against LAPACK zheevr.  Tolerances are FP32-level relative to the spectral radius:
eigenvalues 2e-5, eigenvector orthonormality 1e-4, residual 2e-5, subspace projector 2e-4.
"""
import numpy as np
import pytest

from oracle import forge_oracle as fo

pytestmark = pytest.mark.gpu


def _hf(m):
    import forge_gb300 as fg
    hf = fg.HartreeFock(fg.Setup(ntheta=m, numk=1))
    hf.set_precision("mixed")
    return hf


@pytest.mark.parametrize("m", [2, 5])
def test_mixed_zheevr_random(lib, m):
    hf = _hf(m)
    N = hf.N
    rng = np.random.default_rng(N)
    mats = []
    for _ in range(2):
        A = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
        mats.append((A + A.conj().T) / 2)
    iu = N // 2 + 10
    w, Z, info = hf.zheevr_batch(np.stack([np.tril(M) for M in mats], axis=2), iu)
    assert info == 0
    for b, M in enumerate(mats):
        wo, Zo = fo.eigh_lower(M, iu)
        scale = np.max(np.abs(np.linalg.eigvalsh(M)))
        assert np.max(np.abs(w[:, b] - wo)) <= 2e-5 * scale
        X = Z[:, :, b]
        assert np.max(np.abs(X.conj().T @ X - np.eye(iu))) <= 1e-4
        assert np.max(np.abs(M @ X - X * w[:, b])) <= 2e-5 * scale * np.sqrt(N)
        n = N // 2 - 9
        assert np.max(np.abs(X[:, :n] @ X[:, :n].conj().T - Zo[:, :n] @ Zo[:, :n].conj().T)) <= 2e-4
    hf.close()


def test_mixed_zheevr_model_hamiltonian(lib):
    """H(k) of the tight-binding model with a Hartree-Fock mean field (m=5, N=364)."""
    hf = _hf(5)
    so = fo.Setup(ntheta=5, numk=3)
    g = fo.build_geometry(so)
    T = fo.pair_tables(so, g)
    rng = np.random.default_rng(3)
    N = so.ndim
    P = (rng.standard_normal((4, N, N)) + 1j * rng.standard_normal((4, N, N))) * 0.01
    Hs = [fo.hamiltonian(so, g, T, rng.standard_normal(N) * 0.1, P, g.vk(k)) for k in range(3)]
    iu = so.nUpper
    w, Z, info = hf.zheevr_batch(np.stack([np.tril(H) for H in Hs], axis=2), iu)
    assert info == 0
    for b, H in enumerate(Hs):
        wo, Zo = fo.eigh_lower(H, iu)
        assert np.max(np.abs(w[:, b] - wo)) <= 2e-5 * np.max(np.abs(wo))
        X = Z[:, :, b]
        assert np.max(np.abs(X.conj().T @ X - np.eye(iu))) <= 1e-4
    hf.close()


def test_fp64_window_refinement_recovers_fp64_accuracy(lib):
    """The FP64 Rayleigh-Ritz step after the mixed solve (forge_gpu_set_refinement): the refined top
    32 eigenpairs reach FP64-level eigenvalues and orthonormality, the unrefined ones stay FP32-level."""
    hf = _hf(5)
    N = hf.N
    rng = np.random.default_rng(21)
    A = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    M = (A + A.conj().T) / 2
    iu = N // 2 + 10
    wo, Zo = fo.eigh_lower(M, iu)
    scale = np.max(np.abs(np.linalg.eigvalsh(M)))
    hf.set_refinement(0)
    w0, Z0, info0 = hf.zheevr_batch(np.tril(M)[:, :, None], iu)
    hf.set_refinement(32)
    w1, Z1, info1 = hf.zheevr_batch(np.tril(M)[:, :, None], iu)
    assert info0 == 0 and info1 == 0
    win = slice(iu - 32, iu)
    err0 = np.max(np.abs(w0[win, 0] - wo[win]))
    err1 = np.max(np.abs(w1[win, 0] - wo[win]))
    assert err0 >= 1e-9 * scale                  # the mixed solve alone is FP32-accurate
    # Ritz values of an FP32-accurate subspace: errors of second order in the subspace angle
    assert err1 <= 1e-9 * scale
    X = Z1[:, win, 0]
    assert np.max(np.abs(X.conj().T @ X - np.eye(32))) <= 1e-12
    assert np.max(np.abs(M @ X - X * w1[win, 0])) <= 2e-5 * scale * np.sqrt(N)
    # the bands below the window are untouched
    assert np.array_equal(Z1[:, :iu - 32, 0], Z0[:, :iu - 32, 0])
    hf.close()
