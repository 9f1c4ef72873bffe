"""CPU tests of the oracle's C3-reduced solve and projector (nenforceC3 = 1: Solve_C3, GetFock_C3).

The pin is the full solve: on a C3-symmetric input (the non-interacting Hamiltonian), the rotated
eigenvectors and projector images of Solve_C3 must equal what the full solve computes at the
rotated k points.  The only allowed deviation is the C3 accuracy of the geometry (the site map pairs
sites within 1e-3; bands at rotated k agree to about 1e-5 eV).  At the invariant k points the
reference averages a projector with its two images; the expected values apply the same average to
the full solve's projectors.  The cases have no rotated k point where the two bands at the edge of
the bulk projector lie within 1e-3 eV of each other; where they do (m = 2, numk = 6: 1.6e-4 eV), the
geometry's C3 error mixes the pair and the full solve's projector is not a reference for it."""
import numpy as np
import pytest

from oracle import forge_oracle as fo

GEOM_TOL = 1e-4

CASES = [(2, 3, 2, (-1, 1), 0.0), (3, 6, 2, (-1, 1), 2.0), (2, 3, 3, (-1, 1, -1), -1.0)]


def _system(m, numk, L, rl, nf, **kw):
    s = fo.Setup(ntheta=m, numk=numk, nlayers=L, RotateLayers=rl, nfilling=nf, **kw)
    g = fo.build_geometry(s)
    return s, g, fo.pair_tables(s, g)


def test_c3_orbits_of_the_k_grid():
    for numk in (3, 6, 9):
        s = fo.Setup(ntheta=1, numk=numk)
        g = fo.build_geometry(s)
        rel = fo.c3_related_momenta(s, g)
        # rotating three times returns to k; the second related point is the rotation of the first
        for ic in range(1, s.Nk + 1):
            k2, k3 = rel[ic - 1, 1], rel[ic - 1, 2]
            assert rel[k2 - 1, 1] == k3 and rel[k3 - 1, 1] == ic
        inv = [ic for ic in range(1, s.Nk + 1) if rel[ic - 1, 1] == ic]
        assert inv == [ic for ic in range(1, s.Nk + 1) if fo.c3_invariant(numk, ic)]
        assert len(inv) == 3
        reps = fo.c3_representatives(s, rel)
        assert len(reps) == (s.Nk - 3) // 3 + 3
        covered = sorted({int(x) for r in reps for x in rel[r - 1]})
        assert covered == list(range(1, s.Nk + 1))


def test_c3_solve_needs_numk_divisible_by_3():
    s, g, T = _system(1, 4, 2, (-1, 1), 0.0)
    with pytest.raises(ValueError):
        fo.solve_c3(s, g, T, np.zeros(s.ndim), np.zeros((4, s.ndim, s.ndim), complex))


@pytest.mark.parametrize("m,numk,L,rl,nf", CASES)
def test_c3_solve_reproduces_the_full_solve(m, numk, L, rl, nf):
    s, g, T = _system(m, numk, L, rl, nf)
    N, nL = s.ndim, s.nLower
    V0, P0 = np.zeros(N), np.zeros((4, N, N), complex)
    full = fo.solve(s, g, T, V0, P0)
    red = fo.solve_c3(s, g, T, V0, P0)
    assert np.max(np.abs(full["bands"] - red["bands"])) < GEOM_TOL
    # every rotated eigenvector is an eigenvector of H at its own k (a residual test: it holds also
    # where two bands at a window edge are degenerate to the geometry's accuracy)
    for k in range(s.Nk):
        a, b = (int(x) for x in g.kcomp[k])
        H = fo.hamiltonian(s, g, T, V0, P0, g.kvals[a, b])
        X = red["evecs"][:, :, k]
        assert np.max(np.abs(H @ X - X * red["bands"][:, k])) < GEOM_TOL
        assert np.max(np.abs(X.conj().T @ X - np.eye(s.numb))) < 1e-12
    expect = np.zeros_like(red["bulk"])
    for ic in range(1, s.Nk + 1):
        a, b = (int(x) for x in g.kcomp[ic - 1])
        w, Z = fo.eigh_lower(fo.hamiltonian(s, g, T, V0, P0, g.kvals[a, b]), s.nUpper)
        occ = np.conj(Z[:, :nL - 1])
        B = occ @ occ.conj().T
        if fo.c3_invariant(numk, ic):
            expect += fo._c3_orbit_sum(s, g, B, (a, b), (a, b), (a, b)) / 3.0
        else:
            for c in range(4):
                expect[c] += B * fo.bloch_phase_int(a, b, int(g.ucell1[c]), int(g.ucell2[c]), numk)
    assert np.max(np.abs(red["bulk"] - expect)) < GEOM_TOL
    # the average over an orbit keeps the trace: nLower-1 bands per k
    assert abs(np.trace(red["bulk"][0]).real - (nL - 1) * s.Nk) < 1e-9


@pytest.mark.parametrize("m,numk,L,rl,nf", CASES)
def test_c3_window_projector(m, numk, L, rl, nf):
    s, g, T = _system(m, numk, L, rl, nf, degfactor_mode="corrected")
    N = s.ndim
    V0, P0 = np.zeros(N), np.zeros((4, N, N), complex)
    full = fo.solve(s, g, T, V0, P0)
    red = fo.solve_c3(s, g, T, V0, P0)
    se_a, _, mom_a, sv_a, _, _ = fo.sort_energies_1spin(s, g, full["bands"], full["evecs"])
    se_b, _, mom_b, sv_b, _, _ = fo.sort_energies_1spin(s, g, red["bands"], red["evecs"])
    fa, fb = fo.fermi_level(s, se_a, 1), fo.fermi_level(s, se_b, 1)
    assert fa[2:4] == fb[2:4]
    Pa = fo.get_fock_c3(s, g, sv_a, mom_a, fa[2], fa[3], fa[4])
    Pb = fo.get_fock_c3(s, g, sv_b, mom_b, fb[2], fb[3], fb[4])
    assert np.max(np.abs(Pa - Pb)) < GEOM_TOL
    # states away from the invariant k points enter exactly as in GetFock
    keep = [q for q in range(fa[2] - fa[3])
            if not fo.c3_invariant(numk, int(mom_a[q][0]) * numk + int(mom_a[q][1]) + 1)]
    Pc3 = fo.get_fock_c3(s, g, sv_a[:, keep], mom_a[keep], len(keep), 0, 0.0)
    Pgf = fo.get_fock(s, g, sv_a[:, keep], mom_a[keep], len(keep), 0, 0.0)
    assert np.array_equal(Pc3, Pgf)
    # the window keeps its trace: nFermiLevel states (DegFactor spreads the partial ones)
    assert abs(np.trace(Pb[0]).real - fb[0]) < 1e-9


def test_c3_scf_keeps_the_charge():
    s, g, T = _system(2, 3, 2, (-1, 1), 2.0, degfactor_mode="corrected", nenforceC3=1)
    LR = fo.long_range_interaction(s, g)
    r = fo.run_scf(s, g, T, LR, itmax=3)
    expect = (s.nLower - 1) + fo.fortran_nint(s.Nk * s.NeutralityPoint + s.Nk / 2 * s.nfilling) / s.Nk
    assert abs(np.trace(r["P"][0]).real - expect) < 1e-10
    assert np.max(np.abs(r["P"][0] - r["P"][0].conj().T)) < 1e-12
    # the C3 and full SCF differ only through the averages at the invariant k points
    s1, _, _ = _system(2, 3, 2, (-1, 1), 2.0, degfactor_mode="corrected")
    r1 = fo.run_scf(s1, g, T, LR, itmax=3)
    assert abs(r["Etot"] - r1["Etot"]) / s.ndim < 1e-2
