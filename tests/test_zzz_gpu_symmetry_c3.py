"""Parity of the C3-reduced solve on the GPU (forge_gpu_set_c3, nenforceC3 = 1) with the oracle's
Solve_C3 / GetFock_C3 restatement.

The input potential and density matrix are random, so they are not C3-symmetric: the device must
reproduce the reference's imposed symmetry, not the full solve.  Tolerances as in the full-solve
parity tests: bands 1e-9 eV, zFockBulk 1e-8 per k, window eigenvectors equal up to a phase
(|<x|y>| = 1 within 1e-9), SCF trajectories E/atom 1e-7 eV, P(R) 1e-8, occupation counts exact.
This file builds on the per-routine entry points of the other parity files and is collected after them.
"""
import numpy as np
import pytest

from oracle import forge_oracle as fo

pytestmark = pytest.mark.gpu


def _to_P(Pf):
    return np.ascontiguousarray(np.moveaxis(Pf, 2, 0))


def _to_F(P):
    return np.asfortranarray(np.moveaxis(P, 0, 2))


@pytest.mark.parametrize("m,numk", [(2, 3), (3, 6)])
def test_c3_solve_matches_oracle(lib, m, numk):
    import forge_gb300 as fg
    S = fg.Setup(ntheta=m, numk=numk, nenforceC3=1)
    so = fo.Setup(ntheta=m, numk=numk, nenforceC3=1)
    g = fo.build_geometry(so)
    T = fo.pair_tables(so, g)
    N = so.ndim
    rng = np.random.default_rng(7)
    P = (rng.standard_normal((4, N, N)) + 1j * rng.standard_normal((4, N, N))) * 0.01
    V = rng.standard_normal(N) * 0.05
    ref = fo.solve_c3(so, g, T, V, P)
    with fg.HartreeFock(S) as hf:
        B, E, FB, info = hf.Solve(V, _to_F(P), bands=True, vectors=True, bulk=True)
    assert info == 0
    assert np.max(np.abs(B - ref["bands"])) <= 1e-9
    assert np.max(np.abs(_to_P(FB) - ref["bulk"])) <= 1e-8 * so.Nk
    for k in range(so.Nk):
        for b in range(so.numb):
            assert abs(abs(np.vdot(E[:, b, k], ref["evecs"][:, b, k])) - 1.0) <= 1e-9


@pytest.mark.parametrize("mode", ["reference", "corrected"])
def test_c3_scf_matches_oracle(lib, mode):
    import forge_gb300 as fg
    S = fg.Setup(ntheta=2, numk=3, nfilling=2.0, degfactor_mode=mode, nenforceC3=1)
    so = fo.Setup(ntheta=2, numk=3, nfilling=2.0, degfactor_mode=mode, nenforceC3=1)
    g = fo.build_geometry(so)
    T = fo.pair_tables(so, g)
    LR = fo.long_range_interaction(so, g)
    ref = fo.run_scf(so, g, T, LR, itmax=3)
    with fg.HartreeFock(S) as hf:
        hf.LongRangeInteraction(copy_out=False)
        res, reps = hf.RunScf(itmax=3)
        P, dens, V = hf.GetState()
    natoms = so.ndim
    for r, l in zip(reps, ref["logs"]):
        assert abs(r["TotalEnergyIn"] - l.E_in) / natoms <= 1e-7
        assert abs(r["Step"] - l.step) <= 1e-6
        assert (r["nOccStates"], r["nPartOccStates"]) == (l.nocc, l.npart)
        assert abs(r["FermiEnergy"] - l.EF) <= 1e-9
    assert np.max(np.abs(_to_P(P) - ref["P"])) <= 1e-8
    assert np.max(np.abs(V - ref["V"])) <= 1e-7
    assert abs(res["TotalEnergy"] - ref["Etot"]) / natoms <= 1e-7
