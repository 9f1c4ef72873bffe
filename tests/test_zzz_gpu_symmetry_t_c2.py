"""Parity of the symmetry switches of the SCF loop on the GPU (forge_gpu_set_symmetry,
forge_gpu_symmetrize: nenforceT, nenforceC2, nenforceC2T, Main.f90:513-534) with the oracle.

Tolerances as in the full-solve parity tests: P(R) 1e-8 per element (1e-10 for one projector), SCF
trajectories E/atom 1e-7 eV, occupation counts exact.  This file builds on the per-routine entry
points of the other parity files and is collected after them.
"""
import numpy as np
import pytest

from oracle import forge_oracle as fo

pytestmark = pytest.mark.gpu

FLAGS = dict(nenforceT=1, nenforceC2=1, nenforceC2T=1)


def _to_P(Pf):
    return np.ascontiguousarray(np.moveaxis(Pf, 2, 0))


def _to_F(P):
    return np.asfortranarray(np.moveaxis(P, 0, 2))


def test_symmetrize_matches_oracle(lib):
    import forge_gb300 as fg
    S = fg.Setup(ntheta=2, numk=3, nfilling=2.0, degfactor_mode="corrected", **FLAGS)
    so = fo.Setup(ntheta=2, numk=3, nfilling=2.0, degfactor_mode="corrected", **FLAGS)
    g = fo.build_geometry(so)
    T = fo.pair_tables(so, g)
    N = so.ndim
    rng = np.random.default_rng(3)
    P = (rng.standard_normal((4, N, N)) + 1j * rng.standard_normal((4, N, N))) * 0.01
    V = rng.standard_normal(N) * 0.05
    sol = fo.solve(so, g, T, V, P)
    se, _, moms, sv, _, _ = fo.sort_energies_1spin(so, g, sol["bands"], sol["evecs"])
    nF, EF, nocc, npart, deg = fo.fermi_level(so, se)
    ref = fo.enforce_symmetries(so, g, (fo.get_fock(so, g, sv, moms, nocc, npart, deg) + sol["bulk"]) / so.Nk)
    with fg.HartreeFock(S) as hf:
        hf.Solve(V, _to_F(P), bands=False, bulk=False)
        hf.SortEnergies_1Spin()
        hf.GetFock(deg, nocc, npart, copy_out=False)
        Ps = hf.Symmetrize()
    assert np.max(np.abs(_to_P(Ps) - ref)) <= 1e-10


def test_symmetric_scf_matches_oracle(lib):
    import forge_gb300 as fg
    S = fg.Setup(ntheta=2, numk=3, nfilling=2.0, degfactor_mode="corrected", **FLAGS)
    so = fo.Setup(ntheta=2, numk=3, nfilling=2.0, degfactor_mode="corrected", **FLAGS)
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
    assert np.max(np.abs(_to_P(P) - ref["P"])) <= 1e-8
    assert abs(res["TotalEnergy"] - ref["Etot"]) / natoms <= 1e-7
