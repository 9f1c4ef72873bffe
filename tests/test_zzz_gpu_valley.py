"""Parity of the valley projection on the GPU (forge_gpu_set_valley, nenforceValley = 1,
Main.f90:470-500) with the oracle's window_fock.

Tolerances as in the full-solve parity tests: P_new 1e-10 for one projection, SCF trajectories
E/atom 1e-7 eV and P(R) 1e-8, occupation counts exact.  This file builds on the per-routine entry
points of the other parity files and is collected after them.
"""
import numpy as np
import pytest

from oracle import forge_oracle as fo

pytestmark = pytest.mark.gpu


def _to_P(Pf):
    return np.ascontiguousarray(np.moveaxis(Pf, 2, 0))


def _to_F(P):
    return np.asfortranarray(np.moveaxis(P, 0, 2))


def test_valley_get_fock_matches_oracle(lib):
    import forge_gb300 as fg
    kw = dict(ntheta=2, numk=3, nfilling=2.0, degfactor_mode="corrected", nenforceValley=1)
    S, so = fg.Setup(**kw), fo.Setup(**kw)
    g = fo.build_geometry(so)
    T = fo.pair_tables(so, g)
    N = so.ndim
    rng = np.random.default_rng(5)
    P = (rng.standard_normal((4, N, N)) + 1j * rng.standard_normal((4, N, N))) * 0.01
    V = rng.standard_normal(N) * 0.05
    sol = fo.solve(so, g, T, V, P)
    se, _, moms, sv, _, _ = fo.sort_energies_1spin(so, g, sol["bands"], sol["evecs"])
    nF, EF, nocc, npart, deg = fo.fermi_level(so, se)
    ref = (fo.window_fock(so, g, sol, sv, moms, nocc, npart, deg) + sol["bulk"]) / so.Nk
    with fg.HartreeFock(S) as hf:
        hf.Solve(V, _to_F(P), bands=False)
        hf.SortEnergies_1Spin()
        Pn = hf.GetFock(deg, nocc, npart)
    assert np.max(np.abs(_to_P(Pn) - ref)) <= 1e-10


def test_valley_scf_matches_oracle(lib):
    import forge_gb300 as fg
    kw = dict(ntheta=2, numk=3, nfilling=2.0, degfactor_mode="corrected", nenforceValley=1)
    S, so = fg.Setup(**kw), fo.Setup(**kw)
    g = fo.build_geometry(so)
    T = fo.pair_tables(so, g)
    LR = fo.long_range_interaction(so, g)
    ref = fo.run_scf(so, g, T, LR, itmax=3)
    with fg.HartreeFock(S) as hf:
        hf.LongRangeInteraction(copy_out=False)
        res, reps = hf.RunScf(itmax=3)
        P, dens, Vd = hf.GetState()
    natoms = so.ndim
    for r, l in zip(reps, ref["logs"]):
        assert abs(r["TotalEnergyIn"] - l.E_in) / natoms <= 1e-7
        assert abs(r["Step"] - l.step) <= 1e-6
        assert (r["nOccStates"], r["nPartOccStates"]) == (l.nocc, l.npart)
    assert np.max(np.abs(_to_P(P) - ref["P"])) <= 1e-8
    assert abs(res["TotalEnergy"] - ref["Etot"]) / natoms <= 1e-7
