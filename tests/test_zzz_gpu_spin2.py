"""Parity of the spin-polarised SCF (numS = 2) on the GPU with the oracle's run_scf_2spins.

Each spin runs in its own device context; the host joins them (forge_gb300.spin).  Both a
spin-symmetric start (the plain guess copied to spin 2, Main.f90:290-292) and a spin-split start
are compared over three ODA iterations with the tolerances of the numS = 1 SCF parity test:
E/atom 1e-7 eV, Step 1e-6, DensityConvergence 1e-8, P(R) 1e-8, V 1e-7 eV, occupation counts exact.
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


@pytest.mark.parametrize("split", [False, True])
def test_spin_polarised_scf_matches_oracle(lib, split):
    import forge_gb300 as fg
    from forge_gb300.spin import SpinPolarisedScf
    kw = dict(ntheta=2, numk=3, nfilling=2.0, degfactor_mode="corrected")
    so1 = fo.Setup(**kw)
    g = fo.build_geometry(so1)
    T = fo.pair_tables(so1, g)
    LR = fo.long_range_interaction(so1, g)
    P0 = None
    if split:
        P0 = np.stack([fo.plain_guess(fo.Setup(**{**kw, "nfilling": kw["nfilling"] + d}), g, T)[0]
                       for d in (1.0, -1.0)])
    ref = fo.run_scf_2spins(fo.Setup(numS=2, **kw), g, T, LR, P_init=P0, itmax=3)
    natoms = so1.ndim
    with SpinPolarisedScf(fg.Setup(numS=2, **kw)) as scf:
        reps = scf.run(3, P_init=None if P0 is None else [_to_F(p) for p in P0])
        P = [_to_P(p) for p in scf.P]
        V = scf.V
        Etot = scf.total(scf.E)
    assert len(reps) == 3
    for r, l in zip(reps, ref["logs"]):
        assert abs(r.TotalEnergyIn - l.E_in) / natoms <= 1e-7
        assert abs(r.Step - l.step) <= 1e-6
        assert abs(r.DensityConvergence - l.dn_max) <= 1e-8
        assert (sum(r.nOccStates), sum(r.nPartOccStates)) == (l.nocc, l.npart)
        assert abs(r.FermiEnergy - l.EF) <= 1e-9
    assert tuple(reps[-1].nOccStates) == tuple(ref["nocc"])
    for sp in range(2):
        assert np.max(np.abs(P[sp] - ref["P"][sp])) <= 1e-8
        assert np.max(np.abs(V[sp] - ref["V"][sp])) <= 1e-7
    assert abs(Etot - ref["Etot"]) / natoms <= 1e-7
