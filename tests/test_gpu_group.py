"""Uneven-size batch: systems of different ndim solved in one batched eigen-solve
(forge_gpu_solve_group, forge_gpu_scf_iteration_group).

Members: the (2, 3) bilayer (N = 76), the (3, 4) bilayer (N = 148) and the alternating-twist
trilayer at m = 2 (N = 114), each with its own k grid, filling and dielectric constant, as in the
benchmark description's MLP training set (there with m = 8, 12, 16 and the m = 12 trilayer).  Each
member's group result must equal its own single-system solve (FP64: bands 1e-12 eV, window
projectors 1e-10) and three group SCF iterations must follow the oracle (E/atom 1e-7 eV, P 1e-8).
"""
import numpy as np
import pytest

from oracle import forge_oracle as fo

pytestmark = pytest.mark.gpu

MEMBERS = [dict(ntheta=2, numk=3, nfilling=2.0, epsilon=10.0),
           dict(ntheta=3, numk=3, nfilling=-1.0, epsilon=6.0),
           dict(ntheta=2, nlayers=3, RotateLayers=(-1, 1, -1), numk=3, nfilling=0.0, epsilon=15.0)]


def _contexts(precision="fp64"):
    import forge_gb300 as fg
    hs = []
    for kw in MEMBERS:
        hf = fg.HartreeFock(fg.Setup(degfactor_mode="corrected", precision=precision, **kw))
        hf.LongRangeInteraction(copy_out=False)
        hs.append(hf)
    return hs


def test_group_solve_equals_single_solves(lib):
    import forge_gb300 as fg
    hs = _contexts()
    try:
        for h in hs:
            h.PlainGuess()
        single = [h.Solve(None, None, bands=True, vectors=True)[:2] for h in hs]
        info = fg.SolveGroup(hs)
        assert np.all(info == 0)
        for h, (B, Z) in zip(hs, single):
            Bg = h.GetBands()
            assert np.max(np.abs(Bg - B)) <= 1e-12 * max(1.0, np.max(np.abs(B)))
        # the window eigenvectors through the device path: GetFock of the group solve equals the single one
        for h, (B, Z) in zip(hs, single):
            h.SortEnergies_1Spin()
            nF, EF, nocc, npart, deg = h.FermiLevel()
            Pg = h.GetFock(deg, nocc, npart)
            h.Solve(None, None, bands=False)
            h.SortEnergies_1Spin()
            Ps = h.GetFock(deg, nocc, npart)
            assert np.max(np.abs(Pg - Ps)) <= 1e-10
    finally:
        for h in hs:
            h.close()


def test_group_scf_follows_the_oracle(lib):
    import forge_gb300 as fg
    hs = _contexts()
    try:
        E = np.array([h.PlainGuess()[0] for h in hs])
        reps = []
        for _ in range(3):
            r, E, info = fg.ScfIterationGroup(hs, E)
            assert info == 0
            reps.append(r)
        states = [h.GetState() for h in hs]
    finally:
        for h in hs:
            h.close()
    for b, kw in enumerate(MEMBERS):
        so = fo.Setup(degfactor_mode="corrected", **kw)
        ref = fo.run_scf(so, itmax=3)
        for it, l in enumerate(ref["logs"]):
            r = reps[it][b]
            assert abs(r["TotalEnergyIn"] - l.E_in) / so.ndim <= 1e-7, (b, it)
            assert (r["nOccStates"], r["nPartOccStates"]) == (l.nocc, l.npart)
        P = np.moveaxis(states[b][0], 2, 0)
        assert np.max(np.abs(P - ref["P"])) <= 1e-8, b


def test_group_mixed_solve_matches_fp64_group(lib):
    import forge_gb300 as fg
    hs64, hsmx = _contexts("fp64"), _contexts("mixed")
    try:
        for a, b in zip(hs64, hsmx):
            a.PlainGuess()
            P = a.GetState()[0]
            b.SetState(P)
            b.PrepareState()
        fg.SolveGroup(hs64)
        fg.SolveGroup(hsmx)
        for a, b in zip(hs64, hsmx):
            # the mixed window bands after the FP64 window Rayleigh-Ritz (second order in the FP32
            # leakage of the 32-band span: 1e-8 at the window's top band)
            assert np.max(np.abs(a.GetBands() - b.GetBands())) <= 1e-8
    finally:
        for h in hs64 + hsmx:
            h.close()
