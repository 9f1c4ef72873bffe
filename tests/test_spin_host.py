"""CPU test of the two-spin SCF host logic (forge_gb300.spin): with each per-spin device context
replaced by a CPU model of the same routines (the oracle's Solve, SortEnergies_1Spin, GetFock and
energy functions), SpinPolarisedScf must follow the oracle's numS = 2 SCF (run_scf_2spins).  The
merge and Fermi level run in the library's host code (forge_host_fermi_2spins)."""
import numpy as np
import pytest

from oracle import forge_oracle as fo


def _to_P(Pf):
    return np.ascontiguousarray(np.moveaxis(Pf, 2, 0))


def _to_F(P):
    return np.asfortranarray(np.moveaxis(P, 0, 2))


class OracleSpinEngine:
    """CPU model of one per-spin device context: the HartreeFock methods SpinPolarisedScf calls."""

    def __init__(self, so, g, T, LR):
        self.so, self.g, self.T, self.LR = so, g, T, LR
        self.P = np.zeros((4, so.ndim, so.ndim), complex)
        self.sol = None
        self.sorted = None

    def LongRangeInteraction(self, copy_out=True):
        return self.LR.copy() if copy_out else None

    def PlainGuess(self):
        self.P, _ = fo.plain_guess(self.so, self.g, self.T)
        return (0.0, 0.0, 0.0, 0.0), 0

    def GetState(self):
        return _to_F(self.P), np.real(np.diagonal(self.P[0])).copy(), None

    def SetState(self, zFock):
        self.P = _to_P(zFock)

    def Energies(self, zFock=None):
        P = self.P if zFock is None else _to_P(zFock)
        return fo.kinetic_energy(self.so, self.T, P), fo.fock_energy(self.so, self.T, P), 0.0, 0.0

    def Solve(self, Potential=None, zFock=None, bands=True, vectors=False, bulk=False):
        self.sol = fo.solve(self.so, self.g, self.T, np.asarray(Potential), self.P)
        return None, None, None, 0

    def GetBands(self):
        return np.asfortranarray(self.sol["bands"])

    def SortEnergies_1Spin(self):
        se, idx, moms, sv, _, _ = fo.sort_energies_1spin(self.so, self.g, self.sol["bands"], self.sol["evecs"])
        self.sorted = (moms, sv)
        return se, moms, idx

    def GetFock(self, DegFactor, nOccStates, nPartOccStates, copy_out=True):
        moms, sv = self.sorted
        Pw = fo.window_fock(self.so, self.g, self.sol, sv, moms, nOccStates, nPartOccStates, DegFactor)
        self.Pn = (Pw + self.sol["bulk"]) / complex(float(self.so.Nk), 0.0)
        return _to_F(self.Pn)

    def Symmetrize(self, copy_out=True):
        self.Pn = fo.enforce_symmetries(self.so, self.g, self.Pn)
        return _to_F(self.Pn)

    def SetPotential(self, Potential):
        self.V = np.asarray(Potential)

    def EnergyForms(self):
        # kinetic energy linear, Fock energy -Q(P, P) / 2 with Q a quadratic form
        Q = lambda P: -2.0 * fo.fock_energy(self.so, self.T, P)   # noqa: E731
        qa, qb = Q(self.P), Q(self.Pn)
        qab = 0.5 * (Q(self.P + self.Pn) - qa - qb)
        f = np.array([fo.kinetic_energy(self.so, self.T, self.P), fo.kinetic_energy(self.so, self.T, self.Pn),
                      qa, qab, qb, 0.0])
        return f, np.real(np.diagonal(self.P[0])).copy(), np.real(np.diagonal(self.Pn[0])).copy()

    def Mix(self, Step):
        d0 = np.real(np.diagonal(self.P[0])).copy()
        self.P = Step * self.Pn + (1.0 - Step) * self.P
        d = np.real(np.diagonal(self.P[0])).copy()
        return d, float(np.max(np.abs(d - d0)))


@pytest.mark.parametrize("split,flags", [(False, {}), (True, {}), (True, dict(nenforceT=1, nenforceC2=1)),
                                         (True, dict(nenforceValley=1))])
def test_spin_scf_host_logic_follows_the_oracle(lib, split, flags):
    import forge_gb300 as fg
    from forge_gb300.spin import SpinPolarisedScf
    kw = dict(ntheta=1, numk=3, nfilling=2.0, degfactor_mode="corrected", **flags)
    so1 = fo.Setup(**kw)
    so2 = fo.Setup(numS=2, **kw)
    g = fo.build_geometry(so1)
    T = fo.pair_tables(so1, g)
    LR = fo.long_range_interaction(so1, g)
    P0 = None
    if split:
        P0 = np.stack([fo.plain_guess(fo.Setup(**{**kw, "nfilling": kw["nfilling"] + d}), g, T)[0]
                       for d in (1.0, -1.0)])
    ref = fo.run_scf_2spins(so2, g, T, LR, P_init=P0, itmax=3)
    engines = [OracleSpinEngine(so1, g, T, LR) for _ in range(2)]
    scf = SpinPolarisedScf(fg.Setup(numS=2, **kw), engines=engines)
    reps = scf.run(3, P_init=None if P0 is None else [_to_F(p) for p in P0])
    assert len(reps) == len(ref["logs"]) == 3
    for r, l in zip(reps, ref["logs"]):
        assert r.TotalEnergyIn == pytest.approx(l.E_in, abs=1e-10)
        assert r.Step == pytest.approx(l.step, abs=1e-12)
        assert r.DensityConvergence == pytest.approx(l.dn_max, abs=1e-12)
        assert sum(r.nOccStates) == l.nocc and sum(r.nPartOccStates) == l.npart
        assert r.FermiEnergy == l.EF
    for sp in range(2):
        assert np.max(np.abs(_to_P(scf.P[sp]) - ref["P"][sp])) <= 1e-12
        assert np.max(np.abs(scf.V[sp] - ref["V"][sp])) <= 1e-11
    assert scf.total(scf.E) == pytest.approx(ref["Etot"], abs=1e-10)


def test_spin_scf_rejects_numS1(lib):
    import forge_gb300 as fg
    from forge_gb300.spin import SpinPolarisedScf
    with pytest.raises(ValueError):
        SpinPolarisedScf(fg.Setup(ntheta=1, numk=3), engines=[None, None])


def test_spin_scf_output_files(lib, tmp_path):
    """Energy / Convergence / Bands-nspin1,2 / Fock-nspin1,2 files of a numS = 2 run (Main.f90:596-672):
    the numS = 2 columns, one line per iteration, and Fock files that read back to the state."""
    import forge_gb300 as fg
    from forge_gb300.spin import SpinPolarisedScf
    kw = dict(ntheta=1, numk=3, nfilling=2.0, degfactor_mode="corrected")
    so1 = fo.Setup(**kw)
    g = fo.build_geometry(so1)
    T = fo.pair_tables(so1, g)
    LR = fo.long_range_interaction(so1, g)
    S2 = fg.Setup(numS=2, **kw)
    scf = SpinPolarisedScf(S2, geometry=fg.build_geometry(fg.Setup(**kw)),
                           engines=[OracleSpinEngine(so1, g, T, LR) for _ in range(2)])
    out, fock = tmp_path / "output", tmp_path / "dataFock"
    out.mkdir()
    fock.mkdir()
    reps = scf.run(2, output_dir=str(out), fock_dir=str(fock))
    params = fg.parameters_string(S2)
    assert "-numS2-" in params
    energy = (out / ("Energy" + params)).read_text().splitlines()
    conv = (out / ("Convergence" + params)).read_text().splitlines()
    assert len(energy) == len(conv) == 2
    for line_e, line_c, r in zip(energy, conv, reps):
        e = [float(x) for x in line_e.split()]
        c = [float(x) for x in line_c.split()]
        assert e[0] == r.it and c[0] == r.it
        assert e[1:] == pytest.approx([r.TotalEnergyIn, r.KineticEnergyIn, r.FockEnergyIn, r.HartreeEnergyIn,
                                       r.HubbardEnergyIn], abs=1e-9)
        assert c[1:] == pytest.approx([r.DensityConvergence, r.Step, r.TotalEnergyIn - r.TotalEnergy], abs=1e-6)
    for sp in (1, 2):
        assert (out / (f"Bands-nspin{sp}" + params)).stat().st_size > 0
        back = fg.read_fock(S2, str(fock / (f"Fock-nspin{sp}" + params)))
        Pf = scf.P[sp - 1]
        low = np.tril(np.ones((S2.to_struct().ndim,) * 2, bool))
        assert np.array_equal(back[:, :, 0][low], Pf[:, :, 0][low])
        assert np.array_equal(back[:, :, 1:], Pf[:, :, 1:])


def test_spin_scf_resumes_from_fock_files(lib, tmp_path):
    """nRead = 1 (Main.f90:186-234): a numS = 2 checkpoint gives each spin its own file; a numS = 1
    checkpoint starts both spins from Fock-nspin1."""
    import forge_gb300 as fg
    from forge_gb300.spin import SpinPolarisedScf
    kw = dict(ntheta=1, numk=3, nfilling=2.0, degfactor_mode="corrected")
    so1 = fo.Setup(**kw)
    g = fo.build_geometry(so1)
    T = fo.pair_tables(so1, g)
    LR = fo.long_range_interaction(so1, g)
    S1, S2 = fg.Setup(**kw), fg.Setup(numS=2, **kw)

    def make():
        return SpinPolarisedScf(S2, engines=[OracleSpinEngine(so1, g, T, LR) for _ in range(2)])

    a = make()
    P0 = np.stack([fo.plain_guess(fo.Setup(**{**kw, "nfilling": kw["nfilling"] + d}), g, T)[0] for d in (1.0, -1.0)])
    a.run(1, P_init=[_to_F(p) for p in P0], fock_dir=str(tmp_path))
    b = make()
    b.read_state(str(tmp_path))
    low = np.tril(np.ones(a.P[0].shape[:2], bool))
    for sp in range(2):
        # the file holds the lower triangle of R = 0 (the upper is its conjugate) and the other cells in full
        assert np.array_equal(b.P[sp][:, :, 0][low], a.P[sp][:, :, 0][low])
        assert np.array_equal(b.P[sp][:, :, 1:], a.P[sp][:, :, 1:])
    assert not np.array_equal(b.P[0], b.P[1])
    # a numS = 1 checkpoint starts both spins alike
    fg.write_fock(S1, _to_F(P0[0]), str(tmp_path / ("Fock-nspin1" + fg.parameters_string(S1))))
    c = make()
    c.read_state(str(tmp_path), setup_in=S1)
    assert np.array_equal(c.P[0], c.P[1])
