"""CPU tests of the oracle's spin-polarised path (numS = 2): the merge of SortEnergies_2Spins on
hand-worked lists, the reduction of a spin-symmetric state to the numS = 1 SCF, spin-swap
equivariance, charge counting and the quadratic ODA energy."""
import numpy as np
import pytest

from oracle import forge_oracle as fo


def test_sort_energies_2spins_front_copy_reads_spin2_at_spin1_counter():
    # numk=1, numb=6, windows (2, 5): one state of each spin copied in front, states 2..4 merged,
    # tails appended spin 1 first.  The front spin-2 entry is se2(ncount1) = se2(2) = 0.5, not se2(1).
    se1 = [0.0, 1.0, 2.0, 3.0, 4.0, 5.0]
    se2 = [10.0, 0.5, 1.5, 2.5, 3.5, 4.5]
    e, lab = fo.sort_energies_2spins(1, 6, [[2, 2], [5, 5]], se1, se2)
    assert e.tolist() == [0.0, 0.5, 0.5, 1.0, 1.5, 2.0, 2.5, 3.0, 4.0, 5.0, 3.5, 4.5]
    assert lab.tolist() == [1, 2, 2, 1, 2, 1, 2, 1, 1, 1, 2, 2]


def test_sort_energies_2spins_runs_extend_past_the_window():
    # a spin-1 run that starts inside the window continues to the end of the run (HartreeFock.f90:962)
    se1 = [0.0, 1.0, 1.1, 1.2, 1.3, 9.0]
    se2 = [0.0, 2.0, 3.0, 4.0, 5.0, 6.0]
    e, lab = fo.sort_energies_2spins(1, 6, [[2, 2], [4, 4]], se1, se2)
    assert e.tolist() == [0.0, 2.0, 1.0, 1.1, 1.2, 1.3, 2.0, 9.0, 3.0, 4.0, 5.0, 6.0]
    assert lab.tolist() == [1, 2, 1, 1, 1, 1, 2, 1, 2, 2, 2, 2]
    assert (lab == 1).sum() == 6 and (lab == 2).sum() == 6


def test_sort_energies_2spins_merges_the_window_region():
    rng = np.random.default_rng(3)
    numk, numb = 2, 20
    n = numb * numk * numk
    se1 = np.sort(rng.normal(size=n))
    se2 = np.sort(rng.normal(size=n))
    W = np.array([[9, 9], [13, 13]])
    e, lab = fo.sort_energies_2spins(numk, numb, W, se1, se2)
    front = 2 * 8 * numk * numk
    assert lab[:front].tolist() == [1] * (front // 2) + [2] * (front // 2)
    # the front spin-2 block repeats se2 at position 8*Nk + 1
    assert np.all(e[front // 2:front] == se2[8 * numk * numk])
    # the merged part is sorted, and per spin it keeps the order of its own list
    k1 = np.flatnonzero(lab == 1)
    k2 = np.flatnonzero(lab == 2)
    assert np.array_equal(e[k1], se1)
    assert np.array_equal(e[k2[front // 2:]], se2[front // 2:])
    stop = min(k1[12 * numk * numk - 1], k2[12 * numk * numk - 1]) + 1
    assert stop > front and np.all(np.diff(e[front:stop]) >= 0)


def test_fermi_level_2spins_counts_per_spin():
    s = fo.Setup(ntheta=1, numk=1, numS=2, nfilling=0.0)
    assert (s.Nk, s.numb, s.NeutralityPoint) == (1, 20, 10)
    W = fo.window_sort_2spins(s)
    assert W.tolist() == [[9, 9], [13, 13]]
    base = np.arange(20, dtype=np.float64)
    # spin 2 lies 0.3 above spin 1: nFermiLevel = 2*NP*Nk = 20 states, ten of each spin, none partial
    e, lab = fo.sort_energies_2spins(s.numk, s.numb, W, base, base + 0.3)
    nF, EF, nocc, npart, deg = fo.fermi_level_2spins(s, e, lab)
    assert (nF, EF, nocc, npart, deg) == (20, 9.65, [10, 10], [0, 0], 0.0)
    # a spin-1 and a spin-2 state meet at the Fermi level: both are partially occupied, and DegFactor
    # = (nF + npart - nocc) / npart over both spins
    se2 = np.concatenate([base[:8], [8.5, 10.0, 11.5, 12.0], base[12:] + 1.0])
    e, lab = fo.sort_energies_2spins(s.numk, s.numb, W, base, se2)
    assert e[16:23].tolist() == [8.0, 8.5, 9.0, 10.0, 10.0, 11.0, 11.5]
    assert lab[16:23].tolist() == [1, 2, 1, 1, 2, 1, 2]
    nF, EF, nocc, npart, deg = fo.fermi_level_2spins(s, e, lab)
    assert (nF, EF, nocc, npart, deg) == (20, 10.0, [11, 10], [1, 1], 0.5)


@pytest.fixture(scope="module")
def small_system():
    s1 = fo.Setup(ntheta=1, numk=3, nfilling=2.0, degfactor_mode="corrected")
    g = fo.build_geometry(s1)
    T = fo.pair_tables(s1, g)
    LR = fo.long_range_interaction(s1, g)
    return s1, g, T, LR


def _spin2(s1):
    s2 = fo.Setup(**{f.name: getattr(s1, f.name) for f in fo.dataclasses.fields(s1)})
    s2.numS = 2
    return s2


@pytest.mark.parametrize("nfilling,mode,flags", [(0.0, "reference", {}), (2.0, "corrected", {}),
                                                 (-1.0, "reference", {}), (2.0, "corrected", dict(nenforceC3=1)),
                                                 (2.0, "corrected", dict(nenforceValley=1, nenforceC2T=1))])
def test_spin_symmetric_state_reduces_to_numS1(nfilling, mode, flags):
    """With both spins equal, every numS = 2 quantity is the numS = 1 one: nFermiLevel doubles,
    the merged list pairs the spins, DegFactor, the energies (factor 3 - numS) and the potentials
    (Main.f90:577-594) coincide, so the SCF trajectories agree exactly; also with the C3, valley and
    symmetry switches, which act on each spin alone."""
    s1 = fo.Setup(ntheta=1, numk=3, nfilling=nfilling, degfactor_mode=mode, **flags)
    s2 = _spin2(s1)
    g = fo.build_geometry(s1)
    T = fo.pair_tables(s1, g)
    LR = fo.long_range_interaction(s1, g)
    r1 = fo.run_scf(s1, g, T, LR, itmax=3)
    r2 = fo.run_scf_2spins(s2, g, T, LR, itmax=3)
    for sp in range(2):
        assert np.max(np.abs(r2["P"][sp] - r1["P"])) <= 1e-13
        assert np.max(np.abs(r2["V"][sp] - r1["V"])) <= 1e-12
    for a, b in zip(r1["logs"], r2["logs"]):
        assert a.E_in == pytest.approx(b.E_in, abs=1e-10)
        assert a.step == pytest.approx(b.step, abs=1e-12)
        assert (2 * a.nocc, 2 * a.npart) == (b.nocc, b.npart)


def _split_state(s1, g, T):
    """A spin-split start: spin 1 from the guess at filling +1, spin 2 from the guess at filling -1."""
    P = []
    for nf in (s1.nfilling + 1.0, s1.nfilling - 1.0):
        sx = fo.Setup(**{f.name: getattr(s1, f.name) for f in fo.dataclasses.fields(s1)})
        sx.nfilling = nf
        P.append(fo.plain_guess(sx, g, T)[0])
    return np.stack(P)


def test_spin_swap_equivariance(small_system):
    s1, g, T, LR = small_system
    s2 = _spin2(s1)
    P0 = _split_state(s1, g, T)
    a = fo.run_scf_2spins(s2, g, T, LR, P_init=P0, itmax=3)
    b = fo.run_scf_2spins(s2, g, T, LR, P_init=P0[::-1].copy(), itmax=3)
    assert np.max(np.abs(a["P"] - b["P"][::-1])) <= 1e-12
    assert np.max(np.abs(a["V"] - b["V"][::-1])) <= 1e-12
    assert a["Etot"] == pytest.approx(b["Etot"], abs=1e-10)
    assert a["nocc"] == b["nocc"][::-1]


def test_spin_polarised_charge_and_oda(small_system):
    s1, g, T, LR = small_system
    s2 = _spin2(s1)
    P0 = _split_state(s1, g, T)
    r = fo.run_scf_2spins(s2, g, T, LR, P_init=P0, itmax=3, keep_history=True)
    # total charge: both spins' full bands below the window plus nFermiLevel window states over Nk
    nF = 2 * fo.fortran_nint(s1.Nk * s1.NeutralityPoint + s1.Nk / 2 * s1.nfilling)
    tr = sum(np.trace(r["P"][sp, 0]).real for sp in range(2))
    assert abs(tr - (2 * (s1.nLower - 1) + nF / s1.Nk)) < 1e-10
    # the spin-summed energy is exactly quadratic along the ODA line (HartreeFock.f90:1148-1227)
    a, b = r["history"][1]["P"], r["P_new"]
    da = np.stack([np.real(np.diagonal(a[sp, 0])) for sp in range(2)])
    db = np.stack([np.real(np.diagonal(b[sp, 0])) for sp in range(2)])
    xs = (0, .25, .5, .75, 1)
    es = [fo.energies_2spins(s2, T, LR, (1 - x) * a + x * b, (1 - x) * da + x * db).total(s2) for x in xs]
    c = np.polyfit(xs, es, 2)
    assert np.max(np.abs(np.polyval(c, xs) - es)) < 1e-9
    # OptimalStep never raises the energy when it takes the parabola minimum or a downhill full step
    for l in r["logs"]:
        assert l.dE >= -1e-9 or l.step == s2.StepAlternative
