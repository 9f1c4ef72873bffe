"""CPU tests of the oracle's symmetry switches of the SCF loop (Main.f90:513-534: nenforceT, nenforceC2,
nenforceC2T): each symmetrised density matrix has its symmetry, the symmetrisers are idempotent and
commute, and an SCF run with a switch on produces new density matrices with that symmetry."""
import numpy as np
import pytest

from oracle import forge_oracle as fo


@pytest.fixture(scope="module")
def system():
    s = fo.Setup(ntheta=2, numk=3, nfilling=2.0, degfactor_mode="corrected")
    g = fo.build_geometry(s)
    rng = np.random.default_rng(4)
    N = s.ndim
    P = rng.standard_normal((4, N, N)) + 1j * rng.standard_normal((4, N, N))
    return s, g, P


def _with(s, **flags):
    d = {f.name: getattr(s, f.name) for f in fo.dataclasses.fields(s)}
    d.update(flags)
    return fo.Setup(**d)


def _c2(g, M):
    p0 = g.c2pairs - 1
    return np.conj(M[np.ix_(p0, p0)].T)


def _c2t(g, M):
    p0 = g.c2pairs - 1
    return M[np.ix_(p0, p0)].T


def test_each_switch_imposes_its_symmetry(system):
    s, g, P = system
    assert g.c2_count == s.ndim // 2 and np.all(g.c2pairs > 0)
    PT = fo.enforce_symmetries(_with(s, nenforceT=1), g, P)
    assert np.all(PT.imag == 0) and np.array_equal(PT.real, P.real)
    PC = fo.enforce_symmetries(_with(s, nenforceC2=1), g, P)
    PCT = fo.enforce_symmetries(_with(s, nenforceC2T=1), g, P)
    for m in range(4):
        assert np.max(np.abs(PC[m] - _c2(g, PC[m]))) < 1e-15
        assert np.max(np.abs(PCT[m] - _c2t(g, PCT[m]))) < 1e-15
    # no switch: the matrix is returned unchanged
    assert fo.enforce_symmetries(s, g, P) is P


def test_symmetrisers_are_idempotent_and_commute(system):
    s, g, P = system
    for flags in (dict(nenforceT=1), dict(nenforceC2=1), dict(nenforceC2T=1),
                  dict(nenforceT=1, nenforceC2=1, nenforceC2T=1)):
        sx = _with(s, **flags)
        once = fo.enforce_symmetries(sx, g, P)
        assert np.max(np.abs(fo.enforce_symmetries(sx, g, once) - once)) < 1e-15
    # C2 then C2T equals C2T then C2 (both are averages over commuting involutions)
    a = fo.enforce_symmetries(_with(s, nenforceC2T=1), g, fo.enforce_symmetries(_with(s, nenforceC2=1), g, P))
    b = fo.enforce_symmetries(_with(s, nenforceC2=1), g, fo.enforce_symmetries(_with(s, nenforceC2T=1), g, P))
    assert np.max(np.abs(a - b)) < 1e-15


@pytest.mark.parametrize("flags", [dict(nenforceT=1), dict(nenforceC2=1), dict(nenforceC2T=1),
                                   dict(nenforceT=1, nenforceC2=1, nenforceC2T=1)])
def test_scf_new_density_matrices_have_the_symmetry(system, flags):
    s, g, _ = system
    sx = _with(s, **flags)
    T = fo.pair_tables(sx, g)
    LR = fo.long_range_interaction(sx, g)
    r = fo.run_scf(sx, g, T, LR, itmax=3)
    Pn = r["P_new"]
    if flags.get("nenforceT"):
        assert np.all(Pn.imag == 0)
    for m in range(4):
        if flags.get("nenforceC2"):
            assert np.max(np.abs(Pn[m] - _c2(g, Pn[m]))) < 1e-14
        if flags.get("nenforceC2T"):
            assert np.max(np.abs(Pn[m] - _c2t(g, Pn[m]))) < 1e-14
    # the charge is kept: symmetrisation permutes and averages diagonal entries of P(0)
    expect = (s.nLower - 1) + fo.fortran_nint(s.Nk * s.NeutralityPoint + s.Nk / 2 * s.nfilling) / s.Nk
    assert abs(np.trace(Pn[0]).real - expect) < 1e-10
