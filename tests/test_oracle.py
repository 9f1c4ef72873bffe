"""CPU tests of the oracle: self-consistency of its two restatements, the reference's
algebraic invariants, integer maps, and the committed golden fixtures."""
import math
import os

import numpy as np
import pytest

from oracle import forge_oracle as fo

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_setup_derived_parameters():
    # Setup.f90:10, 23-24, 67-69 for the configurations of the build
    for m, L, N in ((5, 2, 364), (10, 2, 1324), (20, 2, 5044), (12, 3, 2814), (31, 2, 11908)):
        s = fo.Setup(ntheta=m, nlayers=L, RotateLayers=(-1, 1, -1)[:L])
        assert s.ndim == N
        assert s.numb == 20 and s.nLower == N // 2 - 9 and s.nUpper == N // 2 + 10
        assert s.NeutralityPoint == 10
    s = fo.Setup(ntheta=1, nlayers=1, RotateLayers=(-1,))
    assert s.ndim == 14 and s.numb == 14 and s.nUpper - s.nLower + 1 == s.numb


def test_neighbor_cells_and_kgrid():
    assert fo.number_neighbor_cells(1) == 4
    u1, u2 = fo.order_neighbor_cells(1, 4)
    assert list(zip(u1, u2)) == [(0, 0), (-1, 0), (-1, 1), (0, -1)]
    comps, flat, vals = fo.sample_bz(3, (1.0, 0.0), (0.0, 1.0))
    assert comps.tolist() == [[a, b] for a in range(3) for b in range(3)]
    assert flat[2, 1] == 2 * 3 + 1 + 1
    assert vals[2, 1, 0] == 2.0 / 3.0 and vals[2, 1, 1] == 1.0 / 3.0


@pytest.mark.parametrize("m,L,rl", [(1, 2, (-1, 1)), (4, 2, (-1, 1)), (3, 3, (-1, 1, -1)), (2, 1, (1,))])
def test_geometry_site_maps(m, L, rl):
    s = fo.Setup(ntheta=m, nlayers=L, RotateLayers=rl, numk=2)
    g = fo.build_geometry(s)
    N = s.ndim
    assert g.coords.shape == (N, 3)
    # C2 pairs every A site of a layer with a B site, C3 maps every site (no ERROR lines)
    assert g.c2_count == N // 2
    assert g.c3_count == N
    assert sorted(g.c3pairs.tolist()) == list(range(1, N + 1))     # C3 map is a permutation
    assert np.all(g.c2pairs[g.c2pairs - 1] == np.arange(1, N + 1))   # C2 map is an involution
    # layer-major ordering with the layer heights of Geometry.f90:164
    per = N // L
    for l in range(L):
        z = g.coords[l * per:(l + 1) * per, 2]
        assert np.all(z == z[0])
    # rigid graphene: nearest-neighbour distance a0 = a/sqrt(3) inside a layer
    X = g.coords[:per]
    d = np.sqrt(((X[:, None, :2] - X[None, :, :2]) ** 2).sum(-1)) + np.eye(per) * 10
    assert abs(d.min() - 1 / math.sqrt(3)) < 1e-9


def test_tables_c_vs_numpy():
    if fo._clib() is None:
        pytest.skip("oracle C library not built")
    s = fo.Setup(ntheta=2, numk=2)
    g = fo.build_geometry(s)
    Tn = fo.pair_tables(s, g, use_c=False)
    Tc = fo.pair_tables(s, g, use_c=True)
    assert np.array_equal(Tn.vm, Tc.vm) and np.array_equal(Tn.vp, Tc.vp)   # same IEEE ops, no FMA
    for a, b in ((Tn.tm, Tc.tm), (Tn.tp, Tc.tp)):
        assert np.max(np.abs(a - b)) <= 1e-15                           # exp() last-place rounding
    assert np.array_equal(fo.long_range_interaction(s, g, use_c=False), fo.long_range_interaction(s, g, use_c=True))


def test_fv_ft_known_values():
    s = fo.Setup()
    # on-site / coincident points vanish (TightBinding.f90:226, HartreeFock.f90:1250)
    assert fo.ft(s, [0, 0, 0], [0, 0, 0]) == 0.0 and fo.fv(s, [0, 0, 0], [0, 0, 0]) == 0.0
    # nearest-neighbour in-plane hopping is -2.7 eV at r = a0
    assert abs(fo.ft(s, [0, 0, 0], [s.a0, 0, 0]) + 2.7) < 1e-12
    # vertical interlayer hopping is +0.48 eV at r = d0
    assert abs(fo.ft(s, [0, 0, 0], [0, 0, s.d0]) - 0.48) < 1e-12
    # far field: dual-gate screening is exponentially small beyond the gate distance
    far = fo.fv(s, [0, 0, 0], [3 * s.xi, 0, 0])
    assert 0 < far < 1e-5
    # near field: unscreened 1/r dominates at short distance
    v = fo.fv(s, [0, 0, 0], [1.0, 0, 0])
    assert 0.9 < v < 1.0


def test_heap_sort_and_fermi():
    rng = np.random.default_rng(0)
    e = np.round(rng.standard_normal(50), 1)   # many ties
    arr = np.stack([e, np.arange(1, 51, dtype=float)], axis=1)
    srt = fo.dsort_lists(arr)
    assert np.all(np.diff(srt[:, 0]) >= 0)
    assert sorted(srt[:, 1].tolist()) == list(range(1, 51))
    assert np.array_equal(e[srt[:, 1].astype(int) - 1], srt[:, 0])
    assert fo.fortran_nint(2.5) == 3 and fo.fortran_nint(-2.5) == -3 and fo.fortran_nint(1.49) == 1
    s = fo.Setup(ntheta=1, numk=2)
    assert fo.zdeg_weight(s, 0.1) == complex(float(np.float32(0.1)), 8.0)
    s.degfactor_mode = "corrected"
    assert fo.zdeg_weight(s, 0.1) == complex(0.1, 0.0)


@pytest.fixture(scope="module")
def scf_m2():
    s = fo.Setup(ntheta=2, numk=3, itmax=3)
    return s, fo.run_scf(s, keep_history=True)


def test_trace_and_storage_invariants(scf_m2):
    s, r = scf_m2
    P = r["P"]
    # Tr P(0) = nLower-1 fully occupied bands + nFermiLevel/Nk window states (Main.f90:290-294, 400)
    expect = (s.nLower - 1) + fo.fortran_nint(s.Nk * s.NeutralityPoint + s.Nk / 2 * s.nfilling) / s.Nk
    assert abs(np.trace(P[0]).real - expect) < 1e-10
    # P(0) is Hermitian when no partially occupied states carry the complex zdeg weight
    assert all(l.npart == 0 for l in r["logs"])
    assert np.max(np.abs(P[0] - P[0].conj().T)) < 1e-12


def test_zheevr_oracle_agrees_with_zheevd(scf_m2):
    """The oracle's eigen-solver is the reference's zheevr (range 'I', 'L' triangle); the FP64 result
    the benchmark description names is LAPACK's zheevd.  On H(k) of an SCF state the two agree:
    eigenvalues 1..nUpper to 1e-12 eV and the projector onto bands 1..nLower-1 to 1e-12."""
    from scipy.linalg import lapack
    s, r = scf_m2
    g, T = r["geometry"], r["tables"]
    for icount in (0, 4):
        H = fo.hamiltonian(s, g, T, r["V"], r["P"], g.vk(icount))
        w_r, z_r = fo.eigh_lower(H, s.nUpper)
        w_d, z_d, info = lapack.zheevd(H, compute_v=1, lower=1)
        assert info == 0
        assert np.max(np.abs(w_r - w_d[:s.nUpper])) <= 1e-12
        k = s.nLower - 1
        P_r = z_r[:, :k] @ z_r[:, :k].conj().T
        P_d = z_d[:, :k] @ z_d[:, :k].conj().T
        assert np.max(np.abs(P_r - P_d)) <= 1e-12


def test_hamiltonian_hermitian_lower_triangle(scf_m2):
    s, r = scf_m2
    g, T = r["geometry"], r["tables"]
    H = fo.hamiltonian(s, g, T, r["V"], r["P"], g.vk(1))
    off = ~np.eye(s.ndim, dtype=bool)
    assert np.max(np.abs((H - H.conj().T)[off])) == 0.0
    # the diagonal is real up to rounding (zheevr reads only its real part)
    assert np.max(np.abs(np.diag(H).imag)) < 1e-12


def test_oda_energy_is_quadratic(scf_m2):
    s, r = scf_m2
    T, LR = r["tables"], r["LR"]
    a, b = r["history"][0]["P"], r["P_new"]
    da, db = np.real(np.diagonal(a[0])), np.real(np.diagonal(b[0]))
    es = [fo.energies(s, T, LR, (1 - x) * a + x * b, (1 - x) * da + x * db).total(s) for x in (0, .25, .5, .75, 1)]
    c = np.polyfit([0, .25, .5, .75, 1], es, 2)
    assert np.max(np.abs(np.polyval(c, [0, .25, .5, .75, 1]) - es)) < 1e-9


def test_golden_fixtures_reproduce():
    path = os.path.join(GOLDEN, "oracle_m1_k3.npz")
    if not os.path.exists(path):
        pytest.skip("golden fixture missing")
    gd = np.load(path)
    s = fo.Setup(ntheta=1, numk=3, itmax=3)
    r = fo.run_scf(s)
    assert np.array_equal(r["geometry"].coords, gd["coords"])
    assert np.max(np.abs(r["P"] - gd["P"])) < 1e-10
    assert np.max(np.abs(np.array([l.E_in for l in r["logs"]]) - gd["E_in"])) < 1e-9
    assert np.max(np.abs(r["LR"] - gd["LR"])) < 1e-13


@pytest.fixture(scope="module")
def m2_fixed_point():
    """The reference's OptimalStep SCF of the (2, 3) bilayer at nu = +2, converged to 1e-11 eV."""
    so = fo.Setup(ntheta=2, numk=3, nfilling=2.0)
    g = fo.build_geometry(so)
    T = fo.pair_tables(so, g)
    LR = fo.long_range_interaction(so, g)
    return so, g, T, LR, fo.run_scf(so, g, T, LR, itmax=400, residual_tol=1e-11)


def test_oracle_pulay_mixing_reaches_the_optimalstep_fixed_point(m2_fixed_point):
    """The oracle's Anderson / Pulay mixer (the library's FORGE_MIX_PULAY restated) converges to the
    fixed point the reference's OptimalStep SCF reaches, in fewer iterations."""
    so, g, T, LR, oda = m2_fixed_point
    pul = fo.run_scf(so, g, T, LR, itmax=400, residual_tol=1e-11, mixer=fo.PulayMixer(6, 0.7))
    assert oda["logs"][-1].residual < 1e-11 and pul["logs"][-1].residual < 1e-11
    assert len(pul["logs"]) < len(oda["logs"])
    assert np.max(np.abs(pul["P"] - oda["P"])) <= 1e-9
    assert abs(pul["Etot"] - oda["Etot"]) / so.ndim <= 1e-9


def test_oracle_linear_mixing_reaches_the_optimalstep_fixed_point(m2_fixed_point):
    """Linear mixing (Step fixed at beta, the library's FORGE_MIX_LINEAR) converges to the fixed point
    of the reference's OptimalStep SCF, and every logged Step is beta."""
    so, g, T, LR, oda = m2_fixed_point
    lin = fo.run_scf(so, g, T, LR, itmax=200, residual_tol=1e-10, linear_beta=0.7)
    assert lin["logs"][-1].residual < 1e-10
    assert all(l.step == 0.7 for l in lin["logs"])
    assert np.max(np.abs(lin["P"] - oda["P"])) <= 1e-8
    assert abs(lin["Etot"] - oda["Etot"]) / so.ndim <= 1e-9


def test_variant_fixtures_reproduce():
    """Regression pins of the switches outside the configured path (C3, symmetry averages, valley
    projection, numS = 2) on the m = 1 cell."""
    import importlib.util
    path = os.path.join(GOLDEN, "oracle_variants_m1_k3.npz")
    if not os.path.exists(path):
        pytest.skip("golden fixture missing")
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    gd = np.load(path)
    for name, r in mg.variant_runs():
        if name == "valley":
            # The m = 1 window has exactly degenerate pairs at E_F; the valley transform's sign of
            # X^H V X inside such a pair depends on LAPACK's basis of the pair, which differs between
            # CPU kernels of the same OpenBLAS build.  Only the guess (before any valley-averaged
            # window) is pinned here; the transform itself is pinned by tests/test_oracle_valley.py.
            assert abs(r["logs"][0].E_in - gd[name + "_E_in"][0]) < 1e-9, name
            continue
        assert np.max(np.abs(np.array([l.E_in for l in r["logs"]]) - gd[name + "_E_in"])) < 1e-9, name
        assert np.max(np.abs(np.array([l.step for l in r["logs"]]) - gd[name + "_step"])) < 1e-9, name
        assert np.max(np.abs(r["P"] - gd[name + "_P"])) < 1e-10, name
