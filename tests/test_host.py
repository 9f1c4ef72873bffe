"""CPU tests of the host side: the library builds and exports every declared entry point,
the C++ host geometry is bit-exact with the oracle, the parameter string follows Main.f90."""
import ctypes
import os
import re

import numpy as np
import pytest

from oracle import forge_oracle as fo

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    names = set()
    for h in ("forge_gpu.h", "forge_host.h", "forge_gpu_selftest.h"):
        txt = open(os.path.join(ROOT, "include", h)).read()
        names |= set(re.findall(r"^\s*(?:int|int64_t|const char\*)\s+(forge_\w+)\s*\(", txt, flags=re.M))
    return names


def test_library_exports_every_declared_symbol(lib):
    declared = _declared_symbols()
    assert len(declared) >= 25
    for name in sorted(declared):
        assert hasattr(lib, name), name


def test_fortran_binding_declares_every_device_entry():
    """The Fortran module written out for a FORGE host binds every entry point of forge_gpu.h, by
    its C name (bind(C, name=...))."""
    txt = open(os.path.join(ROOT, "include", "forge_gpu.h")).read()
    device = set(re.findall(r"^\s*(?:int|int64_t|const char\*)\s+(forge_gpu_\w+)\s*\(", txt, flags=re.M))
    bound = set(re.findall(r'bind\(C, name="(forge_\w+)"\)', open(os.path.join(ROOT, "INTEGRATION.md")).read()))
    assert device and device <= bound, sorted(device - bound)


def test_library_calls_fail_cleanly_without_context(lib):
    # argument checks run before any device work
    assert lib.forge_gpu_solve(None, None, None, None, None, None) < 0
    assert lib.forge_gpu_finalize(None) == 0
    assert lib.forge_gpu_version() == 1


@pytest.mark.parametrize("m,L,rl,numk", [(1, 2, (-1, 1), 3), (5, 2, (-1, 1), 6), (12, 3, (-1, 1, -1), 6),
                                         (31, 2, (-1, 1), 4)])
def test_host_geometry_bit_exact_with_oracle(lib, m, L, rl, numk):
    import forge_gb300 as fg
    g = fg.build_geometry(fg.Setup(ntheta=m, nlayers=L, RotateLayers=rl, numk=numk))
    go = fo.build_geometry(fo.Setup(ntheta=m, nlayers=L, RotateLayers=rl, numk=numk))
    assert np.array_equal(g.Coords, go.coords)
    assert np.array_equal(g.MomentaValues, go.kvals)
    assert np.array_equal(g.nMomentaComponents, go.kcomp)
    assert np.array_equal(g.nMomentaFlattened, go.kflat)
    assert np.array_equal(g.tn[:, 0], go.t1) and np.array_equal(g.tn[:, 1], go.t2) and np.array_equal(g.tn[:, 2], go.t3)
    assert np.array_equal(g.g1, go.g1) and np.array_equal(g.g12, go.g12)
    assert np.array_equal(g.nC2pairs, go.c2pairs) and np.array_equal(g.nC3pairs, go.c3pairs)
    assert (g.c2_count, g.c3_count) == (go.c2_count, go.c3_count)
    assert list(g.nUnitCell_1) == [0, -1, -1, 0] and list(g.nUnitCell_2) == [0, 0, 1, -1]


def test_host_setup_matches_setup_f90(lib):
    import forge_gb300 as fg
    s = fg.Setup(ntheta=31, numk=4, nfilling=2.0, epsilon=10.0).to_struct()
    assert (s.ndim, s.numb, s.nLower, s.nUpper, s.NeutralityPoint, s.numNeighborCells) == (11908, 20, 5945, 5964,
                                                                                            10, 4)
    assert s.alpha == 5.853 / 10.0 and s.tz == 1.35772 and s.r0 == 0.184


def test_parameters_string(lib):
    import forge_gb300 as fg
    p = fg.parameters_string(fg.Setup(ntheta=9, numk=6))
    assert p == "-SSS-filling+0.0-numS1-i9-nlayers2-relax0-eps10.0-U4.00-screen2-xi10.0-delta0.000-numI1-numC3-numk6-dp8.dat"
    p = fg.parameters_string(fg.Setup(ntheta=20, numk=8, nfilling=-2.0, epsilon=8.0), "AB1")
    assert p.startswith("-AB1-filling-2.0-numS1-i20-") and "-eps8.0-" in p


def test_init_without_gpu_reports_error(lib):
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    import forge_gb300 as fg
    with pytest.raises(fg.ForgeError):
        fg.HartreeFock(fg.Setup(ntheta=1, numk=2))


@pytest.mark.parametrize("numk", [6, 12])
def test_plot_bands_matches_oracle(lib, tmp_path, numk):
    import forge_gb300 as fg
    S = fg.Setup(ntheta=2, numk=numk)
    g = fg.build_geometry(S)
    so = fo.Setup(ntheta=2, numk=numk)
    go = fo.build_geometry(so)
    rng = np.random.default_rng(numk)
    bands = rng.standard_normal((so.numb, so.Nk))
    path = str(tmp_path / "bands.dat")
    fg.api.plot_bands(S, g, bands, 0.25, path)
    rows = [list(map(float, l.split())) for l in open(path) if l.strip()]
    ref = fo.plot_bands_lines(so, go, bands, 0.25)
    assert len(rows) == len(ref)
    assert np.max(np.abs(np.array(rows) - np.round(np.array(ref), 8))) <= 1e-8


def _fock_records_reference_order(P, record_bytes):
    """The record stream of Main.f90:647-672, written with plain numpy loops in the Fortran order."""
    N, _, NC = P.shape
    out = bytearray()
    pad = b"\0" * (record_bytes - 16)
    for i in range(N):
        for j in range(i + 1):
            out += np.complex128(P[i, j, 0]).tobytes() + pad
    for m in range(1, NC):
        for i in range(N):
            for j in range(N):
                out += np.complex128(P[i, j, m]).tobytes() + pad
    return bytes(out)


@pytest.mark.parametrize("record_bytes", [16, 64])
def test_fock_checkpoint_format_round_trip(tmp_path, record_bytes):
    """Fock dump / read (Main.f90:647-672, 202-234): byte-identical to the reference's record order
    (gfortran and ifort record lengths), and the read restores the conjugate upper triangle of R = 0."""
    import forge_gb300 as fg
    S = fg.Setup(ntheta=2, numk=1)
    N = S.to_struct().ndim
    rng = np.random.default_rng(7)
    P = (rng.standard_normal((N, N, 4)) + 1j * rng.standard_normal((N, N, 4))).astype(np.complex128)
    P[:, :, 0] = (P[:, :, 0] + P[:, :, 0].conj().T) / 2          # P(R=0) Hermitian
    P = np.asfortranarray(P)
    path = str(tmp_path / f"Fock-nspin1{fg.parameters_string(S)}")
    fg.write_fock(S, P, path, record_bytes)
    data = open(path, "rb").read()
    assert len(data) == (N * (N + 1) // 2 + 3 * N * N) * record_bytes
    assert data == _fock_records_reference_order(P, record_bytes)
    Q = fg.read_fock(S, path, record_bytes)
    assert np.array_equal(Q, P)


def test_fock_checkpoint_rejects_missing_file(tmp_path):
    import forge_gb300 as fg
    with pytest.raises(fg.ForgeError):
        fg.read_fock(fg.Setup(ntheta=2, numk=1), str(tmp_path / "missing"), 16)


@pytest.mark.parametrize("damage", ["truncated", "trailing", "nan", "other_record_length"])
def test_fock_checkpoint_rejects_damaged_file(tmp_path, damage):
    """A restart (Main.f90:202-234) must not load a cut-off, padded or corrupted checkpoint, nor one
    written with another record length: the reader fails with a message instead."""
    import forge_gb300 as fg
    S = fg.Setup(ntheta=2, numk=1)
    N = S.to_struct().ndim
    rng = np.random.default_rng(3)
    P = np.asfortranarray(rng.standard_normal((N, N, 4)) + 1j * rng.standard_normal((N, N, 4)))
    path = str(tmp_path / "Fock")
    fg.write_fock(S, P, path, 16)
    data = bytearray(open(path, "rb").read())
    rb = 16
    if damage == "truncated":
        data = data[: len(data) // 2]
    elif damage == "trailing":
        data += b"\0" * 16
    elif damage == "nan":
        data[16 * 5: 16 * 5 + 8] = np.float64(np.nan).tobytes()
    else:
        rb = 64
    open(path, "wb").write(bytes(data))
    with pytest.raises(fg.ForgeError) as e:
        fg.read_fock(S, path, rb)
    assert ("non-finite" if damage == "nan" else "bytes") in str(e.value)


@pytest.mark.parametrize("n,seed", [(1, 0), (5, 1), (32, 2)])
def test_rayleigh_ritz_small_solve_matches_numpy(n, seed):
    """The nw x nw step of the mixed path's FP64 window refinement (forge_selftest_rr_small, host
    code): the generalised eigenvalues of (G, S) match numpy, G M = S M theta and M^H S M = I."""
    import ctypes as C
    import forge_gb300 as fg
    lib = fg.load_library()
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((200, n)) + 1j * rng.standard_normal((200, n))
    X /= np.linalg.norm(X, axis=0)
    X += 1e-7 * (rng.standard_normal(X.shape) + 1j * rng.standard_normal(X.shape))   # nearly orthonormal
    H = rng.standard_normal((200, 200)) + 1j * rng.standard_normal((200, 200))
    H = (H + H.conj().T) / 2
    G = np.asfortranarray(X.conj().T @ H @ X)
    S = np.asfortranarray(X.conj().T @ X)
    th = np.zeros(n)
    M = np.zeros((n, n), dtype=np.complex128, order="F")
    rc = lib.forge_selftest_rr_small(n, G.ctypes.data_as(C.c_void_p), S.ctypes.data_as(C.c_void_p),
                                     th.ctypes.data_as(C.c_void_p), M.ctypes.data_as(C.c_void_p))
    assert rc == 0
    Ls = np.linalg.cholesky(S)
    Li = np.linalg.inv(Ls)
    ref = np.linalg.eigvalsh(Li @ G @ Li.conj().T)
    scale = max(1.0, np.max(np.abs(ref)))
    assert np.max(np.abs(th - ref)) <= 1e-12 * scale
    assert np.all(np.diff(th) >= 0)
    assert np.max(np.abs(G @ M - S @ M * th)) <= 1e-11 * scale
    assert np.max(np.abs(M.conj().T @ S @ M - np.eye(n))) <= 1e-12


def test_host_sort_energies_2spins_matches_oracle(lib):
    import forge_gb300 as fg
    # the hand-worked lists of the oracle tests, then random per-spin sorted lists with ties
    se1 = [0.0, 1.0, 2.0, 3.0, 4.0, 5.0]
    se2 = [10.0, 0.5, 1.5, 2.5, 3.5, 4.5]
    out = fg.sort_energies_2spins(1, 6, [[2, 2], [5, 5]], np.stack([se1, se2], 1))
    e, lab = fo.sort_energies_2spins(1, 6, [[2, 2], [5, 5]], se1, se2)
    assert np.array_equal(out[:, 0], e) and np.array_equal(out[:, 1], lab)
    rng = np.random.default_rng(11)
    for numk, numb, W in ((2, 20, [[9, 9], [13, 13]]), (3, 20, [[9, 9], [13, 13]]), (1, 14, [[1, 1], [15, 15]]),
                          (2, 8, [[3, 2], [6, 9]])):
        n = numb * numk * numk
        se = np.sort(np.round(rng.normal(size=(n, 2)), 1), axis=0)      # rounding makes equal energies
        out = fg.sort_energies_2spins(numk, numb, W, se)
        e, lab = fo.sort_energies_2spins(numk, numb, np.array(W), se[:, 0], se[:, 1])
        assert np.array_equal(out[:, 0], e) and np.array_equal(out[:, 1], lab), (numk, numb, W)


def test_host_sort_energies_2spins_rejects_windows_outside_the_lists(lib):
    import forge_gb300 as fg
    se = np.zeros((6, 2))
    for W in ([[0, 1], [3, 3]], [[3, 1], [2, 3]], [[2, 2], [8, 3]], [[7, 2], [7, 7]]):
        with pytest.raises(fg.ForgeError):
            fg.sort_energies_2spins(1, 6, np.array(W), se)


@pytest.mark.parametrize("nfilling,split", [(0.0, 0.3), (2.0, 0.0), (-1.5, 0.05), (1.0, 0.0)])
def test_host_fermi_2spins_matches_oracle(lib, nfilling, split):
    import forge_gb300 as fg
    s = fg.Setup(ntheta=1, numk=3, nfilling=nfilling, numS=2)
    so = fo.Setup(ntheta=1, numk=3, nfilling=nfilling, numS=2)
    n = so.numb * so.Nk
    rng = np.random.default_rng(5)
    base = np.sort(np.round(rng.normal(size=n), 2))
    se = np.stack([base, np.sort(base + split * rng.normal(size=n))], 1)
    r = fg.fermi_2spins(s, se)
    e, lab = fo.sort_energies_2spins(so.numk, so.numb, fo.window_sort_2spins(so), se[:, 0], se[:, 1])
    nF, EF, nocc, npart, deg = fo.fermi_level_2spins(so, e, lab)
    assert np.array_equal(r["SortedEnergies_2Spins"][:, 0], e)
    assert (r["nFermiLevel"], r["FermiEnergy"], r["nOccStates"], r["nPartOccStates"]) == (nF, EF, nocc, npart)
    assert r["DegFactor"] == deg


def test_init_rejects_unsupported_setups_before_touching_the_device(lib):
    """forge_gpu_init checks its arguments before any CUDA call: numS = 2 (one context per spin),
    fphase = 1 (the projectors apply no site phase) and numI > 1 are FORGE_ERR_ARG."""
    import ctypes as C
    import forge_gb300 as fg
    g = fg.build_geometry(fg.Setup(ntheta=1, numk=3))
    keep = [np.asfortranarray(a) for a in (g.Coords, g.nUnitCell_1, g.nUnitCell_2, g.tn, g.MomentaValues,
                                          g.nMomentaComponents)]
    for kw in (dict(numS=2), dict(fphase=1)):
        s = fg.Setup(ntheta=1, numk=3, **kw).to_struct()
        ctx = C.c_void_p()
        rc = lib.forge_gpu_init(C.byref(s), *[a.ctypes.data_as(C.c_void_p) for a in keep], C.byref(ctx))
        assert rc == -1          # FORGE_ERR_ARG
        assert not ctx.value
        assert lib.forge_gpu_last_error()
