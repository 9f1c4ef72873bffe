"""LatticeRelaxation (Geometry.f90:279-1135): the C++ host against the oracle, the relaxation's
symmetries, its error path and the displacement-table reader, on CPU.

The displacement tables are the reference's own (tests/golden/relaxation_uq.npz, read out of
Geometry.f90 by tests/golden/make_relaxation_tables.py with the Fortran literal kinds applied).
"""
import math
import os

import numpy as np
import pytest

from oracle import forge_oracle as fo

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _uq(m):
    d = np.load(os.path.join(GOLDEN, "relaxation_uq.npz"))
    return d[f"uqx_{m}"], d[f"uqy_{m}"]


@pytest.mark.parametrize("m", [2, 5, 10])
def test_host_relaxation_matches_oracle(m):
    import forge_gb300 as fg
    uq = _uq(m)
    G = fg.build_geometry(fg.Setup(ntheta=m, numk=2, nrelax=1, relaxation=uq))
    so = fo.Setup(ntheta=m, numk=2, nrelax=1, relax_uq=uq)
    g = fo.build_geometry(so)
    assert np.array_equal(G.Coords, g.coords)                     # same unfused IEEE operations, same libm
    assert np.array_equal(G.nC2pairs, g.c2pairs) and np.array_equal(G.nC3pairs, g.c3pairs)
    N = so.ndim
    assert (G.c2_count, G.c3_count) == (N // 2, N)                  # the maps stay complete
    # the sites did move, by at most the table's bound
    g0 = fo.build_geometry(fo.Setup(ntheta=m, numk=2))
    disp = np.hypot(*(g.coords[:, :2] - g0.coords[:, :2]).T)
    bound = 3 * sum(math.hypot(uq[0][n, k], uq[1][n, k]) for n in range(5) for k in range(5))
    assert 0.0 < disp.max() <= bound


def test_headline_relaxation_coordinates_match_oracle():
    """The 1.05 deg bilayer (m = 31, N = 11908): host coordinates bit for bit against the oracle's
    relaxation of the same rotated sites; every layer-2 site re-indexed; maps complete."""
    import forge_gb300 as fg
    m = 31
    uq = _uq(m)
    G = fg.build_geometry(fg.Setup(ntheta=m, numk=2, nrelax=1, relaxation=uq))
    G0 = fg.build_geometry(fg.Setup(ntheta=m, numk=2))
    so = fo.Setup(ntheta=m, numk=2, nrelax=1, relax_uq=uq)
    c, cnt = fo.lattice_relaxation(so, G0.Coords, tuple(G0.g1), tuple(G0.g12), *uq)
    N = so.ndim
    assert cnt == (N // 4, N // 4)
    assert np.array_equal(G.Coords, c)
    assert (G.c2_count, G.c3_count) == (N // 2, N)


@pytest.mark.parametrize("m", [5, 10])
def test_relaxation_symmetries(m):
    so = fo.Setup(ntheta=m, numk=2, nrelax=1, relax_uq=_uq(m))
    g = fo.build_geometry(so)
    X = g.coords
    N = so.ndim
    # C2 (r -> -r) pairs the sublattices of each layer exactly, C3 maps every site onto its image
    i = np.arange(N)
    assert np.max(np.abs(X[i, :2] + X[g.c2pairs - 1, :2])) < 1e-13
    # (the corner site closing each sublattice block maps to itself by the reference's convention,
    # Geometry.f90:1216-1220: its image lies in a neighbouring cell)
    c, s = -0.5, math.sqrt(3.0) / 2
    R3 = np.array([[c, -s], [s, c]])
    per = N // so.nlayers
    inner = np.setdiff1d(i, [l * per + k for l in range(so.nlayers) for k in (per // 2 - 1, per - 1)])
    assert np.max(np.abs(X[inner, :2] @ R3.T - X[g.c3pairs[inner] - 1, :2])) < 1e-12
    # layer 2 is the x-mirror of layer 1, as sets of sites of each sublattice (the closing corner site
    # of a layer-2 block takes (x, -y) of the mirrored one instead, Geometry.f90:1103-1106)
    h, q = N // 2, N // 4
    for a, b in ((slice(0, q - 1), slice(h, h + q - 1)), (slice(q, h - 1), slice(h + q, N - 1))):
        L1 = X[a, :2] * np.array([-1.0, 1.0])
        L2 = X[b, :2]
        d = np.hypot(L1[:, None, 0] - L2[None, :, 0], L1[:, None, 1] - L2[None, :, 1]).min(axis=1)
        assert np.max(d) < 1e-12
    # heights unchanged
    g0 = fo.build_geometry(fo.Setup(ntheta=m, numk=2))
    assert np.array_equal(X[:, 2], g0.coords[:, 2])


def test_zero_table_keeps_the_rotated_lattice():
    """With no displacement the relaxation only mirrors layer 1 onto layer 2 and re-indexes it: the
    unrelaxed bilayer is mirror symmetric, so the sites come back to rounding."""
    z = (np.zeros((5, 5)), np.zeros((5, 5)))
    for m in (2, 5):
        g = fo.build_geometry(fo.Setup(ntheta=m, numk=2, nrelax=1, relax_uq=z))
        g0 = fo.build_geometry(fo.Setup(ntheta=m, numk=2))
        assert np.max(np.abs(g.coords - g0.coords)) < 1e-14
        assert np.array_equal(g.c2pairs, g0.c2pairs) and np.array_equal(g.c3pairs, g0.c3pairs)


def test_relaxation_error_paths():
    import forge_gb300 as fg
    from forge_gb300.api import ForgeError
    # nrelax = 1 without a table
    with pytest.raises(ForgeError):
        fg.build_geometry(fg.Setup(ntheta=2, numk=2, nrelax=1))
    # a trilayer is not relaxed (Main.f90:157), with or without a table
    G = fg.build_geometry(fg.Setup(ntheta=2, nlayers=3, RotateLayers=(-1, 1, -1), numk=2, nrelax=1))
    assert G.c3_count == G.Coords.shape[0]
    # displacements beyond the 0.25 a matching radius: the reference's ERROR RELAXATION, here an
    # error with the same counts the oracle finds
    ux, uy = _uq(5)
    ux = ux.copy()
    ux[1, 0] = -0.3
    with pytest.raises(ForgeError, match="ERROR RELAXATION"):
        fg.build_geometry(fg.Setup(ntheta=5, numk=2, nrelax=1, relaxation=(ux, uy)))
    so = fo.Setup(ntheta=5, numk=2, nrelax=1, relax_uq=(ux, uy))
    g0 = fo.build_geometry(fo.Setup(ntheta=5, numk=2))
    c, cnt = fo.lattice_relaxation(so, g0.coords, g0.g1, g0.g12, ux, uy)
    assert cnt != (so.ndim // 4, so.ndim // 4) and np.isnan(c).any()


def test_read_displacement_table_applies_fortran_literal_kinds(tmp_path):
    from forge_gb300.relaxation import fortran_real_literal, read_displacement_table
    src = tmp_path / "Geometry.f90"
    src.write_text(
        "  uqx=0.0_dp\n"
        "  if(ntheta.EQ.4)then\n"
        "  uqx(2,1)=-0.1234567890123\n"
        "  uqy(2,1)=0.5_dp\n"
        "  uqx(3,2)=1.5d-3   ! a comment\n"
        "  uqy(5,4)=-2.0e-07\n"
        "  endif\n"
        "  if(ntheta.EQ.14)then\n"
        "  uqx(2,1)=9.0\n"
        "  endif\n")
    ux, uy = read_displacement_table(str(src), 4)
    assert ux[1, 0] == float(np.float32(-0.1234567890123)) != -0.1234567890123
    assert uy[1, 0] == 0.5 and ux[2, 1] == 1.5e-3 and uy[4, 3] == float(np.float32(-2.0e-07))
    assert np.count_nonzero(ux) == 2 and np.count_nonzero(uy) == 2
    ux, uy = read_displacement_table(str(src), 14)
    assert ux[1, 0] == 9.0 and np.count_nonzero(ux) == 1
    ux, uy = read_displacement_table(str(src), 7)
    assert not ux.any() and not uy.any()
    assert fortran_real_literal("0.0_dp") == 0.0
    with pytest.raises(ValueError):
        fortran_real_literal("1.0_sp")


def test_parameters_string_carries_nrelax():
    import forge_gb300 as fg
    assert "-relax1-" in fg.parameters_string(fg.Setup(ntheta=2, numk=2, nrelax=1, relaxation=_uq(2)))
    assert "-relax0-" in fg.parameters_string(fg.Setup(ntheta=2, numk=2))


def test_host_relaxation_entry_checks_its_arguments(lib):
    """The C entries reject null arguments, non-bilayers and bad nrelax before touching memory."""
    import ctypes as C
    import forge_gb300 as fg
    S = fg.Setup(ntheta=2, numk=2)
    s = S.to_struct()
    N = s.ndim
    X = np.zeros((N, 3), order="F")
    g = np.zeros(2)
    u = np.zeros((5, 5), order="F")
    p = lambda a: a.ctypes.data_as(C.c_void_p)   # noqa: E731
    assert lib.forge_host_lattice_relaxation(C.byref(s), None, p(g), p(g), p(u), p(u), None) == -1
    assert lib.forge_host_lattice_relaxation(None, p(X), p(g), p(g), p(u), p(u), None) == -1
    s3 = fg.Setup(ntheta=2, nlayers=3, RotateLayers=(-1, 1, -1), numk=2).to_struct()
    X3 = np.zeros((s3.ndim, 3), order="F")
    assert lib.forge_host_lattice_relaxation(C.byref(s3), p(X3), p(g), p(g), p(u), p(u), None) == -1
    assert b"bilayers only" in lib.forge_gpu_last_error()
    assert lib.forge_host_site_maps(C.byref(s), None, None, None, None) == -1
    buf = C.create_string_buffer(256)
    assert lib.forge_host_parameters_string_relax(C.byref(s), b"SSS", 10, buf, 256) == -1
    assert lib.forge_host_parameters_string_relax(C.byref(s), b"SSS", 1, buf, 256) == 0
    assert b"-relax1-" in buf.value
