"""ctypes binding of the C-ABI (include/forge_gpu.h, include/forge_host.h).

The names mirror the reference's Fortran routines (Solve, SortEnergies_1Spin,
GetFock, GetKineticEnergy, ..., OptimalStep) with the same argument meaning;
arrays are numpy arrays in the reference's column-major layout.  There is no
CPU fallback: every call goes through ``libforge_gpu.so`` and raises
``ForgeError`` when the library or a CUDA device is missing.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os
from typing import Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libforge_gpu.so")

FORGE_PREC_FP64 = 0
FORGE_PREC_MIXED = 1
FORGE_MIX_ODA, FORGE_MIX_PULAY, FORGE_MIX_LINEAR = 0, 1, 2
FORGE_DEG_REFERENCE = 0
FORGE_DEG_CORRECTED = 1
FORGE_ERR_ARG = -1


class ForgeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"forge_gpu error {code}: {msg}")
        self.code = code


class forge_setup(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "nlayers", "ntheta", "numk", "numS", "numI", "numC", "nscreen", "fphase", "ndim", "numb", "nLower", "nUpper",
        "NeutralityPoint", "numNeighborCells", "degfactor_mode", "precision")] + [(n, C.c_double) for n in (
            "nfilling", "U", "epsilon", "Delta", "xi", "alpha", "alphaH", "a0", "r0", "d0", "tz", "EnergyTolerance",
            "StepAlternative")]


class forge_iter_report(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "Step", "DensityConvergence", "TotalEnergyIn", "TotalEnergy", "KineticEnergyIn", "FockEnergyIn",
        "HartreeEnergyIn", "HubbardEnergyIn", "KineticEnergy", "FockEnergy", "HartreeEnergy", "HubbardEnergy",
        "FermiEnergy", "DegFactor", "residual")] + [(n, C.c_int64) for n in (
            "nFermiLevel", "nOccStates", "nPartOccStates", "info", "refined")]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class forge_scf_options(C.Structure):
    _fields_ = [("itmax", C.c_int64), ("residual_tol", C.c_double), ("mixed_until", C.c_int64),
                ("mixed_switch_tol", C.c_double), ("output_dir", C.c_char_p), ("statename", C.c_char_p),
                ("nMomentaFlattened", C.c_void_p), ("g1", C.c_void_p), ("g12", C.c_void_p)]


class forge_scf_result(C.Structure):
    _fields_ = [("iterations", C.c_int64), ("converged", C.c_int64), ("TotalEnergy", C.c_double),
                ("Energies", C.c_double * 4), ("residual", C.c_double), ("seconds", C.c_double),
                ("guess_seconds", C.c_double)]


# exported entry points: name -> argtypes (all return int)
_P = C.c_void_p
_I = C.c_int64
_D = C.c_double
SIGNATURES = {
    "forge_gpu_version": [],
    "forge_gpu_init": [_P, _P, _P, _P, _P, _P, _P, _P],
    "forge_gpu_finalize": [_P],
    "forge_gpu_long_range": [_P, _P],
    "forge_gpu_set_state": [_P, _P],
    "forge_gpu_get_state": [_P, _P, _P, _P],
    "forge_gpu_hamiltonian": [_P, _P, _P, _I, _I, _P],
    "forge_gpu_zheevr_batch": [_P, _I, _P, _I, _P, _P],
    "forge_gpu_solve": [_P, _P, _P, _P, _P, _P],
    "forge_gpu_sort_energies": [_P, _P, _P, _P],
    "forge_gpu_get_bands": [_P, _P],
    "forge_gpu_set_kshard": [_P, _I, _I],
    "forge_gpu_set_bands": [_P, _P],
    "forge_gpu_project_local": [_P, _P],
    "forge_gpu_set_pnew": [_P, _P],
    "forge_gpu_fermi": [_P, _D, _P, _P, _P, _P, _P],
    "forge_gpu_get_fock": [_P, _D, _I, _I, _P],
    "forge_gpu_energies": [_P, _P, _P, _P, _P, _P],
    "forge_gpu_optimal_step": [_P, _P, _P],
    "forge_gpu_energy_forms": [_P, _P, _P, _P],
    "forge_gpu_mix_potential": [_P, _D, _P, _P],
    "forge_gpu_plain_guess": [_P, _P],
    "forge_gpu_prepare_state": [_P, _P],
    "forge_gpu_field_guess": [_P, _P, _P, _P],
    "forge_gpu_scf_iteration": [_P, _P, _P],
    "forge_gpu_solve_group": [_P, _I, _P],
    "forge_gpu_set_potential": [_P, _P],
    "forge_gpu_scf_iteration_group": [_P, _I, _P, _P],
    "forge_gpu_set_precision": [_P, _I],
    "forge_gpu_set_mixing": [_P, _I, _I, C.c_double],
    "forge_gpu_set_refinement": [_P, _I],
    "forge_gpu_set_eigen_refinement": [_P, _I, _D, _D, _I],
    "forge_gpu_last_refined": [_P, _P],
    "forge_selftest_rr_small": [_I, _P, _P, _P, _P],
    "forge_gpu_get_setup": [_P, _P],
    "forge_gpu_synchronize": [_P],
    "forge_gpu_profile": [_P, _I],
    "forge_gpu_timer_mark": [_P, _I],
    "forge_gpu_timer_elapsed": [_P, _I, _I, _P],
    "forge_gpu_profile_read": [_P, _P, _P, _P, _P, _I],
    "forge_gpu_selftest_tc_gemm": [_I, _I, _I, _I, _P, _P, _P],
    "forge_gpu_selftest_tc_gemm_timeout": [_I, _I, _I, _I, _P, _P, _P],
    "forge_gpu_mlp_create": [_I, _I, C.c_uint64, _P],
    "forge_gpu_mlp_destroy": [_P],
    "forge_gpu_mlp_set_params": [_P, _P],
    "forge_gpu_mlp_get_params": [_P, _P, _P],
    "forge_gpu_mlp_set_loss_weights": [_P, _P],
    "forge_gpu_mlp_forward": [_P, _P, _I, _P],
    "forge_gpu_mlp_gradient": [_P, _P, _P, _I, _P, _P],
    "forge_gpu_mlp_train": [_P, _P, _P, _I, _I, _I, _D, C.c_uint64, _P],
    "forge_host_setup": [_P],
    "forge_host_geometry": [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P],
    "forge_host_run_scf": [_P, _P, _P, _P, _P],
    "forge_host_parameters_string": [_P, C.c_char_p, C.c_char_p, _I],
    "forge_host_parameters_string_relax": [_P, C.c_char_p, _I, C.c_char_p, _I],
    "forge_host_lattice_relaxation": [_P, _P, _P, _P, _P, _P, _P],
    "forge_host_site_maps": [_P, _P, _P, _P, _P],
    "forge_host_plot_bands": [_P, _P, _D, _P, _P, _P, C.c_char_p],
    "forge_host_write_fock": [_P, _P, C.c_char_p, _I],
    "forge_host_read_fock": [_P, _P, C.c_char_p, _I],
    "forge_gpu_set_c3": [_P, _I, _P, _P],
    "forge_gpu_set_symmetry": [_P, _I, _I, _I, _P],
    "forge_gpu_set_valley": [_P, _I, _P],
    "forge_gpu_symmetrize": [_P, _P],
    "forge_gpu_order_parameters": [_P, _P, _P, _P],
    "forge_host_sort_energies_2spins": [_I, _I, _P, _P, _P],
    "forge_host_fermi_2spins": [_P, _P, _P, _P, _P, _P, _P, _P],
}

_LIB = None


def load_library(path: Optional[str] = None):
    """Loads libforge_gpu.so (raises ForgeError if it is not built)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ForgeError(-1, f"{p} is not built (run forge_gb300.build.build())")
    lib = C.CDLL(p)
    for name, argt in SIGNATURES.items():
        f = getattr(lib, name)
        f.argtypes = argt
        f.restype = C.c_int
    lib.forge_gpu_last_error.restype = C.c_char_p
    lib.forge_gpu_last_error.argtypes = []
    lib.forge_gpu_launch_count.restype = C.c_int64
    lib.forge_gpu_launch_count.argtypes = []
    lib.forge_gpu_mlp_num_params.restype = C.c_int64
    lib.forge_gpu_mlp_num_params.argtypes = [_P]
    if path is None:
        _LIB = lib
    return lib


def _check(rc: int, allow_info: bool = False) -> int:
    if rc < 0 or (rc > 0 and not allow_info):
        msg = load_library().forge_gpu_last_error().decode(errors="replace")
        raise ForgeError(rc, msg)
    return rc


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f(a, dtype) -> np.ndarray:
    """Fortran-ordered contiguous copy (or view) of a."""
    return np.asfortranarray(np.asarray(a, dtype=dtype))


# ---------------------------------------------------------------------------
# Setup and geometry (host side, Setup.f90 / Geometry.f90 / Main.f90:102-163)
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class Setup:
    """Runtime mirror of Setup.f90's parameters (names as in the reference)."""

    ntheta: int = 9
    nlayers: int = 2
    RotateLayers: Sequence[int] = (-1, 1)
    numk: int = 6
    nfilling: float = 0.0
    U: float = 4.0
    epsilon: float = 10.0
    Delta: float = 0.0
    numI: int = 1
    numC: int = 3
    nscreen: int = 2
    xi: float = 10.0 / 0.246
    fphase: int = 0
    numS: int = 1
    nenforceC3: int = 0
    nenforceC2: int = 0
    nenforceT: int = 0
    nenforceC2T: int = 0
    nenforceValley: int = 0
    EnergyTolerance: float = 0.0001
    StepAlternative: float = 1.0
    degfactor_mode: str = "reference"
    precision: str = "fp64"
    # Setup.f90:12: 1 relaxes bilayers (Main.f90:156-160) with the in-plane displacement table of this
    # ntheta, relaxation = (uqx, uqy), each 5 x 5 with [n-1, m-1] = uqx(n, m)
    # (forge_gb300.relaxation.read_displacement_table reads it from FORGE's Geometry.f90)
    nrelax: int = 0
    relaxation: Optional[tuple] = None

    def to_struct(self) -> forge_setup:
        s = forge_setup()
        s.nlayers, s.ntheta, s.numk, s.numS = self.nlayers, self.ntheta, self.numk, self.numS
        s.numI, s.numC, s.nscreen, s.fphase = self.numI, self.numC, self.nscreen, self.fphase
        s.degfactor_mode = FORGE_DEG_REFERENCE if self.degfactor_mode == "reference" else FORGE_DEG_CORRECTED
        s.precision = FORGE_PREC_MIXED if self.precision == "mixed" else FORGE_PREC_FP64
        s.nfilling, s.U, s.epsilon, s.Delta, s.xi = self.nfilling, self.U, self.epsilon, self.Delta, self.xi
        s.EnergyTolerance, s.StepAlternative = self.EnergyTolerance, self.StepAlternative
        _check(load_library().forge_host_setup(C.byref(s)))
        return s


@dataclasses.dataclass
class Geometry:
    Coords: np.ndarray            # (ndim, 3)
    nUnitCell_1: np.ndarray
    nUnitCell_2: np.ndarray
    tn: np.ndarray                # (2, 3): t1, t2, t3
    g1: np.ndarray
    g12: np.ndarray
    MomentaValues: np.ndarray     # (numk, numk, 2)
    nMomentaComponents: np.ndarray  # (Nk, 2)
    nMomentaFlattened: np.ndarray   # (numk, numk)
    nC2pairs: np.ndarray
    nC3pairs: np.ndarray
    c2_count: int
    c3_count: int


def build_geometry(setup: Setup) -> Geometry:
    """Main.f90:102-163 through forge_host_geometry; for nrelax = 1 and bilayers, LatticeRelaxation
    (forge_host_lattice_relaxation) and then the C2 / C3 maps of the relaxed sites."""
    s = setup.to_struct()
    N, numk = s.ndim, s.numk
    Nk = numk * numk
    out = Geometry(
        Coords=np.zeros((N, 3), order="F"), nUnitCell_1=np.zeros(4, np.int64), nUnitCell_2=np.zeros(4, np.int64),
        tn=np.zeros((2, 3), order="F"), g1=np.zeros(2), g12=np.zeros(2), MomentaValues=np.zeros((numk, numk, 2), order="F"),
        nMomentaComponents=np.zeros((Nk, 2), np.int64, order="F"),
        nMomentaFlattened=np.zeros((numk, numk), np.int64, order="F"), nC2pairs=np.zeros(N, np.int64),
        nC3pairs=np.zeros(N, np.int64), c2_count=0, c3_count=0)
    rl = np.ascontiguousarray(setup.RotateLayers, dtype=np.int64)
    counts = np.zeros(2, np.int64)
    _check(load_library().forge_host_geometry(
        C.byref(s), _ptr(rl), _ptr(out.Coords), _ptr(out.nUnitCell_1), _ptr(out.nUnitCell_2), _ptr(out.tn),
        _ptr(out.g1), _ptr(out.g12), _ptr(out.MomentaValues), _ptr(out.nMomentaComponents),
        _ptr(out.nMomentaFlattened), _ptr(out.nC2pairs), _ptr(out.nC3pairs), _ptr(counts)))
    if setup.nrelax == 1 and setup.nlayers == 2:
        if setup.relaxation is None:
            raise ForgeError(FORGE_ERR_ARG, "nrelax = 1 needs Setup.relaxation = (uqx, uqy), the displacement "
                                            "table of this ntheta")
        uqx, uqy = (_f(np.asarray(u, dtype=np.float64).reshape(5, 5), np.float64) for u in setup.relaxation)
        matched = np.zeros(2, np.int64)
        lib = load_library()
        _check(lib.forge_host_lattice_relaxation(C.byref(s), _ptr(out.Coords), _ptr(out.g1), _ptr(out.g12),
                                                 _ptr(uqx), _ptr(uqy), _ptr(matched)))
        _check(lib.forge_host_site_maps(C.byref(s), _ptr(out.Coords), _ptr(out.nC2pairs), _ptr(out.nC3pairs),
                                        _ptr(counts)))
    out.c2_count, out.c3_count = int(counts[0]), int(counts[1])
    return out


def plot_bands(setup: Setup, geometry: Geometry, Bands: np.ndarray, FermiEnergy: float, path: str) -> None:
    """PlotBands (TightBinding.f90:275-369) through forge_host_plot_bands."""
    s = setup.to_struct()
    B = _f(Bands, np.float64)
    _check(load_library().forge_host_plot_bands(C.byref(s), _ptr(B), FermiEnergy,
                                                 _ptr(_f(geometry.nMomentaFlattened, np.int64)),
                                                 _ptr(np.ascontiguousarray(geometry.g1)),
                                                 _ptr(np.ascontiguousarray(geometry.g12)), path.encode()))


def write_fock(setup: Setup, zFock: np.ndarray, path: str, record_bytes: int = 16) -> None:
    """Fock checkpoint file of Main.f90:647-672 (record_bytes 16: gfortran recl units, 64: ifort's)."""
    s = setup.to_struct()
    _check(load_library().forge_host_write_fock(C.byref(s), _ptr(_f(zFock, np.complex128)), path.encode(),
                                                record_bytes))


def read_fock(setup: Setup, path: str, record_bytes: int = 16) -> np.ndarray:
    """zFock (ndim, ndim, numNeighborCells) from a Fock checkpoint file (Main.f90:202-234)."""
    s = setup.to_struct()
    P = np.zeros((s.ndim, s.ndim, s.numNeighborCells), dtype=np.complex128, order="F")
    _check(load_library().forge_host_read_fock(C.byref(s), _ptr(P), path.encode(), record_bytes))
    return P


def sort_energies_2spins(numk: int, numb: int, WindowSort_2Spins, SortedEnergies_1Spin) -> np.ndarray:
    """SortEnergies_2Spins (HartreeFock.f90:929-1004) through forge_host_sort_energies_2spins.

    WindowSort_2Spins is W(i, spin) (2 x 2), SortedEnergies_1Spin the (numb*Nk, 2) per-spin sorted
    energies; returns SortedEnergies_2Spins (2*numb*Nk, 2): merged energies and spin labels 1.0 / 2.0.
    """
    n = numb * numk * numk
    W = _f(np.asarray(WindowSort_2Spins, dtype=np.int64).reshape(2, 2), np.int64)
    se = _f(np.asarray(SortedEnergies_1Spin, dtype=np.float64).reshape(n, 2), np.float64)
    out = np.zeros((2 * n, 2), dtype=np.float64, order="F")
    _check(load_library().forge_host_sort_energies_2spins(numk, numb, _ptr(W), _ptr(se), _ptr(out)))
    return out


def fermi_2spins(setup: Setup, SortedEnergies_1Spin) -> dict:
    """Main.f90:416-453 (numS = 2) through forge_host_fermi_2spins: the merged list, nFermiLevel,
    FermiEnergy, nOccStates(2), nPartOccStates(2) and DegFactor."""
    s = setup.to_struct()
    n = s.numb * s.numk * s.numk
    se = _f(np.asarray(SortedEnergies_1Spin, dtype=np.float64).reshape(n, 2), np.float64)
    merged = np.zeros((2 * n, 2), dtype=np.float64, order="F")
    nF, EF, deg = C.c_int64(), C.c_double(), C.c_double()
    nocc = np.zeros(2, np.int64)
    npart = np.zeros(2, np.int64)
    _check(load_library().forge_host_fermi_2spins(C.byref(s), _ptr(se), _ptr(merged), C.byref(nF), C.byref(EF),
                                                  _ptr(nocc), _ptr(npart), C.byref(deg)))
    return dict(SortedEnergies_2Spins=merged, nFermiLevel=nF.value, FermiEnergy=EF.value,
                nOccStates=nocc.tolist(), nPartOccStates=npart.tolist(), DegFactor=deg.value)


def parameters_string(setup: Setup, statename: str = "SSS") -> str:
    s = setup.to_struct()
    buf = C.create_string_buffer(256)
    _check(load_library().forge_host_parameters_string_relax(C.byref(s), statename.encode(), setup.nrelax, buf,
                                                             256))
    return buf.value.decode()


# ---------------------------------------------------------------------------
# Device context: the reference's Hartree-Fock routines
# ---------------------------------------------------------------------------
class HartreeFock:
    """One device context; methods mirror HartreeFock.f90 / LapackRoutines.f90 routines."""

    def __init__(self, setup: Setup, geometry: Optional[Geometry] = None):
        self.setup = setup
        self.s = setup.to_struct()
        self.geometry = geometry if geometry is not None else build_geometry(setup)
        g = self.geometry
        self.N = self.s.ndim
        self.Nk = self.s.numk ** 2
        self.numb = self.s.numb
        self._keep = [_f(g.Coords, np.float64), _f(g.nUnitCell_1, np.int64), _f(g.nUnitCell_2, np.int64),
                      _f(g.tn, np.float64), _f(g.MomentaValues, np.float64), _f(g.nMomentaComponents, np.int64)]
        ctx = C.c_void_p()
        lib = load_library()
        _check(lib.forge_gpu_init(C.byref(self.s), *[_ptr(a) for a in self._keep], C.byref(ctx)))
        self.ctx = ctx
        self.lib = lib
        if setup.nenforceC3:
            self.set_c3(setup.nenforceC3)
        if setup.nenforceT or setup.nenforceC2 or setup.nenforceC2T:
            self.set_symmetry(setup.nenforceT, setup.nenforceC2, setup.nenforceC2T)
        if setup.nenforceValley:
            self.set_valley(setup.nenforceValley)

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.forge_gpu_finalize(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- shapes
    def _zfock_shape(self):
        return (self.N, self.N, 4)

    def set_precision(self, precision: str):
        _check(self.lib.forge_gpu_set_precision(self.ctx, FORGE_PREC_MIXED if precision == "mixed" else FORGE_PREC_FP64))

    def set_refinement(self, width: int = 32):
        """FP64 Rayleigh-Ritz refinement of the top `width` bands after each mixed solve (0: off)."""
        _check(self.lib.forge_gpu_set_refinement(self.ctx, width))

    def set_eigen_refinement(self, mode: int = 1, residual_below: float = 0.0, delta: float = 0.0, depth: int = 0):
        """Eigenpair refinement of the mixed solve: 0 off, 1 every mixed solve, 2 once the SCF residual
        is below residual_below (eV); delta (eV) and depth 0 = defaults (1e-3, 4)."""
        _check(self.lib.forge_gpu_set_eigen_refinement(self.ctx, mode, residual_below, delta, depth))

    def last_solve_refined(self) -> int:
        """1 if the last solve's eigenpairs were refined (forge_gpu_set_eigen_refinement)."""
        r = C.c_int64()
        _check(self.lib.forge_gpu_last_refined(self.ctx, C.byref(r)))
        return int(r.value)

    def set_c3(self, nenforceC3: int = 1):
        """nenforceC3 (Setup.f90:27): 1 = Solve_C3 / GetFock_C3, 0 = the full solve."""
        pairs = _f(self.geometry.nC3pairs, np.int64)
        rl = np.ascontiguousarray(self.setup.RotateLayers, dtype=np.int64)
        _check(self.lib.forge_gpu_set_c3(self.ctx, nenforceC3, _ptr(pairs), _ptr(rl)))

    def set_symmetry(self, nenforceT: int = 0, nenforceC2: int = 0, nenforceC2T: int = 0):
        """Symmetry averages of Main.f90:513-534 on every new density matrix of the SCF loop."""
        pairs = _f(self.geometry.nC2pairs, np.int64)
        _check(self.lib.forge_gpu_set_symmetry(self.ctx, nenforceT, nenforceC2, nenforceC2T, _ptr(pairs)))

    def set_valley(self, nenforceValley: int = 1):
        """nenforceValley (Setup.f90:31): the valley average of Main.f90:470-500 on every new window."""
        rl = np.ascontiguousarray(self.setup.RotateLayers, dtype=np.int64)
        _check(self.lib.forge_gpu_set_valley(self.ctx, nenforceValley, _ptr(rl)))

    def Symmetrize(self, copy_out: bool = True):
        """Main.f90:513-534 on the device P_new of GetFock (the switches of set_symmetry)."""
        P = np.zeros(self._zfock_shape(), dtype=np.complex128, order="F") if copy_out else None
        _check(self.lib.forge_gpu_symmetrize(self.ctx, _ptr(P)))
        return P

    def OrderParameters(self) -> dict:
        """Order parameters of the current state P(0): layer and sublattice polarisation, C2T and C3
        breaking norms (the oracle's order_parameters, evaluated on the device)."""
        out = np.zeros(4)
        c2 = _f(self.geometry.nC2pairs, np.int64)
        c3 = _f(self.geometry.nC3pairs, np.int64)
        _check(self.lib.forge_gpu_order_parameters(self.ctx, _ptr(c2), _ptr(c3), _ptr(out)))
        return dict(layer_polarization=float(out[0]), sublattice_polarization=float(out[1]),
                    c2t_breaking=float(out[2]), c3_breaking=float(out[3]))

    def set_mixing(self, mode: str = "oda", depth: int = 6, beta: float = 0.7):
        """SCF mixing: "oda" (the reference's OptimalStep), "pulay" (Anderson / Pulay, `depth` steps) or
        "linear" (P = beta P_new + (1 - beta) P_in)."""
        modes = {"oda": FORGE_MIX_ODA, "pulay": FORGE_MIX_PULAY, "linear": FORGE_MIX_LINEAR}
        if mode not in modes:
            raise ValueError(f"mixing mode {mode!r}: one of {sorted(modes)}")
        _check(self.lib.forge_gpu_set_mixing(self.ctx, modes[mode], depth, beta))

    def LongRangeInteraction(self, copy_out: bool = True) -> Optional[np.ndarray]:
        """HartreeFock.f90:14-53."""
        LR = np.zeros((self.N, self.N), order="F") if copy_out else None
        _check(self.lib.forge_gpu_long_range(self.ctx, _ptr(LR)))
        return LR

    def HamiltonianHartreeFock(self, Potential, zFock, k0: int = 0, nk: int = 1) -> np.ndarray:
        """Lower triangles of H(k) for flat k indices k0..k0+nk-1 (HartreeFock.f90:57-127)."""
        V = None if Potential is None else _f(Potential, np.float64)
        P = None if zFock is None else _f(zFock, np.complex128)
        H = np.zeros((self.N, self.N, nk), dtype=np.complex128, order="F")
        _check(self.lib.forge_gpu_hamiltonian(self.ctx, _ptr(V), _ptr(P), k0, nk, _ptr(H)))
        return H

    def zheevr_batch(self, A: np.ndarray, iu: int, vectors: bool = True):
        """zdiagRed (LapackRoutines.f90:381-433) on a batch A[:, :, b] (lower triangles)."""
        A = _f(A, np.complex128)
        if A.ndim == 2:
            A = A[:, :, None]
        nb = A.shape[2]
        w = np.zeros((iu, nb), order="F")
        Z = np.zeros((self.N, iu, nb), dtype=np.complex128, order="F") if vectors else None
        info = _check(self.lib.forge_gpu_zheevr_batch(self.ctx, nb, _ptr(A), iu, _ptr(w), _ptr(Z)), allow_info=True)
        return w, Z, info

    def Solve(self, Potential=None, zFock=None, bands=True, vectors=False, bulk=False):
        """Solve (HartreeFock.f90:402-483): returns (Bands, zEigenvectors, zFockBulk, info)."""
        V = None if Potential is None else _f(Potential, np.float64)
        P = None if zFock is None else _f(zFock, np.complex128)
        B = np.zeros((self.numb, self.Nk), order="F") if bands else None
        E = np.zeros((self.N, self.numb, self.Nk), dtype=np.complex128, order="F") if vectors else None
        FB = np.zeros(self._zfock_shape(), dtype=np.complex128, order="F") if bulk else None
        info = _check(self.lib.forge_gpu_solve(self.ctx, _ptr(V), _ptr(P), _ptr(B), _ptr(E), _ptr(FB)),
                      allow_info=True)
        return B, E, FB, info

    def SetPotential(self, Potential):
        """Loads the potential of the next solve (for SolveGroup over several contexts)."""
        _check(self.lib.forge_gpu_set_potential(self.ctx, _ptr(_f(Potential, np.float64))))

    def GetBands(self) -> np.ndarray:
        """Bands (numb, Nk) of the last solve (the window eigenvalues nLower..nUpper per k)."""
        B = np.zeros((self.numb, self.Nk), order="F")
        _check(self.lib.forge_gpu_get_bands(self.ctx, _ptr(B)))
        return B

    def SortEnergies_1Spin(self):
        """HartreeFock.f90:885-925: (SortedEnergies, nSortedMomenta, sorted flat icount)."""
        n = self.numb * self.Nk
        e = np.zeros(n)
        m = np.zeros((n, 2), np.int64, order="F")
        idx = np.zeros(n, np.int64)
        _check(self.lib.forge_gpu_sort_energies(self.ctx, _ptr(e), _ptr(m), _ptr(idx)))
        return e, m, idx

    def FermiLevel(self, nfilling: Optional[float] = None):
        """Main.f90:400-412: (nFermiLevel, FermiEnergy, nOccStates, nPartOccStates, DegFactor)."""
        nf, no, npart = C.c_int64(), C.c_int64(), C.c_int64()
        ef, deg = C.c_double(), C.c_double()
        nfill = self.setup.nfilling if nfilling is None else nfilling
        _check(self.lib.forge_gpu_fermi(self.ctx, nfill, C.byref(nf), C.byref(ef), C.byref(no), C.byref(npart),
                                        C.byref(deg)))
        return nf.value, ef.value, no.value, npart.value, deg.value

    def GetFock(self, DegFactor: float, nOccStates: int, nPartOccStates: int, copy_out: bool = True):
        """GetFock + Main.f90:510-511: P_new = (window + zFockBulk)/Nk."""
        P = np.zeros(self._zfock_shape(), dtype=np.complex128, order="F") if copy_out else None
        _check(self.lib.forge_gpu_get_fock(self.ctx, DegFactor, nOccStates, nPartOccStates, _ptr(P)))
        return P

    def Energies(self, zFock=None):
        """GetKineticEnergy, GetFockEnergy, GetHartreeHubbardEnergy: (Kinetic, Fock, Hartree, Hubbard)."""
        P = None if zFock is None else _f(zFock, np.complex128)
        out = [C.c_double() for _ in range(4)]
        _check(self.lib.forge_gpu_energies(self.ctx, _ptr(P), *[C.byref(o) for o in out]))
        return tuple(o.value for o in out)

    def OptimalStep(self, energies_in: Sequence[float]):
        """OptimalStep (HartreeFock.f90:1148-1227) on the device (P_new, P_in): (Step, energies)."""
        E = np.ascontiguousarray(energies_in, dtype=np.float64).copy()
        step = C.c_double()
        _check(self.lib.forge_gpu_optimal_step(self.ctx, C.byref(step), _ptr(E)))
        return step.value, tuple(E)

    def MixPotential(self, Step: float):
        """Main.f90:558-595: returns (DensityConvergence, residual)."""
        dn, res = C.c_double(), C.c_double()
        _check(self.lib.forge_gpu_mix_potential(self.ctx, Step, C.byref(dn), C.byref(res)))
        return dn.value, res.value

    def EnergyForms(self):
        """The energy forms of (P_in, P_new) after GetFock (forge_gpu_energy_forms): (forms[6], density of
        P_in, density of P_new); the kinetic and Fock energies of (1-s) P_in + s P_new are
        (1-s) forms[0] + s forms[1] and -((1-s)^2 forms[2] + 2 s (1-s) forms[3] + s^2 forms[4]) / 2."""
        f = np.zeros(6)
        d, dn = np.zeros(self.N), np.zeros(self.N)
        _check(self.lib.forge_gpu_energy_forms(self.ctx, _ptr(f), _ptr(d), _ptr(dn)))
        return f, d, dn

    def Mix(self, Step: float):
        """P = Step P_new + (1 - Step) P_in on the device (the OptimalStep mix of Main.f90:558-574): returns
        (site densities of the mixed state, DensityConvergence).  The context's potential is the
        numS = 1 one afterwards; a spin-polarised driver replaces it (SetPotential)."""
        dn, _ = self.MixPotential(Step)
        d = np.zeros(self.N)
        _check(self.lib.forge_gpu_get_state(self.ctx, None, _ptr(d), None))
        return d, dn

    def PlainGuess(self):
        E = np.zeros(4)
        info = _check(self.lib.forge_gpu_plain_guess(self.ctx, _ptr(E)), allow_info=True)
        return tuple(E), info

    def SetState(self, zFock):
        P = _f(zFock, np.complex128)
        _check(self.lib.forge_gpu_set_state(self.ctx, _ptr(P)))

    def PrepareState(self):
        E = np.zeros(4)
        _check(self.lib.forge_gpu_prepare_state(self.ctx, _ptr(E)))
        return tuple(E)

    def GetState(self):
        P = np.zeros(self._zfock_shape(), dtype=np.complex128, order="F")
        d = np.zeros(self.N)
        V = np.zeros(self.N)
        _check(self.lib.forge_gpu_get_state(self.ctx, _ptr(P), _ptr(d), _ptr(V)))
        return P, d, V

    def ScfIteration(self, energies: Optional[Sequence[float]] = None):
        E = None if energies is None else np.ascontiguousarray(energies, dtype=np.float64).copy()
        rep = forge_iter_report()
        info = _check(self.lib.forge_gpu_scf_iteration(self.ctx, _ptr(E), C.byref(rep)), allow_info=True)
        return rep.as_dict(), (None if E is None else tuple(E)), info

    def RunScf(self, itmax: int, residual_tol: float = 0.0, mixed_until: int = 0, mixed_switch_tol: float = 0.0,
               zFock_init=None, output_dir: Optional[str] = None, statename: str = "SSS"):
        """Main.f90:236-679 via forge_host_run_scf: (result dict, list of per-iteration reports)."""
        g = self.geometry
        self._flat = _f(g.nMomentaFlattened, np.int64)
        self._g = (np.ascontiguousarray(g.g1, dtype=np.float64), np.ascontiguousarray(g.g12, dtype=np.float64))
        opts = forge_scf_options(itmax, residual_tol, mixed_until, mixed_switch_tol,
                                 None if output_dir is None else output_dir.encode(), statename.encode(),
                                 _ptr(self._flat), _ptr(self._g[0]), _ptr(self._g[1]))
        res = forge_scf_result()
        reps = (forge_iter_report * max(1, itmax))()
        P0 = None if zFock_init is None else _f(zFock_init, np.complex128)
        _check(self.lib.forge_host_run_scf(self.ctx, C.byref(opts), _ptr(P0), C.byref(res), reps))
        out = dict(iterations=res.iterations, converged=bool(res.converged), TotalEnergy=res.TotalEnergy,
                   Energies=tuple(res.Energies), residual=res.residual, seconds=res.seconds,
                   guess_seconds=res.guess_seconds)
        return out, [reps[i].as_dict() for i in range(res.iterations)]

    def synchronize(self):
        _check(self.lib.forge_gpu_synchronize(self.ctx))

    STAGES = ("tables", "long_range", "assemble", "trd_col", "hemv", "trd_finish", "her2k", "bisect", "invit",
              "backtransform", "projector", "window", "sort", "energy", "lr_matvec", "mix", "refine", "oa_gemm", "oa")

    def mark(self, slot: int):
        """Records a CUDA event in `slot` on the context's stream."""
        _check(self.lib.forge_gpu_timer_mark(self.ctx, slot))

    def elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_double()
        _check(self.lib.forge_gpu_timer_elapsed(self.ctx, a, b, C.byref(ms)))
        return ms.value

    def profile(self, enable: bool = True):
        """Resets and enables (or disables) per-stage CUDA-event timing on the context stream."""
        _check(self.lib.forge_gpu_profile(self.ctx, 1 if enable else 0))

    def profile_read(self) -> dict:
        n = len(self.STAGES)
        ms, b, f = np.zeros(n), np.zeros(n), np.zeros(n)
        nl = np.zeros(n, np.int64)
        self.lib.forge_gpu_profile_read(self.ctx, _ptr(ms), _ptr(nl), _ptr(b), _ptr(f), n)
        return {s: dict(ms=float(ms[i]), launches=int(nl[i]), bytes=float(b[i]), flops=float(f[i]))
                for i, s in enumerate(self.STAGES)}


def _ctx_array(contexts: Sequence["HartreeFock"]):
    arr = (C.c_void_p * len(contexts))(*[h.ctx.value if isinstance(h.ctx, C.c_void_p) else h.ctx for h in contexts])
    return arr


def SolveGroup(contexts: Sequence["HartreeFock"]):
    """One batched eigen-solve over every H(k) of several systems of different ndim
    (forge_gpu_solve_group); returns the per-context info counts."""
    lib = load_library()
    info = np.zeros(len(contexts), np.int64)
    _check(lib.forge_gpu_solve_group(_ctx_array(contexts), len(contexts), _ptr(info)), allow_info=True)
    return info


def ScfIterationGroup(contexts: Sequence["HartreeFock"], energies):
    """One SCF iteration of each context with a shared uneven-size batched eigen-solve
    (forge_gpu_scf_iteration_group): returns (reports, energies (n x 4), info)."""
    lib = load_library()
    E = np.ascontiguousarray(energies, dtype=np.float64).reshape(len(contexts), 4).copy()
    reps = (forge_iter_report * len(contexts))()
    info = _check(lib.forge_gpu_scf_iteration_group(_ctx_array(contexts), len(contexts), _ptr(E), reps),
                  allow_info=True)
    return [reps[i].as_dict() for i in range(len(contexts))], E, info
