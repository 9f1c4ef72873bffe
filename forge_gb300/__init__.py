"""GB300-native (sm_103a) engine for FORGE's real-space Hartree-Fock SCF.

The compute path is ``libforge_gpu.so`` (hand-written CUDA for sm_103a behind the
C-ABI of ``include/forge_gpu.h``); this package is the thin Python host that
binds it with ctypes.  Build with ``forge_gb300.build.build()``.
"""
from .api import (FORGE_DEG_CORRECTED, FORGE_DEG_REFERENCE, FORGE_PREC_FP64, FORGE_PREC_MIXED, ForgeError,
                  Geometry, HartreeFock, ScfIterationGroup, Setup, SolveGroup, build_geometry, fermi_2spins,
                  load_library, parameters_string, read_fock, sort_energies_2spins, write_fock)
from .spin import SpinPolarisedScf

__all__ = ["Setup", "Geometry", "HartreeFock", "build_geometry", "load_library", "parameters_string", "ForgeError",
           "read_fock", "write_fock", "sort_energies_2spins", "fermi_2spins",
           "SpinPolarisedScf", "SolveGroup", "ScfIterationGroup",
           "FORGE_PREC_FP64", "FORGE_PREC_MIXED", "FORGE_DEG_REFERENCE", "FORGE_DEG_CORRECTED"]
