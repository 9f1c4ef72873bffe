"""Spin-polarised SCF (numS = 2) on two device contexts, one per spin.

Main.f90:236-679 with numS = 2; the C3, valley and symmetry switches of the Setup act in each spin's
context as in the numS = 1 path.  Each spin has its own context.  That
context holds the spin's density matrix, solves H(k) with the spin's potential, and forms the
spin's new density matrix.  These are the per-spin routines of the numS = 1 path, unchanged.  The
host joins the spins:
- it merges the two sorted band lists and sets one Fermi level (forge_host_fermi_2spins);
- it sums the kinetic and Fock energies over the spins;
- it evaluates the Hartree and Hubbard terms from both densities;
- it takes one OptimalStep for both spins;
- it builds each spin's potential from both densities (Main.f90:586-594).

The two spins' eigen-solves share one batched launch sequence (forge_gpu_solve_group over the two
contexts).  The density matrices stay on the device: each spin's context returns the energy forms
of its (P_in, P_new) pair (forge_gpu_energy_forms), from which the host evaluates OptimalStep's
three spin-summed energies, and mixes in place with the common step.  Per iteration only site
densities, potentials, band energies and a few scalars cross the host boundary.

Arrays follow the reference: zFock(ndim, ndim, numNeighborCells) per spin, column-major.
"""
from __future__ import annotations

import dataclasses
from typing import Optional, Sequence

import numpy as np

import os

from .api import (Geometry, HartreeFock, Setup, SolveGroup, build_geometry, fermi_2spins, parameters_string,
                  plot_bands, read_fock, write_fock)


@dataclasses.dataclass
class SpinIteration:
    """One line of the Convergence / Energy output of Main.f90:612-625 for numS = 2."""

    it: int
    DensityConvergence: float       # max over spins of max_n |n_new - n_old|
    Step: float
    TotalEnergyIn: float
    TotalEnergy: float
    FermiEnergy: float
    nOccStates: tuple
    nPartOccStates: tuple
    DegFactor: float
    KineticEnergyIn: float = 0.0     # summed over the spins
    FockEnergyIn: float = 0.0        # summed over the spins
    HartreeEnergyIn: float = 0.0
    HubbardEnergyIn: float = 0.0


def hartree_hubbard(LR: np.ndarray, dens: Sequence[np.ndarray]) -> tuple:
    """GetHartreeHubbardEnergy (HartreeFock.f90:1066-1092) with dens1 = n_1 - 1/2, dens2 = n_2 - 1/2."""
    d1, d2 = dens[0] - 0.5, dens[1] - 0.5
    sm = d1 + d2
    return 0.5 * float(sm @ (LR @ sm)), float(np.dot(d1, d2))


def potentials(LR: np.ndarray, dens: Sequence[np.ndarray], alphaH: float, U: float) -> list:
    """Main.f90:331-341 / 586-594: V_1 = alphaH LR (n_1 + n_2 - 1) + U (n_2 - 1/2), V_2 with U (n_1 - 1/2)."""
    h = alphaH * (LR @ (dens[0] + dens[1] - 1.0))
    return [h + U * (dens[1] - 0.5), h + U * (dens[0] - 0.5)]


def density(zFock: np.ndarray) -> np.ndarray:
    """Density(:, spin) = real(zFock(n, n, 1, spin)) (Main.f90:294-298)."""
    return np.ascontiguousarray(np.real(np.diagonal(zFock[:, :, 0])))


class SpinPolarisedScf:
    """Main.f90:236-679 for numS = 2 with ODA mixing.

    ``setup.numS`` must be 2.  ``engines`` are the two per-spin engines.  They default to device
    contexts (``HartreeFock`` of the same setup with numS = 1).  Another object with the same
    methods may stand in, for instance a CPU model of the routines in a test.
    """

    def __init__(self, setup: Setup, geometry: Optional[Geometry] = None, engines: Optional[Sequence] = None):
        if setup.numS != 2:
            raise ValueError("SpinPolarisedScf needs numS = 2")
        self.setup = setup
        self.s = setup.to_struct()
        one = dataclasses.replace(setup, numS=1)
        self.geometry = geometry
        if engines is None:
            if self.geometry is None:
                self.geometry = build_geometry(one)
            engines = [HartreeFock(one, self.geometry), HartreeFock(one, self.geometry)]
            self._own = True
        else:
            self._own = False
        self.hf = list(engines)
        self.LR = np.asarray(self.hf[0].LongRangeInteraction())
        self.hf[1].LongRangeInteraction(copy_out=False)
        self._P = None          # host copies of the state, fetched on demand
        self._have_state = False
        self.dens = None
        self.V = None
        self.E = None

    @property
    def P(self):
        """Both spins' zFock (ndim, ndim, numNeighborCells), copied from the engines."""
        if not self._have_state:
            return None
        if self._P is None:
            self._P = [np.asfortranarray(h.GetState()[0]) for h in self.hf]
        return self._P

    def close(self):
        if self._own:
            for h in self.hf:
                h.close()
        self.hf = []

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def total(self, E: Sequence[float]) -> float:
        """TotalEnergy of Main.f90:312 with the factor 3 - numS = 1."""
        s = self.s
        return s.alpha * E[1] + E[0] + s.U * E[3] + s.alphaH * E[2]

    # -- initial state
    def plain_guess(self):
        """Main.f90:236-292 with numS = 2: the non-interacting spin-1 guess, copied to spin 2."""
        E, info = self.hf[0].PlainGuess()
        P1, _, _ = self.hf[0].GetState()
        self.set_state([P1, P1.copy()])
        return info

    def set_state(self, P: Sequence[np.ndarray]):
        """Loads both spins' zFock and forms their energies and potentials (Main.f90:294-346)."""
        P = [np.asfortranarray(np.asarray(p, dtype=np.complex128)) for p in P]
        for sp in range(2):
            self.hf[sp].SetState(P[sp])
        self._P, self._have_state = P, True
        self.dens = [density(p) for p in P]
        kin = fock = 0.0
        for sp in range(2):
            k, f, _, _ = self.hf[sp].Energies()
            kin += k
            fock += f
        self.E = (kin, fock) + hartree_hubbard(self.LR, self.dens)
        self.V = potentials(self.LR, self.dens, self.s.alphaH, self.s.U)

    def read_state(self, fock_dir: str, setup_in: Optional[Setup] = None, statename_in: str = "SSS",
                   record_bytes: int = 16):
        """Checkpoint resume (nRead = 1, Main.f90:186-234): both spins' zFock from the Fock-nspin files
        of the run described by ``setup_in`` (default: this run's setup); a numS = 1 checkpoint
        (Fock-nspin1) starts both spins."""
        sin = self.setup if setup_in is None else setup_in
        params = parameters_string(sin, statename_in)
        P = [read_fock(self.setup, os.path.join(fock_dir, f"Fock-nspin{1 if sin.numS == 1 else sp + 1}" + params),
                       record_bytes) for sp in range(2)]
        self.set_state(P)

    # -- one SCF iteration (Main.f90:365-595)
    def iterate(self, it: int = 0) -> SpinIteration:
        if not self._have_state:
            raise RuntimeError("no state: call plain_guess() or set_state() first")
        s = self.s
        sorted_e = []
        if all(isinstance(h, HartreeFock) for h in self.hf) and not self.setup.nenforceC3 \
                and not self.setup.nenforceValley:
            # both spins' H(k) in one batched eigen-solve (the device group solve)
            for sp in range(2):
                self.hf[sp].SetPotential(self.V[sp])
            info = SolveGroup(self.hf)
            if np.any(info > 0):
                print("zheev failed", int(np.sum(info)))   # LapackRoutines.f90:430 behaviour
        else:
            for sp in range(2):
                _, _, _, info = self.hf[sp].Solve(self.V[sp], None, bands=False)
                if info > 0:
                    print("zheev failed", info)           # LapackRoutines.f90:430 behaviour
        for sp in range(2):
            e, _, _ = self.hf[sp].SortEnergies_1Spin()
            sorted_e.append(e)
        fl = fermi_2spins(self.setup, np.stack(sorted_e, 1))
        deg = fl["DegFactor"]
        nocc, npart = fl["nOccStates"], fl["nPartOccStates"]
        for sp in range(2):
            self.hf[sp].GetFock(deg, nocc[sp], npart[sp], copy_out=False)
        if self.setup.nenforceT or self.setup.nenforceC2 or self.setup.nenforceC2T:
            # Main.f90:513-534 on each spin's new zFock
            for sp in range(2):
                self.hf[sp].Symmetrize(copy_out=False)
        # OptimalStep (HartreeFock.f90:1148-1227) over the spin-summed energy, from each spin's energy
        # forms of (P_in, P_new): the kinetic energy is linear and the Fock energy quadratic in the step
        forms = [self.hf[sp].EnergyForms() for sp in range(2)]

        def energies_at(t: float) -> tuple:
            u = 1.0 - t
            kin = fock = 0.0
            for f, _, _ in forms:
                kin += u * f[0] + t * f[1]
                fock += -0.5 * (u * u * f[2] + 2.0 * u * t * f[3] + t * t * f[4])
            d = [u * din + t * dnew for _, din, dnew in forms]
            return (kin, fock) + hartree_hubbard(self.LR, d)

        c0 = self.total(self.E)
        t1 = self.total(energies_at(1.0))
        t2 = self.total(energies_at(0.5))
        c1 = 4.0 * t2 - t1 - 3.0 * c0
        c2 = t1 - c0 - c1
        if c2 > 0 and abs(-c1 / 2.0 / c2 - .5) < 0.5:
            step = -c1 / 2.0 / c2
        elif t1 < c0:
            step = 1.0
        else:
            step = s.StepAlternative
        mixed = [self.hf[sp].Mix(step) for sp in range(2)]
        dens = [np.asarray(d) for d, _ in mixed]
        dn = max(float(m) for _, m in mixed)
        E = energies_at(step)[:2] + hartree_hubbard(self.LR, dens)
        Ein = self.E
        self._P = None
        self.dens, self.E = dens, E
        self.V = potentials(self.LR, dens, s.alphaH, s.U)
        return SpinIteration(it, dn, step, self.total(Ein), self.total(E), fl["FermiEnergy"], tuple(nocc),
                             tuple(npart), deg, *Ein)

    def run(self, itmax: int, density_tol: float = 0.0, P_init: Optional[Sequence[np.ndarray]] = None,
            output_dir: Optional[str] = None, fock_dir: Optional[str] = None, statename: str = "SSS") -> list:
        """The SCF loop: itmax iterations (the reference's stop), or fewer once DensityConvergence
        drops below ``density_tol`` (> 0).

        With ``output_dir`` every iteration appends to Energy<parameters> and Convergence<parameters>
        and rewrites Bands-nspin1/2<parameters> (Main.f90:596-639, numS = 2 columns: the energies
        summed over the spins); with ``fock_dir`` it rewrites Fock-nspin1/2<parameters> in the
        reference's record order (Main.f90:645-672)."""
        if P_init is not None:
            self.set_state(P_init)
        elif not self._have_state:
            self.plain_guess()
        params = parameters_string(self.setup, statename) if (output_dir or fock_dir) else ""
        fe = fc = None
        if output_dir:
            fe = open(os.path.join(output_dir, "Energy" + params), "w")
            fc = open(os.path.join(output_dir, "Convergence" + params), "w")
        reports = []
        try:
            for it in range(1, itmax + 1):
                r = self.iterate(it)
                reports.append(r)
                if output_dir:
                    self._write_outputs(r, output_dir, params, fe, fc)
                if fock_dir:
                    for sp in range(2):
                        write_fock(self.setup, self.P[sp], os.path.join(fock_dir, f"Fock-nspin{sp + 1}" + params))
                if density_tol > 0 and r.DensityConvergence < density_tol:
                    break
        finally:
            for f in (fe, fc):
                if f is not None:
                    f.close()
        return reports

    def _write_outputs(self, r: SpinIteration, output_dir: str, params: str, fe, fc):
        g = self.geometry if self.geometry is not None else build_geometry(dataclasses.replace(self.setup, numS=1))
        for sp in range(2):
            plot_bands(self.setup, g, self.hf[sp].GetBands(), r.FermiEnergy,
                       os.path.join(output_dir, f"Bands-nspin{sp + 1}" + params))
        fc.write(f"{float(r.it):5.1f}   {r.DensityConvergence:9.6f}   {r.Step:5.3f}   "
                 f"{r.TotalEnergyIn - r.TotalEnergy:24.9f}   \n")
        fe.write(f"{float(r.it):5.1f}   {r.TotalEnergyIn:24.9f}   {r.KineticEnergyIn:24.9f}   "
                 f"{r.FockEnergyIn:24.9f}   {r.HartreeEnergyIn:24.9f}   {r.HubbardEnergyIn:24.9f}   \n")
        fe.flush()
        fc.flush()
