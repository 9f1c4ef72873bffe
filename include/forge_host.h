/*
 * forge_host.h -- host side of the GB300 Hartree-Fock engine (the part of FORGE's
 * Fortran driver that stays on the CPU: Setup.f90, Geometry.f90 and the SCF control
 * of Main.f90), in C++ because no Fortran compiler is available for this build.
 * A Fortran host keeps its own Setup/Geometry/Main and binds only forge_gpu.h.
 */
#ifndef FORGE_HOST_H
#define FORGE_HOST_H

#include <stdint.h>

#include "forge_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Setup.f90:6-69: fills the derived fields (ndim, numb, nLower, nUpper, NeutralityPoint,
 * numNeighborCells, alpha, alphaH, a0, r0, d0, tz) from the primary ones already set in *s
 * (nlayers, ntheta, numk, numS, numI, numC, nscreen, fphase, nfilling, U, epsilon, Delta, xi,
 * EnergyTolerance, StepAlternative, degfactor_mode, precision). */
int forge_host_setup(forge_setup* s);

/* Main.f90:102-163 with Geometry.f90:14-273 and 1140-1223.  Output arrays (column-major):
 * Coords (ndim x 3), nUnitCell_1/2 (4), tn (2 x 3: t1, t2, t3), g1 (2), g12 (2),
 * MomentaValues (numk x numk x 2), nMomentaComponents (Nk x 2), nMomentaFlattened (numk x numk),
 * nC2pairs / nC3pairs (ndim, 1-based) and the two site-map counts (may be NULL). */
int forge_host_geometry(const forge_setup* s, const int64_t* RotateLayers, double* Coords, int64_t* nUnitCell_1,
                        int64_t* nUnitCell_2, double* tn, double* g1, double* g12, double* MomentaValues,
                        int64_t* nMomentaComponents, int64_t* nMomentaFlattened, int64_t* nC2pairs,
                        int64_t* nC3pairs, int64_t* counts);

/* LatticeRelaxation (Geometry.f90:279-1135), called by Main.f90:156-160 for nrelax = 1 and bilayers,
 * between the rotation of the sites and the C2 / C3 maps.  Coords (ndim x 3, column-major, the
 * rotated sites of forge_host_geometry) is updated in place: layer 1 moves by half the displacement
 * field sum of the 30 Fourier terms built from g1, g12 and the tables uqx, uqy (5 x 5, column-major:
 * uqx[(n-1) + 5*(m-1)] = uqx(n, m); the reference hard-codes one table per ntheta = 2..35 at
 * Geometry.f90:305-1056 and leaves other ntheta at zero), layer 2 becomes its x-mirror, re-indexed
 * onto the unrelaxed layer-2 sites.  matched (2, may be NULL) receives the two layer-2 quarter counts.
 * FORGE_ERR_ARG when nlayers != 2, or when a count is not ndim/4 (the reference's ERROR RELAXATION;
 * the unmatched sites are then NaN, where the reference leaves them undefined). */
int forge_host_lattice_relaxation(const forge_setup* s, double* Coords, const double* g1, const double* g12,
                                  const double* uqx, const double* uqy, int64_t* matched);

/* C2_RelatedPoints / C3_RelatedPoints (Geometry.f90:1140-1223) of the given sites: the 1-based maps
 * nC2pairs / nC3pairs (ndim, may be NULL) and the two match counts (may be NULL).  Run after
 * forge_host_lattice_relaxation, as Main.f90:162-163 does. */
int forge_host_site_maps(const forge_setup* s, const double* Coords, int64_t* nC2pairs, int64_t* nC3pairs,
                         int64_t* counts);

typedef struct forge_scf_options {
    int64_t itmax;              /* Setup.f90:53 */
    double residual_tol;        /* > 0: stop once the mean-field residual is below it (eV) */
    int64_t mixed_until;        /* iterations run with FORGE_PREC_MIXED before switching to FP64 (0 = never) */
    double mixed_switch_tol;    /* > 0: switch to FP64 once the residual is below this (eV) */
    const char* output_dir;     /* NULL: no Energy / Convergence / Bands files */
    const char* statename;      /* label of the solution (Setup.f90:15), NULL = "SSS" */
    const int64_t* nMomentaFlattened; /* with g1, g12: enables the Bands file (Main.f90:601-610) */
    const double* g1;
    const double* g12;
} forge_scf_options;

typedef struct forge_scf_result {
    int64_t iterations;
    int64_t converged;
    double TotalEnergy;
    double Energies[4];         /* Kinetic, Fock, Hartree, Hubbard of the final state */
    double residual;
    double seconds;             /* wall time of the SCF loop (after the initial guess) */
    double guess_seconds;       /* wall time of the initial guess */
} forge_scf_result;

/* Main.f90:236-679 (numS = 1): initial guess (plain, or zFock_init when not NULL), energies,
 * potential, then the SCF loop with ODA mixing.  reports (may be NULL) receives one entry per
 * iteration (capacity opts->itmax). */
int forge_host_run_scf(forge_ctx* ctx, const forge_scf_options* opts, const double* zFock_init,
                       forge_scf_result* result, forge_iter_report* reports);

/* SortEnergies_2Spins (HartreeFock.f90:929-1004), same arguments: WindowSort_2Spins is the 2 x 2
 * column-major window table W(i, spin), SortedEnergies_1Spin the (numb*Nk) x 2 column-major per-spin
 * sorted energies (forge_gpu_sort_energies of each spin), SortedEnergies_2Spins the (2*numb*Nk) x 2
 * output: the merged energies, then the spin label of each (1.0 or 2.0).  The first (W(1,sp)-1)*Nk
 * states of each spin are copied in front, the states up to Nk*(W(2,sp)-1) are merged, the tails are
 * appended spin 1 first; as in the reference, the spin-2 front block repeats the spin-2 energy at
 * position (W(1,1)-1)*Nk+1.  FORGE_ERR_ARG when a window lies outside 1..numb+1. */
int forge_host_sort_energies_2spins(int64_t numk, int64_t numb, const int64_t* WindowSort_2Spins,
                                    const double* SortedEnergies_1Spin, double* SortedEnergies_2Spins);

/* Main.f90:416-453 (numS = 2): nWindowSort_2Spins = (NP-1, NP+3) for both spins, the merge above,
 * nFermiLevel = 2*nint(Nk*NP + Nk/2*nfilling), FermiEnergy between merged states nFermiLevel and
 * nFermiLevel+1, nOccStates(2) / nPartOccStates(2) counted per spin label, and DegFactor over both
 * spins (0 when no state is partially occupied).  SortedEnergies_2Spins may be NULL. */
int forge_host_fermi_2spins(const forge_setup* s, const double* SortedEnergies_1Spin, double* SortedEnergies_2Spins,
                            int64_t* nFermiLevel, double* FermiEnergy, int64_t* nOccStates, int64_t* nPartOccStates,
                            double* DegFactor);

/* PlotBands (TightBinding.f90:275-369): writes Bands(numb, Nk) - FermiEnergy along the
 * K - Gamma - M - K path of k-grid points to the file `path` (the reference's unit 99). */
int forge_host_plot_bands(const forge_setup* s, const double* Bands, double FermiEnergy,
                          const int64_t* nMomentaFlattened, const double* g1, const double* g12, const char* path);

/* Fock checkpoint files (Main.f90:647-672 write, Main.f90:202-234 read): a direct-access
 * unformatted file of one complex(dp) value per record: R = 0 as the lower triangle row by row
 * (for i: for j <= i: zFock(i, j, 1)), then each cell m = 2..numNeighborCells in full, row by row
 * (for i: for j: zFock(i, j, m)).  Reading restores the upper triangle of R = 0 as the conjugate.
 * record_bytes is the record length: 16 for recl = 2*dp in bytes (gfortran), 64 for ifort's default
 * 4-byte record units; the value sits at the start of each record.  zFock is ndim x ndim x
 * numNeighborCells complex, column-major.  The file name the reference uses is
 * dataFock/Fock-nspin1 followed by forge_host_parameters_string. */
int forge_host_write_fock(const forge_setup* s, const double* zFock, const char* path, int64_t record_bytes);
int forge_host_read_fock(const forge_setup* s, double* zFock, const char* path, int64_t record_bytes);

/* The parameter string of Main.f90:180-183 used in output file names (nrelax 0); the _relax form
 * takes Setup.f90:12's nrelax (0..9). */
int forge_host_parameters_string(const forge_setup* s, const char* statename, char* buf, int64_t buflen);
int forge_host_parameters_string_relax(const forge_setup* s, const char* statename, int64_t nrelax, char* buf,
                                       int64_t buflen);

#ifdef __cplusplus
}
#endif
#endif /* FORGE_HOST_H */
