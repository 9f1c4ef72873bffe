"""Generates tests/golden/oracle_cfg1_fixed_point.npz: the oracle's converged SCF state on the
(10, 11) bilayer (N = 1324, 12 x 12 k grid, nu = +2, eps = 10, corrected DegFactor), the workload
of the mixed-precision accuracy claims.

The oracle runs the plain guess and Anderson / Pulay mixing (depth 6, beta 0.7, the library's
FORGE_MIX_PULAY restated) until the mean-field residual is below 1e-10 eV, and keeps what a GPU run
can be compared with without the 112 MB density matrix: the energies, the window bands and Fermi
level, the site densities and potential, P(R) on the short bonds (|r_i - r_j + R| < 1.6 a), and the
order parameters.  About 20 minutes on 8 cores.  Run from the repository root:

    python tests/golden/make_cfg1_fixed_point.py
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import forge_oracle as fo  # noqa: E402

BOND_CUTOFF = 1.6


def short_bonds(g: fo.Geometry, cutoff: float = BOND_CUTOFF) -> np.ndarray:
    """(i, j, c) with |r_i - (r_j - R_c)| < cutoff (in the xy plane), c = 0..3."""
    X = np.asarray(g.coords)
    t1, t2 = np.asarray(g.t1), np.asarray(g.t2)
    out = []
    for c in range(4):
        R = g.ucell1[c] * t1 + g.ucell2[c] * t2
        d2 = ((X[:, None, :2] - (X[None, :, :2] - R[None, None, :])) ** 2).sum(-1)
        i, j = np.nonzero(d2 < cutoff ** 2)
        out.append(np.stack([i, j, np.full_like(i, c)], axis=1))
    return np.concatenate(out).astype(np.int64)


def main():
    s = fo.Setup(ntheta=10, numk=12, nfilling=2.0, epsilon=10.0, degfactor_mode="corrected")
    t0 = time.time()
    r = fo.run_scf(s, itmax=60, residual_tol=1e-10, mixer=fo.PulayMixer(6, 0.7))
    g = r["geometry"]
    bonds = short_bonds(g)
    P = r["P"]
    op = fo.order_parameters(s, g, P)
    logs = r["logs"]
    np.savez_compressed(
        os.path.join(HERE, "oracle_cfg1_fixed_point.npz"),
        residuals=np.array([l.residual for l in logs]), E_in=np.array([l.E_in for l in logs]),
        Etot=np.float64(r["Etot"]), energies=np.array([r["E"].kinetic, r["E"].fock, r["E"].hartree, r["E"].hubbard]),
        bands=r["bands"], EF=np.float64(r["EF"]), nocc=np.int64(r["nocc"]), npart=np.int64(r["npart"]),
        dens=r["dens"], V=r["V"], bonds=bonds, P_bonds=P[bonds[:, 2], bonds[:, 0], bonds[:, 1]],
        order=np.array([op[k] for k in sorted(op)]), order_names=np.array(sorted(op)))
    print(f"{len(logs)} iterations, residual {logs[-1].residual:.2e}, E/atom {r['Etot'] / s.ndim:.12f}, "
          f"{time.time() - t0:.0f} s")


if __name__ == "__main__":
    main()
