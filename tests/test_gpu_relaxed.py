"""The SCF on a relaxed bilayer (nrelax = 1, LatticeRelaxation of Geometry.f90:279-1135) against
the oracle: the device path takes the relaxed sites through forge_gpu_init, so the pair tables, the
long-range kernel and every SCF quantity follow them.  (5, 6) bilayer with the reference's table
for ntheta = 5, 3 x 3 k, nu = +2, three ODA iterations; tolerances as in test_gpu_parity.py."""
import os

import numpy as np
import pytest

from oracle import forge_oracle as fo

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_relaxed_bilayer_scf_matches_oracle(lib):
    import forge_gb300 as fg
    d = np.load(os.path.join(GOLDEN, "relaxation_uq.npz"))
    uq = (d["uqx_5"], d["uqy_5"])
    kw = dict(ntheta=5, numk=3, nfilling=2.0, epsilon=10.0, nrelax=1)
    S = fg.Setup(relaxation=uq, **kw)
    so = fo.Setup(relax_uq=uq, **kw)
    ref = fo.run_scf(so, itmax=3)
    assert np.array_equal(fg.build_geometry(S).Coords, ref["geometry"].coords)
    with fg.HartreeFock(S) as hf:
        hf.LongRangeInteraction(copy_out=False)
        E, _ = hf.PlainGuess()
        reps = []
        for _ in range(3):
            rep, E, _ = hf.ScfIteration(E)
            reps.append(rep)
        P, dens, V = hf.GetState()
        bands = hf.GetBands()
    N = so.ndim
    for r, l in zip(reps, ref["logs"]):
        assert abs(r["TotalEnergyIn"] - l.E_in) / N <= 1e-7, (r["TotalEnergyIn"], l.E_in)
        assert (r["nOccStates"], r["nPartOccStates"]) == (l.nocc, l.npart)
    assert np.max(np.abs(np.moveaxis(P, 2, 0) - ref["P"])) <= 1e-8
    assert np.max(np.abs(bands - ref["bands"])) <= 1e-9
    # the relaxation changes the state: the unrelaxed SCF's first energy differs
    ref0 = fo.run_scf(fo.Setup(**{k: v for k, v in kw.items() if k != "nrelax"}), itmax=1)
    assert abs(ref0["logs"][0].E_in - ref["logs"][0].E_in) / N > 1e-6
