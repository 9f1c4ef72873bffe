"""Linear mixing (FORGE_MIX_LINEAR, the benchmark description's "linear mixing 0.3"; the reference
mixes with OptimalStep only) on the GPU against the oracle's run_scf(linear_beta=0.3): the (5, 6)
bilayer, 6 x 6 k grid, charge neutrality, eps = 10, ten iterations from the plain guess; E/atom
1e-7 eV per iteration, DensityConvergence 1e-8, occupation counts exact, P(R) 1e-8, every Step
exactly 0.3.  Collected last: it takes the oracle about a minute."""
import numpy as np
import pytest

from oracle import forge_oracle as fo

pytestmark = pytest.mark.gpu


def test_m5_bilayer_linear_mixing_matches_oracle(lib):
    import forge_gb300 as fg
    kw = dict(ntheta=5, numk=6, nfilling=0.0, epsilon=10.0)
    S = fg.Setup(**kw)
    so = fo.Setup(**kw)
    with fg.HartreeFock(S) as hf:
        hf.LongRangeInteraction(copy_out=False)
        hf.set_mixing("linear", beta=0.3)
        E, _ = hf.PlainGuess()
        reps = []
        for _ in range(10):
            rep, E, _ = hf.ScfIteration(E)
            reps.append(rep)
        P, dens, V = hf.GetState()
    ref = fo.run_scf(so, itmax=10, linear_beta=0.3)
    N = so.ndim
    assert len(reps) == len(ref["logs"]) == 10
    for r, l in zip(reps, ref["logs"]):
        assert r["Step"] == 0.3
        assert abs(r["TotalEnergyIn"] - l.E_in) / N <= 1e-7, (r["TotalEnergyIn"], l.E_in)
        assert abs(r["DensityConvergence"] - l.dn_max) <= 1e-8
        assert (r["nOccStates"], r["nPartOccStates"]) == (l.nocc, l.npart)
    assert np.max(np.abs(np.moveaxis(P, 2, 0) - ref["P"])) <= 1e-8
