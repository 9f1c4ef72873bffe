"""Learned warm start: the MLP kernels' gradients against the FP64 CPU oracle, training reduces
the loss, and the trained network starts the SCF closer to convergence than the plain guess."""
import numpy as np
import pytest

from oracle import mlp_oracle

pytestmark = pytest.mark.gpu


def test_mlp_forward_and_gradient_match_oracle(lib):
    from forge_gb300.warmstart import Mlp
    rng = np.random.default_rng(0)
    din, dout, n = 12, 2, 300
    net = Mlp(din, dout, seed=3)
    X = rng.standard_normal((n, din)).astype(np.float32)
    T = rng.standard_normal((n, dout)).astype(np.float32)
    p = net.params(bf16=True).astype(np.float64)
    y_ref, _ = mlp_oracle.forward(p, X.astype(np.float64), din, dout)
    y = net.forward(X)
    assert np.max(np.abs(y - y_ref)) <= 1e-4 * (1 + np.max(np.abs(y_ref)))
    G, loss = net.gradient(X, T)
    loss_ref, G_ref = mlp_oracle.loss_and_grad(p, X, T, np.ones(dout), din, dout)
    assert abs(loss - loss_ref) <= 1e-4 * loss_ref
    assert np.linalg.norm(G - G_ref) <= 1e-4 * np.linalg.norm(G_ref)
    net.close()


def test_mlp_training_reduces_loss(lib):
    from forge_gb300.warmstart import Mlp
    rng = np.random.default_rng(1)
    X = rng.standard_normal((4096, 6)).astype(np.float32)
    T = np.stack([np.sin(X[:, 0]) * X[:, 1], np.cos(X[:, 2] + X[:, 3])], axis=1).astype(np.float32)
    net = Mlp(6, 2, seed=1)
    _, l0 = net.gradient(X, T)
    l1 = net.train(X, T, epochs=30, batch=256, lr=2e-3, seed=0)
    assert l1 < 0.2 * l0
    net.close()


def _converged_state(m, nu, numk=3):
    import forge_gb300 as fg
    S = fg.Setup(ntheta=m, numk=numk, nfilling=nu)
    hf = fg.HartreeFock(S)
    hf.LongRangeInteraction(copy_out=False)
    res, reps = hf.RunScf(itmax=80, residual_tol=1e-7)
    P, dens, V = hf.GetState()
    return S, hf, P, dens, reps


def test_warm_start_beats_plain_guess(lib):
    import forge_gb300 as fg
    from forge_gb300 import warmstart as wsm
    samples = []
    for m, nu in ((3, 2.0), (4, 2.0), (4, 0.0), (3, -2.0)):
        S, hf, P, dens, _ = _converged_state(m, nu)
        samples.append(wsm.training_samples(S, hf.geometry, P, dens))
        hf.close()
    ws = wsm.WarmStart(seed=0)
    ws.fit(samples, epochs=60, lr=2e-3)
    # unseen cell: m = 5 at nu = +2
    S = fg.Setup(ntheta=5, numk=3, nfilling=2.0)
    counts = {}
    for mode in ("plain", "warm"):
        with fg.HartreeFock(S) as hf:
            hf.LongRangeInteraction(copy_out=False)
            if mode == "plain":
                E, _ = hf.PlainGuess()
            else:
                E = wsm.apply(hf, S, ws)
                r_ws, r_zero = hf.warm_start_residuals
                assert r_ws < r_zero, (r_ws, r_zero)
            n = 0
            res = 1.0
            while res > 1e-6 and n < 80:
                rep, E, _ = hf.ScfIteration(E)
                res = rep["residual"]
                n += 1
            counts[mode] = n
    assert counts["warm"] < counts["plain"], counts


def test_shipped_warm_start_on_the_10_11_bilayer(lib):
    """The shipped network (trained on the m = 8, 12, 16 bilayers and the m = 12 trilayer) on the
    (10, 11) bilayer at nu = +2, eps = 10 (N = 1324, 12 x 12 k): the mixed-precision SCF with the
    eigenpair refinement and Pulay mixing reaches 1e-7 eV from the warm start in no more iterations
    than from the plain guess (measured on GB300: 7 and 7, no gain at this size), and both runs end
    on the same state.  The gain of a network trained on related cells is shown on the m = 5 cell by
    test_warm_start_beats_plain_guess."""
    import forge_gb300 as fg
    from forge_gb300 import warmstart as wsm
    S = fg.Setup(ntheta=10, numk=12, nfilling=2.0, epsilon=10.0, degfactor_mode="corrected", precision="mixed")
    out = {}
    for mode in ("plain", "warm"):
        with fg.HartreeFock(S) as hf:
            hf.LongRangeInteraction(copy_out=False)
            hf.set_mixing("pulay", 6, 0.7)
            hf.set_eigen_refinement(2, 1e-4)
            if mode == "plain":
                E, _ = hf.PlainGuess()
            else:
                E = wsm.apply(hf, S)
                assert hf.warm_start_used, hf.warm_start_residuals
            n, rep = 0, {"residual": 1.0}
            while rep["residual"] > 1e-7 and n < 40:
                rep, E, _ = hf.ScfIteration(E)
                n += 1
            P, dens, V = hf.GetState()
            out[mode] = dict(n=n, res=rep["residual"], E=rep["TotalEnergy"], dens=dens)
    assert out["plain"]["res"] <= 1e-7 and out["warm"]["res"] <= 1e-7, out
    assert out["warm"]["n"] <= out["plain"]["n"], {k: v["n"] for k, v in out.items()}
    assert abs(out["warm"]["E"] - out["plain"]["E"]) / 1324 <= 1e-7
    assert np.max(np.abs(out["warm"]["dens"] - out["plain"]["dens"])) <= 1e-7
