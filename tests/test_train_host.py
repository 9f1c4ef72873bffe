"""Host logic of the warm-start training driver (forge_gb300.train_warmstart), without a GPU: the
batched convergence loop only iterates the systems above the tolerance, stops at its deadline, and
the sample collection caches each converged system so that a later run converges only the rest."""
import json
import os

import numpy as np

from forge_gb300 import train_warmstart as tw

SYSTEMS = [(8, 2, 6, 2.0, 10.0), (8, 2, 6, 0.0, 10.0), (12, 2, 6, 2.0, 10.0), (16, 2, 4, 2.0, 10.0)]


class _Ctx:
    """A context whose residual drops tenfold per iteration from 10^-(m/8)."""

    def __init__(self, S):
        self.m = S.ntheta
        self.n = 0
        self.closed = False

    def close(self):
        self.closed = True


def _open(S):
    return _Ctx(S), (1.0, 2.0, 3.0, 4.0)


class _Group:
    def __init__(self):
        self.calls = []

    def __call__(self, ctxs, E):
        self.calls.append(len(ctxs))
        reps = []
        for c in ctxs:
            c.n += 1
            reps.append({"residual": 10.0 ** (-(c.m / 8.0) - c.n)})
        return reps, E + 1.0, 0


class _Clock:
    def __init__(self, step):
        self.t, self.step = 0.0, step

    def __call__(self):
        self.t += self.step
        return self.t


def test_converge_group_iterates_only_the_systems_above_tolerance():
    grp = _Group()
    out = tw.converge_group(SYSTEMS, tol=1e-5, open_context=_open, group_iteration=grp)
    iters = [n for _, _, n, _ in out]
    # 10^-(m/8 + n) <= 1e-5: m = 8 -> n = 4, m = 12 -> 4 (1.5 + 4 > 5), m = 16 -> 3
    assert iters == [4, 4, 4, 3]
    assert all(res <= 1e-5 for _, _, _, res in out)
    assert grp.calls == [4, 4, 4, 3]        # the converged m = 16 system leaves the batch
    assert [S.ntheta for S, _, _, _ in out] == [8, 8, 12, 16]


def test_converge_group_stops_at_its_deadline():
    grp = _Group()
    clock = _Clock(1.0)
    out = tw.converge_group(SYSTEMS, tol=1e-5, open_context=_open, group_iteration=grp, deadline=2.5, clock=clock)
    assert grp.calls == [4, 4]              # clock reads 1, 2 start iterations; 3 is past the deadline
    assert all(res > 1e-5 for _, _, _, res in out)


def test_collect_samples_caches_and_resumes(tmp_path):
    cache = str(tmp_path / "cache")
    sampled = []

    def sample(S, hf):
        sampled.append(S.ntheta)
        k = S.ntheta
        return (np.full((k, 2), k, np.float32), np.full((k, 1), k, np.float32), np.zeros((1, 3), np.float32),
                np.zeros((1, 2), np.float32))

    lines = []

    def conv(group, tol, degfactor, deadline):
        return tw.converge_group(group, tol=tol, degfactor=degfactor, deadline=deadline, open_context=_open,
                                 group_iteration=_Group(), clock=lambda: 0.0)

    # first run: the budget allows the first group of two systems only
    clock = _Clock(1.0)
    got = tw.collect_samples(SYSTEMS, cache=cache, group_size=2, budget_s=1.5, converge=conv, sample=sample,
                             clock=clock, log=lines.append)
    assert [int(s[0][0, 0]) for s in got] == [8, 8]
    assert sorted(os.listdir(cache)) == sorted(tw.cache_name(s) for s in SYSTEMS[:2])
    assert all(json.loads(l)["used"] for l in lines)
    # second run: the cached systems are loaded, the other two converge, the order is the systems'
    sampled.clear()
    got = tw.collect_samples(SYSTEMS, cache=cache, group_size=2, converge=conv, sample=sample, log=lines.append)
    assert sampled == [12, 16]
    assert [int(s[0][0, 0]) for s in got] == [8, 8, 12, 16]
    assert len(os.listdir(cache)) == 4
