"""Host logic of the learned warm start (forge_gb300.warmstart.apply), without a GPU.

The fallback rule of the learned start: the network's field is used only if its first residual beats
the plain guess's, and the plain guess is the fallback otherwise.  A network that outputs NaN / Inf, or a
residual comparison that is undefined (NaN), must also fall back, and the device must never see a
non-finite field.  The device calls are replaced by a recording fake.
"""
import numpy as np
import pytest


class _FakeLib:
    def __init__(self, residuals):
        self.residuals = residuals
        self.field_calls = 0

    def forge_gpu_field_guess(self, ctx, P, E, res):
        import ctypes as C
        self.field_calls += 1
        r = np.ctypeslib.as_array(C.cast(res, C.POINTER(C.c_double)), shape=(2,))
        r[:] = self.residuals
        e = np.ctypeslib.as_array(C.cast(E, C.POINTER(C.c_double)), shape=(4,))
        e[:] = (1.0, 2.0, 3.0, 4.0)
        return 0


class _FakeHF:
    def __init__(self, residuals, N=8):
        self.N = N
        self.setup = None
        self.geometry = None
        self.ctx = None
        self.lib = _FakeLib(residuals)
        self.plain_calls = 0

    def PlainGuess(self):
        self.plain_calls += 1
        return (9.0, 9.0, 9.0, 9.0), 0


class _FakeNet:
    def __init__(self, N, bad=False):
        self.N, self.bad = N, bad

    def predict(self, setup, geo):
        dn = np.zeros(self.N)
        if self.bad:
            dn[3] = np.nan
        bonds = np.array([[0, 1, 0], [1, 0, 0]], dtype=np.int64)
        return dn, bonds, np.array([[0.1, 0.0], [0.1, 0.0]])


@pytest.mark.parametrize("residuals,bad,used", [((0.1, 0.2), False, True),     # network better: used
                                                ((0.3, 0.2), False, False),    # worse: plain guess
                                                ((np.nan, 0.2), False, False),  # undefined: plain guess
                                                ((0.1, 0.2), True, False)])    # NaN field: never uploaded
def test_warm_start_falls_back_to_the_plain_guess(residuals, bad, used):
    from forge_gb300 import warmstart
    hf = _FakeHF(residuals)
    E = warmstart.apply(hf, None, ws=_FakeNet(hf.N, bad))
    assert hf.warm_start_used is used
    assert hf.plain_calls == (0 if used else 1)
    assert hf.lib.field_calls == (0 if bad else 1)
    assert E == ((1.0, 2.0, 3.0, 4.0) if used else (9.0, 9.0, 9.0, 9.0))
