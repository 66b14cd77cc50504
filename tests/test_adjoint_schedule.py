"""The backward schedule of the differentiable rollout (shamrock_gb300.adjoint), on CPU
with a stand-in library: each checkpoint segment is recorded once, step by step on one
context per step of the segment, each step starting from the state the previous step's
context holds after its step, and then reversed from the last step to the first on the
context that recorded it, with the same start state and precision tier."""

import ctypes as C

import pytest
import torch

from shamrock_gb300 import _lib as L
from shamrock_gb300 import adjoint


class _FakeLib:
    def __init__(self, log):
        self.log = log
        self.next_id = 1000

    def gbsph_adjoint_record(self, handle, start, cfg, t, dt, kk, after, stream):
        self.next_id += 1
        after._obj.n = self.next_id  # marks the state this context holds after its step
        self.log.append(("record", handle, start._obj.n, cfg._obj.precision, t, dt, kk,
                         self.next_id))
        return 0

    def gbsph_adjoint_reverse(self, handle, start, cfg, dt, cot, g, stream):
        self.log.append(("reverse", handle, start._obj.n, cfg._obj.precision, dt))
        g._obj.value = 1.0
        return 0


class _FakeContext:
    made = []

    def __init__(self, device=0):
        self.handle = len(_FakeContext.made)
        self.lib = _FakeContext.lib
        _FakeContext.made.append(self)

    def check(self, rc):
        assert rc == 0
        return rc


class _FakeModel:
    def __init__(self):
        class _Dev:
            device = 0

        self._dev = _Dev()

    def _lib(self):
        return self._dev

    def _config_struct(self, tier):
        c = L.Config()
        c.precision = tier
        return c


def _checkpoint(n, marker):
    snap = {k: torch.zeros(3, n, dtype=torch.float64) for k in ("xyz", "vxyz", "axyz")}
    snap.update({k: torch.zeros(n, dtype=torch.float64) for k in ("hpart", "uint", "duint")})
    snap["marker"] = marker
    return snap


@pytest.mark.parametrize("n_steps,k", [(7, 3), (6, 3), (4, 1), (5, 5)])
def test_segments_recorded_once_and_reversed(monkeypatch, n_steps, k):
    log = []
    _FakeContext.made = []
    _FakeContext.lib = _FakeLib(log)
    monkeypatch.setattr(adjoint.L, "Context", _FakeContext)
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **kw: None)
    # a checkpoint's Particles struct carries its step index in n (the rows are unused)
    real_particles_of = adjoint._particles_of

    def particles_of(snap):
        p = real_particles_of(snap)
        p.n = snap["marker"]
        return p

    monkeypatch.setattr(adjoint, "_particles_of", particles_of)
    m = _FakeModel()
    r = adjoint._Rollout(m, n_steps, k)
    r.records = [(0.1 * j, 0.01 * (j + 1), 1 + j % 2, j % 3) for j in range(n_steps)]
    r.checkpoints = {j: _checkpoint(2, j) for j in range(0, n_steps, k)}
    cot = adjoint._zero_cot(2, "cpu")
    g = r.backward(cot)
    assert g == n_steps  # one unit per reversed step
    assert len(_FakeContext.made) == k  # one context per step of a segment, made once
    # replay the expected schedule
    i = 0
    for s0 in reversed(range(0, n_steps, k)):
        s1 = min(s0 + k, n_steps)
        held = {}
        start = s0  # the checkpoint's marker
        for j in range(s0, s1):
            op, handle, st, prec, t, dt, kk, after = log[i]
            assert op == "record" and handle == j - s0 and st == start
            assert (t, dt, kk, prec) == r.records[j][:3] + (r.records[j][3],)
            held[j] = start
            start = after
            i += 1
        for j in reversed(range(s0, s1)):
            op, handle, st, prec, dt = log[i]
            assert op == "reverse" and handle == j - s0 and st == held[j]
            assert prec == r.records[j][3] and dt == r.records[j][1]
            i += 1
    assert i == len(log)


def test_large_segments_use_one_context(monkeypatch):
    """Past MAX_POOLED_PARTICLES particles times steps per segment the backward pass keeps
    to the model's own context."""
    called = []
    monkeypatch.setattr(adjoint._Rollout, "_backward_one_context", lambda self, cot: called.append("one") or 0.0)
    monkeypatch.setattr(adjoint._Rollout, "_backward_pooled", lambda self, cot: called.append("pool") or 0.0)
    r = adjoint._Rollout(_FakeModel(), 10, 5)
    cot = adjoint._zero_cot(8, "cpu")
    monkeypatch.setattr(adjoint, "MAX_POOLED_PARTICLES", 40)
    r.backward(cot)
    monkeypatch.setattr(adjoint, "MAX_POOLED_PARTICLES", 39)
    r.backward(cot)
    r1 = adjoint._Rollout(_FakeModel(), 10, 1)  # one step per segment: one context anyway
    r1.backward(cot)
    assert called == ["pool", "one", "pool"]
