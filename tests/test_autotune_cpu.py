"""The autotuners' host logic on a fake solver (no GPU): every candidate is timed, the fastest is
applied, the state is restored, and a stored choice is reused without timing."""
import json

import numpy as np

from festung_gb300 import _lib as L
from festung_gb300 import autotune as AT


class FakeSolver:
    """Records the calls the tuners make; a launch option's cost comes from `cost`."""

    K, p, limiter = 128, 2, 'linear'

    def __init__(self, cost):
        self.cost = cost
        self.options = {L.OPT_FLAGS: 0, L.OPT_GRAPH_STEPS: 12, L.OPT_ADJ_WARPS: 2, L.OPT_OP_BLOCK: 128,
                        L.OPT_TAYLOR_MASS: 1, L.OPT_ADJ_GRAPH: 1, L.OPT_ADJ_STREAMS: 3}
        self.state = np.arange(12.0).reshape(4, 3)
        self.calls = []

    def set_option(self, option, value):
        self.options[option] = value

    def get_option(self, option):
        return self.options[option]

    def get_state(self):
        return self.state.copy()

    def set_state(self, c):
        self.state = np.array(c, copy=True)

    def time_steps(self, nSteps, nStep0, tau):
        self.calls.append(('steps', self.options[L.OPT_FLAGS], self.options[L.OPT_GRAPH_STEPS]))
        self.state = self.state + 1.0   # the tuner must put the state back
        return nSteps * self.cost(self.options)

    def forward_record(self, nSteps, tau, nSnapshots):
        self.calls.append(('record', self.options[L.OPT_ADJ_WARPS], nSnapshots))
        self.state = self.state + 1.0

    def backward(self, g):
        self.calls.append(('backward', self.options[L.OPT_ADJ_WARPS]))
        _now[0] += 1e-3 * self.cost(self.options)   # the tuner's (fake) wall clock sees the cost
        return np.zeros_like(g), None


_now = [0.0]


def test_tune_adjoint_times_every_width_and_applies_the_fastest(monkeypatch):
    _now[0] = 0.0
    monkeypatch.setattr(AT.time, 'perf_counter', lambda: _now[0])
    costs = {1: 3.0, 2: 1.0, 4: 5.0}
    # the sweep launched directly (adjGraph 0) is faster here, and three streams
    s = FakeSolver(lambda o: costs[o[L.OPT_ADJ_WARPS]] * (0.5 if o[L.OPT_ADJ_GRAPH] == 0 else 1.0)
                   * (1.0 if o[L.OPT_ADJ_STREAMS] == 3 else 1.5))
    before = s.get_state()
    best, table = AT.tune_adjoint(s, 1e-3, nSteps=4, nSnapshots=2, reps=2)
    assert [r['adjWarps'] for r in table if 'adjGraph' not in r] == [1, 2, 4]
    assert best['adjWarps'] == 2 and s.get_option(L.OPT_ADJ_WARPS) == 2
    # then the other sweep form on the best width, then the other stream counts (no faster here)
    assert table[-3]['adjWarps'] == 2 and table[-3]['adjGraph'] == 0
    assert abs(table[-3]['ms_backward'] - 0.5) < 1e-9
    assert best['adjGraph'] == 0 and s.get_option(L.OPT_ADJ_GRAPH) == 0
    assert [r['adjStreams'] for r in table[-2:]] == [1, 2]
    assert best['adjStreams'] == 3 and s.get_option(L.OPT_ADJ_STREAMS) == 3
    assert np.array_equal(s.get_state(), before)
    # every width: reps + 1 recorded runs (the first captures the sweep's graph), each with the
    # requested snapshots, and a backward after each; the best width four times (both sweep
    # forms, then the two other stream counts)
    for w in (1, 2, 4):
        n = 12 if w == 2 else 3
        assert s.calls.count(('record', w, 2)) == n
        assert s.calls.count(('backward', w)) == n


def test_tune_picks_the_fastest_launch_configuration_and_caches_it(tmp_path):
    def cost(o):
        return (1.0 + (0.5 if o[L.OPT_FLAGS] & L.FLAG_NO_PDL else 0.0) + abs(o[L.OPT_GRAPH_STEPS] - 24) / 100
                + (0.1 if o[L.OPT_OP_BLOCK] == 128 else 0.0) + 0.05 * o[L.OPT_TAYLOR_MASS])

    s = FakeSolver(cost)
    before = s.get_state()
    cache = str(tmp_path / 'tune.json')
    best, table = AT.tune(s, 1e-3, nSteps=8, reps=2, fused_ok=True, cache=cache, key='k')
    # separate passes: every operator block size; the fused pipeline: its one kernel shape; then
    # the other Taylor mass correction once on the best of those
    assert len(table) == 2 * len(AT.GRAPH_STEPS) * len(AT.OP_BLOCKS) + 2 * len(AT.GRAPH_STEPS) + 1
    assert best['graphSteps'] == 24 and not best['flags'] & L.FLAG_NO_PDL and best['opBlock'] == 64
    assert s.get_option(L.OPT_GRAPH_STEPS) == 24 and s.get_option(L.OPT_OP_BLOCK) == 64
    assert best['taylorMass'] == 0 and s.get_option(L.OPT_TAYLOR_MASS) == 0
    assert np.array_equal(s.get_state(), before)
    stored = json.load(open(cache))
    assert stored['k']['best']['graphSteps'] == 24
    # a second call with the same key applies the stored choice without timing anything
    s2 = FakeSolver(cost)
    best2, _ = AT.tune(s2, 1e-3, cache=cache, key='k')
    assert best2 == stored['k']['best'] and s2.calls == []
    assert s2.get_option(L.OPT_GRAPH_STEPS) == 24
