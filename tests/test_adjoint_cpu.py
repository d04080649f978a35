"""CPU checks of the adjoint's oracle and of the checkpointing schedule (no GPU).

The oracle's gradients (reverse sweep with the transposed assembled operators) must match
central finite differences of its own forward run, and its forward run must be the reference
restatement's run; the checkpointing schedule must reverse every step once, in order, within
its slots, and recompute no step more often than the binomial bound allows.
"""
import math

import numpy as np
import pytest

KW = dict(hmax=2 ** -3, p=2, numSteps=8, tEnd=8 * 2e-4)


@pytest.fixture(scope='module')
def oracle_case():
    from oracle import adjoint as OA
    o = OA.AdjointOracle(**KW)
    o.set_modes(OA.mode_velocities())
    tgt = OA.AdjointOracle(adjointTarget=True, **KW)
    c0 = o.pd.cDisc
    cstar = tgt.forward(c0, KW['numSteps'])
    cT = o.forward(c0, KW['numSteps'])
    g0, gth = o.backward(cT - cstar)
    return o, c0, cstar, g0, gth


def test_oracle_forward_is_the_reference_run(oracle_case):
    from oracle import advection as adv
    o, c0, *_ = oracle_case
    ref = adv.main(testcase='adjoint', **KW)
    assert np.array_equal(o.forward(c0, KW['numSteps']), ref.cDisc)


def test_oracle_gradient_matches_finite_differences(oracle_case):
    o, c0, cstar, g0, gth = oracle_case
    rng = np.random.default_rng(3)
    h = 1e-6
    J = lambda c: 0.5 * float(np.sum((o.forward(c, KW['numSteps']) - cstar) ** 2))
    for _ in range(2):
        d = rng.standard_normal(c0.shape)
        fd = (J(c0 + h * d) - J(c0 - h * d)) / (2 * h)
        assert abs(fd - np.sum(g0 * d)) <= 1e-7 * abs(fd)
    th0 = o.pd.theta.copy()
    for _ in range(2):
        d = rng.standard_normal(th0.size)
        o.set_theta(th0 + h * d)
        Jp = J(c0)
        o.set_theta(th0 - h * d)
        Jm = J(c0)
        fd = (Jp - Jm) / (2 * h)
        assert abs(fd - gth @ d) <= 1e-7 * abs(fd)
    o.set_theta(th0)


def simulate(actions, start, nSteps):
    """Runs the action list: returns the reversed steps, slots used, steps advanced per step.
    The forward phase runs actions[:start] and then carries the state on to the last step."""
    slots = {0: 0}
    reversed_steps, used, advanced = [], {0}, np.zeros(nSteps, dtype=int)
    w = 0
    for i, (op, arg) in enumerate(actions):
        if i == start:
            w = nSteps
        if op == 0:
            w = slots[arg]
        elif op == 1:
            advanced[w:w + arg] += 1
            w += arg
        elif op == 2:
            slots[arg] = w
            used.add(arg)
        else:
            assert i >= start
            assert w == arg, 'reverse step %d with the state of step %d' % (arg, w)
            reversed_steps.append(arg)
            w = arg + 1
    return reversed_steps, used, advanced


@pytest.mark.parametrize('nSteps,nSnap', [(1, 0), (7, 0), (10, 3), (20, 4), (200, 20), (50, 1), (33, 2)])
def test_checkpoint_schedule_reverses_every_step_within_its_slots(lib, nSteps, nSnap):
    from festung_gb300 import _lib as L
    actions, start = L.checkpoint_schedule(nSteps, nSnap)
    rev, used, advanced = simulate(actions, start, nSteps)
    assert rev == list(range(nSteps - 1, -1, -1))
    slots = nSteps if nSnap <= 0 or nSnap >= nSteps else nSnap
    assert max(used) < slots
    # binomial bound: no step advanced more than r times, beta(s, r) = C(s + r, s) >= nSteps
    s = slots - 1
    r = 1
    while s > 0 and math.comb(s + r, s) < nSteps:
        r += 1
    if s > 0:
        assert advanced.max() <= r
    if slots == nSteps:
        assert advanced.max() <= 1      # every state stored once, nothing recomputed


def test_gradient_workload_schedule_recomputes_what_the_cost_model_says(lib):
    """200 steps with 20 slots: the record's checkpointing actions advance 199 steps (the last
    step follows them), and the reverse sweep advances 180 steps, stores 180 checkpoints and
    reverses 200 steps (each of which recomputes two of its three SSP-RK3 stages in the
    unlimited scheme)."""
    from festung_gb300 import _lib as L
    actions, start = L.checkpoint_schedule(200, 20)
    a = np.asarray(actions).reshape(-1, 2)
    fwd, bwd = a[:start], a[start:]
    assert fwd[fwd[:, 0] == 1, 1].sum() == 199
    assert bwd[bwd[:, 0] == 1, 1].sum() == 180
    assert (bwd[:, 0] == 3).sum() == 200
    assert (bwd[:, 0] == 2).sum() == 180


@pytest.mark.parametrize('p,steps', [(1, 6), (2, 6), (3, 3)])
def test_limited_oracle_gradient_matches_finite_differences(p, steps):
    """The scheme with the linear limiter.  The limiter is piecewise rational; directions scaled
    by each coefficient's magnitude keep the near-zero elements (where the 1e-8 tolerance sets
    the limiter factor) in their linear regime, and there the adjoint matches central
    differences of the full run and of the run with the limiter's choices frozen."""
    from oracle import adjoint as OA
    kw = dict(hmax=2 ** -3, p=p, numSteps=steps, tEnd=steps * 2e-4)
    o = OA.LimitedAdjointOracle(**kw)
    o.set_modes(OA.mode_velocities())
    c0 = o.pd.cDisc
    cstar = OA.LimitedAdjointOracle(adjointTarget=True, **kw).forward(c0, steps)
    cT = o.forward(c0, steps)
    assert np.linalg.norm(o.forward(c0, steps, frozen=True) - cT) <= 1e-14 * np.linalg.norm(cT)
    g0, gth = o.backward(cT - cstar)
    h = 1e-5
    rng = np.random.default_rng(5)
    d = rng.standard_normal(c0.shape) * np.abs(c0)
    J = lambda c, fr: 0.5 * float(np.sum((o.forward(c, steps, frozen=fr) - cstar) ** 2))
    for fr in (True, False):
        fd = (J(c0 + h * d, fr) - J(c0 - h * d, fr)) / (2 * h)
        o.forward(c0, steps)                        # the base point's choices again
        assert abs(fd - float(np.sum(g0 * d))) <= 1e-6 * abs(fd)
    th0 = o.pd.theta.copy()
    dt = rng.standard_normal(th0.size) * np.abs(th0)
    o.op.set_theta(th0 + h * dt)
    Jp = J(c0, False)
    o.op.set_theta(th0 - h * dt)
    Jm = J(c0, False)
    o.op.set_theta(th0)
    assert abs((Jp - Jm) / (2 * h) - float(gth @ dt)) <= 1e-6 * abs((Jp - Jm) / (2 * h))


def test_limited_oracle_forward_is_the_reference_run():
    from oracle import adjoint as OA
    from oracle import advection as adv
    kw = dict(hmax=2 ** -3, p=2, numSteps=5, tEnd=5 * 2e-4)
    o = OA.LimitedAdjointOracle(**kw)
    ref = adv.main(testcase='adjoint', isSlopeLim=True, typeSlopeLim='linear', **kw).cDisc
    assert np.linalg.norm(o.forward(o.pd.cDisc, 5) - ref) <= 1e-14 * np.linalg.norm(ref)


@pytest.mark.parametrize('typ', ['strict', 'hierarch_vert'])
def test_limiter_replay_is_the_run_and_its_complex_step_is_its_derivative(typ):
    """The oracle's frozen replay of a strict- or hierarchical-limiter run (used to check the
    GPU adjoints) reproduces the run, and its complex-step derivative agrees with central
    differences of the replay at a step below the smallest winner's |v_n - c -+ tol|."""
    from oracle import adjoint as OA
    kw = dict(hmax=2 ** -3, p=3, numSteps=2, tEnd=2 * 1e-4)
    o = OA.LimiterReplayOracle(typ=typ, **kw)
    c0 = o.pd.cDisc
    cT = o.forward(c0, kw['numSteps'])
    cR = o.forward(c0, kw['numSteps'], frozen=True)
    assert np.linalg.norm(cR - cT) <= 1e-13 * np.linalg.norm(cT)
    assert sum(int(ch[1][q]['active'].sum()) for st in o.choices for ch in st for q in ch[1]
               if isinstance(q, int)) > 0
    w = np.random.default_rng(2).standard_normal(c0.shape)
    J = lambda c: np.sum(w * c)
    d = np.random.default_rng(3).standard_normal(c0.shape)
    cs = float(np.imag(J(o.forward(c0 + 1e-30j * d, kw['numSteps'], frozen=True)))) / 1e-30
    # these runs have a winner within about 1e-10 of a pole: central differences converge like
    # h^2 only below it (strict: 3.7e-3, 3.8e-5, 6.7e-7 at h = 1e-11, 1e-12, 1e-13)
    err = []
    for h in (1e-12, 1e-13):
        fd = (J(o.forward(c0 + h * d, kw['numSteps'], frozen=True)) - J(o.forward(c0 - h * d, kw['numSteps'], frozen=True))) / (2 * h)
        err.append(abs(fd - cs) / abs(cs))
    assert err[1] <= 1e-5 and err[1] < err[0], (err, cs)
