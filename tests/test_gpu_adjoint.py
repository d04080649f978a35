"""GPU adjoint: gradients through the C-ABI against the oracle's transposed assembled operators
(and, with the linear limiter, the oracle's limiter adjoint) and against central finite
differences of the GPU forward run.

Bars: FP64 relative L2 <= 1e-11 against the oracle (dJ/dc0 and dJ/dtheta; the reduction orders
differ); FP64 finite differences (h = 1e-6) within 1e-7 of the adjoint's directional derivative;
the checkpointed and stage-recomputing sweeps bitwise equal to the fully stored one; FP32
within 1e-3 of FP64.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


def oracle_gradient(kw):
    from oracle import adjoint as OA
    o = OA.AdjointOracle(**kw)
    o.set_modes(OA.mode_velocities())
    tgt = OA.AdjointOracle(adjointTarget=True, **kw)
    c0 = o.pd.cDisc
    cstar = tgt.forward(c0, kw['numSteps'])
    cT = o.forward(c0, kw['numSteps'])
    g0, gth = o.backward(cT - cstar)
    return c0, cstar, 0.5 * float(np.sum((cT - cstar) ** 2)), g0, gth


CASES = [dict(hmax=2 ** -3, p=2, numSteps=10, tEnd=10 * 2e-4),
         dict(hmax=2 ** -3, p=1, numSteps=10, tEnd=10 * 4e-4),
         dict(hmax=2 ** -4, p=3, numSteps=6, tEnd=6 * 1e-4)]


@pytest.mark.parametrize('kw', CASES, ids=['p2', 'p1', 'p3'])
def test_fp64_gradient_matches_oracle(lib, kw):
    from festung_gb300 import adjoint as AD
    c0, cstar, Jo, og0, ogth = oracle_gradient(kw)
    pd = AD.setup(precision='fp64', **kw)
    try:
        J, g0, gth = AD.misfit_gradient(pd, c0, pd.theta, cstar)
    finally:
        pd.solver.close()
    assert abs(J - Jo) <= 1e-12 * Jo
    assert rel(g0, og0) <= 1e-11
    assert rel(gth, ogth) <= 1e-11


def test_checkpointed_sweep_equals_stored_sweep(lib):
    from festung_gb300 import adjoint as AD
    kw = dict(hmax=2 ** -4, p=2, numSteps=30, tEnd=30 * 2e-4)
    c0, cstar, *_ = oracle_gradient(dict(kw, numSteps=1, tEnd=2e-4))
    pd = AD.setup(precision='fp64', **kw)
    try:
        ref = AD.misfit_gradient(pd, c0, pd.theta, cstar, nSnapshots=0)
        for snaps in (1, 3, 7, kw['numSteps']):   # binomial, and every state without the stages
            got = AD.misfit_gradient(pd, c0, pd.theta, cstar, nSnapshots=snaps)
            assert got[0] == ref[0]
            assert np.array_equal(got[1], ref[1]) and np.array_equal(got[2], ref[2])
    finally:
        pd.solver.close()


@pytest.mark.parametrize('p', [1, 2, 3])
def test_fp32_sweeps_agree_bitwise_across_checkpoints_and_split_widths(lib, p):
    """FP32: binomial and stage-recomputing sweeps equal the stored one bit for bit, and the
    warp-role split of the stage kernel gives the same bits at 1, 2 and 4 warps per role."""
    from festung_gb300 import _lib as L
    from festung_gb300 import adjoint as AD
    kw = dict(hmax=2 ** -4, p=p, numSteps=12, tEnd=12 * 1e-4)
    c0, cstar, *_ = oracle_gradient(dict(kw, numSteps=1, tEnd=1e-4))
    pd = AD.setup(precision='fp32', **kw)
    try:
        assert pd.solver.get_option(L.OPT_ADJ_WARPS) == 2
        ref = AD.misfit_gradient(pd, c0, pd.theta, cstar, nSnapshots=0)
        for warps in (1, 2, 4):
            pd.solver.set_option(L.OPT_ADJ_WARPS, warps)
            for snaps in (0, 1, 4, kw['numSteps']):
                got = AD.misfit_gradient(pd, c0, pd.theta, cstar, nSnapshots=snaps)
                assert got[0] == ref[0]
                assert np.array_equal(got[1], ref[1]) and np.array_equal(got[2], ref[2]), (warps, snaps)
    finally:
        pd.solver.close()


def test_adjoint_autotuner_applies_a_width_and_keeps_the_gradient(lib):
    from festung_gb300 import _lib as L
    from festung_gb300 import adjoint as AD
    from festung_gb300 import autotune as AT
    kw = dict(hmax=2 ** -4, p=2, numSteps=10, tEnd=10 * 1e-4)
    c0, cstar, *_ = oracle_gradient(dict(kw, numSteps=1, tEnd=1e-4))
    pd = AD.setup(precision='fp32', **kw)
    try:
        ref = AD.misfit_gradient(pd, c0, pd.theta, cstar, nSnapshots=3)
        best, table = AT.tune_adjoint(pd.solver, pd.tau, nSteps=6, nSnapshots=3, reps=1)
        assert [r["adjWarps"] for r in table if "adjGraph" not in r] == [1, 2, 4]
        assert pd.solver.get_option(L.OPT_ADJ_WARPS) == best['adjWarps']
        got = AD.misfit_gradient(pd, c0, pd.theta, cstar, nSnapshots=3)
        assert np.array_equal(got[1], ref[1]) and np.array_equal(got[2], ref[2])
    finally:
        pd.solver.close()


def test_fp64_gradient_matches_finite_differences(lib):
    from festung_gb300 import adjoint as AD
    kw = dict(hmax=2 ** -5, p=2, numSteps=60, tEnd=60 * 2e-4)
    tg = AD.setup(precision='fp64', adjointTarget=True, **kw)
    tg.solver.step(kw['numSteps'], 0, tg.tau)
    cstar = tg.solver.get_state()
    tg.solver.close()
    pd = AD.setup(precision='fp64', **kw)
    try:
        c0 = np.asfortranarray(pd._cDisc)
        J, g0, gth = AD.misfit_gradient(pd, c0, pd.theta, cstar, nSnapshots=8)
        rng = np.random.default_rng(7)
        h = 1e-6
        for _ in range(3):
            d = rng.standard_normal(c0.shape)
            fd = (AD.misfit(pd, c0 + h * d, pd.theta, cstar) - AD.misfit(pd, c0 - h * d, pd.theta, cstar)) / (2 * h)
            assert abs(fd - np.sum(g0 * d)) <= 1e-7 * abs(fd)
            dt = rng.standard_normal(gth.size)
            fd = (AD.misfit(pd, c0, pd.theta + h * dt, cstar) - AD.misfit(pd, c0, pd.theta - h * dt, cstar)) / (2 * h)
            assert abs(fd - gth @ dt) <= 1e-7 * abs(fd)
    finally:
        pd.solver.close()


def test_fp32_gradient_close_to_fp64(lib):
    from festung_gb300 import adjoint as AD
    kw = dict(hmax=2 ** -4, p=2, numSteps=40, tEnd=40 * 2e-4)
    c0, cstar, *_ = oracle_gradient(dict(kw, numSteps=1, tEnd=2e-4))
    out = {}
    for prec in ('fp64', 'fp32'):
        pd = AD.setup(precision=prec, **kw)
        try:
            out[prec] = AD.misfit_gradient(pd, c0, pd.theta, cstar)
        finally:
            pd.solver.close()
    assert rel(out['fp32'][1], out['fp64'][1]) <= 1e-3
    assert rel(out['fp32'][2], out['fp64'][2]) <= 1e-3


def test_autograd_function_gives_the_adjoint_gradient(lib):
    torch = pytest.importorskip('torch')
    from festung_gb300 import adjoint as AD
    kw = dict(hmax=2 ** -3, p=2, numSteps=10, tEnd=10 * 2e-4)
    c0, cstar, Jo, og0, ogth = oracle_gradient(kw)
    pd = AD.setup(precision='fp64', **kw)
    try:
        x = torch.tensor(np.ascontiguousarray(c0), dtype=torch.float64, requires_grad=True)
        th = torch.tensor(pd.theta, dtype=torch.float64, requires_grad=True)
        cT = AD.AdvectionSolve.apply(x, th, pd.solver, kw['numSteps'], pd.tau, 0)
        J = 0.5 * ((cT - torch.from_numpy(np.ascontiguousarray(cstar))) ** 2).sum()
        J.backward()
        assert rel(x.grad.numpy(), og0) <= 1e-11
        assert rel(th.grad.numpy(), ogth) <= 1e-11
    finally:
        pd.solver.close()


def limited_oracle_gradient(kw):
    from oracle import adjoint as OA
    o = OA.LimitedAdjointOracle(**kw)
    o.set_modes(OA.mode_velocities())
    c0 = o.pd.cDisc
    cstar = OA.LimitedAdjointOracle(adjointTarget=True, **kw).forward(c0, kw['numSteps'])
    cT = o.forward(c0, kw['numSteps'])
    g0, gth = o.backward(cT - cstar)
    return c0, cstar, 0.5 * float(np.sum((cT - cstar) ** 2)), g0, gth


LIMITED = [dict(hmax=2 ** -3, p=2, numSteps=8, tEnd=8 * 2e-4),
           dict(hmax=2 ** -3, p=1, numSteps=8, tEnd=8 * 2e-4),
           dict(hmax=2 ** -3, p=3, numSteps=4, tEnd=4 * 2e-4)]


@pytest.mark.parametrize('kw', LIMITED, ids=['p2', 'p1', 'p3'])
@pytest.mark.parametrize('snaps', [0, 3])
def test_limited_fp64_gradient_matches_oracle(lib, kw, snaps):
    """The linear limiter's adjoint (frozen choices recomputed from the recorded limiter inputs)
    against the oracle's, written in the reference's Taylor basis; both stage storage and
    recomputing checkpoints."""
    from festung_gb300 import adjoint as AD
    c0, cstar, Jo, og0, ogth = limited_oracle_gradient(kw)
    pd = AD.setup(precision='fp64', isSlopeLim=True, **kw)
    try:
        J, g0, gth = AD.misfit_gradient(pd, c0, pd.theta, cstar, nSnapshots=snaps)
    finally:
        pd.solver.close()
    assert abs(J - Jo) <= 1e-12 * Jo
    assert rel(g0, og0) <= 1e-11
    assert rel(gth, ogth) <= 1e-11


REPLAY_CASES = [dict(hmax=2 ** -3, p=2, numSteps=4, tEnd=4 * 2e-4),
                 dict(hmax=2 ** -3, p=3, numSteps=3, tEnd=3 * 1e-4)]


@pytest.mark.parametrize('lim', ['strict', 'hierarch_vert'])
@pytest.mark.parametrize('kw', REPLAY_CASES, ids=['p2', 'p3'])
def test_taylor_limiter_gradient_matches_oracle_replay(lib, kw, lim):
    """The strict and the hierarchical limiter's adjoints against the oracle's replay of the same
    run with its choices frozen: the complex-step derivative Im J(c0 + i h d) / h of that replay
    is the exact directional derivative of the piece the run sits on (real differences would
    need h below the smallest |v_n - c -+ tol| of a winner, about 1e-10 here).  Along random
    directions of the initial coefficients, with stored stages and with recomputing
    checkpoints."""
    from oracle import adjoint as OA
    from festung_gb300 import adjoint as AD
    o = OA.LimiterReplayOracle(typ=lim, **kw)
    c0 = o.pd.cDisc
    cstar = OA.LimiterReplayOracle(typ=lim, adjointTarget=True, **kw).forward(c0, kw['numSteps'])
    cT = o.forward(c0, kw['numSteps'])
    Jo = 0.5 * float(np.sum((cT - cstar) ** 2))
    pd = AD.setup(precision='fp64', isSlopeLim=True, typeSlopeLim=lim, **kw)
    try:
        for snaps in (0, 2):
            J, g0, gth = AD.misfit_gradient(pd, c0, pd.theta, cstar, nSnapshots=snaps)
            assert abs(J - Jo) <= 1e-12 * Jo
            rng = np.random.default_rng(7)
            for _ in range(3):
                d = rng.standard_normal(c0.shape)
                cz = o.forward(c0 + 1e-30j * d, kw['numSteps'], frozen=True)
                dj = float(np.imag(0.5 * np.sum((cz - cstar) ** 2))) / 1e-30
                # near a pole of dm / den a rounding difference between the two runs moves the
                # derivative by up to eps / |den| relative
                assert abs(float(np.sum(g0 * d)) - dj) <= 1e-6 * abs(dj), (float(np.sum(g0 * d)), dj)
    finally:
        pd.solver.close()


def test_limited_theta_gradient_matches_finite_differences(lib):
    """Velocity perturbations move every element together and stay on one side of the
    limiter's switches at h = 1e-6: the adjoint matches central differences.  (Random
    perturbations of the initial coefficients cross a switch somewhere on a mesh this size;
    the oracle test checks those directions on the run with frozen choices.)"""
    from festung_gb300 import adjoint as AD
    kw = dict(hmax=2 ** -6, p=2, numSteps=40, tEnd=40 * 2e-4)
    tg = AD.setup(precision='fp64', adjointTarget=True, isSlopeLim=True, **kw)
    tg.solver.step(kw['numSteps'], 0, tg.tau)
    cstar = tg.solver.get_state()
    tg.solver.close()
    pd = AD.setup(precision='fp64', isSlopeLim=True, **kw)
    try:
        c0 = np.asfortranarray(pd._cDisc)
        J, g0, gth = AD.misfit_gradient(pd, c0, pd.theta, cstar, nSnapshots=0)
        rng = np.random.default_rng(11)
        h = 1e-6
        for _ in range(2):
            dt = rng.standard_normal(gth.size) * np.abs(pd.theta)
            fd = (AD.misfit(pd, c0, pd.theta + h * dt, cstar) - AD.misfit(pd, c0, pd.theta - h * dt, cstar)) / (2 * h)
            assert abs(fd - gth @ dt) <= 1e-7 * abs(fd)
    finally:
        pd.solver.close()


HIER = [dict(hmax=2 ** -5, p=2, numSteps=20, tEnd=20 * 2e-4),
        dict(hmax=2 ** -5, p=3, numSteps=10, tEnd=10 * 1e-4, jitter=0.1, meshSeed=5),
        dict(hmax=2 ** -5, p=1, numSteps=20, tEnd=20 * 2e-4)]


def _hier_case(kw, precision='fp64', lim='hierarch_vert'):
    from festung_gb300 import adjoint as AD
    args = dict(kw, isSlopeLim=True, typeSlopeLim=lim)
    tg = AD.setup(precision='fp64', adjointTarget=True, **args)
    tg.solver.step(kw['numSteps'], 0, tg.tau)
    cstar = tg.solver.get_state()
    tg.solver.close()
    return AD.setup(precision=precision, **args), cstar


@pytest.mark.parametrize('lim', ['hierarch_vert', 'strict'])
@pytest.mark.parametrize('kw', HIER, ids=['p2', 'p3-jitter', 'p1'])
def test_hierarchical_gradient_matches_finite_differences(lib, kw, lim):
    """The hierarchical vertex limiter's adjoint (core/applySlopeLimiterTaylorHierarchicalVertex.m)
    and the strict limiter's (core/applySlopeLimiterTaylorStrict.m), choices recomputed from the
    recorded Taylor inputs, against central differences (h = 1e-6) of the GPU forward run: along
    velocity directions scaled by |theta|, and along c0 itself (a direction that moves every
    element together and stays on one side of the switches)."""
    from festung_gb300 import adjoint as AD
    pd, cstar = _hier_case(kw, lim=lim)
    try:
        c0 = np.asfortranarray(pd._cDisc)
        J, g0, gth = AD.misfit_gradient(pd, c0, pd.theta, cstar, nSnapshots=0)
        h = 1e-6
        rng = np.random.default_rng(5)
        for _ in range(2):
            dt = rng.standard_normal(gth.size) * np.abs(pd.theta)
            if lim == 'strict' and kw['p'] == 3:
                # The strict limiter at p = 3 has switches within a relative 1e-7 of this run in
                # these directions: on one side of the base point the one-sided difference
                # converges like h to the adjoint, on the other it does not.  The adjoint must
                # be one of the two one-sided derivatives.
                hs = 1e-7
                f0 = AD.misfit(pd, c0, pd.theta, cstar)
                fp = AD.misfit(pd, c0, pd.theta + hs * dt, cstar)
                fm = AD.misfit(pd, c0, pd.theta - hs * dt, cstar)
                err = min(abs((fp - f0) / hs - gth @ dt), abs((f0 - fm) / hs - gth @ dt))
                assert err <= 1e-4 * abs(gth @ dt), (fp, fm, f0, gth @ dt)
                continue
            fd = (AD.misfit(pd, c0, pd.theta + h * dt, cstar) - AD.misfit(pd, c0, pd.theta - h * dt, cstar)) / (2 * h)
            assert abs(fd - gth @ dt) <= 1e-6 * abs(fd), (fd, gth @ dt)
        fd = (AD.misfit(pd, c0 * (1 + h), pd.theta, cstar) - AD.misfit(pd, c0 * (1 - h), pd.theta, cstar)) / (2 * h)
        assert abs(fd - float(np.sum(g0 * c0))) <= 1e-6 * abs(fd), (fd, float(np.sum(g0 * c0)))
    finally:
        pd.solver.close()


@pytest.mark.parametrize('lim', ['hierarch_vert', 'strict'])
@pytest.mark.parametrize('precision', ['fp64', 'fp32'])
def test_hierarchical_checkpointed_sweep_equals_stored_sweep(lib, precision, lim):
    from festung_gb300 import adjoint as AD
    pd, cstar = _hier_case(HIER[0], precision, lim)
    try:
        c0 = np.asfortranarray(pd._cDisc)
        ref = AD.misfit_gradient(pd, c0, pd.theta, cstar, nSnapshots=0)
        for snaps in (3, HIER[0]['numSteps']):
            got = AD.misfit_gradient(pd, c0, pd.theta, cstar, nSnapshots=snaps)
            assert got[0] == ref[0]
            assert np.array_equal(got[1], ref[1]) and np.array_equal(got[2], ref[2])
    finally:
        pd.solver.close()


STREAM_CASES = [dict(precision='fp32', kw=dict(hmax=2 ** -4, p=2, numSteps=24, tEnd=24 * 1e-4)),
                dict(precision='fp64', kw=dict(hmax=2 ** -4, p=1, numSteps=16, tEnd=16 * 2e-4, isSlopeLim=True)),
                dict(precision='fp32', kw=dict(hmax=2 ** -4, p=2, numSteps=16, tEnd=16 * 2e-4, isSlopeLim=True)),
                dict(precision='fp32', kw=dict(hmax=2 ** -4, p=3, numSteps=10, tEnd=10 * 1e-4, isSlopeLim=True,
                                               typeSlopeLim='hierarch_vert')),
                dict(precision='fp64', kw=dict(hmax=2 ** -4, p=3, numSteps=10, tEnd=10 * 1e-4, isSlopeLim=True,
                                               typeSlopeLim='strict'))]


@pytest.mark.parametrize('case', STREAM_CASES, ids=['unlimited-p2', 'linear-p1', 'linear-p2', 'hier-p3', 'strict-p3'])
def test_stream_sweeps_equal_one_stream_sweep(lib, case):
    """DGADV_OPT_ADJ_STREAMS: the recomputation and the limiter adjoint's scatters on a second
    stream, one reversed step ahead of the reverse stages, and the advances between checkpoints
    on a third (with renamed checkpoint slots), give bitwise the gradients of one stream;
    DGADV_OPT_ADJ_GRAPH: the sweep captured in a graph (and replayed) or launched directly gives
    the same bits; with every stage stored and for binomial and every-state checkpoints."""
    from festung_gb300 import _lib as L
    from festung_gb300 import adjoint as AD
    kw = case['kw']
    tg = AD.setup(precision='fp64', adjointTarget=True, **kw)
    tg.solver.step(kw['numSteps'], 0, tg.tau)
    cstar = tg.solver.get_state()
    tg.solver.close()
    pd = AD.setup(precision=case['precision'], **kw)
    try:
        assert pd.solver.get_option(L.OPT_ADJ_STREAMS) == 3
        c0 = np.asfortranarray(pd._cDisc)
        ref = AD.misfit_gradient(pd, c0, pd.theta, cstar, nSnapshots=0)
        for streams in (1, 2, 3):
            pd.solver.set_option(L.OPT_ADJ_STREAMS, streams)
            for graph in (1, 0):                  # the sweep as one CUDA graph, or launched directly
                pd.solver.set_option(L.OPT_ADJ_GRAPH, graph)
                for snaps in (0, 3, 5, kw['numSteps']):
                    for _ in range(2):
                        got = AD.misfit_gradient(pd, c0, pd.theta, cstar, nSnapshots=snaps)
                        assert got[0] == ref[0]
                        assert np.array_equal(got[1], ref[1]) and np.array_equal(got[2], ref[2]), (streams, graph, snaps)
    finally:
        pd.solver.close()


def test_strict_adjoint_differs_from_hierarchical(lib):
    """The strict limiter's adjoint is its own: on a p = 3 run where both limiters act, the two
    gradients differ (the strict limiter rescales every higher degree by each order's factor
    and reconstructs from the data already limited)."""
    from festung_gb300 import adjoint as AD
    kw = HIER[1]
    out = {}
    for lim in ('hierarch_vert', 'strict'):
        pd, cstar = _hier_case(kw, lim=lim)
        try:
            c0 = np.asfortranarray(pd._cDisc)
            out[lim] = AD.misfit_gradient(pd, c0, pd.theta, cstar, nSnapshots=0)
        finally:
            pd.solver.close()
    assert np.all(np.isfinite(out['strict'][1])) and np.all(np.isfinite(out['strict'][2]))
    assert not np.array_equal(out['strict'][1], out['hierarch_vert'][1])
