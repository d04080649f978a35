"""Implicit time stepping on the GPU (dgadv_step_implicit / dgadv_solve_stationary) against the
oracle's sparse direct solves (oracle/implicit.py).

Bars: FP64 with GMRES to a relative residual of 1e-13: relative L2 difference of the
coefficients <= 1e-10 and the same L2 error to 1e-10 relative; FP32 (residual 1e-6) within 1e-4.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


def gpu(**kw):
    from festung_gb300 import advection_implicit_gpu as AI
    pd = AI.main(**kw)
    pd.solver.close()
    return pd


def oracle(**kw):
    from oracle import implicit as I
    return I.main(**kw)


CASES = [
    dict(testcase='transient', p=1, ordRK=2, hmax=1 / 4, numSteps=4, tEnd=0.4),
    dict(testcase='transient', p=2, ordRK=3, hmax=1 / 4, numSteps=4, tEnd=0.4),
    dict(testcase='transient', p=3, ordRK=4, hmax=1 / 4, numSteps=3, tEnd=0.3),
    dict(testcase='transient', p=0, ordRK=1, hmax=1 / 4, numSteps=4, tEnd=0.4),
    dict(testcase='transient_ode', p=1, ordRK=3, hmax=1 / 3, numSteps=4, tEnd=2),
    dict(testcase='solid_body', p=2, ordRK=3, hmax=1 / 8, numSteps=5, tEnd=0.5),
    dict(testcase='solid_body', p=1, ordRK=1, hmax=1 / 8, numSteps=5, tEnd=2.0),
    dict(testcase='stationary', p=1, hmax=1 / 6),
    dict(testcase='stationary', p=2, hmax=1 / 6),
    dict(testcase='stationary', p=3, hmax=1 / 3),
]


@pytest.mark.parametrize('kw', CASES, ids=lambda kw: '-'.join('%s=%s' % (k, v) for k, v in kw.items()))
def test_fp64_matches_oracle(lib, kw):
    g = gpu(precision='fp64', krylovTol=1e-13, **kw)
    o = oracle(**kw)
    assert rel(g.cDisc, o.cDisc) <= 1e-10
    assert abs(g.error - o.error) <= 1e-10 * max(o.error, 1e-3)
    assert g.relres <= 1e-13 and g.iterations > 0


@pytest.mark.parametrize('kw', CASES[:3] + CASES[7:8], ids=lambda kw: kw['testcase'] + '-p%d' % kw['p'])
def test_fp32_close_to_oracle(lib, kw):
    g = gpu(precision='fp32', **kw)
    o = oracle(**kw)
    assert rel(g.cDisc, o.cDisc) <= 1e-4


def test_stationary_converges_at_order_p_plus_1(lib):
    errs = [gpu(precision='fp64', testcase='stationary', p=2, hmax=2.0 ** -l / 3, krylovTol=1e-12).error
            for l in (1, 2, 3)]
    eoc = [np.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert min(eoc) > 2.85, eoc


def test_iteration_limit_reports_no_convergence(lib):
    from festung_gb300 import _lib as L
    with pytest.raises(L.DgadvError) as e:
        gpu(precision='fp64', testcase='stationary', p=2, hmax=1 / 6, krylovMaxIter=3)
    assert e.value.status == L.DGADV_ENOCONV


def test_implicit_handle_refuses_explicit_steps(lib):
    from festung_gb300 import _lib as L
    from festung_gb300 import advection_implicit_gpu as AI
    from festung_gb300.solver import DeviceSolver
    pd = AI.main(precision='fp64', testcase='transient', p=1, hmax=1 / 4, numSteps=1, tEnd=0.1)
    try:
        with pytest.raises(L.DgadvError) as e:
            pd.solver.step(1, 0, 0.1)
        assert e.value.status == L.DGADV_EUNSUPPORTED
    finally:
        pd.solver.close()
    g = pd.g
    with pytest.raises(L.DgadvError):       # no limiter on an implicit handle
        DeviceSolver(g['coordV'], g['V0T'], 1, 1, isSlopeLim=True, flags=L.FLAG_IMPLICIT)
    s = DeviceSolver(g['coordV'], g['V0T'], 1, 1)
    try:
        s.set_velocity_function((L.VEL_ROTATION, []))
        with pytest.raises(L.DgadvError) as e:   # an explicit handle refuses implicit steps
            s.step_implicit(1, 0, 0.1, 2)
        assert e.value.status == L.DGADV_EINVAL
    finally:
        s.close()


def test_graph_and_eager_arnoldi_steps_agree_bitwise(lib):
    """The Arnoldi steps replayed as CUDA graphs give the eager launches' results bit for bit."""
    from festung_gb300 import _lib as L
    from festung_gb300 import advection_implicit_gpu as AI
    out = []
    for flags in (0, L.FLAG_NO_GRAPH):
        pd = AI.Struct(dict(testcase='transient', p=2, ordRK=3, hmax=1 / 4, numSteps=3, tEnd=0.3,
                            precision='fp64'))
        pd.problemName = 'advection_implicit_gpu'
        for f in AI.PRE:
            pd = f(pd)
        try:
            pd.solver.set_option(L.OPT_FLAGS, flags)
            it, rr = pd.solver.step_implicit(3, 0, pd.tau, 3, 1e-13)
            out.append((pd.solver.get_state(), it))
        finally:
            pd.solver.close()
    assert np.array_equal(out[0][0], out[1][0]) and out[0][1] == out[1][1]
