"""The implicit problem's oracle (oracle/implicit.py) pinned by its convergence orders: the
reference's advection_implicit/doConvergenceTest.m measures these rates; its own tests hold no
golden values.  Spatial order p + 1 on the stationary case (meshes hmax = 2^-l / 3 as there),
temporal order ordRK on the transient ODE case (c = exp(-t), zero velocity)."""
import numpy as np
import pytest

from oracle import implicit as I


@pytest.mark.parametrize('p', [1, 2])
def test_stationary_converges_at_order_p_plus_1(p):
    errs = [I.main(testcase='stationary', p=p, hmax=2.0 ** -l / 3).error for l in (1, 2, 3)]
    eoc = [np.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert min(eoc) > p + 1 - 0.15, eoc


@pytest.mark.parametrize('ordRK', [1, 2, 3, 4])
def test_dirk_converges_at_its_order(ordRK):
    errs = [I.main(testcase='transient_ode', p=1, ordRK=ordRK, hmax=1 / 3, numSteps=4 * 2 ** l).error
            for l in (1, 2, 3)]
    eoc = [np.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert min(eoc) > ordRK - 0.15, eoc


def test_dirk_tables_are_stiffly_accurate_and_consistent():
    for o in (1, 2, 3, 4):
        t, a, b, c = I.rungeKuttaImplicit(o, 0.1, 1.0)
        assert np.allclose(b, a[-1]) and abs(b.sum() - 1.0) < 1e-14
        assert np.allclose(t, 1.0 + 0.1 * a.sum(axis=1))
        assert np.all(np.diag(a) > 0) and np.allclose(np.triu(a, 1), 0.0)


def test_transient_matches_the_explicit_problem_data():
    """'transient' of the implicit problem approaches its exact solution as h and tau shrink."""
    e1 = I.main(testcase='transient', p=1, hmax=1 / 6, numSteps=20).error
    e2 = I.main(testcase='transient', p=1, hmax=1 / 12, numSteps=40).error
    assert e2 < e1 / 3
