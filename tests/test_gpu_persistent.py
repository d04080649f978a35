"""GPU: the persistent time step (one cooperative launch per step, grid barriers between the
phases) gives the separate-kernel pipeline's results bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [dict(testcase='gauss_slot', hmax=2 ** -4, p=2, tEnd=0.03, numSteps=30, isSlopeLim=True),
         dict(testcase='gauss_slot', hmax=2 ** -4, p=1, tEnd=0.03, numSteps=30, isSlopeLim=True),
         dict(testcase='gauss_slot', hmax=2 ** -4, p=3, tEnd=0.01, numSteps=10, isSlopeLim=True),
         dict(testcase='gauss_slot', hmax=2 ** -4, p=2, tEnd=0.03, numSteps=30),
         dict(testcase='gauss_slot', hmax=2 ** -4, p=1, tEnd=0.03, numSteps=30, ordRK=1),
         dict(testcase='solid_body', hmax=2 ** -5, p=2, tEnd=0.03, numSteps=30, isSlopeLim=True, ordRK=2)]


def run(flags, precision, kw):
    from festung_gb300 import advection_gpu as G
    pd = G.main(precision=precision, gpuFlags=flags, **kw)
    pd.solver.close()
    return pd.cDisc


@pytest.mark.parametrize('kw', CASES, ids=['p2lim', 'p1lim', 'p3lim', 'p2', 'p1rk1', 'p2rk2lim'])
@pytest.mark.parametrize('precision', ['fp32', 'fp64'])
def test_persistent_step_is_bitwise_the_pipeline(lib, kw, precision):
    from festung_gb300 import _lib as L
    a = run(L.FLAG_PERSIST, precision, kw)
    b = run(0, precision, kw)
    assert np.array_equal(a, b)
    c = run(L.FLAG_PERSIST | L.FLAG_NO_GRAPH, precision, kw)
    assert np.array_equal(c, b)


def test_persistent_step_on_an_ensemble(lib):
    from festung_gb300 import _lib as L
    from festung_gb300 import ensemble as E
    out = []
    for flags in (0, L.FLAG_PERSIST):
        ens = E.Ensemble([0, 1, 2, 3, 4], precision='fp32', numSteps=20, hmax=2 ** -4, flags=flags)
        try:
            ens.step(20)
            out.append(ens.states())
        finally:
            ens.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)
