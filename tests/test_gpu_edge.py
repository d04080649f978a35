"""GPU edge cases against the oracle: the smallest and ragged meshes domainSquare makes (2, 8,
18 and 50 triangles: one partial block, vertex patches that are all boundary), one-step runs,
every degree and limiter, FP64 at the FP64 bar (10 x the oracle's roundoff spread where that
is larger)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MESHES = [1.0, 0.5, 1 / 3, 0.2]
VARIANTS = [(0, False, 'linear'), (1, True, 'linear'), (2, True, 'linear'), (2, False, 'linear'),
            (3, True, 'hierarch_vert'), (2, True, 'strict'), (3, True, 'strict')]


@pytest.mark.parametrize('hmax', MESHES, ids=['K2', 'K8', 'K18', 'K50'])
@pytest.mark.parametrize('p,lim,typ', VARIANTS, ids=['p0', 'p1lin', 'p2lin', 'p2', 'p3hier', 'p2strict', 'p3strict'])
def test_tiny_and_ragged_meshes_match_oracle(lib, hmax, p, lim, typ):
    from festung_gb300 import advection_gpu as G
    from oracle import matfree as MF
    kw = dict(testcase='gauss_slot', hmax=hmax, p=p, tEnd=0.01, numSteps=3, isSlopeLim=lim, typeSlopeLim=typ)
    pd = G.main(precision='fp64', **kw)
    pd.solver.close()
    o = MF.main_matfree(**kw).cDisc
    tol = max(1e-12, 10 * MF.roundoff_spread(**kw))
    assert np.linalg.norm(pd.cDisc - o) <= tol * max(np.linalg.norm(o), 1e-300)


@pytest.mark.parametrize('precision', ['fp32', 'fp64', 'df32'])
def test_single_step_and_zero_steps(lib, precision):
    from festung_gb300 import advection_gpu as G
    from oracle import matfree as MF
    kw = dict(testcase='gauss_slot', hmax=2 ** -4, p=2, tEnd=1e-3, numSteps=1, isSlopeLim=True)
    pd = G.main(precision=precision, **kw)
    s = pd.solver
    c1 = np.array(pd.cDisc)
    s.step(0, 1, pd.tau)                 # zero steps: a no-op
    assert np.array_equal(s.get_state(), c1)
    s.close()
    o = MF.main_matfree(**kw).cDisc
    tol = {'fp64': 1e-12, 'df32': 1e-11, 'fp32': 1e-6}[precision]
    assert np.linalg.norm(c1 - o) <= tol * np.linalg.norm(o)
