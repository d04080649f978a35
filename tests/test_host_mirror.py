"""Host side of advection_gpu (CPU): synthetic inputs and set-up data equal the oracle's."""
import numpy as np
import pytest

from festung_gb300 import advection_gpu as AG
from festung_gb300 import testcases as TC
from oracle import advection as adv
from oracle import assembly as A
from oracle import testcases as OT


@pytest.mark.parametrize('jitter,seed', [(0.0, 0), (0.2, 3), (0.1, 99)])
def test_meshes_match_oracle(jitter, seed):
    coordV, V0T, dim, h = TC.square_coords(2 ** -4)
    coordV = TC.jitter_coords(coordV, h, jitter, seed)
    g = OT.jittered_square(2 ** -4, jitter, seed)
    assert np.array_equal(coordV, g.coordV) and np.array_equal(V0T, g.V0T)


@pytest.mark.parametrize('seed', [0, 1, 2, 17])
def test_ensemble_parameters_match_oracle(seed):
    a, b = TC.ensemble_params(seed), OT.ensemble_params(seed)
    for k in a:
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k


def test_transient_terms_are_the_reference_functions():
    pd = {'testcase': 'transient'}
    TC.configure(pd)
    po = adv.Struct(testcase='transient', p=1)
    adv.configureProblem(po)
    rng = np.random.default_rng(1)
    x, y = rng.random(100), rng.random(100)
    for t in (0.0, 0.3, 1.7):
        g = {'const': 1.0, 'exp_neg': np.exp(-t)}
        f = sum(g[fn] * fun(x, y) for fn, fun in pd['fTerms'])
        cD = sum(g[fn] * fun(x, y) for fn, fun in pd['cDTerms'])
        assert np.allclose(f, po.fCont(t, x, y), rtol=1e-13, atol=1e-12)
        assert np.allclose(cD, po.cDCont(t, x, y), rtol=1e-14, atol=1e-14)


def test_setup_projections_match_oracle(lib):
    from festung_gb300 import _lib as L
    po = adv.Struct(testcase='gauss_slot', hmax=2 ** -3, p=2, numSteps=1)
    for f in (adv.configureProblem, adv.preprocessProblem):
        po = f(po)
    g = L.grid_build(po.g.coordV, po.g.V0T)
    tables = AG.Tables(po.N)
    c = AG.project(g, tables, po.c0Cont, 5, po.hatM)
    co = A.projectFuncCont2DataDisc(po.g, po.c0Cont, 5, po.hatM, po.basesOnQuad)
    assert np.allclose(c, co, rtol=0, atol=1e-14)
    u = lambda x, y: 0.5 - y
    v = lambda x, y: x - 0.5
    vn = AG.normal_velocity(g, tables, u, v, 5)
    vno = A.computeFuncContNuOnQuadEdge(po.g, lambda a, b: u(a, b), lambda a, b: v(a, b), 5)
    assert np.array_equal(vn, vno)
    err = AG.l2_error(g, tables, co, po.c0Cont, 5)
    assert abs(err - A.computeL2Error(po.g, co, po.c0Cont, 5, po.basesOnQuad)) < 1e-14
