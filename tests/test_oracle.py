"""Oracle pins (CPU).  The reference stores no golden vectors; the oracle is pinned by analytic
identities, by the theoretical convergence order on the reference's analytical test case and by
the agreement of its two independent restatements (sparse operators vs matrix-free)."""
import numpy as np
import pytest

from oracle import advection as adv
from oracle import basis as B
from oracle import grid as G
from oracle import matfree as MF


@pytest.mark.parametrize('p', [0, 1, 2, 3, 4])
def test_hatM_is_identity_to_quadrature_precision(p):
    """The modal basis is orthonormal (core/phi.m:40-61); hatM uses 15-digit rule constants."""
    N = B.N_of_p(p)
    hatM = B.integrateRefElemPhiPhi(N, B.computeBasesOnQuad(N))
    assert np.abs(hatM - np.eye(N)).max() < 2e-14


@pytest.mark.parametrize('qOrd', range(0, 10))
def test_2d_rules_integrate_monomials(qOrd):
    Q1, Q2, W = B.quadRule2D(qOrd)
    from math import factorial
    tol = 1e-14 if qOrd not in (4, 6) else 2e-14     # orders 4 and 6 have 15-digit literals
    for a in range(0, qOrd + 1):
        for b in range(0, qOrd + 1 - a):
            exact = factorial(a) * factorial(b) / factorial(a + b + 2)
            assert abs(np.sum(W * Q1 ** a * Q2 ** b) - exact) < tol


def test_collapsed_rule_matches_triquad_definition():
    """Orders >= 7 use the collapsed-square rule with qOrd^2 points (core/triquad.m:30-78)."""
    Q1, Q2, W = B.quadRule2D(7)
    assert Q1.size == 49 and abs(W.sum() - 0.5) < 1e-15
    assert np.all(Q1 >= 0) and np.all(Q2 >= 0) and np.all(Q1 + Q2 <= 1)


def test_domain_square_counts():
    g = G.domainSquare(2 ** -3)
    dim = 8
    assert g.numT == 2 * dim ** 2 and g.numV == (dim + 1) ** 2
    assert g.numE == 2 * dim * (dim + 1) + dim ** 2
    assert np.all(g.areaT > 0)
    # each interior edge is shared by two elements, boundary edges carry ids 1..4
    assert np.sum(g.T0E[:, 1] == 0) == 4 * dim
    assert set(np.unique(g.idE)) == {0, 1, 2, 3, 4}


def test_outward_normals_and_edge_maps_are_consistent():
    g = G.domainSquare(2 ** -3)
    mid = g.baryE0T - g.baryT[:, None, :]
    assert np.all(np.einsum('knm,knm->kn', mid, g.nuE0T) > 0)
    for nn in range(3):
        for np_ in range(3):
            M = g.markE0TE0T[nn][np_].tocoo()
            assert np.array_equal(g.E0T[M.row, nn], g.E0T[M.col, np_])


@pytest.mark.parametrize('kw', [
    dict(p=1, isSlopeLim=True), dict(p=2, isSlopeLim=True), dict(p=2),
    dict(p=3, isSlopeLim=True, typeSlopeLim='hierarch_vert'),
    dict(p=2, isSlopeLim=True, typeSlopeLim='strict'),
    dict(p=1, testcase='transient', tEnd=0.1)])
def test_sparse_and_matrix_free_restatements_agree(kw):
    base = dict(testcase='gauss_slot', hmax=2 ** -3, tEnd=0.03, numSteps=12)
    base.update(kw)
    a = adv.main(**base)
    b = MF.main_matfree(**base)
    tol = 1e-13
    if base.get('typeSlopeLim') == 'hierarch_vert' and base['p'] == 3:
        tol = max(tol, 10 * MF.roundoff_spread(**base))   # ill-conditioned limiter factors
    assert np.linalg.norm(a.cDisc - b.cDisc) / np.linalg.norm(a.cDisc) < tol


@pytest.mark.parametrize('p', [1, 2])
def test_convergence_order_on_transient_case(p):
    """advection/doConvergenceTest.m:57-107: EOC of the L2 error is about p+1."""
    errs = []
    for l in (1, 2, 3):
        pd = MF.main_matfree(testcase='transient', hmax=2 ** -l / 3, p=p, tEnd=0.2,
                             numSteps=2 ** p * 10 * 2 ** l)
        errs.append(pd.error)
    eoc = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert eoc[-1] > p + 1 - 0.25


def test_p0_is_first_order_upwind_finite_volume():
    """With p = 0 one stage is c_k' = -(1/|T_k|) sum_e |E| (u.n)^up c_upwind."""
    pd = adv.Struct(testcase='gauss_slot', hmax=2 ** -3, p=0, numSteps=1, tEnd=1e-3)
    for f in (adv.configureProblem, adv.preprocessProblem, adv.initializeProblem):
        pd = f(pd)
    mf = MF.MatFree(pd)
    ops = mf.stage_ops(0.0)
    c = pd.cDisc
    cdot = np.linalg.solve(mf.M, mf.rhs(c, ops)[..., None])[..., 0]
    g = pd.g
    K = g.numT
    vbar = ops['vN'][:, :, 0]                   # one Gauss point: u.n at the edge midpoint
    cell = c[:, 0] * np.sqrt(2)                 # cell mean of phi_1 = sqrt(2)
    expect = np.zeros(K)
    for n in range(3):
        kp = mf.nbr[:, n]
        up = np.where(vbar[:, n] > 0, cell, np.where(kp >= 0, cell[np.maximum(kp, 0)], 0.0))
        expect -= g.areaE0T[:, n] * vbar[:, n] * up
    expect /= g.areaT
    assert np.allclose(cdot[:, 0] * np.sqrt(2), expect, rtol=1e-12, atol=1e-14)


def test_mass_conserved_for_divergence_free_field_tangent_to_boundary():
    """Streamfunction velocities have u.n = 0 on the square's boundary: the DG scheme and the
    mean-preserving limiter conserve sum_k |T_k| cbar_k."""
    pd = MF.main_matfree(testcase='ensemble', instanceSeed=5, hmax=2 ** -3, p=2, tEnd=0.02,
                         numSteps=10, isSlopeLim=True, jitter=0.0)
    pd0 = adv.Struct(testcase='ensemble', instanceSeed=5, hmax=2 ** -3, p=2, numSteps=10,
                     tEnd=0.02, isSlopeLim=True, jitter=0.0)
    for f in (adv.configureProblem, adv.preprocessProblem, adv.initializeProblem):
        pd0 = f(pd0)
    m0 = np.sum(pd0.g.areaT * pd0.cDisc[:, 0])
    m1 = np.sum(pd.g.areaT * pd.cDisc[:, 0])
    assert abs(m1 - m0) < 1e-13 * max(1.0, abs(m0))


def test_roundoff_spread_is_small_except_hierarchical_p3():
    kw = dict(testcase='gauss_slot', hmax=2 ** -3, tEnd=0.02, numSteps=6, isSlopeLim=True)
    assert MF.roundoff_spread(p=2, **kw) < 1e-13
    assert MF.roundoff_spread(p=3, typeSlopeLim='hierarch_vert', **kw) < 1e-7
