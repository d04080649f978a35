"""The ``advection_implicit`` problem: diagonally implicit Runge-Kutta steps of the DG advection
operator with a sparse direct solve per stage (oracle restatement).

Test infrastructure: see ``oracle/__init__.py``.  Follows:
  advection_implicit/configureProblem.m (defaults: p = 2, ordRK = min(p + 1, 4),
  qOrd = 2p + 1, domainSquare without the PDE toolbox), advection_implicit/getTestcase.m
  ('solid_body', 'stationary', 'transient_ode', 'transient'),
  advection_implicit/preprocessProblem.m (reference integrals with the rule of order qOrd),
  advection_implicit/computeDerivedGridData.m, advection_implicit/initializeProblem.m,
  advection_implicit/solveStep.m, advection_implicit/preprocessSubStep.m (assembly at the stage
  time with order qOrd), advection_implicit/solveSubStep.m (the stage solve),
  advection_implicit/postprocessStep.m, advection_implicit/postprocessProblem.m (L2 error with
  order qOrd + 1), and core/rungeKuttaImplicit.m (the DIRK tables).

Per stage i of a step from t0:
  (M + tau a_ii A) x_i = tau a_ii sysV(t_i) + M c^n + sum_{j<i} tau a_ij rhs_j,
  rhs_i = sysV(t_i) - A x_i,     A = -G1 - G2 + R,   sysV = L - K_D - K_N,
and c^{n+1} = x_S (the tables are stiffly accurate).  Stationary: A x = sysV.
"""
import numpy as np
import scipy.sparse as sp
from scipy.sparse.linalg import spsolve

from . import assembly as A
from . import basis as B
from . import grid as G
from .advection import Struct, setdefault


def rungeKuttaImplicit(ordRK, tau, t0):
    """core/rungeKuttaImplicit.m: nodes t, matrix A, weights b (the last row of A), c."""
    if ordRK == 1:
        a = np.array([[1.0]])
    elif ordRK == 2:
        lam = 0.5 * (2 - np.sqrt(2.0))
        a = np.array([[lam, 0.0], [1 - lam, lam]])
    elif ordRK == 3:
        alpha = 0.4358665215084589994160194511935568425292
        beta = 0.5 * (1. + alpha)
        b1 = -0.25 * (6 * alpha * alpha - 16 * alpha + 1)
        b2 = 0.25 * (6 * alpha * alpha - 20 * alpha + 5)
        a = np.array([[alpha, 0, 0], [beta - alpha, alpha, 0], [b1, b2, alpha]])
    elif ordRK == 4:
        g = 1. / 4.
        a = np.array([[g, 0, 0, 0, 0],
                      [1. / 2., g, 0, 0, 0],
                      [17. / 50., -1. / 25., g, 0, 0],
                      [371. / 1360., -137. / 2720., 15. / 544., g, 0],
                      [25. / 24., -49. / 48., 125. / 16., -85. / 12., g]])
    else:
        raise ValueError('Function is not defined for order<1 or order>4.')
    b = a[-1, :].copy()
    c = a.sum(axis=1)
    return t0 + c * tau, a, b, c


def get_testcase(pd):
    """advection_implicit/getTestcase.m."""
    tc = pd.testcase
    zero = lambda t, x1, x2: np.zeros(np.broadcast(x1, x2).shape)
    if tc == 'solid_body':
        Gf = lambda x1, x2, a, b: (1 / 0.15) * np.sqrt((x1 - a) ** 2 + (x2 - b) ** 2)
        slot = lambda x1, x2: (((x1 - 0.5) ** 2 + (x2 - 0.75) ** 2 <= 0.0225)
                               & ((x1 <= 0.475) | (x1 >= 0.525) | (x2 >= 0.85))).astype(np.float64)
        d = dict(isAnalytical=False, isStationary=False,
                 c0Cont=lambda x1, x2: (slot(x1, x2)
                                        + (1 - Gf(x1, x2, 0.5, 0.25)) * ((x1 - 0.5) ** 2 + (x2 - 0.25) ** 2 <= 0.0225)
                                        + 0.25 * (1 + np.cos(np.pi * Gf(x1, x2, 0.25, 0.5)))
                                        * ((x1 - 0.25) ** 2 + (x2 - 0.5) ** 2 <= 0.0225)),
                 fCont=zero, u1Cont=lambda t, x1, x2: 0.5 - x2, u2Cont=lambda t, x1, x2: x1 - 0.5,
                 cDCont=zero, gNCont=zero, numSteps=320, tEnd=2 * np.pi)
    elif tc in ('stationary', 'transient'):
        stat = tc == 'stationary'
        if stat:
            cCont = lambda t, x1, x2: np.cos(7 * x1) * np.cos(7 * x2)
        else:
            cCont = lambda t, x1, x2: np.cos(7 * x1) * np.cos(7 * x2) + np.exp(-t)
        u1 = lambda t, x1, x2: np.exp(0.5 * (x1 + x2))
        u2 = lambda t, x1, x2: np.exp(0.5 * (x1 - x2))

        def f(t, x1, x2):
            out = (-7 * u1(t, x1, x2) * np.sin(7 * x1) * np.cos(7 * x2)
                   - 7 * u2(t, x1, x2) * np.cos(7 * x1) * np.sin(7 * x2)
                   + 0.5 * (u1(t, x1, x2) - u2(t, x1, x2)) * cCont(t, x1, x2))
            return out if stat else -np.exp(-t) + out
        d = dict(isAnalytical=True, isStationary=stat, cCont=cCont, u1Cont=u1, u2Cont=u2, fCont=f,
                 c0Cont=lambda x1, x2: cCont(0, x1, x2), cDCont=cCont,
                 gNCont=(lambda t, x1, x2: -7 * np.cos(7 * x1) * np.sin(7 * x2)) if stat else zero,
                 numSteps=1 if stat else 10, tEnd=10 if stat else 2)
    elif tc == 'transient_ode':
        cCont = lambda t, x1, x2: np.exp(-t) * np.ones(np.broadcast(x1, x2).shape)
        d = dict(isAnalytical=True, isStationary=False, cCont=cCont, u1Cont=zero, u2Cont=zero,
                 fCont=lambda t, x1, x2: -cCont(t, x1, x2), c0Cont=lambda x1, x2: cCont(0, x1, x2),
                 cDCont=cCont, gNCont=zero, numSteps=4, tEnd=2)
    else:
        raise ValueError('Invalid testcase "%s".' % tc)
    for k, v in d.items():
        setdefault(pd, k, v)
    # no edge carries the Neumann id -1 of 'stationary': every boundary edge is Dirichlet
    pd.generateMarkE0TbdrN = lambda g: np.zeros((g.numT, 3), dtype=bool)
    return pd


def configureProblem(pd):
    setdefault(pd, 'testcase', 'solid_body')
    setdefault(pd, 'hmax', 2 ** -6)
    setdefault(pd, 'p', 2)
    setdefault(pd, 'ordRK', min(pd.p + 1, 4))
    setdefault(pd, 'qOrd', 2 * pd.p + 1)
    get_testcase(pd)
    assert 0 <= pd.p <= 4 and 1 <= pd.ordRK <= 4 and pd.hmax > 0 and pd.numSteps > 0
    pd.generateGridData = G.domainSquare
    return pd


def preprocessProblem(pd):
    g = pd.generateGridData(pd.hmax)
    pd.g = g
    pd.K, pd.N = g.numT, B.N_of_p(pd.p)
    pd.tau = pd.tEnd / pd.numSteps
    g.markE0Tint = g.idE0T == 0
    g.markE0TbdrN = pd.generateMarkE0TbdrN(g)
    g.markE0TbdrD = ~(g.markE0Tint | g.markE0TbdrN)
    G.computeDerivedGridData(g)
    q = pd.qOrd
    pd.basesOnQuad = B.computeBasesOnQuad(pd.N, [q, q + 1])
    pd.hatM = B.integrateRefElemPhiPhi(pd.N, pd.basesOnQuad, q)
    pd.hatG = B.integrateRefElemDphiPhiPhi(pd.N, pd.basesOnQuad, q)
    pd.hatRdiagOnQuad = B.integrateRefEdgePhiIntPhiIntPerQuad(pd.N, pd.basesOnQuad, q)
    pd.hatRoffdiagOnQuad = B.integrateRefEdgePhiIntPhiExtPerQuad(pd.N, pd.basesOnQuad, q)
    pd.globM = A.assembleMatElemPhiPhi(g, pd.hatM)
    return pd


def initializeProblem(pd):
    pd.isFinished = False
    if not pd.isStationary:
        pd.cDisc = A.projectFuncCont2DataDisc(pd.g, pd.c0Cont, pd.qOrd, pd.hatM, pd.basesOnQuad)
    return pd


def assemble(pd, t):
    """advection_implicit/preprocessSubStep.m: the operators and right-hand side at time t."""
    g, q, N = pd.g, pd.qOrd, pd.N
    fDisc = A.projectFuncCont2DataDisc(g, lambda x1, x2: pd.fCont(t, x1, x2), q, pd.hatM, pd.basesOnQuad)
    u1Disc = A.projectFuncCont2DataDisc(g, lambda x1, x2: pd.u1Cont(t, x1, x2), q, pd.hatM, pd.basesOnQuad)
    u2Disc = A.projectFuncCont2DataDisc(g, lambda x1, x2: pd.u2Cont(t, x1, x2), q, pd.hatM, pd.basesOnQuad)
    vN = A.computeFuncContNuOnQuadEdge(g, lambda x1, x2: pd.u1Cont(t, x1, x2),
                                       lambda x1, x2: pd.u2Cont(t, x1, x2), q)
    globG = A.assembleMatElemDphiPhiFuncDisc(g, pd.hatG, u1Disc, u2Disc)
    globR = A.assembleMatEdgePhiPhiValUpwind(g, ~g.markE0TbdrN, pd.hatRdiagOnQuad, pd.hatRoffdiagOnQuad, vN)
    globKD = A.assembleVecEdgePhiIntFuncContVal(g, g.markE0TbdrD, lambda x1, x2: pd.cDCont(t, x1, x2),
                                                vN, N, pd.basesOnQuad, q)

    def gNUpwind(x1, x2):
        v = pd.gNCont(t, x1, x2)
        return (v <= 0) * v
    globKN = A.assembleVecEdgePhiIntFuncCont(g, g.markE0TbdrN, gNUpwind, N, pd.basesOnQuad, q)
    globL = pd.globM @ fDisc.reshape(-1)
    sysA = (-globG[0] - globG[1] + globR).tocsc()
    return sysA, globL - globKD - globKN


def solveStep(pd, nStep):
    """advection_implicit/solveStep.m + the sub-step loop of solveSubStep.m."""
    K, N = pd.K, pd.N
    if pd.isStationary:
        sysA, sysV = assemble(pd, 0.0)
        pd.cDisc = spsolve(sysA, sysV).reshape(K, N)
        return pd
    t, a, _, _ = rungeKuttaImplicit(pd.ordRK, pd.tau, (nStep - 1) * pd.tau)
    c0 = pd.cDisc.reshape(-1)
    M = pd.globM.tocsc()
    rhs = []
    x = c0
    for i in range(len(t)):
        sysA, sysV = assemble(pd, t[i])
        sysR = (pd.tau * a[i, i]) * sysV + M @ c0
        for j in range(i):
            sysR = sysR + (pd.tau * a[i, j]) * rhs[j]
        x = spsolve((M + (pd.tau * a[i, i]) * sysA).tocsc(), sysR)
        rhs.append(sysV - sysA @ x)
    pd.cDisc = x.reshape(K, N)
    return pd


def postprocessProblem(pd):
    f = (lambda x1, x2: pd.cCont(pd.tEnd, x1, x2)) if 'cCont' in pd else pd.c0Cont
    pd.error = A.computeL2Error(pd.g, pd.cDisc, f, pd.qOrd + 1, pd.basesOnQuad)
    return pd


def main(problemData=None, **kwargs):
    """main('advection_implicit', key, value, ...) (main.m:115-178)."""
    pd = Struct(problemData or {})
    pd.update(kwargs)
    pd.problemName = 'advection_implicit'
    for f in (configureProblem, preprocessProblem, initializeProblem):
        pd = f(pd)
    nSteps = 1 if pd.isStationary else pd.numSteps
    for n in range(1, nSteps + 1):
        solveStep(pd, n)
    return postprocessProblem(pd)
