"""The ``transport`` problem, configuration 'rotation' on the unit square (oracle restatement).

Test infrastructure: see ``oracle/__init__.py``.  Follows transport/configureProblem.m (source
'rotation', grid 'square', no coupling, no mass check), transport/preprocessProblem.m,
transport/computeDerivedGridData.m, transport/initializeProblem.m, transport/solveStep.m,
transport/preprocessSubStep.m, transport/solveSubStep.m, transport/postprocessSubStep.m,
transport/postprocessStep.m, core/computeMask.m and core/projectDataQ0T2DataDisc.m.

Each species s carries its depth-integrated concentration c_s h (the unknown) and its
concentration c_s.  Per Runge-Kutta stage and species:
  * the advective term of c_s with the depth-integrated velocity (u h, v h) is assembled only
    over the species' active elements (its mask): rows and columns of inactive elements drop
    out, and an active element's outflow counts only across edges to active elements or the
    boundary (the masked branches of core/assembleMatElemDphiPhiFuncDiscVec.m:115-141 and
    core/assembleMatEdgePhiPhiValUpwind.m, restated here);
  * the SSP update acts on c_s h; c_s = Pi(c_s h / h) at the quadrature points; c_s is limited
    (linear vertex limiter, zero Dirichlet data), and c_s h = Pi(c_s h);
  * after the step the mask is recomputed from the last limiter call's vertex-patch extremes:
    max over the element's vertices of (max - min) >= maskTol ('vertex-based').
The reference keeps hatM = I (transport/preprocessProblem.m), so every projection here is
(sum_q W_q f_q phi_i(q)) without a mass solve, and globM = 2|T| I.
"""
import numpy as np
import scipy.sparse as sp

from . import assembly as A
from . import basis as B
from . import grid as G
from . import limiter as LM
from .advection import Struct, setdefault


def rotation_data(pd):
    """transport/configureProblem.m, configureRotation: depth 0.1, rotating velocity, four discs
    of radius^2 0.0225 / sqrt(2) times the species index and the depth."""
    h = lambda t, x1, x2: 0.1 * np.ones(np.broadcast(x1, x2).shape)
    pd.hCont = h
    pd.uHCont = lambda t, x1, x2: h(t, x1, x2) * (0.5 - x2)
    pd.vHCont = lambda t, x1, x2: h(t, x1, x2) * (x1 - 0.5)
    r = 0.0225 / np.sqrt(2)

    def cH0(x1, x2):
        return ((((x1 - 0.5) ** 2 + (x2 - 0.75) ** 2 <= r) * 1.0
                 + ((x1 - 0.25) ** 2 + (x2 - 0.5) ** 2 <= r)
                 + ((x1 - 0.5) ** 2 + (x2 - 0.25) ** 2 <= r)
                 + ((x1 - 0.75) ** 2 + (x2 - 0.5) ** 2 <= r)) * h(0, x1, x2))
    pd.cH0Cont = [(lambda s: (lambda x1, x2: s * cH0(x1, x2)))(s + 1) for s in range(pd.numSpecies)]
    return pd


def configureProblem(pd):
    setdefault(pd, 'p', 1)
    setdefault(pd, 'ordRK', min(pd.p + 1, 3))
    setdefault(pd, 'numSpecies', 1)
    setdefault(pd, 'maskTol', 1e-6)
    setdefault(pd, 'isMask', True)
    setdefault(pd, 'hmax', 2 ** -6)
    setdefault(pd, 'numSteps', 3124)
    setdefault(pd, 'tEnd', (pd.numSteps / 3142) * 2 * np.pi)
    assert 1 <= pd.p <= 4 and 1 <= pd.ordRK <= 3
    return rotation_data(pd)


def preprocessProblem(pd):
    g = G.domainSquare(pd.hmax)
    # every boundary edge has id 3 (Dirichlet), transport/preprocessProblem.m 'square'
    idE = np.zeros(g.numE, dtype=np.int64)
    bx, by = g.baryE[:, 0], g.baryE[:, 1]
    idE[(by == 0) | (bx == 1) | (by == 1) | (bx == 0)] = 3
    g.idE = idE
    g.idE0T = idE[g.E0T]
    g.markE0Tint = g.idE0T == 0
    g.markE0TbdrN = g.idE0T == 1
    g.markE0TbdrD = (g.idE0T == 2) | (g.idE0T == 3) | (g.idE0T == 4)
    bdrV = np.zeros(g.numV, dtype=bool)
    bdrV[g.V0E[g.E0T.T[g.markE0TbdrD.T]].ravel()] = True
    g.markV0TbdrD = bdrV[g.V0T]
    G.computeDerivedGridData(g)
    pd.g = g
    pd.K, pd.N = g.numT, B.N_of_p(pd.p)
    pd.tau = pd.tEnd / pd.numSteps
    pd.basesOnQuad = B.computeBasesOnQuad(pd.N)
    LM.computeTaylorBasesV0T(g, pd.N, pd.basesOnQuad)
    pd.hatM = np.eye(pd.N)
    pd.hatG = B.integrateRefElemDphiPhiPhi(pd.N, pd.basesOnQuad)
    pd.hatRdiagOnQuad = B.integrateRefEdgePhiIntPhiIntPerQuad(pd.N, pd.basesOnQuad)
    pd.hatRoffdiagOnQuad = B.integrateRefEdgePhiIntPhiExtPerQuad(pd.N, pd.basesOnQuad)
    pd.globM = A.assembleMatElemPhiPhi(g, pd.hatM)
    pd.globMDiscTaylor = LM.assembleMatElemPhiDiscPhiTaylor(g, pd.N, pd.basesOnQuad)
    return pd


def project_q0t(pd, dataQ0T, qOrd):
    """core/projectDataQ0T2DataDisc.m with refElemPhiPhi = I: sum_q W_q data_q phi_i(q)."""
    qOrd = max(qOrd, 1)
    _, _, W = B.quadRule2D(qOrd)
    return dataQ0T @ (W[:, None] * pd.basesOnQuad.phi2D[qOrd][:, :pd.N])


def project_func(pd, f, qOrd):
    """projectFuncCont2DataDisc with hatM = I."""
    qOrd = max(qOrd, 1)
    Q1, Q2, W = B.quadRule2D(qOrd)
    F = f(G.mapRef2Phy(pd.g, 0, Q1, Q2), G.mapRef2Phy(pd.g, 1, Q1, Q2))
    return F @ (W[:, None] * pd.basesOnQuad.phi2D[qOrd][:, :pd.N])


def at_q0t(pd, dataDisc):
    """dataDisc * phi2D{max(2p,1)}': values at the volume quadrature points."""
    return dataDisc @ pd.basesOnQuad.phi2D[max(2 * pd.p, 1)][:, :pd.N].T


def limit(pd, conc):
    """applySlopeLimiterDisc with the linear limiter and zero Dirichlet data (minMaxV0T too)."""
    zeroD = np.zeros((pd.K, 3))
    return LM.applySlopeLimiterDisc(pd.g, conc, pd.g.markV0TbdrD, zeroD, pd.globM, pd.globMDiscTaylor,
                                    pd.basesOnQuad, 'linear')


def compute_mask(mm, tol):
    """core/computeMask.m, 'vertex-based'."""
    mn, mx = mm
    return np.max(mx - mn, axis=1) >= tol


def initializeProblem(pd):
    p = pd.p
    pd.h0Disc = project_func(pd, lambda x1, x2: pd.hCont(0, x1, x2), 2 * p + 1)
    hQ0T = at_q0t(pd, pd.h0Disc)
    pd.cDisc, pd.concDisc, pd.mask = [], [], []
    for s in range(pd.numSpecies):
        cH = project_func(pd, pd.cH0Cont[s], 2 * p + 1)
        conc = project_q0t(pd, at_q0t(pd, cH) / hQ0T, 2 * p)
        conc, mm = limit(pd, conc)
        cH = project_q0t(pd, at_q0t(pd, conc) * hQ0T, 2 * p)
        pd.cDisc.append(cH)
        pd.concDisc.append(conc)
        pd.mask.append(compute_mask(mm, pd.maskTol) if pd.isMask else np.ones(pd.K, dtype=bool))
    pd.isFinished = False
    return pd


def masked_operator(pd, uHDisc, vHDisc, vN, mask):
    """sysA = -G1 - G2 + R over the active elements (K_e N x K_e N)."""
    g, N = pd.g, pd.N
    Ke = int(mask.sum())
    hatG = pd.hatG
    G1 = sp.csr_matrix((Ke * N, Ke * N))
    G2 = sp.csr_matrix((Ke * N, Ke * N))
    B_ = g.B[mask]
    for l in range(N):
        G1 = G1 + sp.kron(sp.diags(uHDisc[mask, l] * B_[:, 1, 1]), hatG[:, :, l, 0]) \
                - sp.kron(sp.diags(uHDisc[mask, l] * B_[:, 1, 0]), hatG[:, :, l, 1])
        G2 = G2 - sp.kron(sp.diags(vHDisc[mask, l] * B_[:, 0, 1]), hatG[:, :, l, 0]) \
                + sp.kron(sp.diags(vHDisc[mask, l] * B_[:, 0, 0]), hatG[:, :, l, 1])
    # upwind flux, masked branch with area factors (core/assembleMatEdgePhiPhiValUpwind.m,
    # _withAreaE0Tbdr): an active element's outflow across edge nn counts if an active element
    # lies across it or the edge is on the boundary
    R_ = sp.csr_matrix((Ke * N, Ke * N))
    val = vN[mask]
    for nn in range(3):
        area = g.areaE0TbdrNotN[nn][mask]
        mk = [g.markE0TE0T[nn][q].tocsr()[mask][:, mask] for q in range(3)]
        anyN = np.asarray((mk[0] + mk[1] + mk[2]).sum(axis=1)).ravel() > 0
        markElemEdges = anyN | (g.idE0T[mask, nn] != 0)
        for r in range(val.shape[2]):
            v = val[:, nn, r]
            R_ = R_ + sp.kron(sp.diags(area * v * (markElemEdges & (v > 0))), pd.hatRdiagOnQuad[:, :, nn, r],
                              format='csr')
        for q in range(3):
            RknTimesVal = sp.csr_matrix((Ke * N, N))
            for r in range(val.shape[2]):
                v = val[:, nn, r]
                RknTimesVal = RknTimesVal + sp.kron(sp.csr_matrix((area * v * (v < 0))[:, None]),
                                                    pd.hatRoffdiagOnQuad[:, :, nn, q, r], format='csr')
            R_ = R_ + A.kronVec(mk[q], RknTimesVal)
    return (-G1 - G2 + R_).tocsr()


def solveStep(pd, nStep):
    """transport/solveStep.m with the sub-steps of preprocessSubStep.m / solveSubStep.m."""
    K, N, p = pd.K, pd.N, pd.p
    t, omega = A.rungeKuttaExplicit(pd.ordRK, pd.tau, (nStep - 1) * pd.tau)
    cH0 = [c.copy() for c in pd.cDisc]
    cH = [c.copy() for c in pd.cDisc]
    conc = [c.copy() for c in pd.concDisc]
    detJ = 2 * pd.g.areaT
    mms = [None] * pd.numSpecies
    for i in range(len(t)):
        ti = t[i]
        uHDisc = project_func(pd, lambda x1, x2: pd.uHCont(ti, x1, x2), 2 * p)
        vHDisc = project_func(pd, lambda x1, x2: pd.vHCont(ti, x1, x2), 2 * p)
        vN = A.computeFuncContNuOnQuadEdge(pd.g, lambda x1, x2: pd.uHCont(ti, x1, x2),
                                           lambda x1, x2: pd.vHCont(ti, x1, x2), 2 * p + 1)
        hQ0T = at_q0t(pd, project_func(pd, lambda x1, x2: pd.hCont(ti, x1, x2), 2 * p))
        for s in range(pd.numSpecies):
            adv = np.zeros(K * N)
            m = pd.mask[s]
            if m.any():
                sysA = masked_operator(pd, uHDisc, vHDisc, vN, m)
                ind = np.repeat(m, N)
                adv[ind] = sysA @ conc[s][m].reshape(-1)
            cDot = (-adv).reshape(K, N) / detJ[:, None]          # globM = 2|T| I
            cH[s] = omega[i] * cH0[s] + (1 - omega[i]) * (cH[s] + pd.tau * cDot)
            c = project_q0t(pd, at_q0t(pd, cH[s]) / hQ0T, 2 * p)
            c, mms[s] = limit(pd, c)
            conc[s] = c
            cH[s] = project_q0t(pd, at_q0t(pd, c) * hQ0T, 2 * p)
    pd.cDisc, pd.concDisc = cH, conc
    for s in range(pd.numSpecies):      # transport/postprocessStep.m
        if pd.isMask:
            pd.mask[s] = compute_mask(mms[s], pd.maskTol)
    return pd


def main(problemData=None, **kwargs):
    pd = Struct(problemData or {})
    pd.update(kwargs)
    pd.problemName = 'transport'
    for f in (configureProblem, preprocessProblem, initializeProblem):
        pd = f(pd)
    for n in range(1, pd.numSteps + 1):
        solveStep(pd, n)
    return pd
