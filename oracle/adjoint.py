"""Oracle of the discrete adjoint (test infrastructure; see ``oracle/__init__.py``).

The reference has no adjoint.  This file builds the reference's own assembled operators of one
explicit stage and differentiates the time loop with them:
    cDot = M^-1 (G1 + G2 - R) c = A c        advection/solveSubStep.m:62-66 (sources zero)
    c^(s+1) = w_s c^n + (1 - w_s) (c^(s) + tau A c^(s))          advection/solveSubStep.m:83
with G1, G2 from core/assembleMatElemDphiPhiFuncDisc.m:181-202, R from
core/assembleMatEdgePhiPhiValUpwind.m:261-299 and M from core/assembleMatElemPhiPhi.m:88-100.
The reverse sweep applies the transposed sparse matrices (SciPy):
    dJ/dc^n  += w_s mu,     mu <- (1 - w_s) mu + (1 - w_s) tau A^T mu,
and the gradient with respect to the coefficients theta_m of u = sum_m theta_m u_m adds
(1 - w_s) tau mu^T A_m c^(s), where A_m is the operator assembled with mode m's velocity and the
upwind choice of the base velocity (the flux is piecewise linear in u).
"""
import numpy as np
import scipy.sparse as sp
from scipy.sparse.linalg import splu

from . import advection as adv
from . import assembly as A
from . import testcases as TC


def assemble_flux_frozen(g, markE0Tbdr, hatRdiag, hatRoffdiag, valOnQuad, maskOnQuad):
    """R of core/assembleMatEdgePhiPhiValUpwind.m:261-299 with the upwind selection (v > 0 own
    trace, v < 0 neighbour trace) taken from maskOnQuad and the values from valOnQuad."""
    K, _, R = valOnQuad.shape
    N = hatRdiag.shape[0]
    ret = sp.csr_matrix((K * N, K * N))
    for nn in range(3):
        mk = g.markE0TE0T[nn]
        anyN = np.asarray((mk[0] + mk[1] + mk[2]).sum(axis=1)).ravel() > 0
        markElemEdges = anyN | (g.idE0T[:, nn] != 0)
        Rkn = markE0Tbdr[:, nn] * g.areaE0T[:, nn]
        for r in range(R):
            v, m = valOnQuad[:, nn, r], maskOnQuad[:, nn, r]
            d = Rkn * v * (markElemEdges & (m > 0))
            ret = ret + sp.kron(sp.diags(d), hatRdiag[:, :, nn, r], format='csr')
        for np_ in range(3):
            RknTimesVal = sp.csr_matrix((K * N, N))
            for r in range(R):
                v, m = valOnQuad[:, nn, r], maskOnQuad[:, nn, r]
                s = sp.csr_matrix((Rkn * v * (m < 0))[:, None])
                RknTimesVal = RknTimesVal + sp.kron(s, hatRoffdiag[:, :, nn, np_, r], format='csr')
            ret = ret + A.kronVec(g.markE0TE0T[nn][np_], RknTimesVal)
    return ret


def velocity_data(pd, u1, u2):
    """u1Disc, u2Disc (order 2p) and vNormalOnQuadEdge (order 2p+1) of a velocity
    (advection/preprocessSubStep.m:72-79)."""
    g, p = pd.g, pd.p
    u1Disc = A.projectFuncCont2DataDisc(g, lambda x1, x2: u1(0, x1, x2), 2 * p, pd.hatM, pd.basesOnQuad)
    u2Disc = A.projectFuncCont2DataDisc(g, lambda x1, x2: u2(0, x1, x2), 2 * p, pd.hatM, pd.basesOnQuad)
    vN = A.computeFuncContNuOnQuadEdge(g, lambda x1, x2: u1(0, x1, x2), lambda x1, x2: u2(0, x1, x2), 2 * p + 1)
    return u1Disc, u2Disc, vN


def stage_matrix(pd, u1Disc, u2Disc, vN, vMask):
    """G1 + G2 - R (sparse), R with the upwind choice of vMask."""
    G = A.assembleMatElemDphiPhiFuncDisc(pd.g, pd.hatG, u1Disc, u2Disc)
    R = assemble_flux_frozen(pd.g, ~pd.g.markE0TbdrN, pd.hatRdiagOnQuad, pd.hatRoffdiagOnQuad, vN, vMask)
    return (G[0] + G[1] - R).tocsr()


class AdjointOracle:
    """Forward run and reverse sweep of the unlimited scheme with the assembled operators."""

    def __init__(self, **kw):
        kw = dict(kw)
        kw.setdefault('testcase', 'adjoint')
        kw['isSlopeLim'] = False
        pd = adv.Struct(kw)
        pd.problemName = 'advection'
        for f in (adv.configureProblem, adv.preprocessProblem, adv.initializeProblem):
            pd = f(pd)
        self.pd = pd
        self.lu = splu(pd.globM.tocsc())
        u1Disc, u2Disc, vN = velocity_data(pd, pd.u1Cont, pd.u2Cont)
        self.vN = vN
        self.B = stage_matrix(pd, u1Disc, u2Disc, vN, vN)
        self.omega = A.rungeKuttaExplicit(pd.ordRK, pd.tau, 0.0)[1]   # (t, omega)
        self.modes = []

    def set_theta(self, theta):
        """Base velocity u = sum_m theta_m u_m (with its own upwind choice)."""
        u1, u2 = TC.streamfunction_velocity([k for k, _ in TC.ADJOINT_MODES], [l for _, l in TC.ADJOINT_MODES],
                                            np.asarray(theta, dtype=np.float64))
        u1Disc, u2Disc, vN = velocity_data(self.pd, u1, u2)
        self.vN = vN
        self.B = stage_matrix(self.pd, u1Disc, u2Disc, vN, vN)

    def set_modes(self, velocities):
        """Mode matrices G1 + G2 - R of each velocity (u1, u2) with the base upwind choice."""
        self.modes = [stage_matrix(self.pd, *velocity_data(self.pd, u1, u2), self.vN) for u1, u2 in velocities]

    def A(self, c):
        return self.lu.solve(self.B @ c)

    def AT(self, mu):
        return self.B.T @ self.lu.solve(mu)        # M is symmetric

    def forward(self, c0, nSteps):
        tau = self.pd.tau
        c = np.asarray(c0, dtype=np.float64).reshape(-1).copy()
        self.stages = []
        for _ in range(nSteps):
            cs = [c]
            for w in self.omega:
                cs.append(w * c + (1 - w) * (cs[-1] + tau * self.A(cs[-1])))
            self.stages.append(cs[:-1])
            c = cs[-1]
        return c.reshape(self.pd.K, self.pd.N)

    def backward(self, dJdcT):
        tau = self.pd.tau
        lam = np.asarray(dJdcT, dtype=np.float64).reshape(-1).copy()
        gth = np.zeros(len(self.modes))
        for cs in reversed(self.stages):
            mu, accn = lam, np.zeros_like(lam)
            for s in reversed(range(len(self.omega))):
                w = self.omega[s]
                coef = (1 - w) * tau
                accn += w * mu
                if self.modes:
                    Mmu = self.lu.solve(mu)
                    gth += coef * np.array([Mmu @ (Bm @ cs[s]) for Bm in self.modes])
                mu = (1 - w) * mu + coef * self.AT(mu)
            lam = accn + mu
        return lam.reshape(self.pd.K, self.pd.N), gth


def mode_velocities():
    return [TC.mode_velocity(m) for m in range(len(TC.ADJOINT_MODES))]
