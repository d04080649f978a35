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
from . import matfree as MF
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


# ---------------------------------------------------------------------------------------------
# The limited scheme (linear vertex-based limiter): the limiter is piecewise rational in its
# input; with its discrete choices frozen (the vertex whose factor is the element's alpha, the
# branch of core/computeVertexBasedLimiter.m:78-106 taken there, the clip, and which element of
# the vertex patch holds the extreme, or the Dirichlet data), it is differentiable.  Ties go to
# the first vertex and to the lowest element index; Dirichlet data wins a tie with an element.
# The vector-Jacobian product is written in the reference's Taylor basis
# (core/applySlopeLimiterTaylorLinear.m:108-122 through core/projectDataDisc2DataTaylor.m and
# core/projectDataTaylor2DataDisc.m): dJ/dx = P^T (dlimit/dcT)^T P^-T dJ/dout, P = MDT^-1 M.
TOL = 1.e-8


def patch_extremes(mf, val, markV0TbdrD, dataV0T):
    """Per (element, local vertex): patch min / max as the forward computes them (with the
    reference's shift) and their sources: the element index, or -1 for Dirichlet data."""
    g = mf.pd.g
    mn, mx = mf.patch_minmax(val, markV0TbdrD, dataV0T)
    ptr, idx = mf.ptr, mf.idx
    nV = len(ptr) - 1
    amin = np.empty(nV, dtype=np.int64)
    amax = np.empty(nV, dtype=np.int64)
    for v in range(nV):
        e = np.sort(idx[ptr[v]:ptr[v + 1]])
        vv = val[e]
        amin[v] = e[np.argmin(vv)]      # first (lowest index) attaining the extreme
        amax[v] = e[np.argmax(vv)]
    srcMin = amin[g.V0T].copy()
    srcMax = amax[g.V0T].copy()
    valD = np.full(g.V0T.shape, np.nan)
    valD[markV0TbdrD] = dataV0T[markV0TbdrD]
    hasD = ~np.isnan(valD)
    srcMin[hasD & (valD <= val[amin[g.V0T]])] = -1
    srcMax[hasD & (valD >= val[amax[g.V0T]])] = -1
    return mn, mx, srcMin, srcMax


def limiter_choices(mf, cT, markV0TbdrD, dataV0T):
    """alpha and the frozen choices of the linear limiter on Taylor coefficients cT."""
    phiV = mf.pd.basesOnQuad.phiTaylorV0T
    K = cT.shape[0]
    cbar = cT[:, 0]
    v = cbar[:, None] + cT[:, 1:2] * phiV[:, :, 1] + cT[:, 2:3] * phiV[:, :, 2]
    mn, mx, sMin, sMax = patch_extremes(mf, cbar, markV0TbdrD, dataV0T)
    dV, dMin, dMax = v - cbar[:, None], mn - cbar[:, None], mx - cbar[:, None]
    neg = dV < dMin + TOL
    pos = dV > dMax - TOL
    a = np.ones_like(dV)
    raw = np.full_like(dV, np.nan)
    with np.errstate(divide='ignore', invalid='ignore'):
        raw[neg] = dMin[neg] / (dV[neg] - TOL)
        raw[pos] = dMax[pos] / (dV[pos] + TOL)
    m = neg | pos
    a[m] = np.fmax(0, np.fmin(1, raw[m]))
    alpha = np.fmin(np.fmin(a[:, 0], a[:, 1]), a[:, 2])
    ns = np.argmax(a == alpha[:, None], axis=1)          # first vertex attaining alpha
    r = np.arange(K)
    isPos, isNeg = pos[r, ns], neg[r, ns] & ~pos[r, ns]
    den = np.where(isPos, dV[r, ns] + TOL, dV[r, ns] - TOL)
    dm = np.where(isPos, dMax[r, ns], dMin[r, ns])
    src = np.where(isPos, sMax[r, ns], sMin[r, ns])
    rr = raw[r, ns]
    active = (isPos | isNeg) & (alpha < 1) & (rr > 0) & (rr < 1)   # alpha varies with the data here
    mval = np.where(isPos, mx[r, ns], mn[r, ns])
    return dict(alpha=alpha, ns=ns, den=den, dm=dm, src=src, active=active, isPos=isPos,
                mval=mval, phi1=phiV[r, ns, 1], phi2=phiV[r, ns, 2])


def limit_frozen(cT, ch):
    """The linear limiter with the choices ch held fixed (a smooth function of cT): the
    derivative that limiter_vjp_taylor transposes."""
    alpha = ch['alpha'].copy()
    act = ch['active']
    m = np.where(ch['src'] >= 0, cT[np.maximum(ch['src'], 0), 0], ch['mval'])
    dV = cT[:, 1] * ch['phi1'] + cT[:, 2] * ch['phi2']
    den = np.where(ch['isPos'], dV + TOL, dV - TOL)
    alpha[act] = ((m - cT[:, 0]) / den)[act]
    out = cT.copy()
    lim = ch['alpha'] < 1
    out[lim, 1] = alpha[lim] * cT[lim, 1]
    out[lim, 2] = alpha[lim] * cT[lim, 2]
    out[lim, 3:] = 0.0
    return out


def limiter_vjp_taylor(cT, ch, lamL):
    """(d limitTaylor / d cT)^T lamL for the linear limiter with frozen choices ch."""
    alpha = ch['alpha']
    lim = alpha < 1
    g = lamL.copy()
    g[lim, 1] = alpha[lim] * lamL[lim, 1]
    g[lim, 2] = alpha[lim] * lamL[lim, 2]
    g[lim, 3:] = 0.0
    s = lamL[:, 1] * cT[:, 1] + lamL[:, 2] * cT[:, 2]        # dJ / d alpha
    act = ch['active']
    den, dm = ch['den'], ch['dm']
    g[act, 0] -= s[act] / den[act]                            # d dm / d cbar = -1
    g[act, 1] -= s[act] * dm[act] / den[act] ** 2 * ch['phi1'][act]
    g[act, 2] -= s[act] * dm[act] / den[act] ** 2 * ch['phi2'][act]
    nl = act & (ch['src'] >= 0)
    np.add.at(g[:, 0], ch['src'][nl], s[nl] / den[nl])        # the extreme's element
    return g


class LimitedAdjointOracle:
    """Forward run and reverse sweep of the scheme with the linear limiter (solution limiting,
    and time-derivative limiting at p >= 2, advection/solveSubStep.m:69-98)."""

    def __init__(self, **kw):
        kw = dict(kw)
        kw.setdefault('testcase', 'adjoint')
        kw['isSlopeLim'] = True
        kw['typeSlopeLim'] = 'linear'
        self.op = AdjointOracle.__new__(AdjointOracle)
        AdjointOracle.__init__(self.op, **dict(kw, isSlopeLim=False))
        pd = adv.Struct(kw)
        pd.problemName = 'advection'
        for f in (adv.configureProblem, adv.preprocessProblem, adv.initializeProblem):
            pd = f(pd)
        self.pd = pd
        self.mf = MF.MatFree(pd)
        self.P = np.linalg.solve(self.mf.MDT, self.mf.M)        # Taylor = P modal
        self.Pinv = np.linalg.solve(self.mf.M, self.mf.MDT)
        self.omega = self.op.omega

    def set_modes(self, velocities):
        self.op.set_modes(velocities)

    def T(self, c):
        return np.einsum('kij,kj->ki', self.P, c)

    def Tinv(self, cT):
        return np.einsum('kij,kj->ki', self.Pinv, cT)

    def forward(self, c0, nSteps, frozen=False):
        """frozen=True replays the choices of the last unfrozen run (for finite differences of
        the differentiable branch)."""
        pd, g = self.pd, self.pd.g
        K, N = pd.K, pd.N
        tau = pd.tau
        none = np.zeros((K, 3), dtype=bool)
        cD = np.zeros((K, 3))                                   # the adjoint case: c_D = 0
        c = np.asarray(c0, dtype=np.float64).reshape(K, N).copy()
        if not frozen:
            self.rec, self.choices = [], []
        for n in range(nSteps):
            cn = c
            stages, chs = [], []
            for s, w in enumerate(self.omega):
                cdot = self.op.A(c.reshape(-1)).reshape(K, N)
                cdotRaw = cdot
                chd = None
                if pd.p > 1:
                    cT = self.T(cdot)
                    if frozen:
                        cTL = limit_frozen(cT, self.choices[n][s][0])
                    else:
                        chd = limiter_choices(self.mf, cT, none, np.full((K, 3), np.nan))
                        cTL = self.mf.limit_taylor(cT, none, np.full((K, 3), np.nan), 'linear')
                    cdot = self.Tinv(cTL + np.einsum('kij,kj->ki', self.mf.Mcorr, cT - cTL))
                y = w * cn + (1 - w) * (c + tau * cdot)
                if frozen:
                    c = self.Tinv(limit_frozen(self.T(y), self.choices[n][s][1]))
                else:
                    stages.append((c, cdotRaw, y))
                    chs.append((chd, limiter_choices(self.mf, self.T(y), g.markV0TbdrD, cD)))
                    c = self.mf.limit_disc(y, g.markV0TbdrD, cD)
            if not frozen:
                self.rec.append(stages)
                self.choices.append(chs)
        return c

    def backward(self, dJdcT):
        pd, g = self.pd, self.pd.g
        K, N = pd.K, pd.N
        tau = pd.tau
        none = np.zeros((K, 3), dtype=bool)
        cD = np.zeros((K, 3))
        lam = np.asarray(dJdcT, dtype=np.float64).reshape(K, N).copy()
        gth = np.zeros(len(self.op.modes))
        PinvT = lambda x: np.einsum('kji,kj->ki', self.Pinv, x)
        PT = lambda x: np.einsum('kji,kj->ki', self.P, x)
        for stages in reversed(self.rec):
            mu, accn = lam, np.zeros_like(lam)
            for s in reversed(range(len(self.omega))):
                w = self.omega[s]
                cs, cdotRaw, y = stages[s]
                # solution limiter
                yT = self.T(y)
                ch = limiter_choices(self.mf, yT, g.markV0TbdrD, cD)
                muY = PT(limiter_vjp_taylor(yT, ch, PinvT(mu)))
                accn += w * muY
                lamDot = (1 - w) * tau * muY
                # time-derivative limiter with the Taylor mass correction
                if pd.p > 1:
                    dT = self.T(cdotRaw)
                    chd = limiter_choices(self.mf, dT, none, np.full((K, 3), np.nan))
                    lT = PinvT(lamDot)
                    McT = np.einsum('kji,kj->ki', self.mf.Mcorr, lT)
                    lamDot = PT(McT + limiter_vjp_taylor(dT, chd, lT - McT))
                flat = lamDot.reshape(-1)
                if self.op.modes:
                    Mmu = self.op.lu.solve(flat)
                    gth += np.array([Mmu @ (Bm @ cs.reshape(-1)) for Bm in self.op.modes])
                mu = (1 - w) * muY + self.op.AT(flat).reshape(K, N)
            lam = accn + mu
        return lam, gth


# ---------------------------------------------------------------------------------------------
# The strict limiter (core/applySlopeLimiterTaylorStrict.m:111-150) with its choices frozen.
# The forward limits the orders o = p..1 in turn, each on the data already limited: a
# sub-limiter's vertex values are the degree-(p - o + 1) reconstruction about a derivative of
# order o - 1, and every DOF of degree >= o is scaled by the order's factor.  With the choices
# held (per order and element: the winning sub-limiter, vertex and branch, and the source of the
# patch extreme: an element, the element's own vertex value above order 1, or boundary data),
# the run is a smooth function of its input, and central differences of that replay give the
# exact directional derivative of the piece the run sits on, with no switch to cross.  That is
# what the GPU's strict-limiter adjoint is checked against.


def strict_choices(mf, cT, markV0TbdrD, dataV0T):
    """Runs the strict limiter on Taylor coefficients cT as the forward does (matfree.limit_taylor)
    and returns (limited, choices): per order o, alpha_o and the winner of each element (the
    first sub-limiter and vertex attaining alpha_o), whether alpha_o varies with the data there
    (a branch ratio strictly inside (0, 1)), and the extreme's source (patch_extremes)."""
    from . import basis as B
    from . import limiter as L
    phiV = mf.pd.basesOnQuad.phiTaylorV0T
    K, N = cT.shape
    p = B.p_of_N(N)
    r = np.arange(K)
    lim = cT.copy()
    chs = {}
    for o in range(p, 0, -1):
        facs, raws, dms, poss, srcs, mvals, subs = [], [], [], [], [], [], []
        aO = np.ones(K)
        for i in range(1, o + 1):
            ind = L.mult2ind(np.array([o - i, i - 1])[None, :] + L.multiindex(p - o + 1))
            v = A.computeFuncDiscAtPoints(lim[:, ind], phiV[:, :, 0:ind.size])
            data = v if o > 1 else dataV0T
            aO = np.fmin(aO, mf.vertex_limiter(lim[:, ind[0]], v, markV0TbdrD, data))
            c = lim[:, ind[0]]
            mn, mx, sMin, sMax = patch_extremes(mf, c, markV0TbdrD, data)
            dV, dMin, dMax = v - c[:, None], mn - c[:, None], mx - c[:, None]
            neg = dV < dMin + TOL
            pos = dV > dMax - TOL
            with np.errstate(divide='ignore', invalid='ignore'):
                raw = np.where(pos, dMax / (dV + TOL), np.where(neg, dMin / (dV - TOL), np.nan))
            for n in range(3):
                br = neg[:, n] | pos[:, n]
                facs.append(np.where(br, np.fmax(0, np.fmin(1, raw[:, n])), 1.0))
                raws.append(raw[:, n])
                dms.append(np.where(pos[:, n], dMax[:, n], dMin[:, n]))
                poss.append(pos[:, n])
                srcs.append(np.where(pos[:, n], sMax[:, n], sMin[:, n]))
                mvals.append(np.where(pos[:, n], mx[:, n], mn[:, n]))
                subs.append(i)
        F = np.stack(facs, axis=1)
        w = np.argmax(F == aO[:, None], axis=1)                    # first winner
        pick = lambda arrs: np.stack(arrs, axis=1)[r, w]
        rw = pick(raws)
        chs[o] = dict(alpha=aO, i=np.array(subs)[w], n=w % 3, isPos=pick(poss), src=pick(srcs),
                      mval=pick(mvals), active=(aO < 1) & (rw > 0) & (rw < 1))
        lim[:, o * (o + 1) // 2:] = aO[:, None] * lim[:, o * (o + 1) // 2:]
    return lim, chs


def strict_frozen(mf, cT, chs):
    """The strict limiter with the choices chs held: on the elements where alpha_o varies with
    the data it is the winner's ratio (ext - c) / (v_n - c +- tol), recomputed from cT; elsewhere
    the recorded factor."""
    from . import basis as B
    from . import limiter as L
    phiV = mf.pd.basesOnQuad.phiTaylorV0T
    K, N = cT.shape
    p = B.p_of_N(N)
    lim = cT.copy()
    for o in range(p, 0, -1):
        ch = chs[o]
        alpha = ch['alpha'].astype(cT.dtype)
        for i in range(1, o + 1):
            sel = np.nonzero(ch['active'] & (ch['i'] == i))[0]
            if sel.size == 0:
                continue
            ind = L.mult2ind(np.array([o - i, i - 1])[None, :] + L.multiindex(p - o + 1))
            n = ch['n'][sel]
            v = np.sum(lim[sel][:, ind] * phiV[sel, n, 0:ind.size], axis=1)
            c = lim[sel, ind[0]]
            src = ch['src'][sel]
            own = v if o > 1 else ch['mval'][sel]                    # Dirichlet: own value / data
            ext = np.where(src >= 0, cT[np.maximum(src, 0), ind[0]], own)
            den = (v - c) + np.where(ch['isPos'][sel], TOL, -TOL)
            alpha[sel] = (ext - c) / den
        lim[:, o * (o + 1) // 2:] = alpha[:, None] * lim[:, o * (o + 1) // 2:]
    return lim


def hier_choices(mf, cT, markV0TbdrD, dataV0T):
    """The hierarchical vertex limiter (core/applySlopeLimiterTaylorHierarchicalVertex.m:124-168)
    on Taylor coefficients cT, as the forward runs it (matfree.limit_taylor), with its choices:
    per order o the factor alpha_o of its sub-limiters (linear reconstructions of the input) and
    the winner as in strict_choices, and per degree d the order whose alpha holds the running
    maximum A_d = max(alpha_p, ..., alpha_d) (the first, highest, on ties)."""
    from . import basis as B
    from . import limiter as L
    phiV = mf.pd.basesOnQuad.phiTaylorV0T
    K, N = cT.shape
    p = B.p_of_N(N)
    r = np.arange(K)
    lim = np.zeros_like(cT)
    lim[:, 0] = cT[:, 0]
    run = np.zeros(K)
    runOrd = np.full(K, p)
    chs = {'runOrd': {}}
    for o in range(p, 0, -1):
        facs, raws, poss, srcs, mvals, subs = [], [], [], [], [], []
        aO = np.ones(K)
        for i in range(1, o + 1):
            ind = L.mult2ind(np.array([o - i, i - 1])[None, :] + L.multiindex(1))
            v = A.computeFuncDiscAtPoints(cT[:, ind], phiV[:, :, 0:3])
            data = v if o > 1 else dataV0T
            aO = np.fmin(aO, mf.vertex_limiter(cT[:, ind[0]], v, markV0TbdrD, data))
            c = cT[:, ind[0]]
            mn, mx, sMin, sMax = patch_extremes(mf, c, markV0TbdrD, data)
            dV, dMin, dMax = v - c[:, None], mn - c[:, None], mx - c[:, None]
            neg = dV < dMin + TOL
            pos = dV > dMax - TOL
            with np.errstate(divide='ignore', invalid='ignore'):
                raw = np.where(pos, dMax / (dV + TOL), np.where(neg, dMin / (dV - TOL), np.nan))
            for n in range(3):
                br = neg[:, n] | pos[:, n]
                facs.append(np.where(br, np.fmax(0, np.fmin(1, raw[:, n])), 1.0))
                raws.append(raw[:, n])
                poss.append(pos[:, n])
                srcs.append(np.where(pos[:, n], sMax[:, n], sMin[:, n]))
                mvals.append(np.where(pos[:, n], mx[:, n], mn[:, n]))
                subs.append(i)
        F = np.stack(facs, axis=1)
        w = np.argmax(F == aO[:, None], axis=1)
        pick = lambda arrs: np.stack(arrs, axis=1)[r, w]
        rw = pick(raws)
        chs[o] = dict(alpha=aO, i=np.array(subs)[w], n=w % 3, isPos=pick(poss), src=pick(srcs),
                      mval=pick(mvals), active=(aO < 1) & (rw > 0) & (rw < 1))
        runOrd = np.where((o == p) | (aO > run), o, runOrd)
        run = np.fmax(run, aO)
        chs['runOrd'][o] = runOrd.copy()
        d = np.arange(o * (o + 1) // 2, (o + 1) * (o + 2) // 2)
        lim[:, d] = run[:, None] * cT[:, d]
    return lim, chs


def hier_frozen(mf, cT, chs):
    """The hierarchical limiter with the choices chs held: each order's factor is its winner's
    ratio where it varies with the data (else the recorded factor), computed from the input cT,
    and degree d is scaled by the factor of the order recorded as holding A_d."""
    from . import basis as B
    from . import limiter as L
    phiV = mf.pd.basesOnQuad.phiTaylorV0T
    K, N = cT.shape
    p = B.p_of_N(N)
    r = np.arange(K)
    fac = {}
    for o in range(p, 0, -1):
        ch = chs[o]
        alpha = ch['alpha'].astype(cT.dtype)
        for i in range(1, o + 1):
            sel = np.nonzero(ch['active'] & (ch['i'] == i))[0]
            if sel.size == 0:
                continue
            ind = L.mult2ind(np.array([o - i, i - 1])[None, :] + L.multiindex(1))
            n = ch['n'][sel]
            v = np.sum(cT[sel][:, ind] * phiV[sel, n, 0:3], axis=1)
            c = cT[sel, ind[0]]
            src = ch['src'][sel]
            own = v if o > 1 else ch['mval'][sel]
            ext = np.where(src >= 0, cT[np.maximum(src, 0), ind[0]], own)
            den = (v - c) + np.where(ch['isPos'][sel], TOL, -TOL)
            alpha[sel] = (ext - c) / den
        fac[o] = alpha
    lim = np.zeros_like(cT)
    lim[:, 0] = cT[:, 0]
    for o in range(p, 0, -1):
        F = np.stack([fac[q] for q in range(1, p + 1)], axis=1)      # column q - 1: order q
        A_d = F[r, chs['runOrd'][o] - 1]
        d = np.arange(o * (o + 1) // 2, (o + 1) * (o + 2) // 2)
        lim[:, d] = A_d[:, None] * cT[:, d]
    return lim


class LimiterReplayOracle:
    """Forward run of the scheme with the strict (or, typ='hierarch_vert', the hierarchical
    vertex) limiter (solution limiting, and time-derivative
    limiting with the Taylor mass correction at p >= 2, advection/solveSubStep.m:69-98); with
    frozen=True the run replays the choices of the last unfrozen run.  The replay is rational in
    c0 and takes complex input: Im J(c0 + i h d) / h is the exact directional derivative of the
    piece (complex step, Squire and Trapp 1998), also next to the poles of dm / den where a
    winner's v_n - c is of the order of tol and real differences need h below |den|."""

    def __init__(self, typ='strict', **kw):
        kw = dict(kw)
        kw.setdefault('testcase', 'adjoint')
        kw['isSlopeLim'] = True
        kw['typeSlopeLim'] = typ
        self.choose, self.frozen = {'strict': (strict_choices, strict_frozen),
                                    'hierarch_vert': (hier_choices, hier_frozen)}[typ]
        self.op = AdjointOracle.__new__(AdjointOracle)
        AdjointOracle.__init__(self.op, **dict(kw, isSlopeLim=False))
        pd = adv.Struct(kw)
        pd.problemName = 'advection'
        for f in (adv.configureProblem, adv.preprocessProblem, adv.initializeProblem):
            pd = f(pd)
        self.pd = pd
        self.mf = MF.MatFree(pd)
        self.P = np.linalg.solve(self.mf.MDT, self.mf.M)
        self.Pinv = np.linalg.solve(self.mf.M, self.mf.MDT)
        self.omega = self.op.omega

    def T(self, c):
        return np.einsum('kij,kj->ki', self.P, c)

    def Tinv(self, cT):
        return np.einsum('kij,kj->ki', self.Pinv, cT)

    def forward(self, c0, nSteps, frozen=False):
        pd, g = self.pd, self.pd.g
        K, N = pd.K, pd.N
        tau = pd.tau
        nan3 = np.full((K, 3), np.nan)
        cD = np.zeros((K, 3))                                   # the adjoint case: c_D = 0
        c = np.array(c0, dtype=np.complex128 if np.iscomplexobj(c0) else np.float64).reshape(K, N)
        if not frozen:
            self.choices = []
        def opA(v):   # the real operator on a real or complex state
            if np.iscomplexobj(v):
                return self.op.A(v.real.copy()) + 1j * self.op.A(v.imag.copy())
            return self.op.A(v)
        for n in range(nSteps):
            cn = c
            chs = []
            for s, w in enumerate(self.omega):
                cdot = opA(c.reshape(-1)).reshape(K, N)
                chd = None
                if pd.p > 1:
                    cT = self.T(cdot)
                    if frozen:
                        cTL = self.frozen(self.mf, cT, self.choices[n][s][0])
                    else:   # the Dirichlet vertices with no data (advection/solveSubStep.m:76)
                        cTL, chd = self.choose(self.mf, cT, g.markV0TbdrD, nan3)
                    cdot = self.Tinv(cTL + np.einsum('kij,kj->ki', self.mf.Mcorr, cT - cTL))
                y = w * cn + (1 - w) * (c + tau * cdot)
                yT = self.T(y)
                if frozen:
                    c = self.Tinv(self.frozen(self.mf, yT, self.choices[n][s][1]))
                else:
                    yL, chs_y = self.choose(self.mf, yT, g.markV0TbdrD, cD)
                    chs.append((chd, chs_y))
                    c = self.Tinv(yL)
            if not frozen:
                self.choices.append(chs)
        return c
