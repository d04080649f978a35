"""Matrix-free restatement of the advection stage (oracle, large meshes).

Test infrastructure: see ``oracle/__init__.py``.

The same arithmetic as ``oracle.advection`` (which assembles the reference's sparse operators),
applied element by element with numpy batched operations so that meshes with 10^5..10^6
triangles run in minutes:
  * volume term      G_k = sum_l u1_kl (B22 hatG(:,:,l,1) - B21 hatG(:,:,l,2))
                           + u2_kl (B11 hatG(:,:,l,2) - B12 hatG(:,:,l,1))
    (core/assembleMatElemDphiPhiFuncDisc.m:181-202);
  * upwind edge term with the element-centric neighbour map instead of markE0TE0T
    (core/assembleMatEdgePhiPhiValUpwind.m:261-299);
  * block mass solves, Taylor projections and the Taylor mass correction per element
    (advection/solveSubStep.m:62-83, core/projectDataDisc2DataTaylor.m:56-61);
  * vertex patch min/max over a CSR vertex -> element map instead of the K x K masks
    markV0TT0V, with the same global shift of the centroid values
    (core/computeMinMaxV0TElementPatch.m:66-112).
It is checked against the sparse-operator restatement in the tests.
"""
import numpy as np

from . import advection as adv
from . import assembly as A
from . import basis as B
from . import limiter as L


def neighbour_maps(g):
    """nbr[k,n] = element across edge n of k (or -1), nbrEdge[k,n] = its local edge index."""
    K = g.numT
    e = g.E0T
    t0, t1 = g.T0E[e, 0] - 1, g.T0E[e, 1] - 1
    n0, n1 = g.E0E[e, 0] - 1, g.E0E[e, 1] - 1
    me = np.arange(K)[:, None]
    first = t0 == me
    nbr = np.where(first, t1, t0)
    nbrEdge = np.where(first, n1, n0)
    nbrEdge = np.where(nbr >= 0, nbrEdge, -1)
    return nbr.astype(np.int64), nbrEdge.astype(np.int64)


def vertex_csr(V0T, numV):
    """CSR map vertex -> elements containing it (element ids ascending per vertex)."""
    K = V0T.shape[0]
    v = V0T.ravel()
    el = np.repeat(np.arange(K), 3)
    order = np.lexsort((el, v))
    counts = np.bincount(v, minlength=numV)
    ptr = np.concatenate([[0], np.cumsum(counts)])
    return ptr, el[order]


def batched_mass_blocks(g, hatM):
    return g.detJ0T[:, None, None] * hatM[None, :, :]


def taylor_blocks(g, N, bases):
    """Per-element N x N blocks of M_DT (order 2p+1) and M_T (order 2p), as the reference's
    assembleMatElemPhiDiscPhiTaylor / assembleMatElemPhiTaylorPhiTaylor."""
    MDT = L.assembleMatElemPhiDiscPhiTaylor(g, N, bases)
    MT = L.assembleMatElemPhiTaylorPhiTaylor(g, N)
    K = g.numT

    def blocks(Msp):
        Mc = Msp.tocoo()
        out = np.zeros((K, N, N))
        k = Mc.row // N
        out[k, Mc.row % N, Mc.col % N] = Mc.data
        return out
    return blocks(MDT), blocks(MT)


class MatFree:
    """Holds a preprocessed oracle problem and advances it with matrix-free stages."""

    def __init__(self, pd, rounding='lu'):
        """``rounding='inverse'`` applies explicit block inverses instead of LU solves for the
        Taylor projections: the same algebra with different rounding, used to measure how
        sensitive a configuration is to roundoff (the spread that bounds any parity claim)."""
        self.pd = pd
        self.rounding = rounding
        g, N = pd.g, pd.N
        self.nbr, self.nbrEdge = neighbour_maps(g)
        self.ptr, self.idx = vertex_csr(g.V0T, g.numV)
        self.M = batched_mass_blocks(g, pd.hatM)
        if pd.isSlopeLim:
            self.MDT, MT = taylor_blocks(g, N, pd.basesOnQuad)
            d = np.einsum('kii->ki', MT)
            self.Mcorr = MT / d[:, :, None]
        self._ops = None

    # ------------------------------------------------------------------ operators of a stage
    def stage_ops(self, t):
        pd = self.pd
        if self._ops is not None and pd.isTimeIndependentData:
            return self._ops
        g, p, N = pd.g, pd.p, pd.N
        u1 = A.projectFuncCont2DataDisc(g, lambda a, b: pd.u1Cont(t, a, b), 2 * p, pd.hatM, pd.basesOnQuad)
        u2 = A.projectFuncCont2DataDisc(g, lambda a, b: pd.u2Cont(t, a, b), 2 * p, pd.hatM, pd.basesOnQuad)
        f = A.projectFuncCont2DataDisc(g, lambda a, b: pd.fCont(t, a, b), 2 * p, pd.hatM, pd.basesOnQuad)
        vN = A.computeFuncContNuOnQuadEdge(g, lambda a, b: pd.u1Cont(t, a, b),
                                           lambda a, b: pd.u2Cont(t, a, b), 2 * p + 1)
        hG = pd.hatG
        Bm = g.B
        G = (np.einsum('kl,ijl->kij', u1 * Bm[:, 1, 1:2], hG[:, :, :, 0])
             - np.einsum('kl,ijl->kij', u1 * Bm[:, 1, 0:1], hG[:, :, :, 1])
             + np.einsum('kl,ijl->kij', u2 * Bm[:, 0, 0:1], hG[:, :, :, 1])
             - np.einsum('kl,ijl->kij', u2 * Bm[:, 0, 1:2], hG[:, :, :, 0]))
        KD = A.assembleVecEdgePhiIntFuncContVal(g, g.markE0TbdrD, lambda a, b: pd.cDCont(t, a, b),
                                                vN, N, pd.basesOnQuad, pd.qOrd).reshape(-1, N)

        def gNUp(a, b):
            v = pd.gNCont(t, a, b)
            return (v <= 0) * v
        KN = A.assembleVecEdgePhiIntFuncCont(g, g.markE0TbdrN, gNUp, N, pd.basesOnQuad).reshape(-1, N)
        Lv = np.einsum('kij,kj->ki', self.M, f)
        ops = dict(G=G, vN=vN, rhs0=Lv - KD - KN, u1=u1, u2=u2)
        self._ops = ops
        return ops

    def rhs(self, c, ops):
        """L - K_D - K_N + (G1+G2) c - R c for K x N coefficients c."""
        pd, g = self.pd, self.pd.g
        vN = ops['vN']
        out = ops['rhs0'] + np.einsum('kij,kj->ki', ops['G'], c)
        Rd, Ro = pd.hatRdiagOnQuad, pd.hatRoffdiagOnQuad
        R = vN.shape[2]
        markBdr = ~g.markE0TbdrN
        for nn in range(3):
            kp = self.nbr[:, nn]; npn = self.nbrEdge[:, nn]
            interior = kp >= 0
            edgeOk = interior | (g.idE0T[:, nn] != 0)
            area = markBdr[:, nn] * g.areaE0T[:, nn]
            cn = c[np.where(interior, kp, 0)]
            for r in range(R):
                v = vN[:, nn, r]
                dcoef = area * v * (edgeOk & (v > 0))
                out -= dcoef[:, None] * (c @ Rd[:, :, nn, r].T)
                ocoef = area * v * ((v < 0) & interior)
                Roff = Ro[:, :, nn, :, r]                 # N x N x 3 (np)
                out -= ocoef[:, None] * np.einsum('kij,kj->ki', Roff.transpose(2, 0, 1)[np.maximum(npn, 0)], cn)
        return out

    # ------------------------------------------------------------------ limiter pieces
    def to_taylor(self, c):
        if self.rounding == 'inverse':
            if not hasattr(self, '_P'):
                self._P = np.linalg.inv(self.MDT) @ self.M
            return np.einsum('kij,kj->ki', self._P, c)
        return np.linalg.solve(self.MDT, np.einsum('kij,kj->ki', self.M, c)[..., None])[..., 0]

    def from_taylor(self, cT):
        if self.rounding == 'inverse':
            if not hasattr(self, '_Q'):
                self._Q = np.linalg.inv(self.M) @ self.MDT
            return np.einsum('kij,kj->ki', self._Q, cT)
        return np.linalg.solve(self.M, np.einsum('kij,kj->ki', self.MDT, cT)[..., None])[..., 0]

    def patch_minmax(self, valCentroid, markV0TbdrD, dataV0T):
        """computeMinMaxV0TElementPatch over CSR vertex patches."""
        g = self.pd.g
        sPos = abs(np.min(valCentroid)) + 1
        sNeg = abs(np.max(valCentroid)) + 1
        vals = valCentroid[self.idx]
        vmin = np.minimum.reduceat(vals - sNeg, self.ptr[:-1])
        vmax = np.maximum.reduceat(vals + sPos, self.ptr[:-1])
        valD = np.full((g.numT, 3), np.nan)
        valD[markV0TbdrD] = dataV0T[markV0TbdrD]
        mn = np.fmin(vmin[g.V0T] + sNeg, valD)
        mx = np.fmax(vmax[g.V0T] - sPos, valD)
        return mn, mx

    def vertex_limiter(self, valCentroid, valV0T, markV0TbdrD, dataV0T):
        mn, mx = self.patch_minmax(valCentroid, markV0TbdrD, dataV0T)
        dV = valV0T - valCentroid[:, None]
        dMin = mn - valCentroid[:, None]
        dMax = mx - valCentroid[:, None]
        tol = 1.e-8
        markNeg = dV < dMin + tol
        markPos = dV > dMax - tol
        a = np.ones_like(dV)
        with np.errstate(divide='ignore', invalid='ignore'):
            a[markNeg] = np.fmax(0, np.fmin(1, dMin[markNeg] / (dV[markNeg] - tol)))
            a[markPos] = np.fmax(0, np.fmin(1, dMax[markPos] / (dV[markPos] + tol)))
        return np.fmin(np.fmin(a[:, 0], a[:, 1]), a[:, 2])

    def limit_taylor(self, cT, markV0TbdrD, dataV0T, typ):
        pd = self.pd
        phiV = pd.basesOnQuad.phiTaylorV0T
        K, N = cT.shape
        if typ == 'linear':
            valV0T = A.computeFuncDiscAtPoints(cT[:, 0:3], phiV[:, :, 0:3])
            alpha = self.vertex_limiter(cT[:, 0], valV0T, markV0TbdrD, dataV0T)
            return np.concatenate([cT[:, 0:1], alpha[:, None] * cT[:, 1:3],
                                   (alpha == 1)[:, None] * cT[:, 3:]], axis=1)
        p = B.p_of_N(N)
        if typ == 'hierarch_vert':
            lim = np.zeros_like(cT); lim[:, 0] = cT[:, 0]
            alpha = np.zeros(K)
            for o in range(p, 0, -1):
                aO = np.ones(K)
                indDOF = np.arange(o * (o + 1) // 2, (o + 1) * (o + 2) // 2)
                for i in range(1, o + 1):
                    ind = L.mult2ind(np.array([o - i, i - 1])[None, :] + L.multiindex(1))
                    valV0T = A.computeFuncDiscAtPoints(cT[:, ind], phiV[:, :, 0:3])
                    data = valV0T if o > 1 else dataV0T
                    aO = np.fmin(aO, self.vertex_limiter(cT[:, ind[0]], valV0T, markV0TbdrD, data))
                alpha = np.fmax(alpha, aO)
                lim[:, indDOF] = alpha[:, None] * cT[:, indDOF]
            return lim
        if typ == 'strict':
            lim = cT.copy()
            for o in range(p, 0, -1):
                aO = np.ones(K)
                indDOF = np.arange(o * (o + 1) // 2, N)
                for i in range(1, o + 1):
                    ind = L.mult2ind(np.array([o - i, i - 1])[None, :] + L.multiindex(p - o + 1))
                    valV0T = A.computeFuncDiscAtPoints(lim[:, ind], phiV[:, :, 0:ind.size])
                    data = valV0T if o > 1 else dataV0T
                    aO = np.fmin(aO, self.vertex_limiter(lim[:, ind[0]], valV0T, markV0TbdrD, data))
                lim[:, indDOF] = aO[:, None] * lim[:, indDOF]
            return lim
        raise ValueError(typ)

    def limit_disc(self, c, markV0TbdrD, dataV0T):
        cT = self.to_taylor(c)
        return self.from_taylor(self.limit_taylor(cT, markV0TbdrD, dataV0T, self.pd.typeSlopeLim))

    # ------------------------------------------------------------------ time stepping
    def step(self, nStep):
        pd, g = self.pd, self.pd.g
        K, N = pd.K, pd.N
        t, omega = A.rungeKuttaExplicit(pd.ordRK, pd.tau, (nStep - 1) * pd.tau)
        c0 = pd.cDisc
        c = c0
        for s in range(len(omega)):
            ops = self.stage_ops(t[s])
            cdot = np.linalg.solve(self.M, self.rhs(c, ops)[..., None])[..., 0]
            if pd.p > 1 and pd.isSlopeLim:
                cT = self.to_taylor(cdot)
                cTL = self.limit_taylor(cT, g.markV0TbdrD, np.full((K, 3), np.nan), pd.typeSlopeLim)
                cT = cTL + np.einsum('kij,kj->ki', self.Mcorr, cT - cTL)
                cdot = self.from_taylor(cT)
            new = omega[s] * c0 + (1 - omega[s]) * (c + pd.tau * cdot)
            if pd.isSlopeLim:
                tBC = A.getdefault(t, s + 2, t[0] + pd.tau)
                cDV0T = A.computeFuncContV0T(g, lambda a, b: pd.cDCont(tBC, a, b))
                new = self.limit_disc(new, g.markV0TbdrD, cDV0T)
            c = new
        pd.cDisc = c
        return c

    def run(self, nsteps=None):
        pd = self.pd
        n0 = pd.get('nStep', 0)
        n = pd.numSteps - n0 if nsteps is None else nsteps
        for s in range(n0 + 1, n0 + n + 1):
            self.step(s)
        pd.nStep = n0 + n
        return pd


def main_matfree(problemData=None, rounding='lu', **kwargs):
    """Same pre/loop/post phases as ``oracle.advection.main`` with matrix-free stages."""
    pd = adv.Struct(problemData or {})
    pd.update(kwargs)
    pd.problemName = 'advection'
    for f in (adv.configureProblem, adv.preprocessProblem):
        pd = f(pd)
    mf = MatFree(pd, rounding=rounding)
    # initializeProblem with this object's limiter (advection/initializeProblem.m:46-86)
    pd.isFinished = False
    pd.cDisc = A.projectFuncCont2DataDisc(pd.g, pd.c0Cont, pd.qOrd, pd.hatM, pd.basesOnQuad)
    if pd.isSlopeLim:
        cDV0T = A.computeFuncContV0T(pd.g, lambda x1, x2: pd.cDCont(0, x1, x2))
        pd.cDisc = mf.limit_disc(pd.cDisc, pd.g.markV0TbdrD, cDV0T)
    pd.initialError = A.computeL2Error(pd.g, pd.cDisc, pd.c0Cont, 2 * pd.p, pd.basesOnQuad)
    mf.run()
    return adv.postprocessProblem(pd)


def roundoff_spread(**kwargs):
    """Relative L2 distance between two roundings of the same oracle computation."""
    a = main_matfree(rounding='lu', **kwargs).cDisc
    b = main_matfree(rounding='inverse', **kwargs).cDisc
    return float(np.linalg.norm(a - b) / np.linalg.norm(a))
