"""Global sparse assembly, projections and errors (oracle restatement).

Test infrastructure: see ``oracle/__init__.py``.  Follows:
  core/assembleMatElemPhiPhi.m:88-100, core/assembleMatElemDphiPhiFuncDisc.m:181-202 (vector
  branch, which for affine triangles equals core/assembleMatElemDphiPhiFuncDiscVec.m:117-141),
  core/assembleMatEdgePhiPhiValUpwind.m:261-299 (no-area branch), core/kronVec.m:78-104,
  core/assembleVecEdgePhiIntFuncContVal.m:162-185, core/assembleVecEdgePhiIntFuncCont.m:86-136,
  core/projectFuncCont2DataDisc.m:94-102, core/computeFuncContNuOnQuadEdge.m:46-67,
  core/computeFuncContV0T.m:41-51, core/computeFuncDiscAtPoints.m:43-55,
  core/computeL2Error.m:97-114, core/rungeKuttaExplicit.m:64-78.

Vectors of the stage loop are element-major (index k*N+i), as ``reshape(cDisc', K*N, 1)``
in the reference.
"""
import numpy as np
import scipy.sparse as sp

from .basis import quadRule1D, quadRule2D, gammaMap, seqsum
from .grid import mapRef2Phy


def block_diag_sparse(blocks):
    """Sparse K*N x K*N matrix with the dense N x N blocks[k] on the diagonal."""
    K, N, _ = blocks.shape
    rows = (np.arange(K)[:, None, None] * N + np.arange(N)[None, :, None]) * np.ones((1, 1, N), np.int64)
    cols = (np.arange(K)[:, None, None] * N + np.arange(N)[None, None, :]) * np.ones((1, N, 1), np.int64)
    return sp.csr_matrix((blocks.ravel(), (rows.ravel(), cols.ravel())), shape=(K * N, K * N))


def kronVec(A, B):
    """kronVec(A, B) for sparse A (K x K) and B (K*N x nb) (core/kronVec.m:78-104):
    block (k, kp) of the result is A(k,kp) * B(k*N:(k+1)*N, :)."""
    A = sp.coo_matrix(A)
    B = sp.csr_matrix(B)
    ma, na = A.shape
    mb, nb = B.shape
    mc = mb // ma
    Bd = B.toarray().reshape(ma, mc, nb)
    k, kp, v = A.row, A.col, A.data
    rows = (k[:, None, None] * mc + np.arange(mc)[None, :, None]) * np.ones((1, 1, nb), np.int64)
    cols = (kp[:, None, None] * nb + np.arange(nb)[None, None, :]) * np.ones((1, mc, 1), np.int64)
    vals = v[:, None, None] * Bd[k]
    return sp.csr_matrix((vals.ravel(), (rows.ravel(), cols.ravel())), shape=(mb, na * nb))


def assembleMatElemPhiPhi(g, hatM):
    return sp.kron(sp.diags(g.detJ0T), hatM, format='csr')


def assembleMatElemDphiPhiFuncDisc(g, hatG, u1Disc, u2Disc):
    """{G1, G2} for dataDisc = {u1Disc, u2Disc}, J0T = {g.B}."""
    K, dataN = u1Disc.shape
    N = hatG.shape[0]
    ret = []
    for m, U in enumerate((u1Disc, u2Disc)):
        Rs = np.zeros((K * N, N))
        for l in range(dataN):
            a = (U[:, l] * g.B[:, 1 - m, 1 - m])[:, None]
            b = (U[:, l] * g.B[:, 1 - m, m])[:, None]
            Rs = Rs + np.kron(a, hatG[:, :, l, m]) - np.kron(b, hatG[:, :, l, 1 - m])
        ret.append(block_diag_sparse(Rs.reshape(K, N, N)))
    return ret


def assembleMatEdgePhiPhiValUpwind(g, markE0Tbdr, hatRdiag, hatRoffdiag, valOnQuad):
    """Upwind edge matrix R (no-area branch)."""
    K, _, R = valOnQuad.shape
    N = hatRdiag.shape[0]
    ret = sp.csr_matrix((K * N, K * N))
    for nn in range(3):
        mk = g.markE0TE0T[nn]
        anyN = np.asarray((mk[0] + mk[1] + mk[2]).sum(axis=1)).ravel() > 0
        markElemEdges = anyN | (g.idE0T[:, nn] != 0)
        Rkn = markE0Tbdr[:, nn] * g.areaE0T[:, nn]
        for r in range(R):
            v = valOnQuad[:, nn, r]
            d = Rkn * v * (markElemEdges & (v > 0))
            ret = ret + sp.kron(sp.diags(d), hatRdiag[:, :, nn, r], format='csr')
        for np_ in range(3):
            RknTimesVal = sp.csr_matrix((K * N, N))
            for r in range(R):
                v = valOnQuad[:, nn, r]
                s = sp.csr_matrix((Rkn * v * (v < 0))[:, None])
                RknTimesVal = RknTimesVal + sp.kron(s, hatRoffdiag[:, :, nn, np_, r], format='csr')
            ret = ret + kronVec(g.markE0TE0T[nn][np_], RknTimesVal)
    return ret


def assembleVecEdgePhiIntFuncContVal(g, markE0Tbdr, funcCont, valOnQuad, N, bases, qOrd):
    """Dirichlet inflow vector K_D (no-area branch)."""
    Q, W = quadRule1D(qOrd)
    ret = np.zeros((g.numT, N))
    for n in range(3):
        Q1, Q2 = gammaMap(n, Q)
        funcOnQuad = funcCont(mapRef2Phy(g, 0, Q1, Q2), mapRef2Phy(g, 1, Q1, Q2))
        Kkn = markE0Tbdr[:, n] * g.areaE0T[:, n]
        v = valOnQuad[:, n, :]
        for i in range(N):
            integral = (funcOnQuad * ((v < 0) * v)) @ (W * bases.phi1D[qOrd][:, i, n])
            ret[:, i] = ret[:, i] + Kkn * integral
    return ret.reshape(-1)


def assembleVecEdgePhiIntFuncCont(g, markE0T, funcCont, N, bases, qOrd=None):
    """Neumann vector K_N (coefE0T = areaE0T)."""
    if qOrd is None:
        qOrd = 2 * int(round((np.sqrt(8 * N + 1) - 3) / 2)) + 1
    Q, W = quadRule1D(qOrd)
    ret = np.zeros((g.numT, N))
    for n in range(3):
        Q1, Q2 = gammaMap(n, Q)
        funcQ0E = funcCont(mapRef2Phy(g, 0, Q1, Q2), mapRef2Phy(g, 1, Q1, Q2))
        markCoef = markE0T[:, n] * g.areaE0T[:, n]
        for i in range(N):
            ret[:, i] = ret[:, i] + markCoef * (funcQ0E @ (W * bases.phi1D[qOrd][:, i, n]))
    return ret.reshape(-1)


def projectFuncCont2DataDisc(g, funcCont, qOrd, hatM, bases):
    qOrd = max(qOrd, 1)
    Q1, Q2, W = quadRule2D(qOrd)
    N = hatM.shape[0]
    F = funcCont(mapRef2Phy(g, 0, Q1, Q2), mapRef2Phy(g, 1, Q1, Q2))
    rhs = F @ (W[:, None] * bases.phi2D[qOrd][:, :N])
    return np.linalg.solve(hatM.T, rhs.T).T


def computeFuncContNuOnQuadEdge(g, f1, f2, qOrd):
    Q, W = quadRule1D(qOrd)
    ret = np.zeros((g.numT, 3, len(W)))
    for n in range(3):
        Q1, Q2 = gammaMap(n, Q)
        X1, X2 = mapRef2Phy(g, 0, Q1, Q2), mapRef2Phy(g, 1, Q1, Q2)
        ret[:, n, :] = g.nuE0T[:, n, 0:1] * f1(X1, X2) + g.nuE0T[:, n, 1:2] * f2(X1, X2)
    return ret


def computeFuncContV0T(g, funcCont):
    return np.stack([funcCont(g.coordV0T[:, n, 0], g.coordV0T[:, n, 1]) for n in range(3)], axis=1)


def computeFuncDiscAtPoints(funcDisc, phiAtPoints):
    """ret(:,i) = sum(funcDisc .* phiAtPoints(:,i,:), 2), summed left to right."""
    K, N = funcDisc.shape
    ret = np.zeros((K, phiAtPoints.shape[1]))
    for i in range(phiAtPoints.shape[1]):
        acc = np.zeros(K)
        for j in range(N):
            acc = acc + funcDisc[:, j] * phiAtPoints[:, i, j]
        ret[:, i] = acc
    return ret


def computeL2Error(g, dataDisc, funcCont, qOrd, bases):
    qOrd = max(qOrd, 1)
    Q1, Q2, W = quadRule2D(qOrd)
    N = dataDisc.shape[1]
    X1, X2 = mapRef2Phy(g, 0, Q1, Q2), mapRef2Phy(g, 1, Q1, Q2)
    cEx = funcCont(X1, X2)
    cApprx = dataDisc @ bases.phi2D[qOrd][:, :N].T
    return float(np.sqrt(2 * np.dot(((cApprx - cEx) ** 2) @ W, g.areaT)))


def rungeKuttaExplicit(ordRK, tau, t0):
    if ordRK == 1:
        return np.array([t0]), np.array([0.0])
    if ordRK == 2:
        return t0 + np.array([0.0, 1.0]) * tau, np.array([0.0, 0.5])
    if ordRK == 3:
        return t0 + np.array([0.0, 1.0, 0.5]) * tau, np.array([0.0, 3 / 4, 1 / 3])
    raise ValueError('Order %d not implemented' % ordRK)


def getdefault(v, idx, default):
    """core/getdefault.m:54-95 for a vector and a 1-based scalar index."""
    return v[idx - 1] if idx <= len(v) else default


__all__ = [n for n in dir() if not n.startswith('_')] + ['seqsum', 'quadRule2D']
