"""Vertex-based Taylor slope limiter (oracle restatement).

Test infrastructure: see ``oracle/__init__.py``.  Follows:
  core/phiTaylorPhy.m:70-135, core/phiTaylorRef.m:51-53, core/computeTaylorBasesV0T.m:50-65,
  core/assembleMatElemPhiDiscPhiTaylor.m:68-77, core/assembleMatElemPhiTaylorPhiTaylor.m:50-64,
  core/projectDataDisc2DataTaylor.m:56-61, core/projectDataTaylor2DataDisc.m:56-61,
  core/computeMinMaxV0TElementPatch.m:66-166 (the markV0TT0V branch, including the global
  shift of the centroid values), core/computeVertexBasedLimiter.m:78-106,
  core/applySlopeLimiterTaylorLinear.m:108-122,
  core/applySlopeLimiterTaylorHierarchicalVertex.m:124-168,
  core/applySlopeLimiterTaylorStrict.m:111-150, core/applySlopeLimiterTaylor.m:69-85,
  core/applySlopeLimiterDisc.m:77-86, core/multiindex.m:42-51, core/mult2ind.m:57-62.

Matlab's ``min``/``max`` ignore NaN; ``np.fmin``/``np.fmax`` do the same.
"""
import math

import numpy as np
import scipy.sparse as sp
from scipy.sparse.linalg import spsolve

from .assembly import block_diag_sparse, computeFuncDiscAtPoints
from .basis import quadRule2D, p_of_N
from .grid import mapRef2Phy


def _rowsum_seq(A, W):
    """A @ W for a K x R matrix, summing over r left to right."""
    acc = np.zeros(A.shape[0])
    for r in range(A.shape[1]):
        acc = acc + A[:, r] * W[r]
    return acc


def phiTaylorPhy(g, i, X1, X2):
    """Taylor basis function i (0-based) of every element at physical points X1, X2 (K x P)."""
    qOrd = int(math.ceil((math.sqrt(8 * (i + 1) + 1) - 3) / 2))
    Q1, Q2, W = quadRule2D(qOrd)
    X1 = np.asarray(X1, dtype=np.float64); X2 = np.asarray(X2, dtype=np.float64)
    if X1.ndim == 1:
        X1 = X1[:, None]; X2 = X2[:, None]
    numP = X1.shape[1]
    dX = np.repeat((2 / np.sqrt(2 * g.areaT))[:, None], numP, axis=1)
    bx = g.baryT[:, 0:1]; by = g.baryT[:, 1:2]
    if i == 0:
        return np.ones_like(X1)
    if i == 1:
        return (X1 - bx) * dX
    if i == 2:
        return (X2 - by) * dX
    mx = mapRef2Phy(g, 0, Q1, Q2) - bx
    my = mapRef2Phy(g, 1, Q1, Q2) - by
    dx, dy = X1 - bx, X2 - by
    if i == 3:
        return (0.5 * dx ** 2 - _rowsum_seq(mx ** 2, W)[:, None]) * dX ** 2
    if i == 4:
        return (dx * dy - _rowsum_seq(2 * (mx * my), W)[:, None]) * dX ** 2
    if i == 5:
        return (0.5 * dy ** 2 - _rowsum_seq(my ** 2, W)[:, None]) * dX ** 2
    if i == 6:
        return (dx ** 3 / 6 - (_rowsum_seq(mx ** 3, W) / 3)[:, None]) * dX ** 3
    if i == 7:
        return (0.5 * dx ** 2 * dy - _rowsum_seq(mx ** 2 * my, W)[:, None]) * dX ** 3
    if i == 8:
        return (0.5 * dx * dy ** 2 - _rowsum_seq(mx * my ** 2, W)[:, None]) * dX ** 3
    if i == 9:
        return (dy ** 3 / 6 - (_rowsum_seq(my ** 3, W) / 3)[:, None]) * dX ** 3
    if i == 10:
        return (dx ** 4 / 24 - (_rowsum_seq(mx ** 4, W) / 12)[:, None]) * dX ** 4
    if i == 11:
        return (dx ** 3 * dy / 6 - (_rowsum_seq(mx ** 3 * my, W) / 3)[:, None]) * dX ** 4
    if i == 12:
        return (dx ** 2 * dy ** 2 / 4 - (_rowsum_seq(mx ** 2 * my ** 2, W) / 2)[:, None]) * dX ** 4
    if i == 13:
        return (dx * dy ** 3 / 6 - (_rowsum_seq(mx * my ** 3, W) / 3)[:, None]) * dX ** 4
    if i == 14:
        return (dy ** 4 / 24 - (_rowsum_seq(my ** 4, W) / 12)[:, None]) * dX ** 4
    raise ValueError('Taylor basis functions for p>4 not implemented')


def phiTaylorRef(g, i, Q1, Q2):
    return phiTaylorPhy(g, i, mapRef2Phy(g, 0, Q1, Q2), mapRef2Phy(g, 1, Q1, Q2))


def computeTaylorBasesV0T(g, N, bases):
    out = np.zeros((g.numT, 3, N))
    for n in range(3):
        for i in range(N):
            out[:, n, i] = phiTaylorPhy(g, i, g.coordV0T[:, n, 0], g.coordV0T[:, n, 1])[:, 0]
    bases.phiTaylorV0T = out
    return bases


def assembleMatElemPhiDiscPhiTaylor(g, N, bases):
    p = p_of_N(N)
    qOrd = max(2 * p + 1, 1)
    Q1, Q2, W = quadRule2D(qOrd)
    blocks = np.zeros((g.numT, N, N))
    PT = [phiTaylorRef(g, j, Q1, Q2) for j in range(N)]
    for i in range(N):
        for j in range(N):
            integ = _rowsum_seq(bases.phi2D[qOrd][:, i][None, :] * PT[j], W)
            blocks[:, i, j] = 2 * g.areaT * integ
    return block_diag_sparse(blocks)


def assembleMatElemPhiTaylorPhiTaylor(g, N):
    p = p_of_N(N)
    qOrd = max(2 * p, 1)
    Q1, Q2, W = quadRule2D(qOrd)
    blocks = np.zeros((g.numT, N, N))
    PT = [phiTaylorRef(g, j, Q1, Q2) for j in range(N)]
    for i in range(N):
        for j in range(N):
            blocks[:, i, j] = 2 * g.areaT * _rowsum_seq(PT[i] * PT[j], W)
    return block_diag_sparse(blocks)


def projectDataDisc2DataTaylor(dataDisc, globM, globMDiscTaylor):
    K, N = dataDisc.shape
    return spsolve(globMDiscTaylor.tocsc(), globM @ dataDisc.reshape(-1)).reshape(K, N)


def projectDataTaylor2DataDisc(dataTaylor, globM, globMDiscTaylor):
    K, N = dataTaylor.shape
    return spsolve(globM.tocsc(), globMDiscTaylor @ dataTaylor.reshape(-1)).reshape(K, N)


def computeMinMaxV0TElementPatch(g, valCentroid, markV0TbdrD, dataV0T):
    shiftToPos = abs(np.min(valCentroid)) + 1
    shiftToNeg = abs(np.max(valCentroid)) + 1
    valPos = valCentroid + shiftToPos
    valNeg = valCentroid - shiftToNeg
    valD = np.full((g.numT, 3), np.nan)
    valD[markV0TbdrD] = dataV0T[markV0TbdrD]
    mn = np.zeros((g.numT, 3)); mx = np.zeros((g.numT, 3))
    for i in range(3):
        M = g.markV0TT0V[i]
        rowmin = np.asarray(M.multiply(valNeg[None, :]).tocsr().min(axis=1).todense()).ravel()
        rowmax = np.asarray(M.multiply(valPos[None, :]).tocsr().max(axis=1).todense()).ravel()
        mn[:, i] = np.fmin(rowmin + shiftToNeg, valD[:, i])
        mx[:, i] = np.fmax(rowmax - shiftToPos, valD[:, i])
    return mn, mx


def computeVertexBasedLimiter(g, valCentroid, valV0T, markV0TbdrD, dataV0T):
    mn, mx = computeMinMaxV0TElementPatch(g, valCentroid, markV0TbdrD, dataV0T)
    dV = valV0T - valCentroid[:, None]
    dMin = mn - valCentroid[:, None]
    dMax = mx - valCentroid[:, None]
    tol = 1.e-8
    markNeg = dV < dMin + tol
    markPos = dV > dMax - tol
    a = np.ones((g.numT, 3))
    with np.errstate(divide='ignore', invalid='ignore'):
        a[markNeg] = np.fmax(0, np.fmin(1, dMin[markNeg] / (dV[markNeg] - tol)))
        a[markPos] = np.fmax(0, np.fmin(1, dMax[markPos] / (dV[markPos] + tol)))
    alpha = np.fmin(np.fmin(a[:, 0], a[:, 1]), a[:, 2])
    return alpha, (mn, mx)


def multiindex(p):
    """Multi-indices of the Taylor DOFs up to degree p, in DOF order."""
    rows = [(0, 0)]
    for ord_ in range(1, p + 1):
        for i in range(1, ord_ + 2):
            rows.append((ord_ - i + 1, i - 1))
    return np.array(rows, dtype=np.int64)


def mult2ind(a):
    """0-based column index of the Taylor DOF with multi-index a (rows of a)."""
    a = np.atleast_2d(a)
    p = a.sum(axis=1)
    return p * (p + 1) // 2 + a[:, 1]


def applySlopeLimiterTaylorLinear(g, dataTaylor, markV0TbdrD, dataV0T, bases):
    valV0T = computeFuncDiscAtPoints(dataTaylor[:, 0:3], bases.phiTaylorV0T[:, :, 0:3])
    alpha, mm = computeVertexBasedLimiter(g, dataTaylor[:, 0], valV0T, markV0TbdrD, dataV0T)
    out = np.concatenate([dataTaylor[:, 0:1], alpha[:, None] * dataTaylor[:, 1:3],
                          (alpha == 1)[:, None] * dataTaylor[:, 3:]], axis=1)
    return out, mm


def applySlopeLimiterTaylorHierarchicalVertex(g, dataTaylor, markV0TbdrD, dataV0T, bases):
    K, N = dataTaylor.shape
    p = p_of_N(N)
    lim = np.zeros_like(dataTaylor)
    lim[:, 0] = dataTaylor[:, 0]
    alpha = np.zeros(K)
    mm = None
    for ord_ in range(p, 0, -1):
        alphaOrd = np.ones(K)
        indDOF = np.arange(ord_ * (ord_ + 1) // 2, (ord_ + 1) * (ord_ + 2) // 2)
        for i in range(1, ord_ + 1):
            mult = np.array([ord_ - i, i - 1])[None, :] + multiindex(1)
            ind = mult2ind(mult)
            valV0T = computeFuncDiscAtPoints(dataTaylor[:, ind], bases.phiTaylorV0T[:, :, 0:3])
            data = valV0T if ord_ > 1 else dataV0T
            alphaTmp, mm = computeVertexBasedLimiter(g, dataTaylor[:, ind[0]], valV0T, markV0TbdrD, data)
            alphaOrd = np.fmin(alphaOrd, alphaTmp)
        alpha = np.fmax(alpha, alphaOrd)
        lim[:, indDOF] = alpha[:, None] * dataTaylor[:, indDOF]
    return lim, mm


def applySlopeLimiterTaylorStrict(g, dataTaylor, markV0TbdrD, dataV0T, bases):
    K, N = dataTaylor.shape
    p = p_of_N(N)
    lim = dataTaylor.copy()
    mm = None
    for ord_ in range(p, 0, -1):
        alphaOrd = np.ones(K)
        indDOF = np.arange(ord_ * (ord_ + 1) // 2, N)
        for i in range(1, ord_ + 1):
            pRec = p - ord_ + 1
            mult = np.array([ord_ - i, i - 1])[None, :] + multiindex(pRec)
            ind = mult2ind(mult)
            valV0T = computeFuncDiscAtPoints(lim[:, ind], bases.phiTaylorV0T[:, :, 0:ind.size])
            data = valV0T if ord_ > 1 else dataV0T
            alphaTmp, mm = computeVertexBasedLimiter(g, lim[:, ind[0]], valV0T, markV0TbdrD, data)
            alphaOrd = np.fmin(alphaOrd, alphaTmp)
        lim[:, indDOF] = alphaOrd[:, None] * lim[:, indDOF]
    return lim, mm


def applySlopeLimiterTaylor(g, dataTaylor, markV0TbdrD, dataV0T, bases, typ='linear'):
    if typ == 'linear':
        return applySlopeLimiterTaylorLinear(g, dataTaylor, markV0TbdrD, dataV0T, bases)
    if typ == 'hierarch_vert':
        return applySlopeLimiterTaylorHierarchicalVertex(g, dataTaylor, markV0TbdrD, dataV0T, bases)
    if typ == 'strict':
        return applySlopeLimiterTaylorStrict(g, dataTaylor, markV0TbdrD, dataV0T, bases)
    raise ValueError('Unknown limiter type')


def applySlopeLimiterDisc(g, dataDisc, markV0TbdrD, dataV0T, globM, globMDiscTaylor, bases, typ):
    dataTaylor = projectDataDisc2DataTaylor(dataDisc, globM, globMDiscTaylor)
    dataTaylor, mm = applySlopeLimiterTaylor(g, dataTaylor, markV0TbdrD, dataV0T, bases, typ)
    return projectDataTaylor2DataDisc(dataTaylor, globM, globMDiscTaylor), mm
