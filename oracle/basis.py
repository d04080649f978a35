"""Quadrature rules, modal basis and reference-element integrals (oracle restatement).

Test infrastructure: see ``oracle/__init__.py``.  Follows, function by function:
  core/quadRule1D.m:48-95, core/quadRule2D.m:64-109, core/triquad.m:30-78 (re-derived from the
  mathematics, not transcribed), core/phi.m:40-61, core/gradPhi.m:42-87, core/gammaMap.m:50-57,
  core/theta.m:109-133, core/computeBasesOnQuad.m:72-134, core/integrateRefElemPhiPhi.m:49-59,
  core/integrateRefElemDphiPhiPhi.m:55-82, core/integrateRefEdgePhiIntPhiIntPerQuad.m:52-66,
  core/integrateRefEdgePhiIntPhiExtPerQuad.m:54-70.

Index conventions: 0-based arrays; basis index i=0..N-1 stands for the reference's i=1..N, edge
index n=0..2 for n=1..3.  Table shapes keep the reference's axis order
(e.g. ``phi1D[qOrd]`` is R x N x 3).
"""
import math

import numpy as np
from scipy.special import roots_jacobi, roots_legendre

SQ2, SQ3, SQ5, SQ6 = math.sqrt(2.0), math.sqrt(3.0), math.sqrt(5.0), math.sqrt(6.0)
SQ10, SQ14, SQ30, SQ70 = math.sqrt(10.0), math.sqrt(14.0), math.sqrt(30.0), math.sqrt(70.0)


def seqsum(v):
    """Left-to-right sum of a short vector (the reference's ``sum`` over quadrature points)."""
    acc = 0.0
    for x in np.asarray(v, dtype=np.float64).ravel():
        acc = acc + x
    return acc


def N_of_p(p):
    return (p + 1) * (p + 2) // 2


def p_of_N(N):
    p = (math.sqrt(8 * N + 1) - 3) / 2
    assert abs(p - round(p)) < 1e-12, 'N does not match a polynomial degree'
    return int(round(p))


# ---------------------------------------------------------------------------------------------
# 1D Gauss-Legendre rules on [0,1]                                  core/quadRule1D.m:48-95
# ---------------------------------------------------------------------------------------------
def quadRule1D(qOrd):
    if qOrd in (0, 1):
        Q = np.array([0.0]); W = np.array([2.0])
    elif qOrd in (2, 3):
        Q = math.sqrt(1 / 3) * np.array([-1.0, 1.0]); W = np.array([1.0, 1.0])
    elif qOrd in (4, 5):
        Q = math.sqrt(3 / 5) * np.array([-1.0, 0.0, 1.0]); W = 1 / 9 * np.array([5.0, 8.0, 5.0])
    elif qOrd in (6, 7):
        Q = np.array([-1.0, -1.0, 1.0, 1.0]) * np.sqrt(
            3 / 7 + np.array([1.0, -1.0, -1.0, 1.0]) * 2 / 7 * math.sqrt(6 / 5))
        W = 1 / 36 * (18 + math.sqrt(30) * np.array([-1.0, 1.0, 1.0, -1.0]))
    elif qOrd in (8, 9):
        Q = np.array([-1.0, -1.0, 0.0, 1.0, 1.0]) * np.sqrt(
            5 + np.array([2.0, -2.0, 0.0, -2.0, 2.0]) * math.sqrt(10 / 7)) / 3
        W = 1 / 900 * (322 + 13 * math.sqrt(70) * np.array([-1.0, 1.0, 0.0, 1.0, -1.0])
                       + np.array([0.0, 0.0, 190.0, 0.0, 0.0]))
    elif qOrd in (10, 11):
        Q = np.array([0.6612093864662645, -0.6612093864662645, -0.2386191860831969,
                      0.2386191860831969, -0.9324695142031521, 0.9324695142031521])
        W = np.array([0.3607615730481386, 0.3607615730481386, 0.4679139345726910,
                      0.4679139345726910, 0.1713244923791704, 0.171324492379170])
    elif qOrd in (12, 13):
        Q = np.array([0.0000000000000000, 0.4058451513773972, -0.4058451513773972,
                      -0.7415311855993945, 0.7415311855993945, -0.9491079123427585,
                      0.9491079123427585])
        W = np.array([0.4179591836734694, 0.3818300505051189, 0.3818300505051189,
                      0.2797053914892766, 0.2797053914892766, 0.1294849661688697,
                      0.1294849661688697])
    else:
        raise ValueError('Order %d not implemented' % qOrd)
    return (Q + 1) / 2, W / 2


# ---------------------------------------------------------------------------------------------
# 2D rules on the reference triangle (0,0),(1,0),(0,1)              core/quadRule2D.m:64-109
# ---------------------------------------------------------------------------------------------
def collapsed_gauss_rule(n):
    """Product rule on the triangle from the collapsed square (role of core/triquad.m:30-78).

    Re-derived: map (s,t) in [0,1]^2 to (x1,x2) = (s(1-t), s t), Jacobian s.  In s use the
    n-point Gauss-Jacobi rule for the weight s (Jacobi(0,1) on [-1,1]), in t the n-point
    Gauss-Legendre rule.  Points are ordered with s fastest, then t; both ascending.
    Exact for polynomials of degree <= 2n-2 on the triangle.
    """
    X, wJ = roots_jacobi(n, 0.0, 1.0)
    order = np.argsort(X); X = X[order]; wJ = wJ[order]
    Y, wL = roots_legendre(n)
    order = np.argsort(Y); Y = Y[order]; wL = wL[order]
    s = (X + 1) / 2; ws = wJ / 4
    t = (1 + Y) / 2; wt = wL / 2
    ss, tt = np.meshgrid(s, t, indexing='ij')      # ss[i,j] = s_i, tt[i,j] = t_j
    yy = tt * ss
    Q1 = (ss - yy).ravel(order='F'); Q2 = yy.ravel(order='F')
    W = np.outer(ws, wt).ravel(order='F')
    return Q1, Q2, W


def quadRule2D(qOrd):
    if qOrd in (0, 1):
        return np.array([1 / 3]), np.array([1 / 3]), np.array([1 / 2])
    if qOrd == 2:
        return (np.array([1 / 6, 2 / 3, 1 / 6]), np.array([1 / 6, 1 / 6, 2 / 3]),
                np.array([1 / 6, 1 / 6, 1 / 6]))
    if qOrd == 3:
        a1 = (3 + math.sqrt(3)) / 6; a2 = (3 - math.sqrt(3)) / 6
        b1 = (6 + math.sqrt(6)) / 10; b2 = (6 - math.sqrt(6)) / 10
        w1 = 1 / 8 + math.sqrt(6) / 72; w2 = 1 / 8 - math.sqrt(6) / 72
        return (np.array([a1 * b1, a2 * b1, a1 * b2, a2 * b2]),
                np.array([a2 * b1, a1 * b1, a2 * b2, a1 * b2]), np.array([w1, w1, w2, w2]))
    if qOrd == 4:
        return (np.array([0.445948490915965, 0.108103018168070, 0.445948490915965,
                          0.091576213509771, 0.816847572980458, 0.091576213509771]),
                np.array([0.108103018168070, 0.445948490915965, 0.445948490915965,
                          0.816847572980458, 0.091576213509771, 0.091576213509771]),
                np.array([0.111690794839005, 0.111690794839005, 0.111690794839005,
                          0.054975871827661, 0.054975871827661, 0.054975871827661]))
    if qOrd == 5:
        a1 = (6 - math.sqrt(15)) / 21; a2 = (6 + math.sqrt(15)) / 21
        w1 = (155 - math.sqrt(15)) / 2400; w2 = (155 + math.sqrt(15)) / 2400
        return (np.array([1 / 3, a1, 1 - 2 * a1, a1, a2, 1 - 2 * a2, a2]),
                np.array([1 / 3, 1 - 2 * a1, a1, a1, 1 - 2 * a2, a2, a2]),
                np.array([9 / 80, w1, w1, w1, w2, w2, w2]))
    if qOrd == 6:
        return (np.array([0.063089014491502, 0.873821971016996, 0.063089014491502,
                          0.249286745170910, 0.501426509658179, 0.249286745170910,
                          0.310352451033785, 0.053145049844816, 0.636502499121399,
                          0.053145049844816, 0.636502499121399, 0.310352451033785]),
                np.array([0.063089014491502, 0.063089014491502, 0.873821971016996,
                          0.249286745170910, 0.249286745170910, 0.501426509658179,
                          0.053145049844816, 0.310352451033785, 0.053145049844816,
                          0.636502499121399, 0.310352451033785, 0.636502499121399]),
                np.array([0.025422453185103, 0.025422453185103, 0.025422453185103,
                          0.058393137863189, 0.058393137863189, 0.058393137863189,
                          0.041425537809187, 0.041425537809187, 0.041425537809187,
                          0.041425537809187, 0.041425537809187, 0.041425537809187]))
    return collapsed_gauss_rule(qOrd)


# ---------------------------------------------------------------------------------------------
# Orthonormal modal basis and its gradient                  core/phi.m:40-61, core/gradPhi.m:42-87
# ---------------------------------------------------------------------------------------------
def phi(i, X1, X2):
    """Basis function i (0-based) on the reference triangle."""
    x, y = np.asarray(X1, dtype=np.float64), np.asarray(X2, dtype=np.float64)
    if i == 0: return SQ2 * np.ones_like(x)
    if i == 1: return 2 - 6 * x
    if i == 2: return 2 * SQ3 * (1 - x - 2 * y)
    if i == 3: return SQ6 * ((10 * x - 8) * x + 1)
    if i == 4: return SQ3 * ((5 * x - 4) * x + (-15 * y + 12) * y - 1)
    if i == 5: return 3 * SQ5 * ((3 * x + 8 * y - 4) * x + (3 * y - 4) * y + 1)
    if i == 6: return 2 * SQ2 * (-1 + (15 + (-45 + 35 * x) * x) * x)
    if i == 7: return 2 * SQ6 * (-1 + (13 + (-33 + 21 * x) * x) * x + (2 + (-24 + 42 * x) * x) * y)
    if i == 8: return 2 * SQ10 * (-1 + (9 + (-15 + 7 * x) * x) * x
                                  + (6 + (-48 + 42 * x) * x + (-6 + 42 * x) * y) * y)
    if i == 9: return 2 * SQ14 * (-1 + (3 + (-3 + x) * x) * x
                                  + (12 + (-24 + 12 * x) * x + (-30 + 30 * x + 20 * y) * y) * y)
    if i == 10: return SQ10 * (1 + (-24 + (126 + (-224 + 126 * x) * x) * x) * x)
    if i == 11: return SQ30 * (1 + (-22 + (105 + (-168 + 84 * x) * x) * x) * x
                               + (-2 + (42 + (-168 + 168 * x) * x) * x) * y)
    if i == 12: return 5 * SQ2 * (1 + (-18 + (69 + (-88 + 36 * x) * x) * x) * x
                                  + (-6 + (102 + (-312 + 216 * x) * x) * x
                                     + (6 + (-96 + 216 * x) * x) * y) * y)
    if i == 13: return SQ70 * (1 + (-12 + (30 + (-28 + 9 * x) * x) * x) * x
                               + (-12 + (132 + (-228 + 108 * x) * x) * x
                                  + (30 + (-300 + 270 * x) * x + (-20 + 180 * x) * y) * y) * y)
    if i == 14: return 3 * SQ10 * (1 + (-4 + (6 + (-4 + x) * x) * x) * x
                                   + (-20 + (60 + (-60 + 20 * x) * x) * x
                                      + (90 + (-180 + 90 * x) * x
                                         + (-140 + 140 * x + 70 * y) * y) * y) * y)
    raise ValueError('basis index out of range')


def gradPhi(i, m, X1, X2):
    """Derivative d/dx_{m} (m=0,1) of basis function i (0-based)."""
    x, y = np.asarray(X1, dtype=np.float64), np.asarray(X2, dtype=np.float64)
    z = np.zeros_like(x); o = np.ones_like(x)
    if m == 0:
        if i == 0: return z
        if i == 1: return -6 * o
        if i == 2: return -2 * SQ3 * o
        if i == 3: return SQ6 * (20 * x - 8)
        if i == 4: return SQ3 * (10 * x - 4)
        if i == 5: return 6 * SQ5 * (3 * x + 4 * y - 2)
        if i == 6: return 2 * SQ2 * (15 + (-90 + 105 * x) * x)
        if i == 7: return 2 * SQ6 * (13 + (-66 + 63 * x) * x + (-24 + 84 * x) * y)
        if i == 8: return 2 * SQ10 * (9 + (-30 + 21 * x) * x + (-48 + 84 * x + 42 * y) * y)
        if i == 9: return 2 * SQ14 * (3 + (-6 + 3 * x) * x + (-24 + 24 * x + 30 * y) * y)
        if i == 10: return SQ10 * (-24 + (252 + (-672 + 504 * x) * x) * x)
        if i == 11: return SQ30 * (-22 + (210 + (-504 + 336 * x) * x) * x
                                   + (42 + (-336 + 504 * x) * x) * y)
        if i == 12: return 5 * SQ2 * (-18 + (138 + (-264 + 144 * x) * x) * x
                                      + (102 + (-624 + 648 * x) * x + (-96 + 432 * x) * y) * y)
        if i == 13: return SQ70 * (-12 + (60 + (-84 + 36 * x) * x) * x
                                   + (132 + (-456 + 324 * x) * x
                                      + (-300 + 540 * x + 180 * y) * y) * y)
        if i == 14: return 3 * SQ10 * (-4 + (12 + (-12 + 4 * x) * x) * x
                                       + (60 + (-120 + 60 * x) * x
                                          + (-180 + 180 * x + 140 * y) * y) * y)
    else:
        if i == 0: return z
        if i == 1: return z
        if i == 2: return -4 * SQ3 * o
        if i == 3: return z
        if i == 4: return 2 * SQ3 * (-15 * y + 6)
        if i == 5: return 6 * SQ5 * (4 * x + 3 * y - 2)
        if i == 6: return z
        if i == 7: return 2 * SQ6 * (2 + (-24 + 42 * x) * x)
        if i == 8: return 2 * SQ10 * (6 + (-48 + 42 * x) * x + (-12 + 84 * x) * y)
        if i == 9: return 2 * SQ14 * (12 + (-24 + 12 * x) * x + (-60 + 60 * x + 60 * y) * y)
        if i == 10: return z
        if i == 11: return SQ30 * (-2 + (42 + (-168 + 168 * x) * x) * x)
        if i == 12: return 5 * SQ2 * (-6 + (102 + (-312 + 216 * x) * x) * x
                                      + (12 + (-192 + 432 * x) * x) * y)
        if i == 13: return SQ70 * (-12 + (132 + (-228 + 108 * x) * x) * x
                                   + (60 + (-600 + 540 * x) * x + (-60 + 540 * x) * y) * y)
        if i == 14: return 3 * SQ10 * (-20 + (60 + (-60 + 20 * x) * x) * x
                                       + (180 + (-360 + 180 * x) * x
                                          + (-420 + 420 * x + 280 * y) * y) * y)
    raise ValueError('basis index out of range')


def gammaMap(n, S):
    """Edge parametrisation of reference edge n (0-based)        core/gammaMap.m:50-57."""
    S = np.asarray(S, dtype=np.float64).ravel()
    if n == 0: return 1 - S, S
    if n == 1: return np.zeros_like(S), 1 - S
    if n == 2: return S, np.zeros_like(S)
    raise ValueError


def theta(nn, np_, X1, X2):
    """Map a point of edge nn to the matching point of the neighbour's edge np
    (core/theta.m:109-133)."""
    z = np.zeros_like(X1)
    table = {
        (0, 0): (1 - X1, 1 - X2), (0, 1): (z, X2), (0, 2): (X1, z),
        (1, 0): (1 - X2, X2), (1, 1): (z, 1 - X2), (1, 2): (X2, z),
        (2, 0): (X1, 1 - X1), (2, 1): (z, X1), (2, 2): (1 - X1, z),
    }
    return table[(nn, np_)]


class Bases:
    """Container of basis values on quadrature points, keyed by quadrature order
    (core/computeBasesOnQuad.m:72-134)."""

    def __init__(self):
        self.phi2D, self.gradPhi2D, self.phi1D, self.thetaPhi1D = {}, {}, {}, {}
        self.gradPhi1D, self.thetaGradPhi1D = {}, {}
        self.phiTaylorV0T = None


def computeBasesOnQuad(N, requiredOrders=None):
    if requiredOrders is None:
        p = p_of_N(N)
        requiredOrders = [2 * p, 2 * p + 1] if p > 0 else [1]
    b = Bases()
    for ord_ in requiredOrders:
        Q1, Q2, _ = quadRule2D(ord_)
        b.phi2D[ord_] = np.stack([phi(i, Q1, Q2) for i in range(N)], axis=1)
        b.gradPhi2D[ord_] = np.stack(
            [np.stack([gradPhi(i, m, Q1, Q2) for i in range(N)], axis=1) for m in range(2)], axis=2)
        Q, _ = quadRule1D(ord_)
        R = len(Q)
        b.phi1D[ord_] = np.zeros((R, N, 3))
        b.gradPhi1D[ord_] = np.zeros((R, N, 3, 2))
        b.thetaPhi1D[ord_] = np.zeros((R, N, 3, 3))
        b.thetaGradPhi1D[ord_] = np.zeros((R, N, 3, 3, 2))
        for nn in range(3):
            X1, X2 = gammaMap(nn, Q)
            for i in range(N):
                b.phi1D[ord_][:, i, nn] = phi(i, X1, X2)
                for m in range(2):
                    b.gradPhi1D[ord_][:, i, nn, m] = gradPhi(i, m, X1, X2)
            for np_ in range(3):
                P1, P2 = theta(nn, np_, X1, X2)
                for i in range(N):
                    b.thetaPhi1D[ord_][:, i, nn, np_] = phi(i, P1, P2)
                    for m in range(2):
                        b.thetaGradPhi1D[ord_][:, i, nn, np_, m] = gradPhi(i, m, P1, P2)
    return b


# ---------------------------------------------------------------------------------------------
# Reference-element integrals
# ---------------------------------------------------------------------------------------------
def integrateRefElemPhiPhi(N, bases, qOrd=None):
    """hatM (core/integrateRefElemPhiPhi.m:49-59)."""
    if qOrd is None:
        qOrd = max(2 * p_of_N(N), 1)
    _, _, W = quadRule2D(qOrd)
    P = bases.phi2D[qOrd]
    ret = np.zeros((N, N))
    for i in range(N):
        for j in range(N):
            ret[i, j] = seqsum(W * P[:, i] * P[:, j])
    return ret


def integrateRefElemDphiPhiPhi(N, bases, qOrd=None):
    """hatG(i,j,l,m) = sum_q W dphi_i/dx_m phi_j phi_l (core/integrateRefElemDphiPhiPhi.m:55-82)."""
    ret = np.zeros((N, N, N, 2))
    if N == 1:
        return ret
    if qOrd is None:
        qOrd = max(2 * p_of_N(N), 1)
    _, _, W = quadRule2D(qOrd)
    P, G = bases.phi2D[qOrd], bases.gradPhi2D[qOrd]
    for i in range(N):
        for j in range(N):
            for l in range(N):
                for m in range(2):
                    ret[i, j, l, m] = seqsum(W * G[:, i, m] * P[:, j] * P[:, l])
    return ret


def integrateRefEdgePhiIntPhiIntPerQuad(N, bases, qOrd=None):
    """hatRdiag N x N x 3 x R (core/integrateRefEdgePhiIntPhiIntPerQuad.m:52-66)."""
    if qOrd is None:
        qOrd = max(2 * p_of_N(N) + 1, 1)
    _, W = quadRule1D(qOrd)
    P = bases.phi1D[qOrd]
    ret = np.zeros((N, N, 3, len(W)))
    for n in range(3):
        for i in range(N):
            for j in range(N):
                ret[i, j, n, :] = P[:, i, n] * P[:, j, n] * W
    return ret


def integrateRefEdgePhiIntPhiExtPerQuad(N, bases, qOrd=None):
    """hatRoffdiag N x N x 3 x 3 x R (core/integrateRefEdgePhiIntPhiExtPerQuad.m:54-70)."""
    if qOrd is None:
        qOrd = 2 * p_of_N(N) + 1
    _, W = quadRule1D(qOrd)
    P, T = bases.phi1D[qOrd], bases.thetaPhi1D[qOrd]
    ret = np.zeros((N, N, 3, 3, len(W)))
    for nn in range(3):
        for np_ in range(3):
            for i in range(N):
                for j in range(N):
                    ret[i, j, nn, np_, :] = P[:, i, nn] * T[:, j, nn, np_] * W
    return ret
