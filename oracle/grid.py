"""Triangular mesh and its incidence data (oracle restatement).

Test infrastructure: see ``oracle/__init__.py``.  Follows core/domainSquare.m:67-105,
core/generateGridData.m:130-198 and advection/computeDerivedGridData.m:66-81.

Integer maps use the reference's 1-based numbering where the reference stores numbers that
mean "element/edge/local index or 0 for none" (T0E, E0E, idE, idE0T): these arrays hold the
reference's values.  Index arrays used to address numpy arrays (V0T, E0T, V0E) are 0-based.

The K x K masks ``markE0TE0T{nn,np}`` and ``markV0TV0T{nn,np}`` are built as scipy sparse
matrices directly.  The reference forms ``markV0TV0T`` from a dense K x K comparison
(core/generateGridData.m:187), which only fits memory for small K; the sparse construction here
yields the same matrix without that intermediate.
"""
import numpy as np
import scipy.sparse as sp


class Grid:
    pass


def colon(a, h, b):
    """Matlab/Octave ``a:h:b`` for the meshes used here: base + i*increment with the last
    point put on ``b`` (the two interpreters differ from this only in the last ulp for
    step sizes that are not powers of two)."""
    n = int(np.floor((b - a) / h + 1e-10)) + 1
    v = a + np.arange(n) * h
    if abs(v[-1] - b) < 1e-10 * max(1.0, abs(b)):
        v[-1] = b
    return v


def domainSquare(h, a=0.0, b=1.0):
    """Friedrichs-Keller triangulation of [a,b]^2 (core/domainSquare.m:67-105)."""
    dim = int(np.ceil((b - a) / h))
    h = (b - a) / dim
    v = colon(a, h, b)
    X, Y = np.meshgrid(v, v)                      # X[i,j] = v[j], Y[i,j] = v[i]
    coordV = np.stack([X.ravel(order='F'), Y.ravel(order='F')], axis=1)
    V0T = square_V0T(dim)
    g = generateGridData(coordV, V0T)
    add_boundary_ids(g, a, b)
    return g


def square_V0T(dim):
    """Triangles of domainSquare: lower-left ones (pattern [1,dim+2,2]) then upper-right ones
    (pattern [dim+2,dim+3,2]); rows whose first vertex is on the top row are removed
    (core/domainSquare.m:94-99).  0-based vertex numbers."""
    r = np.arange(dim * (dim + 1))
    keep = (r + 1) % (dim + 1) != 0
    base = r[keep]
    V0T1 = np.stack([base, base + dim + 1, base + 1], axis=1)
    V0T2 = np.stack([base + dim + 1, base + dim + 2, base + 1], axis=1)
    return np.concatenate([V0T1, V0T2], axis=0).astype(np.int64)


def add_boundary_ids(g, a=0.0, b=1.0):
    """Boundary edge ids south=1, east=2, north=3, west=4 (core/domainSquare.m:100-104)."""
    tol = 10 * np.finfo(np.float64).eps
    idE = np.zeros(g.numE, dtype=np.int64)
    idE[np.abs(g.baryE[:, 1] - a) < tol] = 1
    idE[np.abs(g.baryE[:, 0] - b) < tol] = 2
    idE[np.abs(g.baryE[:, 1] - b) < tol] = 3
    idE[np.abs(g.baryE[:, 0] - a) < tol] = 4
    g.idE = idE
    g.idE0T = idE[g.E0T]


def generateGridData(coordV, V0T):
    """All incidence maps and geometry of a triangulation (core/generateGridData.m:130-198)."""
    g = Grid()
    coordV = np.asarray(coordV, dtype=np.float64)
    V0T = np.asarray(V0T, dtype=np.int64)
    g.coordV, g.V0T = coordV, V0T
    numT, numV = V0T.shape[0], coordV.shape[0]
    g.numT, g.numV = numT, numV
    T1 = np.arange(1, numT + 1)
    # V2T(a,b) = T for every counter-clockwise directed edge (a,b) of T            (:136-137)
    rows = V0T[:, [0, 1, 2]].ravel(); cols = V0T[:, [1, 2, 0]].ravel()
    V2T = sp.csr_matrix((np.repeat(T1, 3), (rows, cols)), shape=(numV, numV))
    g.V2T = V2T
    # edges numbered in column-major order of triu(V2T + V2T')                     (:138-140)
    S = sp.triu(V2T + V2T.T).tocoo()
    order = np.lexsort((S.row, S.col))
    r, c = S.row[order], S.col[order]
    numE = r.size
    V2E = sp.csr_matrix((np.arange(1, numE + 1), (r, c)), shape=(numV, numV))
    V2E = (V2E + V2E.T).tocsr()
    g.V2E = V2E

    def lookup(M, a, b):
        return np.asarray(M[a, b]).ravel().astype(np.int64)

    # edge-wise maps written for triangles in reverse order, last writer wins       (:141-148)
    Trev = np.arange(numT - 1, -1, -1)
    A = V0T[Trev][:, [0, 1, 2]].ravel()          # row-major over (t reversed, n) == idxE(:)
    Bv = V0T[Trev][:, [1, 2, 0]].ravel()
    idxE = lookup(V2E, A, Bv) - 1
    t0 = lookup(V2T, A, Bv)
    t1 = lookup(V2T, Bv, A)
    # position of the last write to each edge = first occurrence in the reversed sequence
    uniq, first_rev = np.unique(idxE[::-1], return_index=True)
    assert uniq.size == numE
    pos = np.empty(numE, dtype=np.int64)
    pos[uniq] = idxE.size - 1 - first_rev
    g.V0E = np.stack([A[pos], Bv[pos]], axis=1)
    g.T0E = np.stack([t0[pos], t1[pos]], axis=1)
    g.numE = numE
    vecE = coordV[g.V0E[:, 1], :] - coordV[g.V0E[:, 0], :]
    g.areaE = np.sqrt(vecE[:, 0] ** 2 + vecE[:, 1] ** 2)
    g.nuE = np.stack([vecE[:, 1], -vecE[:, 0]], axis=1) / g.areaE[:, None]
    x, y = coordV[:, 0], coordV[:, 1]
    v1, v2, v3 = V0T[:, 0], V0T[:, 1], V0T[:, 2]
    g.areaT = (x[v1] * y[v2] + x[v2] * y[v3] + x[v3] * y[v1]
               - x[v1] * y[v3] - x[v2] * y[v1] - x[v3] * y[v2]) / 2
    g.baryT = (coordV[v1, :] + coordV[v2, :] + coordV[v3, :]) / 3
    # E0T(:,n): edge opposite to vertex n                                              (:159)
    g.E0T = np.stack([lookup(V2E, V0T[:, (n + 1) % 3], V0T[:, (n + 2) % 3]) for n in range(3)],
                     axis=1) - 1
    g.areaE0T = g.areaE[g.E0T]
    sigE0T = 1 - 2 * (g.T0E[g.E0T, 1] == T1[:, None]).astype(np.int64)
    g.sigE0T = sigE0T
    g.baryE = 0.5 * (coordV[g.V0E[:, 0], :] + coordV[g.V0E[:, 1], :])
    g.coordV0T = np.stack([coordV[V0T[:, n], :] for n in range(3)], axis=1)      # K x 3 x 2
    g.baryE0T = np.stack([g.baryE[g.E0T[:, n], :] for n in range(3)], axis=1)
    g.nuE0T = np.stack([g.nuE[g.E0T[:, n], :] * sigE0T[:, n:n + 1] for n in range(3)], axis=1)
    E0E = np.zeros((numE, 2), dtype=np.int64)
    for n in range(3):
        Tn = sigE0T[:, n] == 1
        E0E[g.E0T[Tn, n], 0] = n + 1
        E0E[g.E0T[~Tn, n], 1] = n + 1
    g.E0E = E0E
    g.B = np.zeros((numT, 2, 2))
    for m in range(2):
        g.B[:, m, 0] = g.coordV0T[:, 1, m] - g.coordV0T[:, 0, m]
        g.B[:, m, 1] = g.coordV0T[:, 2, m] - g.coordV0T[:, 0, m]
    markEint = E0E[:, 1] != 0
    g.markE0TE0T = [[None] * 3 for _ in range(3)]
    for nn in range(3):
        for np_ in range(3):
            idx1 = (E0E[:, 0] == nn + 1) & (E0E[:, 1] == np_ + 1) & markEint
            idx2 = (E0E[:, 1] == nn + 1) & (E0E[:, 0] == np_ + 1) & markEint
            rr = np.concatenate([g.T0E[idx1, 0], g.T0E[idx2, 1]]) - 1
            cc = np.concatenate([g.T0E[idx1, 1], g.T0E[idx2, 0]]) - 1
            M = sp.csr_matrix((np.ones(rr.size), (rr, cc)), shape=(numT, numT))
            M.data[:] = 1.0
            g.markE0TE0T[nn][np_] = M
    g.markV0TV0T = build_markV0TV0T(V0T, numV)
    g.detJ0T = 2 * g.areaT
    return g


def build_markV0TV0T(V0T, numV):
    """markV0TV0T{nn,np}(k,kp) = (V0T(k,nn) == V0T(kp,np)) as sparse K x K matrices."""
    numT = V0T.shape[0]
    out = [[None] * 3 for _ in range(3)]
    for np_ in range(3):
        # for each vertex, the elements whose local vertex np_ is that vertex
        col_by_vertex = sp.csr_matrix((np.ones(numT), (V0T[:, np_], np.arange(numT))),
                                      shape=(numV, numT))
        for nn in range(3):
            sel = sp.csr_matrix((np.ones(numT), (np.arange(numT), V0T[:, nn])),
                                shape=(numT, numV))
            M = (sel @ col_by_vertex).tocsr()
            M.data[:] = 1.0
            out[nn][np_] = M
    return out


def mapRef2Phy(g, i, X1, X2):
    """Physical coordinate i of reference points X1, X2 in every element: K x R
    (core/generateGridData.m:195-196)."""
    X1 = np.asarray(X1, dtype=np.float64).reshape(1, -1)
    X2 = np.asarray(X2, dtype=np.float64).reshape(1, -1)
    return (g.B[:, i, 0:1] * X1 + g.B[:, i, 1:2] * X2) + g.coordV0T[:, 0, i:i + 1] * np.ones_like(X1)


def computeDerivedGridData(g):
    """advection/computeDerivedGridData.m:66-81."""
    g.markV0TT0V = []
    for n in range(3):
        M = (g.markV0TV0T[n][0] + g.markV0TV0T[n][1] + g.markV0TV0T[n][2]).tocsr()
        M.data[:] = 1.0
        g.markV0TT0V.append(M)
    g.areaE0TbdrN = g.markE0TbdrN * g.areaE0T
    g.areaE0TbdrD = [g.areaE0T[:, n] * g.markE0TbdrD[:, n] for n in range(3)]
    g.areaE0TbdrNotN = [g.areaE0T[:, n] * ~g.markE0TbdrN[:, n] for n in range(3)]
    return g
