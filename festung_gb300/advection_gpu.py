"""The ``advection_gpu`` problem: the step-function interface of FESTUNG's ``advection`` problem
with the stage loop on the GPU.

The reference drives a problem through ``main(problemName, key, value, ...)`` (main.m:115-178):
pre-processing steps configureProblem, preprocessProblem, initializeProblem; then per time step
preprocessStep, solveStep, postprocessStep, outputStep until ``isFinished``; then
postprocessProblem.  This module provides the same functions over the same ``problemData``
fields (``cDisc`` K x N, ``K``, ``N``, ``tau``, ``isFinished``, ``error``, ...), so
``main('advection_gpu', ...)`` is a drop-in for ``main('advection', ...)`` on triangles.

Differences in mechanism (not in results):
  * preprocessProblem uploads the mesh, tables and the (time-independent) velocity once; the
    reference re-assembles sparse operators every stage (advection/preprocessSubStep.m:56-99).
  * solveStep enqueues one time step with all its RK stages (advection/solveStep.m:57-73 and the
    sub-steps advection/solveSubStep.m:57-99) and returns without waiting; ``cDisc`` is read back
    lazily, when postprocessProblem or the caller asks for it.
  * source and Dirichlet data are time-separable terms (see ``festung_gb300.testcases``).
Host-side set-up work (projections of the initial data and of the velocity, boundary vectors,
L2 error) runs in numpy with the library's quadrature rules and basis values, as the
reference's host code does with its core functions.
"""
import numpy as np

from . import _lib as L
from . import testcases as TC
from .solver import DeviceSolver


class Struct(dict):
    def __getattr__(self, k):
        try:
            return self[k]
        except KeyError as e:
            raise AttributeError(k) from e

    def __setattr__(self, k, v):
        self[k] = v


def setdefault(pd, key, value):
    if key not in pd:
        pd[key] = value


# ---------------------------------------------------------------------------------------------
# Host-side set-up helpers (restate the reference's core functions for the set-up phase).
class Tables:
    """Quadrature rules and basis values by quadrature order (core/computeBasesOnQuad.m)."""

    def __init__(self, N):
        self.N = N
        self._r2, self._r1, self._phi2D, self._phi1D = {}, {}, {}, {}

    def rule2(self, qOrd):
        if qOrd not in self._r2:
            self._r2[qOrd] = L.quad_rule_2d(qOrd)
        return self._r2[qOrd]

    def rule1(self, qOrd):
        if qOrd not in self._r1:
            self._r1[qOrd] = L.quad_rule_1d(qOrd)
        return self._r1[qOrd]

    def phi2D(self, qOrd):
        if qOrd not in self._phi2D:
            Q1, Q2, _ = self.rule2(qOrd)
            self._phi2D[qOrd] = L.basis_eval(self.N, Q1, Q2)
        return self._phi2D[qOrd]

    def phi1D(self, qOrd):
        """R x N x 3: basis on the edge points gammaMap(n, Q) (core/gammaMap.m:50-57)."""
        if qOrd not in self._phi1D:
            Q, _ = self.rule1(qOrd)
            out = np.zeros((Q.size, self.N, 3))
            for n in range(3):
                X1, X2 = gamma_map(n, Q)
                out[:, :, n] = L.basis_eval(self.N, X1, X2)
            self._phi1D[qOrd] = out
        return self._phi1D[qOrd]


def gamma_map(n, S):
    S = np.asarray(S, dtype=np.float64)
    if n == 0:
        return 1 - S, S
    if n == 1:
        return np.zeros_like(S), 1 - S
    return S, np.zeros_like(S)


def map_ref_to_phy(g, i, X1, X2):
    X1 = np.asarray(X1).reshape(1, -1); X2 = np.asarray(X2).reshape(1, -1)
    return (g['B'][:, i, 0:1] * X1 + g['B'][:, i, 1:2] * X2) + g['coordV0T'][:, 0, i:i + 1] * np.ones_like(X1)


def project(g, tables, func, qOrd, hatM):
    """projectFuncCont2DataDisc (core/projectFuncCont2DataDisc.m:94-102)."""
    qOrd = max(qOrd, 1)
    Q1, Q2, W = tables.rule2(qOrd)
    F = func(map_ref_to_phy(g, 0, Q1, Q2), map_ref_to_phy(g, 1, Q1, Q2))
    rhs = F @ (W[:, None] * tables.phi2D(qOrd))
    return np.linalg.solve(hatM.T, rhs.T).T


def normal_velocity(g, tables, u1, u2, qOrd):
    """computeFuncContNuOnQuadEdge (core/computeFuncContNuOnQuadEdge.m:46-67): K x 3 x R."""
    Q, _ = tables.rule1(qOrd)
    out = np.zeros((g['numT'], 3, Q.size))
    for n in range(3):
        X1, X2 = gamma_map(n, Q)
        x, y = map_ref_to_phy(g, 0, X1, X2), map_ref_to_phy(g, 1, X1, X2)
        out[:, n, :] = g['nuE0T'][:, n, 0:1] * u1(x, y) + g['nuE0T'][:, n, 1:2] * u2(x, y)
    return out


def dirichlet_vector(g, tables, markD, func, vN, qOrd):
    """assembleVecEdgePhiIntFuncContVal (core/assembleVecEdgePhiIntFuncContVal.m:162-185): K x N."""
    Q, W = tables.rule1(qOrd)
    P = tables.phi1D(qOrd)
    out = np.zeros((g['numT'], tables.N))
    for n in range(3):
        X1, X2 = gamma_map(n, Q)
        f = func(map_ref_to_phy(g, 0, X1, X2), map_ref_to_phy(g, 1, X1, X2))
        Kkn = markD[:, n] * g['areaE0T'][:, n]
        v = vN[:, n, :]
        out += Kkn[:, None] * ((f * ((v < 0) * v)) @ (W[:, None] * P[:, :, n]))
    return out


def l2_error(g, tables, cDisc, func, qOrd):
    """computeL2Error (core/computeL2Error.m:97-114)."""
    qOrd = max(qOrd, 1)
    Q1, Q2, W = tables.rule2(qOrd)
    x, y = map_ref_to_phy(g, 0, Q1, Q2), map_ref_to_phy(g, 1, Q1, Q2)
    d = cDisc @ tables.phi2D(qOrd).T - func(x, y)
    return float(np.sqrt(2 * np.dot((d ** 2) @ W, g['areaT'])))


def vertex_values(g, func):
    """computeFuncContV0T (core/computeFuncContV0T.m:41-51): K x 3."""
    return np.stack([func(g['coordV0T'][:, n, 0], g['coordV0T'][:, n, 1]) for n in range(3)], axis=1)


# ---------------------------------------------------------------------------------------------
# Step functions
def configureProblem(pd):
    """advection/configureProblem.m:61-151 (triangle path)."""
    setdefault(pd, 'testcase', 'solid_body')
    setdefault(pd, 'hmax', 2 ** -6)
    setdefault(pd, 'isQuadri', False)
    setdefault(pd, 'p', 0)
    setdefault(pd, 'qOrd', 2 * pd.p + 1)
    setdefault(pd, 'ordRK', min(pd.p + 1, 3))
    setdefault(pd, 'numSteps', 100)
    setdefault(pd, 'tEnd', (pd.numSteps / (3142 * 1.5)) * 2 * np.pi)
    setdefault(pd, 'isSlopeLim', False)
    setdefault(pd, 'typeSlopeLim', 'linear')
    setdefault(pd, 'isVisSol', False)          # the reference defaults to true (writes files)
    setdefault(pd, 'outputFrequency', 100)
    setdefault(pd, 'outputBasename', 'output/advection_' + pd.typeSlopeLim)
    setdefault(pd, 'outputTypes', ['vtk'])
    setdefault(pd, 'precision', 'fp64')
    setdefault(pd, 'device', 0)
    setdefault(pd, 'gpuFlags', 0)
    setdefault(pd, 'setupOnDevice', True)      # projections, velocity data, L2 errors on the GPU
    assert not pd.isQuadri, 'advection_gpu supports triangles only (isQuadri = false).'
    assert 0 <= pd.p <= 4, 'Polynomial order must be zero to four.'
    assert 1 <= pd.ordRK <= 3, 'Order of Runge Kutta must be zero to three.'
    assert pd.hmax > 0, 'Maximum edge length must be positive.'
    assert pd.numSteps > 0, 'Number of time steps must be positive.'
    assert (not pd.isSlopeLim) or pd.p > 0, 'Slope limiting only available for p > 0.'
    TC.configure(pd)
    pd.deviceFns = TC.device_functions(pd) if pd.setupOnDevice else None
    return pd


def host_preprocess(pd):
    """The host part of advection/preprocessProblem.m:48-112: grid, markers, tables, the
    separable right-hand-side terms, and (without device functions for the case) the velocity
    data (advection/preprocessSubStep.m:72-79, time-independent); no device work."""
    coordV, V0T, dim, h = TC.square_coords(pd.hmax)
    coordV = TC.jitter_coords(coordV, h, pd.jitter, pd.meshSeed)
    g = L.grid_build(coordV, V0T)
    g['coordV'], g['V0T'] = coordV, V0T
    g['idE'] = TC.boundary_ids(g['baryE'])
    g['idE0T'] = g['idE'][g['E0T']]
    g['markE0Tint'] = g['idE0T'] == 0
    g['markE0TbdrN'] = np.zeros((g['numT'], 3), dtype=bool)
    g['markE0TbdrD'] = ~(g['markE0Tint'] | g['markE0TbdrN'])
    pd.g = g
    pd.K = g['numT']
    pd.N = (pd.p + 1) * (pd.p + 2) // 2
    pd.tau = pd.tEnd / pd.numSteps
    tables = Tables(pd.N)
    pd.tables = tables
    qv = max(2 * pd.p, 1)
    _, _, W = tables.rule2(qv)
    P = tables.phi2D(qv)
    pd.hatM = (W[:, None] * P).T @ P
    if not pd.get('deviceFns'):
        pd.u1Disc = project(g, tables, pd.u1Cont, 2 * pd.p, pd.hatM)
        pd.u2Disc = project(g, tables, pd.u2Cont, 2 * pd.p, pd.hatM)
    if not pd.get('deviceFns') or pd.cDTerms:     # the Dirichlet vectors need it on the host
        pd.vNormalOnQuadEdge = normal_velocity(g, tables, pd.u1Cont, pd.u2Cont, 2 * pd.p + 1)
    # separable right-hand-side terms rhs_m = M f_m - K_D,m  (K_N = 0: no Neumann data)
    terms = {}
    detJ = g['detJ0T']
    for fn, f in pd.fTerms:
        fd = project(g, tables, f, 2 * pd.p, pd.hatM)
        terms.setdefault(fn, [np.zeros((pd.K, pd.N)), np.zeros((pd.K, 3))])[0][...] += \
            detJ[:, None] * (fd @ pd.hatM.T)
    for fn, f in pd.cDTerms:
        e = terms.setdefault(fn, [np.zeros((pd.K, pd.N)), np.zeros((pd.K, 3))])
        e[0][...] -= dirichlet_vector(g, tables, g['markE0TbdrD'], f, pd.vNormalOnQuadEdge, pd.qOrd)
        e[1][...] += vertex_values(g, f)
    codes = {'const': L.TIME_CONST, 'exp_neg': L.TIME_EXP_NEG}
    names = sorted(terms)
    pd.srcTimeFn = [codes[n] for n in names]
    pd.srcRhs = [terms[n][0] for n in names]
    pd.srcCD = [terms[n][1] for n in names] if pd.cDTerms else None
    return pd


def instance_mesh(pd):
    """The mesh of one problem as DeviceSolver takes it (also one instance of an ensemble)."""
    g = pd.g
    return dict(coordV=g['coordV'], V0T=g['V0T'], idE0T=g['idE0T'], markE0TbdrD=g['markE0TbdrD'],
                markE0TbdrN=g['markE0TbdrN'])


def preprocessProblem(pd):
    """advection/preprocessProblem.m:48-112: grid, markers, tables; device upload."""
    host_preprocess(pd)
    m = instance_mesh(pd)
    pd.solver = DeviceSolver(m['coordV'], m['V0T'], pd.p, pd.ordRK, precision=pd.precision,
                             isSlopeLim=pd.isSlopeLim, typeSlopeLim=pd.typeSlopeLim,
                             idE0T=m['idE0T'], markE0TbdrD=m['markE0TbdrD'],
                             markE0TbdrN=m['markE0TbdrN'], device=pd.device, flags=pd.gpuFlags)
    for opt, val in (pd.get('gpuOptions') or {}).items():     # {DGADV_OPT_*: value}
        pd.solver.set_option(opt, val)
    if pd.deviceFns:
        pd.solver.set_velocity_function(pd.deviceFns['u'])
    else:
        pd.solver.set_velocity(pd.u1Disc, pd.u2Disc, pd.vNormalOnQuadEdge)
    pd.solver.set_source_terms(pd.srcTimeFn, pd.srcRhs, pd.srcCD)
    return pd


def initializeProblem(pd):
    """advection/initializeProblem.m:46-86: L2 projection of c0, initial limiting, error."""
    pd.isFinished = False
    if pd.deviceFns:
        pd.solver.project_state(pd.deviceFns['c0'], 0.0, pd.qOrd)
    else:
        pd.solver.set_state(project(pd.g, pd.tables, pd.c0Cont, pd.qOrd, pd.hatM))
    if pd.isSlopeLim:
        pd.solver.limit_state(0.0)
    pd._cDisc = np.ascontiguousarray(pd.solver.get_state())
    pd._stale = False
    if pd.deviceFns:
        pd.initialError = pd.solver.l2_error(pd.deviceFns['c0'], 0.0, 2 * pd.p)
    else:
        pd.initialError = l2_error(pd.g, pd.tables, pd._cDisc, pd.c0Cont, 2 * pd.p)
    if pd.isVisSol:
        pd.solver.output(pd.outputBasename, 0, pd.outputTypes)
    return pd


def cDisc(pd):
    """Current coefficients K x N (read back from the device when stale)."""
    if pd._stale:
        pd._cDisc = np.ascontiguousarray(pd.solver.get_state())
        pd._stale = False
    return pd._cDisc


def preprocessStep(pd, nStep):
    return pd


def solveStep(pd, nStep):
    """One SSP-RK step with all sub-steps, enqueued on the device (advection/solveStep.m:57-73)."""
    pd.solver.step(1, nStep - 1, pd.tau)
    pd._stale = True
    return pd


def postprocessStep(pd, nStep):
    """advection/postprocessStep.m:54-61 (cDisc is read back lazily)."""
    pd.isFinished = nStep >= pd.numSteps
    return pd


def outputStep(pd, nStep):
    """advection/outputStep.m:53-66: nodal values of u_h every outputFrequency steps, written to
    <outputBasename>.<nStep>.vtu / .plt by the library's writer thread (the call only enqueues)."""
    if pd.isVisSol and nStep % pd.outputFrequency == 0:
        pd.solver.output(pd.outputBasename, nStep, pd.outputTypes)
    return pd


def postprocessProblem(pd):
    """advection/postprocessProblem.m:43-82 (output, then the error against the exact or the
    initial data)."""
    if pd.isVisSol:
        pd.solver.output(pd.outputBasename, pd.numSteps, pd.outputTypes)
        pd.solver.output_wait()
    pd.cDisc = cDisc(pd)
    if pd.deviceFns:
        if pd.isAnalytical:
            pd.error = pd.solver.l2_error(pd.deviceFns['cCont'], pd.tEnd, pd.qOrd)
        else:
            pd.error = pd.solver.l2_error(pd.deviceFns['c0'], 0.0, pd.qOrd)
        return pd
    if pd.isAnalytical:
        f = lambda x1, x2: pd.cCont(pd.tEnd, x1, x2)
    else:
        f = pd.c0Cont
    pd.error = l2_error(pd.g, pd.tables, pd.cDisc, f, pd.qOrd)
    return pd


PRE = (configureProblem, preprocessProblem, initializeProblem)
STEP = (preprocessStep, solveStep, postprocessStep, outputStep)
POST = (postprocessProblem,)


def main(problemData=None, **kwargs):
    """main('advection_gpu', key, value, ...) (main.m:115-178)."""
    pd = Struct(problemData or {})
    pd.update(kwargs)
    pd.problemName = 'advection_gpu'
    for f in PRE:
        pd = f(pd)
    nStep = 0
    while not pd.isFinished:
        nStep += 1
        for f in STEP:
            pd = f(pd, nStep)
    for f in POST:
        pd = f(pd)
    return pd
