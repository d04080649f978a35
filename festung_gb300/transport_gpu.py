"""The ``transport_gpu`` problem: FESTUNG's ``transport`` problem (configuration 'rotation', grid
'square', no coupling to a flow model) with every stage on the GPU.

Several species on one mesh, each advected as its depth-integrated concentration c h with the
depth-integrated velocity (u h, v h), only over its active elements, and limited as a
concentration c = c h / h (transport/solveSubStep.m).  The step functions follow the reference:
  configureProblem      transport/configureProblem.m, 'rotation' (depth 0.1, rotating velocity,
                        four discs of value (species index) x depth; p = 1, ordRK = min(p+1, 3))
  preprocessProblem     transport/preprocessProblem.m ('square': every boundary edge id 3)
  initializeProblem     transport/initializeProblem.m (dgadv_transport_init)
  solveStep             transport/solveStep.m and its sub-steps (dgadv_transport_step)
  postprocessStep       transport/postprocessStep.m (masks; cDisc read back lazily)
The reference keeps hatM = I, so projections here are sum_q W_q f_q phi_i(q) without a solve.
Fields: ``cDisc`` (list of K x N c h), ``concDisc`` (list of K x N c), ``mask`` (list of K).
"""
import numpy as np

from . import _lib as L
from . import advection_gpu as AG
from . import testcases as TC
from .solver import DeviceSolver

Struct = AG.Struct


def configureProblem(pd):
    AG.setdefault(pd, 'p', 1)
    AG.setdefault(pd, 'ordRK', min(pd.p + 1, 3))
    AG.setdefault(pd, 'numSpecies', 1)
    AG.setdefault(pd, 'maskTol', 1e-6)
    AG.setdefault(pd, 'isMask', True)
    AG.setdefault(pd, 'hmax', 2 ** -6)
    AG.setdefault(pd, 'numSteps', 3124)
    AG.setdefault(pd, 'tEnd', (pd.numSteps / 3142) * 2 * np.pi)
    AG.setdefault(pd, 'precision', 'fp64')
    AG.setdefault(pd, 'device', 0)
    assert 1 <= pd.p <= 3 and 1 <= pd.ordRK <= 3 and pd.numSpecies >= 1
    depth = 0.1
    pd.hCont = lambda t, x1, x2: depth * np.ones(np.broadcast(x1, x2).shape)
    pd.uHCont = lambda t, x1, x2: pd.hCont(t, x1, x2) * (0.5 - x2)
    pd.vHCont = lambda t, x1, x2: pd.hCont(t, x1, x2) * (x1 - 0.5)
    r = 0.0225 / np.sqrt(2)

    def cH0(x1, x2):
        return ((((x1 - 0.5) ** 2 + (x2 - 0.75) ** 2 <= r) * 1.0
                 + ((x1 - 0.25) ** 2 + (x2 - 0.5) ** 2 <= r)
                 + ((x1 - 0.5) ** 2 + (x2 - 0.25) ** 2 <= r)
                 + ((x1 - 0.75) ** 2 + (x2 - 0.5) ** 2 <= r)) * pd.hCont(0, x1, x2))
    pd.cH0Cont = [(lambda s: (lambda x1, x2: s * cH0(x1, x2)))(s + 1) for s in range(pd.numSpecies)]
    return pd


def preprocessProblem(pd):
    coordV, V0T, dim, h = TC.square_coords(pd.hmax)
    g = L.grid_build(coordV, V0T)
    g['coordV'], g['V0T'] = coordV, V0T
    bx, by = g['baryE'][:, 0], g['baryE'][:, 1]
    idE = np.zeros(g['numE'], dtype=np.int64)
    idE[(by == 0) | (bx == 1) | (by == 1) | (bx == 0)] = 3
    g['idE0T'] = idE[g['E0T']]
    g['markE0TbdrN'] = g['idE0T'] == 1
    g['markE0TbdrD'] = (g['idE0T'] == 2) | (g['idE0T'] == 3) | (g['idE0T'] == 4)
    pd.g = g
    pd.K = g['numT']
    pd.N = (pd.p + 1) * (pd.p + 2) // 2
    pd.tau = pd.tEnd / pd.numSteps
    pd.tables = AG.Tables(pd.N)
    pd.hatM = np.eye(pd.N)
    pd.solver = DeviceSolver(coordV, V0T, pd.p, pd.ordRK, precision=pd.precision, isSlopeLim=True,
                             typeSlopeLim='linear', idE0T=g['idE0T'], markE0TbdrD=g['markE0TbdrD'],
                             markE0TbdrN=g['markE0TbdrN'], device=pd.device)
    # transport/preprocessSubStep.m: u h, v h projected with order 2p, the normal component at
    # the order-(2p+1) edge points (time-independent here)
    u1 = lambda x1, x2: pd.uHCont(0, x1, x2)
    u2 = lambda x1, x2: pd.vHCont(0, x1, x2)
    pd.solver.set_velocity(AG.project(g, pd.tables, u1, 2 * pd.p, pd.hatM),
                           AG.project(g, pd.tables, u2, 2 * pd.p, pd.hatM),
                           AG.normal_velocity(g, pd.tables, u1, u2, 2 * pd.p + 1))
    return pd


def initializeProblem(pd):
    g, q = pd.g, 2 * pd.p + 1
    hDisc = AG.project(g, pd.tables, lambda x1, x2: pd.hCont(0, x1, x2), q, pd.hatM)
    cH0 = np.stack([AG.project(g, pd.tables, f, q, pd.hatM) for f in pd.cH0Cont], axis=2)
    pd.solver.transport_init(hDisc, cH0, pd.maskTol, pd.isMask)
    pd.isFinished = False
    return pd


def preprocessStep(pd, nStep):
    return pd


def solveStep(pd, nStep):
    pd.solver.transport_step(1, nStep - 1, pd.tau)
    return pd


def postprocessStep(pd, nStep):
    pd.isFinished = nStep >= pd.numSteps
    return pd


def outputStep(pd, nStep):
    return pd


def postprocessProblem(pd):
    out = [pd.solver.transport_get(s) for s in range(pd.numSpecies)]
    pd.cDisc = [o[0] for o in out]
    pd.concDisc = [o[1] for o in out]
    pd.mask = [o[2] for o in out]
    return pd


PRE = (configureProblem, preprocessProblem, initializeProblem)
STEP = (preprocessStep, solveStep, postprocessStep, outputStep)
POST = (postprocessProblem,)


def main(problemData=None, **kwargs):
    """main('transport_gpu', key, value, ...) (main.m:115-178)."""
    pd = Struct(problemData or {})
    pd.update(kwargs)
    pd.problemName = 'transport_gpu'
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
