"""The ``advection_implicit_gpu`` problem: the step functions of FESTUNG's ``advection_implicit``
problem with the stage solves on the GPU.

The reference (advection_implicit/*.m) integrates with diagonally implicit Runge-Kutta methods of
order 1..4 (core/rungeKuttaImplicit.m) and solves each stage, or the stationary problem, with a
sparse direct solver.  Here one ``dgadv_step_implicit`` call runs a whole step: every stage is a
matrix-free GMRES solve on the device (``DGADV_FLAG_IMPLICIT`` handle).  The step functions and
``problemData`` fields follow the reference:
  configureProblem      advection_implicit/configureProblem.m (p = 2, ordRK = min(p+1, 4),
                        qOrd = 2p+1, hmax = 2^-6), test cases of getTestcase.m
  preprocessProblem     advection_implicit/preprocessProblem.m (grid, markers, device upload)
  initializeProblem     advection_implicit/initializeProblem.m (projection of c0)
  solveStep             advection_implicit/solveStep.m + its sub-steps
  postprocessStep       advection_implicit/postprocessStep.m
  postprocessProblem    advection_implicit/postprocessProblem.m (L2 error, rule of order qOrd+1)
Keys beyond the reference: precision ('fp64' | 'fp32'), krylovTol, krylovMaxIter,
krylovRestart, device.  ``pd.iterations`` counts GMRES iterations.
"""
import numpy as np

from . import _lib as L
from . import advection_gpu as AG
from . import testcases as TC
from .solver import DeviceSolver

Struct = AG.Struct


def configureProblem(pd):
    AG.setdefault(pd, 'testcase', 'solid_body')
    AG.setdefault(pd, 'hmax', 2 ** -6)
    AG.setdefault(pd, 'p', 2)
    AG.setdefault(pd, 'ordRK', min(pd.p + 1, 4))
    AG.setdefault(pd, 'qOrd', 2 * pd.p + 1)
    AG.setdefault(pd, 'precision', 'fp64')
    AG.setdefault(pd, 'device', 0)
    AG.setdefault(pd, 'krylovTol', 1e-12 if pd.precision == 'fp64' else 1e-6)
    AG.setdefault(pd, 'krylovMaxIter', 4000)
    AG.setdefault(pd, 'krylovRestart', 50)
    AG.setdefault(pd, 'isVisSol', False)      # the reference defaults to true (writes files)
    AG.setdefault(pd, 'outputFrequency', 50)
    AG.setdefault(pd, 'outputBasename', 'output/advection_implicit')
    AG.setdefault(pd, 'outputTypes', ['vtk', 'tec'])
    TC.configure_implicit(pd)
    assert 0 <= pd.p <= 3, 'the device kernels cover p = 0..3'
    assert 1 <= pd.ordRK <= 4, 'Order of Runge-Kutta method must be one to four.'
    assert pd.hmax > 0 and pd.numSteps > 0
    return pd


def preprocessProblem(pd):
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
    tables = AG.Tables(pd.N)
    pd.tables = tables
    _, _, W = tables.rule2(pd.qOrd)
    P = tables.phi2D(pd.qOrd)
    pd.hatM = (W[:, None] * P).T @ P
    pd.solver = DeviceSolver(coordV, V0T, pd.p, 1, precision=pd.precision, idE0T=g['idE0T'],
                             markE0TbdrD=g['markE0TbdrD'], markE0TbdrN=g['markE0TbdrN'],
                             device=pd.device, flags=L.FLAG_IMPLICIT)
    pd.solver.set_velocity_function(pd.implicitFns['u'])
    # separable right-hand side M f_m - K_D,m (advection_implicit/preprocessSubStep.m: fDisc and
    # K_D with the rule of order qOrd)
    terms = {}
    if pd.cDTerms:
        vN = AG.normal_velocity(g, tables, pd.u1Cont, pd.u2Cont, pd.qOrd)
    for fn, f in pd.fTerms:
        fd = AG.project(g, tables, f, pd.qOrd, pd.hatM)
        terms.setdefault(fn, np.zeros((pd.K, pd.N)))[...] += g['detJ0T'][:, None] * (fd @ pd.hatM.T)
    for fn, f in pd.cDTerms:
        terms.setdefault(fn, np.zeros((pd.K, pd.N)))[...] -= AG.dirichlet_vector(
            g, tables, g['markE0TbdrD'], f, vN, pd.qOrd)
    codes = {'const': L.TIME_CONST, 'exp_neg': L.TIME_EXP_NEG}
    names = sorted(terms)
    pd.solver.set_source_terms([codes[n] for n in names], [terms[n] for n in names])
    return pd


def initializeProblem(pd):
    pd.isFinished = False
    pd.iterations = 0
    if not pd.isStationary:
        pd.solver.project_state(pd.implicitFns['c0'], 0.0, pd.qOrd)
        if pd.isVisSol:
            pd.solver.output(pd.outputBasename, 0, pd.outputTypes)
    return pd


def preprocessStep(pd, nStep):
    return pd


def solveStep(pd, nStep):
    kr = dict(tol=pd.krylovTol, maxIter=pd.krylovMaxIter, restart=pd.krylovRestart)
    if pd.isStationary:
        it, pd.relres = pd.solver.solve_stationary(**kr)
    else:
        it, pd.relres = pd.solver.step_implicit(1, nStep - 1, pd.tau, pd.ordRK, **kr)
    pd.iterations += it
    return pd


def postprocessStep(pd, nStep):
    pd.isFinished = pd.isStationary or nStep >= pd.numSteps
    return pd


def outputStep(pd, nStep):
    if pd.isVisSol and nStep % pd.outputFrequency == 0:
        pd.solver.output(pd.outputBasename, nStep, pd.outputTypes)
    return pd


def postprocessProblem(pd):
    if pd.isVisSol:
        pd.solver.output(pd.outputBasename, pd.numSteps, pd.outputTypes)
        pd.solver.output_wait()
    pd.cDisc = pd.solver.get_state()
    fns = pd.implicitFns
    if pd.isAnalytical:
        if 'cCont' in fns:
            pd.error = pd.solver.l2_error(fns['cCont'], pd.tEnd, pd.qOrd + 1)
        else:   # 'transient_ode': c(t) = exp(-t), constant in space
            pd.error = pd.solver.l2_error((L.FN_CONST, [np.exp(-pd.tEnd)]), pd.tEnd, pd.qOrd + 1)
    else:
        pd.error = pd.solver.l2_error(fns['c0'], 0.0, pd.qOrd + 1)
    return pd


PRE = (configureProblem, preprocessProblem, initializeProblem)
STEP = (preprocessStep, solveStep, postprocessStep, outputStep)
POST = (postprocessProblem,)


def main(problemData=None, **kwargs):
    """main('advection_implicit_gpu', key, value, ...) (main.m:115-178)."""
    pd = AG.Struct(problemData or {})
    pd.update(kwargs)
    pd.problemName = 'advection_implicit_gpu'
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
