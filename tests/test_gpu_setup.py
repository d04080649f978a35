"""Set-up on the device: projections, velocity data and L2 errors from the built-in test cases'
device functions, against the oracle's projectFuncCont2DataDisc / computeL2Error and against the
host set-up path.

Bars (FP64): projections within 1e-13 of the oracle (max norm, the data are O(1); the quadrature
points are computed with the oracle's roundings, so the indicator functions of 'solid_body' and
'gauss_slot' agree point by point); steps driven by device velocity data within 1e-12 of steps
driven by the host arrays; L2 errors within 1e-12 relative of the oracle.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = ['solid_body', 'gauss_slot', 'transient', 'ensemble', 'adjoint']


def _host_problem(testcase, p, precision='fp64', hmax=2 ** -4, **kw):
    """configureProblem + the host path of preprocessProblem (host projections)."""
    from festung_gb300 import advection_gpu as G
    args = dict(testcase=testcase, hmax=hmax, p=p, precision=precision, setupOnDevice=False)
    if testcase == 'ensemble':
        args['instanceSeed'] = 3
    args.update(kw)
    pd = G.Struct(args)
    pd.problemName = 'advection_gpu'
    G.configureProblem(pd)
    G.preprocessProblem(pd)
    return pd


def _oracle(pd):
    from oracle import basis as B
    from oracle import grid as OG
    g = OG.generateGridData(pd.g['coordV'], pd.g['V0T'])
    bases = B.computeBasesOnQuad(pd.N)
    return g, bases, B.integrateRefElemPhiPhi(pd.N, bases)


@pytest.mark.parametrize('testcase', CASES)
@pytest.mark.parametrize('p', [0, 1, 2, 3])
def test_projection_matches_oracle(lib, testcase, p):
    from festung_gb300 import testcases as TC
    from oracle import assembly as A
    pd = _host_problem(testcase, p)
    s = pd.solver
    try:
        s.project_state(TC.device_functions(pd)['c0'], 0.0, pd.qOrd)
        c = s.get_state()
    finally:
        s.close()
    g, bases, hatM = _oracle(pd)
    ref = A.projectFuncCont2DataDisc(g, pd.c0Cont, pd.qOrd, hatM, bases)
    assert np.abs(c - ref).max() < 1e-13


@pytest.mark.parametrize('testcase', CASES)
@pytest.mark.parametrize('p', [1, 2])
def test_device_velocity_steps_match_host_velocity(lib, testcase, p):
    from festung_gb300 import testcases as TC
    pd = _host_problem(testcase, p)
    s = pd.solver
    try:
        c0 = np.asfortranarray(np.random.default_rng(p).standard_normal((pd.K, pd.N)))
        s.set_state(c0)
        s.step(5, 0, 1e-3)
        ref = s.get_state()
        s.set_velocity_function(TC.device_functions(pd)['u'])
        s.set_state(c0)
        s.step(5, 0, 1e-3)
        got = s.get_state()
    finally:
        s.close()
    assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize('testcase', ['solid_body', 'transient', 'ensemble'])
@pytest.mark.parametrize('p', [0, 1, 2, 3])
def test_l2_error_matches_oracle(lib, testcase, p):
    from festung_gb300 import testcases as TC
    from oracle import assembly as A
    pd = _host_problem(testcase, p)
    s = pd.solver
    c = np.asfortranarray(np.random.default_rng(7).standard_normal((pd.K, pd.N)) * 0.1)
    fn = TC.device_functions(pd)
    f, t = (fn['cCont'], 0.3) if 'cCont' in fn else (fn['c0'], 0.0)
    fh = (lambda x1, x2: pd.cCont(t, x1, x2)) if 'cCont' in fn else pd.c0Cont
    try:
        s.set_state(c)
        err = s.l2_error(f, t, 2 * p + 1)
    finally:
        s.close()
    g, bases, _ = _oracle(pd)
    ref = A.computeL2Error(g, c, fh, 2 * p + 1, bases)
    assert abs(err - ref) <= 1e-12 * ref


def test_fp32_handle_projects_in_fp64_then_rounds(lib):
    from festung_gb300 import testcases as TC
    pd64 = _host_problem('gauss_slot', 2)
    pd32 = _host_problem('gauss_slot', 2, precision='fp32')
    try:
        for pd in (pd64, pd32):
            pd.solver.project_state(TC.device_functions(pd)['c0'], 0.0, pd.qOrd)
        c64, c32 = pd64.solver.get_state(), pd32.solver.get_state()
    finally:
        pd64.solver.close(); pd32.solver.close()
    assert np.array_equal(c32, c64.astype(np.float32).astype(np.float64))


def test_ensemble_per_instance_functions(lib):
    """One function per instance: each instance's projection, velocity data and L2 error equal
    the single-instance handle's."""
    from festung_gb300 import advection_gpu as G
    from festung_gb300 import ensemble as E
    from festung_gb300 import testcases as TC
    from festung_gb300.solver import DeviceSolver
    seeds = [0, 1, 4]
    pds = [E.instance_problem(sd, hmax=2 ** -4, p=1) for sd in seeds]
    fns = [TC.device_functions(pd) for pd in pds]
    s = DeviceSolver(None, None, 1, 2, precision='fp64', isSlopeLim=True,
                     instances=[G.instance_mesh(pd) for pd in pds])
    try:
        s.set_velocity_function([f['u'] for f in fns])
        s.project_state([f['c0'] for f in fns], 0.0, pds[0].qOrd)
        s.limit_state(0.0)
        s.step(4, 0, 5e-4)
        errs = s.l2_error([f['c0'] for f in fns], 0.0, 3)
        whole = s.l2_error(fns[0]['c0'], 0.0, 3)
        got = s.split(s.get_state())
    finally:
        s.close()
    assert errs.shape == (3,)
    for pd, f, c, e in zip(pds, fns, got, errs):
        one = DeviceSolver(pd.g['coordV'], pd.g['V0T'], 1, 2, precision='fp64', isSlopeLim=True)
        try:
            one.set_velocity_function(f['u'])
            one.project_state(f['c0'], 0.0, pd.qOrd)
            one.limit_state(0.0)
            one.step(4, 0, 5e-4)
            assert np.array_equal(one.get_state(), c)
            assert one.l2_error(f['c0'], 0.0, 3) == pytest.approx(e, rel=1e-14)
        finally:
            one.close()
    assert whole > 0


def test_invalid_functions_are_rejected(lib):
    from festung_gb300 import _lib as L
    pd = _host_problem('solid_body', 1)
    s = pd.solver
    try:
        for bad in [(L.FN_GAUSS, [0.5, 0.5]), (L.VEL_ROTATION, []), (99, [])]:
            with pytest.raises(L.DgadvError) as e:
                s.project_state(bad, 0.0, 3)
            assert e.value.status == L.DGADV_EINVAL
        with pytest.raises(L.DgadvError):
            s.set_velocity_function((L.FN_CONST, [1.0]))
        with pytest.raises(L.DgadvError):
            s.set_velocity_function((L.VEL_STREAM, [1.0, 1.0]))
        with pytest.raises(L.DgadvError):
            s.project_state([(L.FN_CONST, [1.0])] * 2, 0.0, 3)     # one instance, two functions
        with pytest.raises(L.DgadvError):
            s.project_state((L.FN_CONST, [1.0]), 0.0, 21)
        s.project_state((L.FN_CONST, [2.0]), 0.0, 3)
        c = s.get_state()
    finally:
        s.close()
    assert np.allclose(c[:, 0], 2.0 / np.sqrt(2.0)) and np.abs(c[:, 1:]).max() < 1e-14
