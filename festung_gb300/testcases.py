"""Built-in test cases of the ``advection_gpu`` problem (host side).

'solid_body' and 'transient' are the reference's cases (advection/configureProblem.m:106-133);
'gauss_slot' is the rotating Gaussian hump plus slotted cylinder of the benchmark workloads and
'ensemble' a seeded random instance (8-mode streamfunction velocity, Gaussian hump, jittered
mesh).  Source and Dirichlet data are given as time-separable terms
``[(timeFn, spatial function), ...]`` with timeFn in {'const', 'exp_neg'} (g(t) = 1 or e^-t),
which is what the device solver evaluates per stage.

Meshes: domainSquare (core/domainSquare.m:67-105) on [0,1]^2, optionally with seeded jitter
of the interior nodes (numpy default_rng, a fixed call order).
"""
import numpy as np


def square_coords(hmax, a=0.0, b=1.0):
    """Vertex coordinates of domainSquare and its triangles (0-based, counter-clockwise)."""
    dim = int(np.ceil((b - a) / hmax))
    h = (b - a) / dim
    n = int(np.floor((b - a) / h + 1e-10)) + 1
    v = a + np.arange(n) * h
    if abs(v[-1] - b) < 1e-10 * max(1.0, abs(b)):
        v[-1] = b
    X, Y = np.meshgrid(v, v)
    coordV = np.stack([X.ravel(order='F'), Y.ravel(order='F')], axis=1)
    r = np.arange(dim * (dim + 1))
    base = r[(r + 1) % (dim + 1) != 0]
    V0T = np.concatenate([np.stack([base, base + dim + 1, base + 1], 1),
                          np.stack([base + dim + 1, base + dim + 2, base + 1], 1)], 0)
    return coordV, V0T.astype(np.int64), dim, h


def jitter_coords(coordV, h, jitter, seed, a=0.0, b=1.0):
    if jitter <= 0:
        return coordV
    rng = np.random.default_rng(seed)
    d = rng.uniform(-1.0, 1.0, size=coordV.shape) * (jitter * h)
    interior = ((coordV[:, 0] > a) & (coordV[:, 0] < b) & (coordV[:, 1] > a) & (coordV[:, 1] < b))
    out = coordV.copy()
    out[interior] += d[interior]
    return out


def boundary_ids(baryE, a=0.0, b=1.0):
    """idE of domainSquare: south 1, east 2, north 3, west 4 (core/domainSquare.m:100-104)."""
    tol = 10 * np.finfo(np.float64).eps
    idE = np.zeros(baryE.shape[0], dtype=np.int64)
    idE[np.abs(baryE[:, 1] - a) < tol] = 1
    idE[np.abs(baryE[:, 0] - b) < tol] = 2
    idE[np.abs(baryE[:, 1] - b) < tol] = 3
    idE[np.abs(baryE[:, 0] - a) < tol] = 4
    return idE


def slotted_cylinder(x1, x2):
    return (((x1 - 0.5) ** 2 + (x2 - 0.75) ** 2 <= 0.0225)
            & ((x1 <= 0.475) | (x1 >= 0.525) | (x2 >= 0.85))).astype(np.float64)


def ensemble_params(seed):
    """Random instance: mesh level, degree, streamfunction modes, hump centre and width."""
    rng = np.random.default_rng(seed)
    level = int(rng.choice([5, 6, 7]))
    p = int(rng.choice([1, 2]))
    k = rng.integers(1, 4, size=8)
    l = rng.integers(1, 4, size=8)
    a = rng.normal(0.0, 0.1, size=8)
    centre = rng.uniform(0.2, 0.8, size=2)
    width = float(rng.uniform(0.05, 0.15))
    return dict(hmax=2.0 ** -level, p=p, k=k, l=l, a=a, centre=centre, width=width,
                mesh_seed=int(rng.integers(0, 2 ** 31 - 1)))


def streamfunction_velocity(k, l, a):
    """u = (d psi/dy, -d psi/dx), psi = sum_m a_m sin(k_m pi x) sin(l_m pi y)."""
    def u1(x1, x2):
        out = np.zeros(np.broadcast(x1, x2).shape)
        for km, lm, am in zip(k, l, a):
            out = out + am * (lm * np.pi) * np.sin(km * np.pi * x1) * np.cos(lm * np.pi * x2)
        return out

    def u2(x1, x2):
        out = np.zeros(np.broadcast(x1, x2).shape)
        for km, lm, am in zip(k, l, a):
            out = out - am * (km * np.pi) * np.cos(km * np.pi * x1) * np.sin(lm * np.pi * x2)
        return out
    return u1, u2


# Velocity modes of the adjoint workload: psi_m = sin(k_m pi x) sin(l_m pi y), (k_m, l_m) in
# {1..4}^2 (u . n = 0 on the unit square's boundary).
ADJOINT_MODES = [(k, l) for k in (1, 2, 3, 4) for l in (1, 2, 3, 4)]


def adjoint_params(seed):
    """Coefficients of the adjoint workload's streamfunction psi = sum_m theta_m psi_m: base
    theta ~ N(0, 0.1^2); the target run adds N(0, 0.05^2) to 8 of the 16 modes (seeded)."""
    rng = np.random.default_rng(seed)
    theta = rng.normal(0.0, 0.1, size=len(ADJOINT_MODES))
    idx = rng.choice(len(ADJOINT_MODES), size=8, replace=False)
    dtheta = np.zeros(len(ADJOINT_MODES))
    dtheta[idx] = rng.normal(0.0, 0.05, size=8)
    return dict(theta=theta, dtheta=dtheta)


def mode_velocity(m):
    k, l = ADJOINT_MODES[m]
    return streamfunction_velocity([k], [l], [1.0])


# The explicit problem's test cases (configure below; the Matlab folder's configureProblem.m
# defines the same names).
TESTCASES = ('solid_body', 'transient', 'gauss_slot', 'ensemble', 'adjoint')


def configure(pd):
    """Sets c0Cont, u1Cont, u2Cont (time-independent), fTerms, cDTerms, mesh parameters."""
    tc = pd['testcase']
    pd['fTerms'] = []
    pd['cDTerms'] = []
    if pd.get('jitter') is None:
        pd['jitter'] = 0.2 if tc == 'ensemble' else 0.0
    pd.setdefault('meshSeed', 0)
    if tc in ('solid_body', 'gauss_slot'):
        pd['isAnalytical'] = False
        pd['u1Cont'] = lambda x1, x2: 0.5 - x2
        pd['u2Cont'] = lambda x1, x2: x1 - 0.5
        if tc == 'solid_body':
            Gf = lambda x1, x2, a, b: (1 / 0.15) * np.sqrt((x1 - a) ** 2 + (x2 - b) ** 2)
            pd['c0Cont'] = lambda x1, x2: (
                slotted_cylinder(x1, x2)
                + (1 - Gf(x1, x2, 0.5, 0.25)) * ((x1 - 0.5) ** 2 + (x2 - 0.25) ** 2 <= 0.0225)
                + 0.25 * (1 + np.cos(np.pi * Gf(x1, x2, 0.25, 0.5))) * ((x1 - 0.25) ** 2 + (x2 - 0.5) ** 2 <= 0.0225))
        else:
            pd['c0Cont'] = lambda x1, x2: (np.exp(-((x1 - 0.25) ** 2 + (x2 - 0.5) ** 2) / 0.01)
                                           + slotted_cylinder(x1, x2))
    elif tc == 'transient':
        pd['isAnalytical'] = True
        u1 = lambda x1, x2: np.exp(0.5 * (x1 + x2))
        u2 = lambda x1, x2: np.exp(0.5 * (x1 - x2))
        pd['u1Cont'], pd['u2Cont'] = u1, u2
        pd['cCont'] = lambda t, x1, x2: np.cos(7 * x1) * np.cos(7 * x2) + np.exp(-t)
        pd['c0Cont'] = lambda x1, x2: pd['cCont'](0, x1, x2)
        # f(t) = A(x) + e^-t Bf(x), c_D(t) = C(x) + e^-t
        pd['fTerms'] = [
            ('const', lambda x1, x2: (-7 * u1(x1, x2) * np.sin(7 * x1) * np.cos(7 * x2)
                                      - 7 * u2(x1, x2) * np.cos(7 * x1) * np.sin(7 * x2)
                                      + 0.5 * (u1(x1, x2) - u2(x1, x2)) * np.cos(7 * x1) * np.cos(7 * x2))),
            ('exp_neg', lambda x1, x2: -1 + 0.5 * (u1(x1, x2) - u2(x1, x2))),
        ]
        pd['cDTerms'] = [
            ('const', lambda x1, x2: np.cos(7 * x1) * np.cos(7 * x2)),
            ('exp_neg', lambda x1, x2: np.ones(np.broadcast(x1, x2).shape)),
        ]
    elif tc == 'ensemble':
        pd['isAnalytical'] = False
        prm = ensemble_params(pd['instanceSeed'])
        pd['ensembleParams'] = prm
        pd['meshSeed'] = prm['mesh_seed']
        pd['u1Cont'], pd['u2Cont'] = streamfunction_velocity(prm['k'], prm['l'], prm['a'])
        cx, cy = prm['centre']; w2 = prm['width'] ** 2
        pd['c0Cont'] = lambda x1, x2: np.exp(-((x1 - cx) ** 2 + (x2 - cy) ** 2) / w2)
    elif tc == 'adjoint':
        pd['isAnalytical'] = False
        prm = adjoint_params(pd.get('adjointSeed', 0))
        theta = prm['theta'] + (prm['dtheta'] if pd.get('adjointTarget', False) else 0.0)
        pd['theta'] = theta
        pd['u1Cont'], pd['u2Cont'] = streamfunction_velocity([k for k, _ in ADJOINT_MODES],
                                                             [l for _, l in ADJOINT_MODES], theta)
        pd['c0Cont'] = lambda x1, x2: np.exp(-((x1 - 0.4) ** 2 + (x2 - 0.45) ** 2) / 0.01)
    else:
        raise ValueError('Invalid testcase "%s".' % tc)
    return pd


def device_functions(pd):
    """The configured problem's data as device functions (kind, params) of ``dgadv_function``:
    'c0' (initial data), 'u' (velocity) and, for analytical cases, 'cCont' (exact solution,
    evaluated at a time t).  The parameters reproduce the host closures above."""
    from . import _lib as L
    tc = pd['testcase']
    if tc == 'solid_body':
        return dict(c0=(L.FN_SOLID_BODY, []), u=(L.VEL_ROTATION, []))
    if tc == 'gauss_slot':
        return dict(c0=(L.FN_GAUSS_SLOT, []), u=(L.VEL_ROTATION, []))
    if tc == 'transient':
        return dict(c0=(L.FN_TRANSIENT, []), u=(L.VEL_TRANSIENT, []), cCont=(L.FN_TRANSIENT, []))
    if tc == 'ensemble':
        prm = pd['ensembleParams']
        cx, cy = prm['centre']
        return dict(c0=(L.FN_GAUSS, [cx, cy, prm['width'] ** 2]),
                    u=(L.VEL_STREAM, np.concatenate([prm['k'], prm['l'], prm['a']]).astype(np.float64)))
    if tc == 'adjoint':
        k = [km for km, _ in ADJOINT_MODES]
        l = [lm for _, lm in ADJOINT_MODES]
        return dict(c0=(L.FN_GAUSS, [0.4, 0.45, 0.01]),
                    u=(L.VEL_STREAM, np.concatenate([k, l, pd['theta']]).astype(np.float64)))
    return None


# ---------------------------------------------------------------------------------------------
# Test cases of the implicit problem (advection_implicit/getTestcase.m).  Source and Dirichlet
# data as time-separable terms, as above; 'stationary' has no Neumann edge (its id -1 marks
# none), so every boundary edge is Dirichlet.
IMPLICIT_CASES = ('solid_body', 'stationary', 'transient_ode', 'transient')


def configure_implicit(pd):
    """Sets isStationary, isAnalytical, numSteps, tEnd, c0Cont, u1Cont, u2Cont, cCont, fTerms,
    cDTerms and the device functions ('c0', 'u', 'cCont' at a time t) of an implicit case."""
    from . import _lib as L
    tc = pd['testcase']
    cos7 = lambda x1, x2: np.cos(7 * x1) * np.cos(7 * x2)
    u1e = lambda x1, x2: np.exp(0.5 * (x1 + x2))
    u2e = lambda x1, x2: np.exp(0.5 * (x1 - x2))
    adv = lambda x1, x2: (-7 * u1e(x1, x2) * np.sin(7 * x1) * np.cos(7 * x2)
                          - 7 * u2e(x1, x2) * np.cos(7 * x1) * np.sin(7 * x2)
                          + 0.5 * (u1e(x1, x2) - u2e(x1, x2)) * cos7(x1, x2))
    ones = lambda x1, x2: np.ones(np.broadcast(x1, x2).shape)
    if tc == 'solid_body':
        d = dict(isStationary=False, isAnalytical=False, numSteps=320, tEnd=2 * np.pi,
                 u1Cont=lambda x1, x2: 0.5 - x2, u2Cont=lambda x1, x2: x1 - 0.5, fTerms=[], cDTerms=[])
        d['c0Cont'] = configure(dict(testcase='solid_body', jitter=0.0))['c0Cont']   # the explicit case's c0
        fns = dict(c0=(L.FN_SOLID_BODY, []), u=(L.VEL_ROTATION, []))
    elif tc == 'stationary':
        d = dict(isStationary=True, isAnalytical=True, numSteps=1, tEnd=10, u1Cont=u1e, u2Cont=u2e,
                 cCont=lambda t, x1, x2: cos7(x1, x2), c0Cont=cos7,
                 fTerms=[('const', adv)], cDTerms=[('const', cos7)])
        fns = dict(c0=(L.FN_COS7, []), u=(L.VEL_TRANSIENT, []), cCont=(L.FN_COS7, []))
    elif tc == 'transient_ode':
        zero = lambda x1, x2: np.zeros(np.broadcast(x1, x2).shape)
        d = dict(isStationary=False, isAnalytical=True, numSteps=4, tEnd=2, u1Cont=zero, u2Cont=zero,
                 cCont=lambda t, x1, x2: np.exp(-t) * ones(x1, x2), c0Cont=ones,
                 fTerms=[('exp_neg', lambda x1, x2: -ones(x1, x2))], cDTerms=[('exp_neg', ones)])
        fns = dict(c0=(L.FN_CONST, [1.0]), u=(L.VEL_CONST, [0.0, 0.0]))
    elif tc == 'transient':
        d = dict(isStationary=False, isAnalytical=True, numSteps=10, tEnd=2, u1Cont=u1e, u2Cont=u2e,
                 cCont=lambda t, x1, x2: cos7(x1, x2) + np.exp(-t),
                 c0Cont=lambda x1, x2: cos7(x1, x2) + 1.0,
                 fTerms=[('const', adv), ('exp_neg', lambda x1, x2: -1 + 0.5 * (u1e(x1, x2) - u2e(x1, x2)))],
                 cDTerms=[('const', cos7), ('exp_neg', ones)])
        fns = dict(c0=(L.FN_TRANSIENT, []), u=(L.VEL_TRANSIENT, []), cCont=(L.FN_TRANSIENT, []))
    else:
        raise ValueError('Invalid testcase "%s".' % tc)
    for k, v in d.items():
        pd.setdefault(k, v)
    pd['jitter'] = pd.get('jitter') or 0.0
    pd.setdefault('meshSeed', 0)
    pd['implicitFns'] = fns
    return pd
