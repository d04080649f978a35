"""Test cases of the advection problem (oracle side).

Test infrastructure: see ``oracle/__init__.py``.

'solid_body' and 'transient' restate advection/configureProblem.m:106-133 (LeVeque's solid-body
rotation; the analytical transient case used by advection/doConvergenceTest.m).  'gauss_slot' is
the rotating Gaussian hump plus slotted cylinder of the benchmark configurations, and
'ensemble' the seeded random instance (streamfunction of 8 Fourier modes, Gaussian hump), and
'adjoint' the gradient workload (streamfunction of 16 seeded modes, Gaussian hump); these are
new cases defined by formulas.  Meshes come from domainSquare
(advection/configureProblem.m:139-146 without the PDE toolbox), optionally with seeded jitter of
the interior nodes.

The random draws (``ensemble_params``, ``jittered_square``) use numpy's default_rng in a fixed
call order; the product's host code draws the same numbers from the same seeds.
"""
import numpy as np

from .grid import domainSquare, generateGridData, add_boundary_ids, square_V0T, colon


def slotted_cylinder(x1, x2):
    return (((x1 - 0.5) ** 2 + (x2 - 0.75) ** 2 <= 0.0225)
            & ((x1 <= 0.475) | (x1 >= 0.525) | (x2 >= 0.85))).astype(np.float64)


def jittered_square(hmax, jitter, seed):
    """domainSquare mesh whose interior nodes move by U(-jitter*h, jitter*h) per coordinate."""
    dim = int(np.ceil(1.0 / hmax))
    h = 1.0 / dim
    v = colon(0.0, h, 1.0)
    X, Y = np.meshgrid(v, v)
    coordV = np.stack([X.ravel(order='F'), Y.ravel(order='F')], axis=1)
    if jitter > 0:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-1.0, 1.0, size=coordV.shape) * (jitter * h)
        interior = ((coordV[:, 0] > 0) & (coordV[:, 0] < 1) & (coordV[:, 1] > 0) & (coordV[:, 1] < 1))
        coordV = coordV.copy()
        coordV[interior] += d[interior]
    g = generateGridData(coordV, square_V0T(dim))
    add_boundary_ids(g, 0.0, 1.0)
    return g


def ensemble_params(seed):
    """Random instance of the ensemble workload: mesh level, degree, streamfunction and hump."""
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
    """u = (d psi/dy, -d psi/dx) for psi = sum_m a_m sin(k_m pi x) sin(l_m pi y)."""
    def u1(t, x1, x2):
        out = np.zeros(np.broadcast(x1, x2).shape)
        for km, lm, am in zip(k, l, a):
            out = out + am * (lm * np.pi) * np.sin(km * np.pi * x1) * np.cos(lm * np.pi * x2)
        return out

    def u2(t, x1, x2):
        out = np.zeros(np.broadcast(x1, x2).shape)
        for km, lm, am in zip(k, l, a):
            out = out - am * (km * np.pi) * np.cos(km * np.pi * x1) * np.sin(lm * np.pi * x2)
        return out
    return u1, u2


# Adjoint workload (a new item with no counterpart in the reference): streamfunction modes
# psi_m = sin(k_m pi x) sin(l_m pi y), (k_m, l_m) in {1..4}^2.
ADJOINT_MODES = [(k, l) for k in (1, 2, 3, 4) for l in (1, 2, 3, 4)]


def adjoint_params(seed):
    """Base coefficients theta ~ N(0, 0.1^2); the target run adds N(0, 0.05^2) to 8 modes."""
    rng = np.random.default_rng(seed)
    theta = rng.normal(0.0, 0.1, size=len(ADJOINT_MODES))
    idx = rng.choice(len(ADJOINT_MODES), size=8, replace=False)
    dtheta = np.zeros(len(ADJOINT_MODES))
    dtheta[idx] = rng.normal(0.0, 0.05, size=8)
    return dict(theta=theta, dtheta=dtheta)


def mode_velocity(m):
    k, l = ADJOINT_MODES[m]
    return streamfunction_velocity([k], [l], [1.0])


def configure_testcase(pd):
    tc = pd.testcase
    zero = lambda t, x1, x2: np.zeros(np.broadcast(x1, x2).shape)
    pd.isTimeIndependentData = True
    if tc == 'solid_body':
        pd.isAnalytical = False
        Gf = lambda x1, x2, a, b: (1 / 0.15) * np.sqrt((x1 - a) ** 2 + (x2 - b) ** 2)
        pd.c0Cont = lambda x1, x2: (
            slotted_cylinder(x1, x2)
            + (1 - Gf(x1, x2, 0.5, 0.25)) * ((x1 - 0.5) ** 2 + (x2 - 0.25) ** 2 <= 0.0225)
            + 0.25 * (1 + np.cos(np.pi * Gf(x1, x2, 0.25, 0.5))) * ((x1 - 0.25) ** 2 + (x2 - 0.5) ** 2 <= 0.0225))
        pd.fCont = zero
        pd.u1Cont = lambda t, x1, x2: 0.5 - x2
        pd.u2Cont = lambda t, x1, x2: x1 - 0.5
        pd.cDCont = zero
        pd.gNCont = zero
        pd.generateGridData = domainSquare
    elif tc == 'transient':
        pd.isAnalytical = True
        pd.isTimeIndependentData = False
        pd.cCont = lambda t, x1, x2: np.cos(7 * x1) * np.cos(7 * x2) + np.exp(-t)
        pd.u1Cont = lambda t, x1, x2: np.exp(0.5 * (x1 + x2))
        pd.u2Cont = lambda t, x1, x2: np.exp(0.5 * (x1 - x2))
        pd.fCont = lambda t, x1, x2: (
            -np.exp(-t)
            - 7 * pd.u1Cont(t, x1, x2) * np.sin(7 * x1) * np.cos(7 * x2)
            - 7 * pd.u2Cont(t, x1, x2) * np.cos(7 * x1) * np.sin(7 * x2)
            + 0.5 * (pd.u1Cont(t, x1, x2) - pd.u2Cont(t, x1, x2)) * pd.cCont(t, x1, x2))
        pd.c0Cont = lambda x1, x2: pd.cCont(0, x1, x2)
        pd.cDCont = lambda t, x1, x2: pd.cCont(t, x1, x2)
        pd.gNCont = zero
        pd.generateGridData = domainSquare
    elif tc == 'gauss_slot':
        pd.isAnalytical = False
        pd.setdefault('jitter', 0.0)
        pd.setdefault('meshSeed', 0)
        pd.c0Cont = lambda x1, x2: (np.exp(-((x1 - 0.25) ** 2 + (x2 - 0.5) ** 2) / 0.01)
                                    + slotted_cylinder(x1, x2))
        pd.fCont = zero
        pd.u1Cont = lambda t, x1, x2: 0.5 - x2
        pd.u2Cont = lambda t, x1, x2: x1 - 0.5
        pd.cDCont = zero
        pd.gNCont = zero
        if pd.jitter > 0:
            pd.generateGridData = lambda h: jittered_square(h, pd.jitter, pd.meshSeed)
        else:
            pd.generateGridData = domainSquare
    elif tc == 'ensemble':
        pd.isAnalytical = False
        prm = ensemble_params(pd.instanceSeed)
        pd.ensembleParams = prm
        pd.setdefault('jitter', 0.2)
        u1, u2 = streamfunction_velocity(prm['k'], prm['l'], prm['a'])
        cx, cy = prm['centre']; w2 = prm['width'] ** 2
        pd.c0Cont = lambda x1, x2: np.exp(-((x1 - cx) ** 2 + (x2 - cy) ** 2) / w2)
        pd.fCont = zero
        pd.u1Cont = u1
        pd.u2Cont = u2
        pd.cDCont = zero
        pd.gNCont = zero
        pd.generateGridData = lambda h: jittered_square(h, pd.jitter, prm['mesh_seed'])
    elif tc == 'adjoint':
        pd.isAnalytical = False
        prm = adjoint_params(pd.get('adjointSeed', 0))
        theta = prm['theta'] + (prm['dtheta'] if pd.get('adjointTarget', False) else 0.0)
        pd.theta = theta
        u1, u2 = streamfunction_velocity([k for k, _ in ADJOINT_MODES], [l for _, l in ADJOINT_MODES], theta)
        pd.c0Cont = lambda x1, x2: np.exp(-((x1 - 0.4) ** 2 + (x2 - 0.45) ** 2) / 0.01)
        pd.fCont = zero
        pd.u1Cont = u1
        pd.u2Cont = u2
        pd.cDCont = zero
        pd.gNCont = zero
        pd.generateGridData = domainSquare
    else:
        raise ValueError('Invalid testcase "%s".' % tc)
    return pd
