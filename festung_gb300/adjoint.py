"""Gradients through the GPU solver: the discrete adjoint behind ``torch.autograd.Function``.

The reference has no adjoint.  For an unlimited run c(T) = Phi(c0; theta), with the velocity
u = sum_m theta_m u_m over streamfunction modes u_m, ``AdvectionSolve.apply(c0, theta, ...)``
returns c(T) and records the run (``dgadv_forward_record``); ``backward`` maps dJ/dc(T) to
dJ/dc0 and dJ/dtheta with the adjoint kernels (``dgadv_backward``).  The upwind choice is frozen
at the recorded velocity.  Tensors are FP64 on the host (the C-ABI copies them in and out).

``setup(pd)`` prepares a problem of the 'adjoint' test case (16 modes psi_m = sin(k pi x)
sin(l pi y)): it hands the mode velocities to the solver.
"""
import numpy as np

from . import advection_gpu as G
from . import testcases as TC

try:
    import torch
except ImportError:   # the Function needs torch; the rest of the module does not
    torch = None


def mode_data(pd, modes=None):
    """Velocity data of each mode, stacked on a last axis: u1Disc, u2Disc (K x N x M) and
    vNormalOnQuadEdge (K x 3 x R x M), the inputs of dgadv_set_velocity per mode."""
    modes = range(len(TC.ADJOINT_MODES)) if modes is None else modes
    u1s, u2s, vns = [], [], []
    for m in modes:
        u1, u2 = TC.mode_velocity(m)
        u1s.append(G.project(pd.g, pd.tables, u1, 2 * pd.p, pd.hatM))
        u2s.append(G.project(pd.g, pd.tables, u2, 2 * pd.p, pd.hatM))
        vns.append(G.normal_velocity(pd.g, pd.tables, u1, u2, 2 * pd.p + 1))
    return np.stack(u1s, -1), np.stack(u2s, -1), np.stack(vns, -1)


def setup(**kw):
    """configure / preprocess / initialise an 'adjoint' problem and give the solver its modes."""
    kw = dict(kw)
    kw.setdefault('testcase', 'adjoint')
    pd = G.Struct(kw)
    pd.problemName = 'advection_gpu'
    for f in G.PRE:
        pd = f(pd)
    pd.solver.set_velocity_modes(*mode_data(pd))
    pd.solver.set_velocity_theta(pd.theta)
    return pd


if torch is not None:
    class AdvectionSolve(torch.autograd.Function):
        """c(T) = AdvectionSolve.apply(c0, theta, solver, nSteps, tau, nSnapshots)."""

        @staticmethod
        def forward(ctx, c0, theta, solver, nSteps, tau, nSnapshots=0):
            solver.set_velocity_theta(theta.detach().cpu().double().numpy())
            solver.set_state(c0.detach().cpu().double().numpy())
            solver.forward_record(nSteps, tau, nSnapshots)
            ctx.solver = solver
            return torch.from_numpy(np.ascontiguousarray(solver.get_state()))

        @staticmethod
        def backward(ctx, gcT):
            g0, gth = ctx.solver.backward(gcT.detach().cpu().double().numpy())
            return (torch.from_numpy(np.ascontiguousarray(g0)), torch.from_numpy(gth),
                    None, None, None, None)


def misfit_gradient(pd, c0, theta, cTarget, nSnapshots=0):
    """J = 0.5 ||c(T) - cTarget||^2 and its gradients (dJ/dc0, dJ/dtheta) for pd.numSteps steps."""
    s = pd.solver
    s.set_velocity_theta(theta)
    s.set_state(c0)
    s.forward_record(pd.numSteps, pd.tau, nSnapshots)
    r = s.get_state() - cTarget
    J = 0.5 * float(np.sum(r * r))
    g0, gth = s.backward(r)
    return J, g0, gth


def misfit(pd, c0, theta, cTarget):
    """J of a plain forward run (no recording), for finite-difference checks."""
    s = pd.solver
    s.set_velocity_theta(theta)
    s.set_state(c0)
    s.step(pd.numSteps, 0, pd.tau)
    r = s.get_state() - cTarget
    return 0.5 * float(np.sum(r * r))
