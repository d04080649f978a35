"""Ensembles of independent advection problems on one GPU (and sharded across ranks).

The ensemble workload: seeded instances of the 'ensemble' test case.
- Each instance draws its mesh level hmax in {2^-5, 2^-6, 2^-7} (2048 / 8192 / 32768
  triangles), with interior nodes jittered by +-0.2 h.
- It draws its degree p in {1, 2}.
- Its velocity comes from a streamfunction of 8 random Fourier modes.
- Its initial data is a Gaussian hump.
- Every instance runs SSP-RK of order p + 1 (the reference's default,
  advection/configureProblem.m:80), 200 steps of 5e-4, with the linear vertex-based limiter.

The instances of one degree are stacked into one handle (``dgadv_create_ensemble``), each
instance keeping its own limiter extremes.  The degree groups' handles are linked
(``dgadv_link``): one step then launches each stage kernel once for every instance of every
degree, the blocks of each group running that group's kernel code (``linked=False`` steps the
groups on their own streams instead).

``shard(n, rank, world)`` splits instances across ranks with no data exchange: each rank runs
its own instances (weak scaling); results stay on their rank.
"""
import numpy as np

from . import _lib as L
from . import advection_gpu as G
from . import testcases as TC
from .solver import DeviceSolver

STEPS, TAU = 200, 5e-4


def shard(n, rank, world):
    """Instances of this rank: i = rank, rank + world, ... (a balanced mix of sizes)."""
    return list(range(rank, n, world))


def instance_problem(seed, numSteps=STEPS, tau=TAU, **overrides):
    """configureProblem + the host part of preprocessProblem for instance `seed`.  With
    setupOnDevice (the default) the velocity and the initial data stay device functions
    (``pd.deviceFns``); otherwise they are projected on the host (pd.u1Disc, ..., pd.c0)."""
    prm = TC.ensemble_params(seed)
    kw = dict(testcase='ensemble', instanceSeed=seed, hmax=prm['hmax'], p=prm['p'], numSteps=numSteps,
              tEnd=numSteps * tau, isSlopeLim=True, typeSlopeLim='linear')
    kw.update(overrides)
    pd = G.Struct(kw)
    pd.problemName = 'advection_gpu'
    G.configureProblem(pd)
    G.host_preprocess(pd)
    if not pd.deviceFns:
        pd.c0 = G.project(pd.g, pd.tables, pd.c0Cont, pd.qOrd, pd.hatM)
    return pd


class Ensemble:
    """Instances grouped by degree, one stacked handle per group."""

    def __init__(self, seeds, precision='fp32', device=0, flags=0, numSteps=STEPS, tau=TAU, linked=True,
                 **overrides):
        self.seeds = list(seeds)
        self.problems = [instance_problem(s, numSteps, tau, **overrides) for s in self.seeds]
        self.numSteps, self.tau = numSteps, tau
        self.groups = {}
        for i, pd in enumerate(self.problems):
            self.groups.setdefault(pd.p, []).append(i)
        self.solvers = {}
        for p, members in sorted(self.groups.items()):
            pds = [self.problems[i] for i in members]
            pd0 = pds[0]
            s = DeviceSolver(None, None, p, pd0.ordRK, precision=precision, isSlopeLim=pd0.isSlopeLim,
                             typeSlopeLim=pd0.typeSlopeLim, device=device, flags=flags,
                             instances=[G.instance_mesh(pd) for pd in pds])
            if pd0.deviceFns:
                s.set_velocity_function([pd.deviceFns['u'] for pd in pds])
            else:
                s.set_velocity(np.concatenate([pd.u1Disc for pd in pds]),
                               np.concatenate([pd.u2Disc for pd in pds]),
                               np.concatenate([pd.vNormalOnQuadEdge for pd in pds]))
            self.solvers[p] = s
        # link the groups: the largest group's handle steps all of them
        self.primary = None
        # (the linked step runs the separate-pass pipeline: handles created for the fused or
        # the persistent pipeline stay on their own streams)
        if (linked and len(self.solvers) > 1 and precision in ('fp32', 'fp64')
                and not flags & (L.FLAG_FUSE | L.FLAG_PERSIST)):
            self._link()
        self.reset()

    @property
    def dofs(self):
        return sum(pd.K * pd.N for pd in self.problems)

    def dof_stages(self, nSteps):
        return sum(pd.K * pd.N * pd.ordRK for pd in self.problems) * nSteps

    def reset(self):
        """Initial data of every instance, limited (advection/initializeProblem.m:56-67)."""
        for p, members in self.groups.items():
            s = self.solvers[p]
            pds = [self.problems[i] for i in members]
            if pds[0].deviceFns:
                s.project_state([pd.deviceFns['c0'] for pd in pds], 0.0, pds[0].qOrd)
            else:
                s.set_state(np.concatenate([pd.c0 for pd in pds]))
            if pds[0].isSlopeLim:
                s.limit_state(0.0)

    def step(self, nSteps, nStep0=0):
        """Enqueues steps: one linked step for all groups, or each group on its own stream."""
        if self.primary is not None:
            self.primary.step(nSteps, nStep0, self.tau)
            return
        for s in self.solvers.values():
            s.step(nSteps, nStep0, self.tau)

    def unlink(self):
        """Back to one handle per degree group, each on its own stream."""
        if self.primary is not None:
            self.primary.link(None)
            self.primary = None

    def kernels_per_step(self):
        """Launches per time step: of the linked step, or per group."""
        if self.primary is not None:
            return {'linked': self.primary.kernels_per_step()}
        return {int(p): s.kernels_per_step() for p, s in self.solvers.items()}

    def sync(self):
        for s in self.solvers.values():
            s.sync()

    def states(self):
        """Per-instance coefficient arrays (K x N), in seed order."""
        out = [None] * len(self.problems)
        for p, members in self.groups.items():
            parts = self.solvers[p].split(self.solvers[p].get_state())
            for i, c in zip(members, parts):
                out[i] = np.array(c)
        return out

    def _time(self, nSteps, reps):
        """Wall time (s) of nSteps steps of every instance, best of reps, state restored."""
        import time
        saved = {p: s.get_state() for p, s in self.solvers.items()}
        self.step(nSteps)
        self.sync()
        best = float('inf')
        for _ in range(reps):
            t = time.perf_counter()
            self.step(nSteps)
            self.sync()
            best = min(best, time.perf_counter() - t)
        for p, s in self.solvers.items():
            s.set_state(saved[p])
        return best

    def _link(self):
        order = sorted(self.solvers, key=lambda p: -sum(self.problems[i].K for i in self.groups[p]))
        self.primary = self.solvers[order[0]]
        for p in order[1:]:
            self.primary.link(self.solvers[p])

    def tune(self, nSteps=48, reps=3, cache=None):
        """Autotunes the launch configuration (festung_gb300.autotune): for linked groups, the
        linked step's configuration, then each group's on its own stream, and keeps the faster
        of the two schedules (returned under 'schedule' with both times per step)."""
        from . import autotune as AT
        out = {}
        if self.primary is not None:   # the linked step: the primary's launch configuration
            s = self.primary
            key = AT.signature(s, self.tau, s.precision, '|ensemble-linked:%d' % len(self.problems)) if cache else None
            out['linked'] = AT.tune(s, self.tau, nSteps, reps, fused_ok=False, cache=cache, key=key)[0]
            tLinked = self._time(nSteps, reps) / nSteps
            self.unlink()
            out['separate'] = self._tune_groups(nSteps, reps, cache)
            tSep = self._time(nSteps, reps) / nSteps
            chosen = 'linked' if tLinked <= tSep else 'separate'
            if chosen == 'linked':
                self._link()
                # the primary took its own group's configuration while the groups were tuned
                AT.apply(self.primary, out['linked'])
            out['schedule'] = dict(chosen=chosen, ms_per_step={'linked': 1e3 * tLinked, 'separate': 1e3 * tSep})
            return out
        return self._tune_groups(nSteps, reps, cache)

    def _tune_groups(self, nSteps, reps, cache):
        from . import autotune as AT
        out = {}
        for p, s in self.solvers.items():
            pd0 = self.problems[self.groups[p][0]]
            fused_ok = pd0.isSlopeLim and pd0.typeSlopeLim == 'linear' and s.precision != 'df32' and not pd0.cDTerms
            key = AT.signature(s, self.tau, s.precision, '|ensemble:%d' % len(self.groups[p])) if cache else None
            out[p] = AT.tune(s, self.tau, nSteps, reps, fused_ok=fused_ok, cache=cache, key=key)[0]
        return out

    def close(self):
        for s in self.solvers.values():
            s.close()
        self.solvers = {}
