"""Launch-configuration autotuner.

For one handle (one mesh, or one degree group of an ensemble) it times the launch
configurations this library has and keeps the fastest:
- the limiter pipeline: separate passes, or the fused one (linear limiter, zero Dirichlet data);
- programmatic dependent launch on or off;
- the number of time steps per captured CUDA graph;
- the stage operator's elements per CTA, 64 or 128 (one thread per element; separate-pass
  pipeline, and the linked step of an ensemble's degree groups);
- with time-derivative limiting, the Taylor mass correction from stored blocks or rebuilt from
  each element's B (tried on the best configuration of the above).
Each candidate runs ``nSteps`` steps of the handle's own problem after one warm-up call, timed
with CUDA events on the handle's stream; the state is restored afterwards.  The choice can be
kept in a JSON file keyed by the problem's signature and the GPU name, and reused.

``tune_adjoint`` does the same for the reverse sweep: the adjoint stage kernel's warps per role,
i.e. 32, 64 or 128 elements per CTA with four warp roles (three edges, the volume points) per
element, then the sweep as one CUDA graph or launched directly, then on one stream or two.

The limiter kernels keep 128 elements per CTA (the padding unit of every per-element array).
"""
import json
import os
import time

from . import _lib as L

GRAPH_STEPS = (4, 12, 24, 48)


OP_BLOCKS = (128, 64)


def candidates(solver, fused_ok):
    """Launch configurations: pipeline, dependent launch, steps per graph and, for the
    separate-pass pipeline, the stage operator's elements per CTA (one thread per element)."""
    out = []
    for fuse in ((False, True) if fused_ok else (False,)):
        for pdl in (True, False):
            for gs in GRAPH_STEPS:
                flags = (L.FLAG_FUSE if fuse else 0) | (0 if pdl else L.FLAG_NO_PDL)
                for eb in (OP_BLOCKS if not fuse else OP_BLOCKS[:1]):
                    out.append(dict(flags=flags, graphSteps=gs, opBlock=eb))
    return out


def signature(solver, tau, precision, extra=''):
    import torch
    name = torch.cuda.get_device_name(0) if torch.cuda.is_available() else 'cpu'
    return '%s|K=%d|p=%d|%s|%s|tau=%g%s' % (name, solver.K, solver.p, precision, solver.limiter, tau, extra)


def apply(solver, best):
    """Sets a configuration returned by `tune` on `solver`."""
    solver.set_option(L.OPT_FLAGS, best['flags'])
    solver.set_option(L.OPT_GRAPH_STEPS, best['graphSteps'])
    solver.set_option(L.OPT_OP_BLOCK, best.get('opBlock', 128))
    if 'taylorMass' in best:
        solver.set_option(L.OPT_TAYLOR_MASS, best['taylorMass'])


def tune(solver, tau, nSteps=48, reps=3, fused_ok=False, cache=None, key=None):
    """Times every candidate on `solver` and applies the fastest; returns (best, table).
    `cache`: optional JSON path; with `key`, a stored choice is applied without timing."""
    if cache and key and os.path.exists(cache):
        with open(cache) as f:
            stored = json.load(f)
        if key in stored:
            best = stored[key]['best']
            apply(solver, best)
            return best, stored[key]['table']
    state = solver.get_state()
    table = []
    for c in candidates(solver, fused_ok):
        solver.set_option(L.OPT_FLAGS, c['flags'])
        solver.set_option(L.OPT_GRAPH_STEPS, c['graphSteps'])
        solver.set_option(L.OPT_OP_BLOCK, c['opBlock'])
        solver.set_state(state)
        solver.time_steps(nSteps, 0, tau)                 # warm-up: graph capture, first launches
        ms = min(solver.time_steps(nSteps, 0, tau) for _ in range(reps))
        table.append(dict(c, ms_per_step=ms / nSteps))
    best = min(table, key=lambda r: r['ms_per_step'])
    best = dict(flags=best['flags'], graphSteps=best['graphSteps'], opBlock=best['opBlock'],
                ms_per_step=best['ms_per_step'])
    solver.set_option(L.OPT_FLAGS, best['flags'])
    solver.set_option(L.OPT_GRAPH_STEPS, best['graphSteps'])
    solver.set_option(L.OPT_OP_BLOCK, best['opBlock'])
    if solver.p >= 2 and solver.limiter != 'none':
        # with time-derivative limiting: the Taylor mass correction read from stored blocks or
        # rebuilt from B, tried once on the best configuration (the stored blocks win where
        # they stay in L2, the rebuild where they would stream from DRAM)
        cur = solver.get_option(L.OPT_TAYLOR_MASS)
        times = {cur: best['ms_per_step']}
        alt = 1 - cur
        solver.set_option(L.OPT_TAYLOR_MASS, alt)
        solver.set_state(state)
        solver.time_steps(nSteps, 0, tau)
        times[alt] = min(solver.time_steps(nSteps, 0, tau) for _ in range(reps)) / nSteps
        table.append(dict(best, taylorMass=alt, ms_per_step=times[alt]))
        best['taylorMass'] = min(times, key=times.get)
        best['ms_per_step'] = times[best['taylorMass']]
        solver.set_option(L.OPT_TAYLOR_MASS, best['taylorMass'])
    solver.set_state(state)
    if cache and key:
        stored = {}
        if os.path.exists(cache):
            with open(cache) as f:
                stored = json.load(f)
        stored[key] = dict(best=best, table=table)
        with open(cache, 'w') as f:
            json.dump(stored, f, indent=1)
    return best, table


ADJ_WARPS = (1, 2, 4)          # FP32: the warp-role split (bitwise the same gradients)
ADJ_WARPS_FP64 = (0, 1, 2, 4)  # FP64 also times one thread per element (gradients to roundoff)


def tune_adjoint(solver, tau, nSteps=20, nSnapshots=0, reps=3):
    """Times a recorded run of `nSteps` steps and its reverse sweep at every warps-per-role
    setting of the adjoint stage (wall time of dgadv_backward, which synchronises) and applies
    the fastest; returns (best, table).  In FP32 the gradients do not depend on the setting; in
    FP64 the one-thread kernel (0) is timed too, whose gradients agree to roundoff.  The
    handle's state is restored."""
    state = solver.get_state()

    def timed():
        times = []
        for _ in range(reps + 1):   # the first backward captures the sweep's graph
            solver.set_state(state)
            solver.forward_record(nSteps, tau, nSnapshots)
            g = solver.get_state()
            t = time.perf_counter()
            solver.backward(g)
            times.append(time.perf_counter() - t)
        return 1e3 * min(times[1:])

    table = []
    for w in (ADJ_WARPS_FP64 if getattr(solver, 'precision', None) == 'fp64' else ADJ_WARPS):
        solver.set_option(L.OPT_ADJ_WARPS, w)
        table.append(dict(adjWarps=w, ms_backward=timed()))
    best = min(table, key=lambda r: r['ms_backward'])
    solver.set_option(L.OPT_ADJ_WARPS, best['adjWarps'])
    # then the sweep as one CUDA graph or launched directly, on that width
    if hasattr(L, 'OPT_ADJ_GRAPH'):
        cur = solver.get_option(L.OPT_ADJ_GRAPH)
        best = dict(best, adjGraph=cur)
        solver.set_option(L.OPT_ADJ_GRAPH, 1 - cur)
        alt = timed()
        table.append(dict(adjWarps=best['adjWarps'], adjGraph=1 - cur, ms_backward=alt))
        if alt < best['ms_backward']:
            best = dict(best, adjGraph=1 - cur, ms_backward=alt)
        solver.set_option(L.OPT_ADJ_GRAPH, best['adjGraph'])
    # and the sweep on one, two or three streams
    if hasattr(L, 'OPT_ADJ_STREAMS'):
        cur = solver.get_option(L.OPT_ADJ_STREAMS)
        best = dict(best, adjStreams=cur)
        for alt in (n for n in (1, 2, 3) if n != cur):
            solver.set_option(L.OPT_ADJ_STREAMS, alt)
            t = timed()
            table.append(dict(adjWarps=best['adjWarps'], adjGraph=best.get('adjGraph'), adjStreams=alt, ms_backward=t))
            if t < best['ms_backward']:
                best = dict(best, adjStreams=alt, ms_backward=t)
        solver.set_option(L.OPT_ADJ_STREAMS, best['adjStreams'])
    solver.set_state(state)
    return best, table
