"""Benchmark of the explicit DG advection step on one GB300 (or N replicas under torchrun).

Workload (default): the 131072-triangle production case -- domainSquare hmax=2^-8, p=2 (N=6),
SSP-RK3, tau=1e-4, 500 steps per solve, rotating Gaussian hump + slotted cylinder, linear
vertex-based Taylor limiter on.  One bench "step" is one full 500-step solve (1500 RK stages)
from the projected initial data c0 at t = 0.  The headline precision is FP64, the reference's.
Beside it: the FP32 path and the double-float path (DF32: each real a pair of FP32 numbers, ~48
significant bits, on the FP32 units), each with its relative L2 distance to the FP64 result of
the same solve, and the fastest path within the 1e-6 accuracy bar.

Metric: DOF-stage updates per second = K * N * stages / seconds.
  value  -- device time (CUDA events on the library's stream) with the state resident in HBM;
            the state is reset to c0 and L2 is flushed (512 MB memset) before every timed solve.
  e2e    -- the same solve through the C-ABI with host buffers: every step copies c0 in from
            pinned host memory (dgadv_set_state), runs the 500 steps and reads the result back
            (dgadv_get_state); wall-clock time.
  roofline -- the dominant kernel's algorithmic bytes per launch / its live launch time, against
            the measured HBM copy bandwidth; whole_stage: the scope table's bytes per
            element-stage over the mean stage time.  The 131072-triangle working set fits L2;
            hbm_case gives the same operator on 2,097,152 triangles, far beyond L2.
  cpu_baseline -- the oracle's restatement of the reference (per-stage sparse assembly, as the
            reference) on this machine's cores for a bounded sample of stages.

``--impl reference`` times the reference's algorithm on the host (the oracle port; there is no
Matlab/Octave to run the reference itself) on the same workload, a bounded number of RK stages
per bench step.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # Gaussian hump and slotted cylinder in the rotating velocity, linear limiter
    'gauss_slot_131k_p2': dict(testcase='gauss_slot', hmax=2 ** -8, p=2, numSteps=500, tEnd=500 * 1e-4,
                               isSlopeLim=True, typeSlopeLim='linear', ordRK=3),
    # the same operator on a 16x larger mesh (2,097,152 triangles): inputs well beyond L2, used
    # for the DRAM traffic capture of the stage kernels
    'gauss_slot_2M_p2': dict(testcase='gauss_slot', hmax=2 ** -10, p=2, numSteps=500, tEnd=500 * 1e-4,
                             isSlopeLim=True, typeSlopeLim='linear', ordRK=3),
    'gauss_slot_2048_p1': dict(testcase='gauss_slot', hmax=2 ** -5, p=1, numSteps=500, tEnd=0.5,
                               isSlopeLim=True, typeSlopeLim='linear', ordRK=2),
    # 2,097,152 triangles with 10% node jitter, p = 3, hierarchical vertex limiter
    # p = 3 with the hierarchical limiter on the 131072-triangle mesh (profiling captures of the
    # p = 3 stage kernels at a size a full capture handles)
    'gauss_slot_131k_p3_hier': dict(testcase='gauss_slot', hmax=2 ** -8, p=3, numSteps=100, tEnd=100 * 2e-5,
                                    isSlopeLim=True, typeSlopeLim='hierarch_vert', ordRK=3, jitter=0.1,
                                    meshSeed=5),
    'gauss_slot_2M_p3_hier': dict(testcase='gauss_slot', hmax=2 ** -10, p=3, numSteps=100, tEnd=100 * 2e-5,
                                  isSlopeLim=True, typeSlopeLim='hierarch_vert', ordRK=3, jitter=0.1,
                                  meshSeed=5),
}


def dist_env():
    rank = int(os.environ.get('RANK', '0'))
    world = int(os.environ.get('WORLD_SIZE', '1'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return rank, world, local


# ---------------------------------------------------------------------------------------------
def algorithmic_bytes(kind, w, N, Q, R, nc, mtRows=0):
    """Unique bytes per element a launch of each kernel kind must move (its own element's
    inputs and outputs plus the static per-element data; neighbour gathers re-read the same
    arrays and count once).  mtRows: the per-element rows of the time-derivative limiter's Taylor
    mass correction (N(N-1) of Q_k for the linear limiter, N(N+1)/2 packed M_T and the 4 of B
    for the hierarchical one, or the 4 of B when it is rebuilt from B)."""
    csr = 14                                    # vertex CSR (vptr ~ 2 B, vidx 12 B per element)
    if kind == 'op0':                           # stage operator, limiter off: c, c^n, F, Vn, ints, out
        return w * (3 * N + 2 * Q + 3 * R) + 16
    if kind == 'op1':                           # + B, Taylor out, centroid quantities
        return w * (3 * N + 2 * Q + 3 * R + 4 + nc) + 16
    if kind == 'op2':                           # c, F, Vn, B, ints; Taylor(cDot) and q out
        return w * (2 * N + 2 * Q + 3 * R + 4 + nc) + 16
    if kind == 'limdot':                        # cDot in, out, c^n, c^(s-1), correction rows, q in/out
        return w * (4 * N + mtRows + 2 * nc) + 16 + csr
    if kind == 'lim':                           # Taylor in, B, q, modal out
        return w * (2 * N + 4 + nc) + 16 + csr
    raise ValueError(kind)


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed region runs."""
    FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, device):
        self.device = device
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.device), '--query-gpu=' + self.FIELDS,
                 '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in self.lines:
            f = [x.strip() for x in ln.split(',')]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1])); mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == 'active':
                    reasons.add(n)
        if not sm:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': [], 'samples': 0}
        return {'sm_mhz': statistics.median(sm), 'sm_max_mhz': max(mx), 'reasons': sorted(reasons),
                'samples': len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            d = json.load(f)
        return float(d['hbm_gbs']), 'measured'
    except (OSError, KeyError, ValueError):
        return 6800.0, 'fallback'


def setup_problem(wl, precision, device):
    from festung_gb300 import advection_gpu as G
    pd = G.Struct(dict(WORKLOADS[wl], precision=precision, device=device))
    pd.problemName = 'advection_gpu'
    for f in G.PRE:
        pd = f(pd)
    return pd


class OracleStages:
    """Runs RK stages of the oracle restatement (per-stage sparse assembly and solve, as
    advection/preprocessSubStep.m + advection/solveSubStep.m) one at a time: a bounded sample of
    the workload for the CPU baseline."""

    def __init__(self, wl):
        from oracle import advection as adv
        from oracle import assembly as A
        self.adv, self.A = adv, A
        pd = adv.Struct(dict(WORKLOADS[wl]))
        pd.problemName = 'advection'
        for f in (adv.configureProblem, adv.preprocessProblem, adv.initializeProblem):
            pd = f(pd)
        self.pd = pd
        self.S = len(A.rungeKuttaExplicit(pd.ordRK, 1.0, 0.0)[1])
        self.nStep, self.sub = 0, self.S

    def stage(self):
        adv, pd = self.adv, self.pd
        if self.sub >= self.S:
            if self.nStep > 0:
                adv.postprocessStep(pd, self.nStep)
            self.nStep += 1
            pd.t, pd.omega = self.A.rungeKuttaExplicit(pd.ordRK, pd.tau, (self.nStep - 1) * pd.tau)
            pd.cDiscRK = [None] * (len(pd.t) + 1)
            pd.cDiscRK[0] = pd.cDisc.reshape(-1).copy()
            self.sub = 0
        self.sub += 1
        adv.preprocessSubStep(pd, self.nStep, self.sub)
        adv.solveSubStep(pd, self.nStep, self.sub)
        adv.postprocessSubStep(pd, self.nStep, self.sub)

    def dofs_per_stage(self):
        return self.pd.K * self.pd.N


def cpu_baseline(wl, nstages):
    """DOF-stage updates/s of the oracle restatement over ``nstages`` RK stages."""
    o = OracleStages(wl)
    t = time.perf_counter()
    for _ in range(nstages):
        o.stage()
    dt = time.perf_counter() - t
    return o.dofs_per_stage() * nstages / dt, dt, o.pd


def thread_count():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ---------------------------------------------------------------------------------------------
def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    n = str(thread_count())
    for v in ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS'):
        os.environ.setdefault(v, n)
    o = OracleStages(args.workload)
    per = args.ref_stages_per_step
    for _ in range(args.warmup):
        for _ in range(per):
            o.stage()
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        for _ in range(per):
            o.stage()
        times.append(time.perf_counter() - t)
    pd, S = o.pd, o.S
    ms = 1e3 * statistics.mean(times)
    value = o.dofs_per_stage() * per / (ms / 1e3)
    sample = ('%d RK stage(s) of the %s workload per bench step (of %d steps x %d stages per solve), '
              'sparse operators re-assembled every stage as the reference does; %d host threads '
              'allowed to BLAS, the scipy sparse assembly and products run on one'
              % (per, args.workload, pd.numSteps, S, thread_count()))
    line = {
        'impl': 'reference', 'metric': 'DG DOF-stage updates/s', 'value': value,
        'unit': 'DOF-stage/s', 'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': ms,
        'ms_per_step_unit': ('%d RK stage(s) of the workload, a bounded sample: only the DOF-stage '
                             'rate compares with the GPU line, whose step is one full solve' % per),
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f64', 'data': 'synthetic',
        'config': workload_config(args.workload, pd.K, pd.N, S, pd.numSteps),
        'cpu_baseline': {'value': value, 'unit': 'DOF-stage/s', 'cores': 1,
                         'kind': 'port', 'sample': sample},
        'e2e': {'value': value, 'unit': 'DOF-stage/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the stage kernels,
# from single-kernel ncu captures (-k <kernel> -c 1, cold L2 under ncu) of
# `bench.py --ncu-case <workload> --precision <p> --ncu-steps 2`, keyed (workload, precision,
# kernel).
# FP64 floating-point operations per element of the FP64 stage kernels (2 x DFMA + DADD + DMUL
# thread instructions, smsp__sass_thread_inst_executed_op_{dfma,dadd,dmul}_pred_on.sum of one
# single-kernel ncu capture each, divided by the elements), keyed (workload, kernel):
# profiles/stage_kernels_131k_fp64_full.md.
MEASURED_FP64_FLOPS = {('gauss_slot_131k_p2', 'k_stage_op'): 197.1,
                       ('gauss_slot_131k_p2', 'k_limit_dot'): 192.4,
                       ('gauss_slot_131k_p2', 'k_limit'): 117.5}


def fp64_peak(reps=5, n=4096):
    """GB300's FP64 rate as a library reaches it: cuBLAS DGEMM (torch.matmul, float64) of n^3,
    best of reps, CUDA events (TFLOP/s)."""
    import torch
    a = torch.randn(n, n, dtype=torch.float64, device='cuda')
    b = torch.randn_like(a)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = float('inf')
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


MEASURED_TRAFFIC = {('gauss_slot_131k_p2', 'fp32', 'k_stage_op'): 18.4e6,
                    ('gauss_slot_131k_p2', 'fp32', 'k_limit_dot'): 28.4e6,
                    ('gauss_slot_131k_p2', 'fp32', 'k_limit'): 5.8e6,
                    # FP64, element operator on (ncu, one cold launch each; dram read + write)
                    ('gauss_slot_131k_p2', 'fp64', 'k_stage_op'): 58.5e6,
                    ('gauss_slot_131k_p2', 'fp64', 'k_limit_dot'): 54.8e6,
                    ('gauss_slot_131k_p2', 'fp64', 'k_limit'): 9.5e6}


def large_block(device, flush):
    """The large single mesh: 2,097,152 jittered triangles, p = 3, the hierarchical
    vertex limiter, 100 SSP-RK3 steps.  One full solve from the projected initial data in FP32
    and in FP64 after an L2 flush (the working set, >1 GB, is far beyond L2), the FP32 kernels'
    launch times and the dominant kernel's HBM roofline, and FP32's distance to FP64."""
    import torch
    out = {'workload': 'gauss_slot_2M_p3_hier: domainSquare hmax=2^-10 with 10% node jitter '
                       '(2,097,152 triangles), p=3 (N=10), hierarchical vertex limiter, 100 SSP-RK3 '
                       'steps, tau=2e-5, gauss_slot'}
    from festung_gb300 import _lib as L
    states = {}
    for prec in ('fp32', 'fp32_volume_mma', 'fp64'):
        pd = setup_problem('gauss_slot_2M_p3_hier', prec.split('_')[0], device)
        s = pd.solver
        if prec == 'fp32_volume_mma':                # the volume term on the tensor cores
            s.set_option(L.OPT_VOLUME_MMA, 1)
        c0 = np.asfortranarray(pd._cDisc)
        if prec != 'fp64':                           # launch configuration (FP64: seconds per solve)
            from festung_gb300 import autotune as AT
            AT.tune(s, pd.tau, nSteps=8, reps=2)
            s.set_state(c0)
        s.step(5, 0, pd.tau)                        # warm-up (graph capture, first launches)
        s.sync()
        s.set_state(c0)
        flush.zero_()
        torch.cuda.synchronize()
        ms = s.time_steps(pd.numSteps, 0, pd.tau)
        states[prec] = s.get_state()
        K, N, S = pd.K, pd.N, pd.ordRK
        row = {'value': K * N * S * pd.numSteps / (ms / 1e3), 'unit': 'DOF-stage/s', 'ms_per_solve': ms,
               'K': K}
        if prec.startswith('fp32'):
            kpl, nl = s.profile_kernels(4, 0, pd.tau)
            w, Q, R, nc = 4, 12, pd.p + 1, pd.p * (pd.p + 1) // 2
            kinds = ['op2', 'limdot', 'lim']
            names = ['k_stage_op', 'k_limit_dot', 'k_limit']
            shares = [kpl[i] * nl[i] for i in range(3)]
            tot = max(sum(shares), 1e-30)
            dom = int(np.argmax(shares))
            peak, peak_kind = measured_peaks()
            kern = {}
            mtr = mt_rows(s, pd)
            for i in range(3):
                b = algorithmic_bytes(kinds[i], w, N, Q, R, nc, mtr) * K
                live = ms * shares[i] / tot / (nl[i] / 4.0 * pd.numSteps)
                kern[names[i]] = {'ms_per_launch_isolated': kpl[i], 'ms_per_launch_live': live,
                                  'share': shares[i] / tot, 'algorithmic_bytes_per_launch': b,
                                  'achieved_GBps_live': b / (live * 1e-3) / 1e9,
                                  'achieved_GBps_isolated': b / (kpl[i] * 1e-3) / 1e9}
            a = kern[names[dom]]['achieved_GBps_live']
            ai = kern[names[dom]]['achieved_GBps_isolated']
            row['kernels'] = kern
            row['roofline'] = {'bound': 'hbm', 'kernel': names[dom], 'achieved': a, 'peak': peak, 'unit': 'GB/s',
                               'frac': a / peak, 'peak_source': peak_kind, 'achieved_isolated': ai,
                               'frac_isolated': ai / peak}
        out[prec] = row
        s.close()
    rel = lambda a, b: float(np.linalg.norm(states[a] - states[b]) / np.linalg.norm(states[b]))
    out['fp32_vs_fp64_rel_l2'] = rel('fp32', 'fp64')
    out['fp32_volume_mma']['rel_l2_vs_fp64'] = rel('fp32_volume_mma', 'fp64')
    out['fp32_volume_mma']['rel_l2_vs_fp32'] = rel('fp32_volume_mma', 'fp32')
    out['fp32_volume_mma']['speedup_vs_fp32'] = out['fp32']['ms_per_solve'] / out['fp32_volume_mma']['ms_per_solve']
    return out


ADJOINT_WORKLOAD = dict(hmax=2 ** -7, p=2, numSteps=200, tEnd=200 * 2e-4)


def tuned_sweep(s, pd, snaps):
    """The reverse sweep's launch configuration for a checkpoint mode (autotune.tune_adjoint:
    warps per role, graph or direct launches, one or two streams), tuned on a 40-step run with
    the same kind of checkpoints; returns the choice."""
    from festung_gb300 import autotune as AT
    best = AT.tune_adjoint(s, pd.tau, nSteps=40, nSnapshots=0 if snaps == 0 else 4, reps=2)[0]
    return {k: v for k, v in best.items() if k != 'ms_backward'}


def adjoint_block(reps=3, fd_dirs=16):
    """Adjoint cost on the gradient workload (32768 triangles, p = 2, 200 SSP-RK3 steps): wall
    time of dgadv_backward over the wall time of the same run forward (dgadv_set_state +
    dgadv_step + sync), with every stage state stored and with 20 binomial snapshots, each with
    the sweep's launch configuration tuned for it (tuned_sweep); FP64
    central differences (h = 1e-6) against the adjoint's directional derivatives; FP32
    gradients against FP64."""
    from festung_gb300 import adjoint as AD
    kw = ADJOINT_WORKLOAD
    tg = AD.setup(precision='fp64', adjointTarget=True, **kw)
    tg.solver.step(kw['numSteps'], 0, tg.tau)
    cstar = tg.solver.get_state()
    tg.solver.close()
    out, grads = {'workload': 'adjoint: domainSquare hmax=2^-7 (32768 triangles), p=2, 200 SSP-RK3 '
                              'steps, tau=2e-4, 16 streamfunction modes, J = 0.5 ||c(T) - c*||^2'}, {}
    for prec in ('fp64', 'fp32'):
        pd = AD.setup(precision=prec, **kw)
        s = pd.solver
        c0 = np.asfortranarray(pd._cDisc)
        s.set_state(c0); s.step(kw['numSteps'], 0, pd.tau); s.sync()
        tf = []
        for _ in range(reps):
            t = time.perf_counter(); s.set_state(c0); s.step(kw['numSteps'], 0, pd.tau); s.sync()
            tf.append(time.perf_counter() - t)
        row = {'forward_ms': 1e3 * min(tf)}
        for name, snaps in (('stages_stored', 0), ('snapshots_20', 20)):
            launch = tuned_sweep(s, pd, snaps)
            tb, trec = [], []
            for _ in range(reps + 1):
                s.set_velocity_theta(pd.theta); s.set_state(c0)
                t = time.perf_counter(); s.forward_record(kw['numSteps'], pd.tau, snaps); s.sync()
                trec.append(time.perf_counter() - t)
                r = s.get_state() - cstar
                t = time.perf_counter(); g0, gth = s.backward(r); tb.append(time.perf_counter() - t)
            row[name] = {'record_ms': 1e3 * min(trec), 'backward_ms': 1e3 * min(tb[1:]),
                         'backward_over_forward': min(tb[1:]) / min(tf), 'launch': launch}
        grads[prec] = (g0, gth)
        if prec == 'fp64' and fd_dirs:
            rng = np.random.default_rng(0)
            h = 1e-6
            errs = []
            for _ in range(fd_dirs):
                d = rng.standard_normal(c0.shape)
                fd = (AD.misfit(pd, c0 + h * d, pd.theta, cstar) - AD.misfit(pd, c0 - h * d, pd.theta, cstar)) / (2 * h)
                errs.append(abs(fd - float(np.sum(g0 * d))) / abs(fd))
                dt = rng.standard_normal(gth.size)
                fd = (AD.misfit(pd, c0, pd.theta + h * dt, cstar) - AD.misfit(pd, c0, pd.theta - h * dt, cstar)) / (2 * h)
                errs.append(abs(fd - float(gth @ dt)) / abs(fd))
            row['fd_max_rel_err'] = max(errs)
            row['fd_directions'] = 2 * fd_dirs
        out[prec] = row
        s.close()
    rel = lambda a, b: float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))
    out['fp32_vs_fp64_grad_rel_l2'] = {'dJdc0': rel(grads['fp32'][0], grads['fp64'][0]),
                                       'dJdtheta': rel(grads['fp32'][1], grads['fp64'][1])}
    # the same workload with the linear, the hierarchical vertex and the strict limiter on (the
    # adjoint through the limiter's choices)
    out['linear_limiter'] = limited_adjoint_rows(AD, kw, reps, fd_dirs, 'linear')
    out['hierarchical_limiter'] = limited_adjoint_rows(AD, kw, reps, fd_dirs, 'hierarch_vert')
    out['strict_limiter'] = limited_adjoint_rows(AD, kw, reps, fd_dirs, 'strict')
    return out


def limited_adjoint_rows(AD, kw, reps, fd_dirs, lim):
    """Backward over forward with the limiter `lim` on, FP64 and FP32, stages stored and 20
    snapshots; FP64 finite differences in theta over 20 steps and the 200-step sensitivity."""
    kwl = dict(kw, isSlopeLim=True, typeSlopeLim=lim)
    rows = {}
    tg = AD.setup(precision='fp64', adjointTarget=True, **kwl)
    tg.solver.step(kw['numSteps'], 0, tg.tau)
    cstarL = tg.solver.get_state()
    tg.solver.close()
    for prec in ('fp64', 'fp32'):
        pd = AD.setup(precision=prec, **kwl)
        s = pd.solver
        c0 = np.asfortranarray(pd._cDisc)
        s.set_state(c0); s.step(kw['numSteps'], 0, pd.tau); s.sync()
        tf = []
        for _ in range(reps):
            t = time.perf_counter(); s.set_state(c0); s.step(kw['numSteps'], 0, pd.tau); s.sync()
            tf.append(time.perf_counter() - t)
        row = {'forward_ms': 1e3 * min(tf)}
        for name, snaps in (('stages_stored', 0), ('snapshots_20', 20)):
            launch = tuned_sweep(s, pd, snaps)
            tb = []
            for _ in range(reps + 1):
                s.set_velocity_theta(pd.theta); s.set_state(c0)
                s.forward_record(kw['numSteps'], pd.tau, snaps); s.sync()
                r = s.get_state() - cstarL
                t = time.perf_counter(); g0, gth = s.backward(r); tb.append(time.perf_counter() - t)
            row[name] = {'backward_ms': 1e3 * min(tb[1:]), 'backward_over_forward': min(tb[1:]) / min(tf),
                         'launch': launch}
        if prec == 'fp64' and fd_dirs:
            row['fd_theta'] = limited_fd_check(AD, kw, fd_dirs, lim=lim)
            row['sensitivity'] = limited_sensitivity(AD, pd, c0, cstarL, kw['numSteps'])
        rows[prec] = row
        s.close()
    return rows


def limited_fd_check(AD, kw, fd_dirs, steps=20, hs=(1e-7, 1e-8), lim='linear'):
    """Central differences in theta against the limited adjoint on the same mesh over `steps`
    steps, at each step size in `hs`.  The limited map is piecewise smooth: where a perturbation
    of relative size h crosses one of the limiter's switches somewhere on the mesh, the central
    difference averages two slopes.  The hierarchical limiter has many more switches (one per
    order, vertex and sub-limiter) than the linear one: over 20 steps h = 1e-7 crosses some of
    them, h = 1e-8 stays inside one piece."""
    kw20 = dict(kw, numSteps=steps, tEnd=steps * kw['tEnd'] / kw['numSteps'], typeSlopeLim=lim)
    tg = AD.setup(precision='fp64', adjointTarget=True, isSlopeLim=True, **kw20)
    tg.solver.step(steps, 0, tg.tau)
    cstar = tg.solver.get_state()
    tg.solver.close()
    pd = AD.setup(precision='fp64', isSlopeLim=True, **kw20)
    c0 = np.asfortranarray(pd._cDisc)
    _, _, gth = AD.misfit_gradient(pd, c0, pd.theta, cstar)
    rng = np.random.default_rng(1)
    errs = {h: [] for h in hs}
    for _ in range(fd_dirs):
        dt = rng.standard_normal(gth.size) * np.abs(pd.theta)
        for h in hs:
            fd = (AD.misfit(pd, c0, pd.theta + h * dt, cstar) - AD.misfit(pd, c0, pd.theta - h * dt, cstar)) / (2 * h)
            errs[h].append(abs(fd - float(gth @ dt)) / abs(fd))
    pd.solver.close()
    return {'steps': steps, 'directions': fd_dirs,
            'max_rel_err': {'h=%g' % h: max(e) for h, e in errs.items()},
            'median_rel_err': {'h=%g' % h: float(np.median(e)) for h, e in errs.items()}}


def limited_sensitivity(AD, pd, c0, cstar, steps, h=1e-14):
    """How far a relative change h of theta moves c(T) of the limited run: where it is O(1), c(T)
    is not differentiable at any resolvable scale and no finite difference can check a gradient."""
    rng = np.random.default_rng(2)
    dt = rng.standard_normal(pd.theta.size) * np.abs(pd.theta)
    AD.misfit(pd, c0, pd.theta, cstar)
    ca = pd.solver.get_state()
    AD.misfit(pd, c0, pd.theta + h * dt, cstar)
    cb = pd.solver.get_state()
    return {'steps': steps, 'theta_rel_change': h, 'max_abs_change_cT': float(np.abs(cb - ca).max()),
            'max_abs_cT': float(np.abs(ca).max())}


def setup_block(wl, device, reps=2):
    """The steps either side of the time loop on the headline workload (FP32 handle): velocity
    data, projection of the initial data and the L2 error, with the test case's device functions
    (dgadv_set_velocity_function, dgadv_project_state, dgadv_l2_error) and with the host set-up
    (numpy projections, dgadv_set_velocity / dgadv_set_state, numpy L2 error).  Wall time of
    each (best of `reps`), and the whole configure + preprocess + initialize both ways."""
    from festung_gb300 import advection_gpu as G
    out = {'workload': wl, 'precision': 'fp32'}
    whole = {}
    for dev in (True, False):
        ts = []
        for _ in range(reps):
            t = time.perf_counter()
            pd = G.Struct(dict(WORKLOADS[wl], precision='fp32', device=device, setupOnDevice=dev))
            pd.problemName = 'advection_gpu'
            for f in G.PRE:
                pd = f(pd)
            ts.append(time.perf_counter() - t)
            if dev:
                pdDev = pd
            else:
                pdHost = pd
        whole['device' if dev else 'host'] = min(ts)
    out['pre_s'] = whole
    s, fns = pdDev.solver, pdDev.deviceFns

    def best(fn):
        ts = []
        for _ in range(reps + 1):
            t = time.perf_counter(); fn(); ts.append(time.perf_counter() - t)
        return 1e3 * min(ts[1:])
    g, tb, ph = pdHost.g, pdHost.tables, pdHost
    out['device_ms'] = {
        'velocity': best(lambda: s.set_velocity_function(fns['u'])),
        'initial_data': best(lambda: s.project_state(fns['c0'], 0.0, pdDev.qOrd)),
        'l2_error': best(lambda: s.l2_error(fns['c0'], 0.0, pdDev.qOrd))}

    def host_velocity():
        u1 = G.project(g, tb, ph.u1Cont, 2 * ph.p, ph.hatM)
        u2 = G.project(g, tb, ph.u2Cont, 2 * ph.p, ph.hatM)
        vn = G.normal_velocity(g, tb, ph.u1Cont, ph.u2Cont, 2 * ph.p + 1)
        ph.solver.set_velocity(u1, u2, vn)
    out['host_ms'] = {
        'velocity': best(host_velocity),
        'initial_data': best(lambda: ph.solver.set_state(G.project(g, tb, ph.c0Cont, ph.qOrd, ph.hatM))),
        'l2_error': best(lambda: G.l2_error(g, tb, ph.solver.get_state(), ph.c0Cont, ph.qOrd))}
    out['l2_error_device_vs_host_rel'] = abs(s.l2_error(fns['c0'], 0.0, ph.qOrd) -
                                             G.l2_error(g, tb, s.get_state(), ph.c0Cont, ph.qOrd)) / \
        G.l2_error(g, tb, s.get_state(), ph.c0Cont, ph.qOrd)
    pdDev.solver.close()
    pdHost.solver.close()
    return out


IMPLICIT_WORKLOAD = dict(testcase='solid_body', p=2, ordRK=3, hmax=2 ** -6, numSteps=320, tEnd=2 * np.pi)


def implicit_block(device, steps=20, reps=2, with_cpu=True):
    """The implicit problem's default configuration (advection_implicit/configureProblem.m:
    solid body rotation, p = 2, 3-stage DIRK, hmax = 2^-6, 320 steps to 2 pi): wall time per
    step of dgadv_step_implicit (every stage a block-Jacobi GMRES solve to a relative residual
    of 1e-12 in FP64, 1e-6 in FP32), GMRES iterations per stage, and one step of the oracle's
    sparse direct solves (scipy, host) on the same mesh with its difference to the GPU step."""
    from festung_gb300 import advection_implicit_gpu as AI
    from oracle import implicit as I
    out = {'workload': 'advection_implicit defaults: solid_body, hmax=2^-6 (8192 triangles), p=2, '
                       'DIRK3, tau=2pi/320'}
    S = IMPLICIT_WORKLOAD['ordRK']
    first = {}
    for prec in ('fp64', 'fp32'):
        pd = AI.Struct(dict(IMPLICIT_WORKLOAD, precision=prec, device=device))
        pd.problemName = 'advection_implicit_gpu'
        for f in AI.PRE:
            pd = f(pd)
        s = pd.solver
        c0 = np.asfortranarray(s.get_state())
        it1, _ = s.step_implicit(1, 0, pd.tau, pd.ordRK, pd.krylovTol, pd.krylovMaxIter, pd.krylovRestart)
        first[prec] = s.get_state()
        ts, its = [], []
        for _ in range(reps):
            s.set_state(c0)
            t = time.perf_counter()
            it, rr = s.step_implicit(steps, 0, pd.tau, pd.ordRK, pd.krylovTol, pd.krylovMaxIter, pd.krylovRestart)
            ts.append(time.perf_counter() - t)
            its.append(it)
        dt = min(ts)
        out[prec] = {'ms_per_step': 1e3 * dt / steps, 'gmres_iterations_per_stage': its[0] / (steps * S),
                     'value': pd.K * pd.N * S * steps / dt, 'unit': 'DOF-stage/s', 'final_relres': rr,
                     'tol': pd.krylovTol}
        s.close()
    if not with_cpu:
        return out
    # CPU baseline and checker: one step of the oracle restatement (sparse LU per stage)
    o = I.Struct(dict(IMPLICIT_WORKLOAD))
    o.problemName = 'advection_implicit'
    for f in (I.configureProblem, I.preprocessProblem, I.initializeProblem):
        o = f(o)
    t = time.perf_counter()
    I.solveStep(o, 1)
    out['cpu_baseline'] = {'ms_per_step': 1e3 * (time.perf_counter() - t), 'kind': 'port', 'cores': 1,
                           'sample': 'one step of the oracle restatement: assembly and scipy sparse LU '
                                     'per stage, host'}
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    out['fp64_vs_oracle_rel_l2_1step'] = rel(first['fp64'], o.cDisc)
    out['fp32_vs_oracle_rel_l2_1step'] = rel(first['fp32'], o.cDisc)
    return out


def transport_block(device, steps=200, with_cpu=True):
    """The transport problem's 'rotation' configuration (transport/configureProblem.m: 8192
    triangles, p = 1, SSP-RK2, masks on), with 1 and 4 species: wall time per step of
    dgadv_transport_step (FP64), the active fraction of the elements, and one step of the
    oracle restatement on the host with its difference to the GPU step."""
    from festung_gb300 import transport_gpu as TG
    from oracle import transport as TR
    out = {'workload': 'transport rotation: domainSquare hmax=2^-6 (8192 triangles), p=1, SSP-RK2, '
                       'tau=2pi/3142, vertex-based masks (tol 1e-6), FP64'}
    kw = dict(hmax=2 ** -6, numSteps=3124, tEnd=(3124 / 3142) * 2 * np.pi)
    for ns in (1, 4):
        pd = TG.Struct(dict(kw, numSpecies=ns, precision='fp64', device=device))
        pd.problemName = 'transport_gpu'
        for f in TG.PRE:
            pd = f(pd)
        s = pd.solver
        s.transport_step(1, 0, pd.tau)
        first = [s.transport_get(i) for i in range(ns)]
        t = time.perf_counter()
        s.transport_step(steps, 1, pd.tau)
        dt = time.perf_counter() - t
        act = np.mean([s.transport_get(i)[2].mean() for i in range(ns)])
        out['species_%d' % ns] = {'ms_per_step': 1e3 * dt / steps, 'active_fraction': float(act),
                                  'value': ns * pd.K * pd.N * pd.ordRK * steps / dt, 'unit': 'DOF-stage/s'}
        s.close()
        if ns == 1 and with_cpu:
            o = TR.Struct(dict(kw, numSpecies=1))
            o.problemName = 'transport'
            for f in (TR.configureProblem, TR.preprocessProblem, TR.initializeProblem):
                o = f(o)
            t = time.perf_counter()
            TR.solveStep(o, 1)
            out['cpu_baseline'] = {'ms_per_step': 1e3 * (time.perf_counter() - t), 'kind': 'port', 'cores': 1,
                                   'sample': 'one step of the oracle restatement (masked sparse assembly, host)'}
            out['fp64_vs_oracle_rel_l2_1step'] = float(np.linalg.norm(first[0][0] - o.cDisc[0]) /
                                                       np.linalg.norm(o.cDisc[0]))
            out['mask_equal_1step'] = bool(np.array_equal(first[0][2], o.mask[0]))
    return out


def ensemble_block(rank, world, device, n=256, steps=200, reps=3):
    """The ensemble workload: n seeded instances (2048 to 32768 triangles, p in {1, 2}, their own
    velocity fields), 200 steps in FP32 with the linear limiter.  Each degree group is one
    stacked handle; the autotuner tunes the linked step (one launch per stage kernel for all
    instances) and the groups on their own streams, and keeps the faster schedule, which is then
    timed.  Instances are sharded across ranks with no exchange; whole-job DOF-stage/s = all
    ranks' work / the slowest rank's time."""
    import torch
    from festung_gb300 import ensemble as E
    t = time.perf_counter()
    ens = E.Ensemble(E.shard(n, rank, world), precision='fp32', device=device, numSteps=steps)
    setup_s = time.perf_counter() - t
    flush = torch.empty(512 * 2 ** 20, dtype=torch.uint8, device='cuda')
    units = ens.dof_stages(steps)
    tuned = ens.tune()
    ens.step(steps)
    ens.sync()
    times = []
    for _ in range(reps):
        ens.reset()
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ens.step(steps)
        ens.sync()
        times.append(time.perf_counter() - t0)
    dt, u = min(times), float(units)
    if world > 1:
        x = torch.tensor([dt, u], dtype=torch.float64, device='cuda')
        mx = x.clone()
        torch.distributed.all_reduce(mx, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(x, op=torch.distributed.ReduceOp.SUM)
        dt, u = float(mx[0]), float(x[1])
    out = {'workload': 'ensemble: %d seeded instances, hmax in {2^-5,2^-6,2^-7} with 0.2 h jitter, p in {1,2}, '
                       '8-mode streamfunction velocity, Gaussian hump, %d steps of 5e-4, FP32, linear limiter'
                       % (n, steps),
           'instances_this_rank': len(ens.seeds), 'dofs_this_rank': ens.dofs,
           'value': u / dt, 'unit': 'DOF-stage/s', 'ms_per_solve': 1e3 * dt,
           'groups': {int(p): {'instances': len(m), 'elements': int(sum(ens.problems[i].K for i in m))}
                      for p, m in ens.groups.items()},
           'schedule': tuned.get('schedule'), 'kernels_per_step': ens.kernels_per_step(), 'tuned': tuned,
           'host_setup_s': setup_s,
           'timing': 'wall clock of 200 steps after an L2 flush, initial data reset and limited before each, '
                     'in the schedule the autotuner kept (linked: every degree group in one launch per '
                     'stage kernel; separate: one handle per degree on its own stream)'}
    ens.close()
    return out


def workload_config(wl, K, N, S, steps):
    kw = WORKLOADS[wl]
    return {'workload': '%s: domainSquare hmax=2^%d, K=%d triangles, p=%d (N=%d), SSP-RK%d, '
                        '%d steps per solve, %s limiter, %s' % (
                            wl, int(round(np.log2(kw['hmax']))), K, kw['p'], N, S, steps,
                            kw['typeSlopeLim'] if kw['isSlopeLim'] else 'no', kw['testcase']),
            'K': K, 'p': kw['p'], 'N': N, 'rk_stages': S, 'steps_per_solve': steps,
            'limiter': kw['typeSlopeLim'] if kw['isSlopeLim'] else None,
            'l2_flush_between_steps': True, 'parallelism': 'replicas'}


def survey_bytes(w, N, R, nc, limPasses):
    """Algorithmic bytes per element-stage: the operator pass moves w(5N + 3R + 4) + 16 bytes
    (c^(s-1), c^n and c^(s); u1, u2; the edge normal velocities; B; neighbour ids and codes) and
    each limiter pass w(2N + 4 nc) + 26 (state in and out; nc centroid quantities written and
    gathered, vertex min / max written and read; V0T and the vertex CSR)."""
    return w * (5 * N + 3 * R + 4) + 16 + limPasses * (w * (2 * N + 4 * nc) + 26)


def time_solves(s, c0, steps, tau, reps, flush):
    """Device time (ms, CUDA events on the library's stream) of `reps` full solves, each from c0
    at t = 0 after an L2 flush; and the final state of the last one."""
    import torch
    ts = []
    for _ in range(reps):
        s.set_state(c0)
        flush.zero_()
        torch.cuda.synchronize()
        ts.append(s.time_steps(steps, 0, tau))
    return ts, s.get_state()


def kernel_table(s, pd, w, ms_per_solve, profSteps=20):
    """Per-kernel launch times (CUDA events around every launch of a `profSteps`-step profiling
    pass), their shares, and the algorithmic bytes each launch moves; the dominant kernel's
    roofline against the measured HBM copy bandwidth.  `live` splits the timed solve over the
    kernels by their shares (inside the solve the chained kernels overlap through dependent
    launch, so no single launch can be timed there on its own)."""
    kpl, nlaunch = s.profile_kernels(profSteps, 0, pd.tau)
    N, Q, R = pd.N, {0: 1, 1: 3, 2: 6, 3: 12}[pd.p], pd.p + 1
    nc = 1 if pd.typeSlopeLim == 'linear' else pd.p * (pd.p + 1) // 2
    mtRows = mt_rows(s, pd)
    op_kind = 'op0' if not pd.isSlopeLim else ('op2' if pd.p > 1 else 'op1')
    kinds = [op_kind, 'limdot', 'lim']
    names = ['k_stage_op', 'k_limit_dot', 'k_limit']
    shares = [kpl[i] * nlaunch[i] for i in range(3)]
    tot = max(sum(shares), 1e-30)
    peak, peak_kind = measured_peaks()
    kern = {}
    for i in range(3):
        if not nlaunch[i] or kpl[i] <= 0:
            continue
        b = algorithmic_bytes(kinds[i], w, N, Q, R, nc, mtRows) * pd.K
        per_solve = nlaunch[i] / float(profSteps) * pd.numSteps
        live = ms_per_solve * shares[i] / tot / per_solve
        kern[names[i]] = {'ms_per_launch_isolated': kpl[i], 'ms_per_launch_live': live,
                          'launches_per_solve': int(per_solve), 'share': shares[i] / tot,
                          'algorithmic_bytes_per_launch': b,
                          'achieved_GBps_live': b / (live * 1e-3) / 1e9,
                          'achieved_GBps_isolated': b / (kpl[i] * 1e-3) / 1e9}
    dom = max(kern, key=lambda n: kern[n]['share'])
    a, ai = kern[dom]['achieved_GBps_live'], kern[dom]['achieved_GBps_isolated']
    roof = {'bound': 'hbm', 'kernel': dom, 'achieved': a, 'peak': peak, 'unit': 'GB/s', 'frac': a / peak,
            'peak_source': peak_kind,
            'method': 'live: timed solve x kernel share (CUDA events around every launch of a '
                      'profiling pass) / launches per solve',
            'achieved_isolated': ai, 'frac_isolated': ai / peak}
    return kern, roof


def mt_rows(s, pd):
    """Per-element rows the time-derivative limiter reads for its Taylor mass correction."""
    from festung_gb300 import _lib as L
    N = pd.N
    if s.get_option(L.OPT_TAYLOR_MASS):
        return 4
    return N * (N - 1) if pd.typeSlopeLim == 'linear' else N * (N + 1) // 2 + 4


def whole_stage_roofline(pd, w, ms_per_solve):
    """The scope table's algorithmic bytes of a whole stage (operator pass + limiter passes) times
    the elements, over the mean stage time, against the measured HBM copy bandwidth."""
    nc = 1 if pd.typeSlopeLim == 'linear' else pd.p * (pd.p + 1) // 2
    limPasses = 0 if not pd.isSlopeLim else (2 if pd.p >= 2 else 1)
    b = survey_bytes(w, pd.N, pd.p + 1, nc, limPasses)
    stage_ms = ms_per_solve / (pd.numSteps * pd.ordRK)
    peak, peak_kind = measured_peaks()
    a = b * pd.K / (stage_ms * 1e-3) / 1e9
    return {'bytes_per_element_stage': b, 'stage_ms': stage_ms, 'achieved_GBps': a, 'peak': peak,
            'peak_source': peak_kind, 'frac': a / peak}


def hbm_block(device, flush, reps=2):
    """The HBM-bound case of the p = 2 operator: the 131072-triangle workload's operator and
    limiter on a 16x larger mesh (2,097,152 triangles, FP32 working set ~0.5 GB, far beyond
    L2), 500 steps from c0: the whole stage against the scope table's bytes, and each kernel."""
    pd = setup_problem('gauss_slot_2M_p2', 'fp32', device)
    s = pd.solver
    c0 = np.asfortranarray(pd._cDisc)
    from festung_gb300 import autotune as AT
    tuned = AT.tune(s, pd.tau, nSteps=24, reps=2, fused_ok=True)[0]   # launch configuration
    s.set_state(c0)
    s.step(20, 0, pd.tau)                     # warm-up (graph capture, first launches)
    s.sync()
    ts, _ = time_solves(s, c0, pd.numSteps, pd.tau, reps, flush)
    ms = statistics.mean(ts)
    kern, roof = kernel_table(s, pd, 4, ms, profSteps=4)
    out = {'workload': 'gauss_slot_2M_p2: domainSquare hmax=2^-10 (2,097,152 triangles), p=2 (N=6), '
                       'linear limiter, 500 SSP-RK3 steps, tau=1e-4, gauss_slot, FP32; L2 flushed before '
                       'each solve, working set far beyond L2',
           'K': pd.K, 'ms_per_solve': ms, 'value': pd.K * pd.N * pd.ordRK * pd.numSteps / (ms / 1e3),
           'unit': 'DOF-stage/s', 'whole_stage': whole_stage_roofline(pd, 4, ms), 'kernels': kern,
           'roofline': roof, 'launch': tuned}
    s.close()
    return out


def side_path(wl, precision, device, c0, flush, reps, options=None):
    """One precision on the headline workload: `reps` solves from c0 (each after an L2 flush),
    the mean device time and the last final state, with its kernel table."""
    pd = setup_problem(wl, precision, device)
    s = pd.solver
    for o, v in (options or {}).items():
        s.set_option(o, v)
    from festung_gb300 import autotune as AT
    tuned = AT.tune(s, pd.tau, nSteps=48, reps=3, fused_ok=(pd.typeSlopeLim == "linear" and precision != "df32"))[0]
    s.step(pd.numSteps, 0, pd.tau)             # warm-up solve (graph capture, first launches)
    s.sync()
    ts, c = time_solves(s, c0, pd.numSteps, pd.tau, reps, flush)
    ms = statistics.mean(ts)
    units = pd.K * pd.N * pd.ordRK * pd.numSteps
    w = 8 if precision in ('fp64', 'df32') else 4
    kern, roof = kernel_table(s, pd, w, ms)
    s.close()
    return {'value': units / (ms / 1e3), 'unit': 'DOF-stage/s', 'ms_per_solve': ms, 'launch': tuned,
            'kernels': kern, 'roofline': roof, 'whole_stage': whole_stage_roofline(pd, w, ms)}, c


def run_ours(args):
    rank, world, local = dist_env()
    device = local
    import torch
    torch.cuda.set_device(device)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl' if torch.cuda.is_available() else 'gloo')
    from festung_gb300.build import build
    if rank == 0:
        build()
    if world > 1:
        torch.distributed.barrier()
    wl = args.workload
    # the headline: the FP64 path, the reference's own precision
    pd = setup_problem(wl, 'fp64', device)
    s = pd.solver
    steps = pd.numSteps
    S = pd.ordRK
    K, N = pd.K, pd.N
    units = K * N * S * steps
    c0 = np.asfortranarray(pd._cDisc)
    flush = torch.empty(512 * 2 ** 20, dtype=torch.uint8, device='cuda')
    # launch configuration from the autotuner (graph length, dependent launch, pipeline)
    from festung_gb300 import autotune as AT
    tuned = AT.tune(s, pd.tau, nSteps=48, reps=3, fused_ok=(pd.typeSlopeLim == "linear"))[0] \
        if not args.no_tune else None

    # every solve, warm-up and timed, runs the configured 500 steps from c0 at t = 0
    for _ in range(args.warmup):
        s.set_state(c0)
        s.step(steps, 0, pd.tau)
    s.sync()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(device)
    with sampler:
        times, c64 = time_solves(s, c0, steps, pd.tau, args.steps, flush)
    torch.cuda.synchronize()
    total_ms = sum(times)
    if world > 1:
        t = torch.tensor([total_ms], device='cuda')
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = world * units / (ms_per_step / 1e3)
    kern, roof = kernel_table(s, pd, 8, ms_per_step)
    roof['traffic'] = MEASURED_TRAFFIC.get((wl, 'fp64', roof['kernel']))
    roof['note'] = ('L2-resident: the bytes a FP64 stage touches on this mesh (about 120 MB cold per '
                    'stage with the element operator, traffic) fit the 129 MB L2 for the most part, so '
                    'they are served mostly from L2 once a solve runs; the FP64 kernels are bound '
                    'by GB300\'s FP64 rate, not by bandwidth (fp64_rate); the HBM-bound figure is hbm_case')
    # the bound that applies: the FP64 pipe, against cuBLAS DGEMM on the same GPU
    peak64 = fp64_peak()
    rate = {'peak_tflops': peak64, 'peak_source': 'measured: cuBLAS DGEMM 4096^3 (torch.matmul float64)',
            'kernels': {}}
    for name, k in kern.items():
        f = MEASURED_FP64_FLOPS.get((wl, name))
        if f is None:
            continue
        a = f * K / (k['ms_per_launch_live'] * 1e-3) / 1e12
        rate['kernels'][name] = {'fp64_flops_per_element': f, 'achieved_tflops_live': a, 'frac': a / peak64}
    roof['fp64_rate'] = rate

    # end to end through the C-ABI with pinned host buffers: the same solve from c0
    hin = torch.empty((N, K), dtype=torch.float64, pin_memory=True)
    hout = torch.empty((N, K), dtype=torch.float64, pin_memory=True)
    hin.numpy()[...] = c0.T
    cin = hin.numpy().T            # K x N Fortran-ordered view of pinned memory
    cout = hout.numpy().T
    e2e_times = []
    for i in range(max(1, args.steps)):
        torch.cuda.synchronize()
        t = time.perf_counter()
        s.set_state(cin)
        s.step(steps, 0, pd.tau)
        s.get_state(cout)
        e2e_times.append(time.perf_counter() - t)
    e2e_s = statistics.mean(e2e_times)
    if world > 1:
        t = torch.tensor([e2e_s], device='cuda')
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * units / e2e_s
    e2e_equal = bool(np.array_equal(np.array(cout), c64))
    launches = int(s.kernels_per_step() * steps * args.steps)

    result = {
        'metric': 'DG DOF-stage updates/s',
        'metric_note': ('headline: the FP64 path (the reference\'s precision), every timed solve the '
                        'configured 500 steps from c0 at t = 0; fp32 and df32 beside it with their '
                        'relative L2 distance to FP64 after the same solve, and the fastest path within '
                        'the 1e-6 bar in accuracy_bar; adjoint cost ratios in adjoint'),
        'value': value, 'unit': 'DOF-stage/s', 'n_gpus': world, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': ms_per_step,
        'ms_per_step_unit': 'one full solve: %d steps x %d RK stages' % (steps, S),
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
        'data': 'synthetic',
        'config': dict(workload_config(wl, K, N, S, steps), launch=tuned, precision='fp64'),
        'clocks': sampler.summary(),
        'e2e': {'value': e2e_value, 'unit': 'DOF-stage/s', 'h2d_bytes_per_step': K * N * 8,
                'd2h_bytes_per_step': K * N * 8,
                'timing': 'wall clock: dgadv_set_state from pinned host memory + the same 500-step '
                          'solve from c0 + dgadv_get_state to pinned host memory',
                'final_state_equal_to_device_timed': e2e_equal},
        'gpu_launches': launches,
        'roofline': roof,
        'kernels': kern,
        'whole_stage': whole_stage_roofline(pd, 8, ms_per_step),
    }
    s.close()

    if rank == 0 and not args.no_fp64:
        from festung_gb300 import _lib as L
        paths = {'fp64': (value, 0.0)}
        # fp32: everything FP32; df32: everything double-float (~48 bits on the FP32 units);
        # df32_operator_fp32: double-float state, SSP update and limiter, the operator in FP32
        variants = [('fp32', 'fp32', None)]
        if not args.no_df32:
            variants += [('df32', 'df32', None), ('df32_operator_fp32', 'df32', {L.OPT_OPERATOR_FP32: 1})]
        for name, prec, opts in variants:
            row, c = side_path(wl, prec, device, c0, flush, reps=3, options=opts)
            row['rel_l2_vs_fp64'] = float(np.linalg.norm(c - c64) / np.linalg.norm(c64))
            result[name] = row
            paths[name] = (row['value'], row['rel_l2_vs_fp64'])
        result['fp32']['roofline']['note'] = ('L2-resident: the FP32 working set (~31 MB) stays in '
                                              'the 129 MB L2 within a solve; see hbm_case')
        result['fp32']['roofline']['traffic'] = MEASURED_TRAFFIC.get((wl, 'fp32', result['fp32']['roofline']['kernel']))
        within = {k: v for k, v in paths.items() if v[1] <= 1e-6}
        best = max(within, key=lambda k: within[k][0])
        result['accuracy_bar'] = {
            'rel_l2_vs_fp64': 1e-6, 'fastest_path_within_bar': best, 'value': within[best][0],
            'speedup_vs_fp64': within[best][0] / value,
            'paths': {k: {'value': v[0], 'rel_l2_vs_fp64': v[1]} for k, v in paths.items()}}

    if rank == 0 and not args.no_large:
        result['hbm_case'] = hbm_block(device, flush)

    if rank == 0 and not args.no_setup:
        result['setup'] = setup_block(wl, device)

    if rank == 0 and not args.no_large:
        result['large'] = large_block(device, flush)

    if not args.no_ensemble:
        ens = ensemble_block(rank, world, device)
        if rank == 0:
            result['ensemble'] = ens

    if rank == 0 and not args.no_adjoint:
        result['adjoint'] = adjoint_block()

    if rank == 0 and not args.no_implicit:
        result['implicit'] = implicit_block(device, with_cpu=not args.no_cpu)

    if rank == 0 and not args.no_transport:
        result['transport'] = transport_block(device, with_cpu=not args.no_cpu)

    if rank == 0 and not args.no_cpu:
        n = thread_count()
        v, dt, _ = cpu_baseline(wl, args.cpu_stages)
        result['cpu_baseline'] = {
            'value': v, 'unit': 'DOF-stage/s', 'cores': 1, 'kind': 'port',
            'sample': '%d RK stage(s) of the workload with the oracle restatement in FP64 (per-stage sparse '
                      'assembly as the reference; scipy sparse is single-threaded), %.1f s on a %d-core host'
                      % (args.cpu_stages, dt, n)}
    if rank == 0:
        print(json.dumps(result), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=5)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--workload', default='gauss_slot_131k_p2', choices=sorted(WORKLOADS))
    ap.add_argument('--no-fp64', action='store_true')
    ap.add_argument('--no-df32', action='store_true')
    ap.add_argument('--no-adjoint', action='store_true')
    ap.add_argument('--no-ensemble', action='store_true')
    ap.add_argument('--no-tune', action='store_true')
    ap.add_argument('--no-setup', action='store_true')
    ap.add_argument('--no-implicit', action='store_true')
    ap.add_argument('--no-large', action='store_true')
    ap.add_argument('--no-transport', action='store_true')
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--cpu-stages', type=int, default=1)
    ap.add_argument('--ref-stages-per-step', type=int, default=1)
    ap.add_argument('--ncu-case', default=None, choices=sorted(WORKLOADS) + ['adjoint', 'implicit', 'transport'],
                    help='profiling driver: set up the workload and run --ncu-steps steps, no timing')
    ap.add_argument('--ncu-steps', type=int, default=2)
    ap.add_argument('--ncu-hmax-exp', type=int, default=9,
                    help='adjoint profiling case: hmax = 2^-e (9: 524288 triangles, 7: 32768)')
    ap.add_argument('--ncu-snapshots', type=int, default=0,
                    help='adjoint profiling case: checkpoint slots (0: every stage stored)')
    ap.add_argument('--ncu-limited', action='store_true', help='adjoint profiling case: limiter on')
    ap.add_argument('--ncu-lim-type', default='linear', choices=['linear', 'hierarch_vert', 'strict'],
                    help='adjoint profiling case: the limiter (with --ncu-limited)')
    ap.add_argument('--precision', default='fp32', choices=['fp32', 'fp64', 'df32'])
    ap.add_argument('--ncu-option', action='append', default=[],
                    help='profiling driver: DGADV_OPT_* option as NAME=VALUE (e.g. VOLUME_MMA=1)')
    args = ap.parse_args()
    if args.ncu_case == 'adjoint':
        # one recorded run and its reverse sweep (p = 2, hmax = 2^-e), for profiling
        from festung_gb300 import adjoint as AD
        pd = AD.setup(precision=args.precision, hmax=2.0 ** -args.ncu_hmax_exp, p=2, numSteps=args.ncu_steps,
                      tEnd=args.ncu_steps * 2e-5,
                      **({'isSlopeLim': True, 'typeSlopeLim': args.ncu_lim_type} if args.ncu_limited else {}))
        c0 = np.asfortranarray(pd._cDisc)
        AD.misfit_gradient(pd, c0, pd.theta, 0.9 * c0, nSnapshots=args.ncu_snapshots)
        pd.solver.close()
        return 0
    if args.ncu_case == 'implicit':
        # the implicit problem's default configuration, --ncu-steps DIRK steps
        from festung_gb300 import advection_implicit_gpu as AI
        pd = AI.Struct(dict(IMPLICIT_WORKLOAD, precision='fp64' if args.precision == 'df32' else args.precision))
        pd.problemName = 'advection_implicit_gpu'
        for f in AI.PRE:
            pd = f(pd)
        pd.solver.step_implicit(args.ncu_steps, 0, pd.tau, pd.ordRK, pd.krylovTol)
        pd.solver.close()
        return 0
    if args.ncu_case == 'transport':
        # the transport problem's 'rotation' configuration with 4 species, --ncu-steps steps
        from festung_gb300 import transport_gpu as TG
        pd = TG.Struct(dict(hmax=2 ** -6, numSteps=3124, tEnd=(3124 / 3142) * 2 * np.pi, numSpecies=4,
                            precision='fp64' if args.precision == 'df32' else args.precision))
        pd.problemName = 'transport_gpu'
        for f in TG.PRE:
            pd = f(pd)
        pd.solver.transport_step(args.ncu_steps, 0, pd.tau)
        pd.solver.close()
        return 0
    if args.ncu_case:
        from festung_gb300 import _lib as L
        pd = setup_problem(args.ncu_case, args.precision, 0)
        for o in args.ncu_option:
            name, val = o.split('=')
            pd.solver.set_option(getattr(L, 'OPT_' + name), int(val))
        pd.solver.step(args.ncu_steps, 0, pd.tau)
        pd.solver.sync()
        pd.solver.close()
        return 0
    if args.impl == 'reference':
        return run_reference(args)
    return run_ours(args)


if __name__ == '__main__':
    sys.exit(main())
