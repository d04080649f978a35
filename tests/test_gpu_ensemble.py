"""GPU ensembles: instances stacked into one handle per degree, the degree groups linked into one
launch per stage kernel for all of them, give each instance exactly its own single-problem
result.

Bars: bitwise equal to the single-instance handle (FP32 and FP64: the same per-element
arithmetic, the same vertex patches, the instance's own limiter extremes); FP64 relative L2
<= 1e-12 against the oracle.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def single(seed, precision, **kw):
    from festung_gb300 import advection_gpu as G
    from festung_gb300 import testcases as TC
    prm = TC.ensemble_params(seed)
    args = dict(testcase='ensemble', instanceSeed=seed, hmax=prm['hmax'], p=prm['p'], isSlopeLim=True,
                precision=precision)
    args.update(kw)
    pd = G.main(**args)
    pd.solver.close()
    return pd.cDisc


@pytest.mark.parametrize('precision', ['fp32', 'fp64'])
def test_stacked_instances_equal_single_runs_bitwise(lib, precision):
    from festung_gb300 import ensemble as E
    seeds = list(range(6))
    kw = dict(hmax=2 ** -4)                       # 512 triangles each, both degrees
    ens = E.Ensemble(seeds, precision=precision, numSteps=12, tau=5e-4, **kw)
    try:
        assert len(ens.groups) == 2
        ens.step(12)
        got = ens.states()
    finally:
        ens.close()
    for s, c in zip(seeds, got):
        ref = single(s, precision, numSteps=12, tEnd=12 * 5e-4, **kw)
        assert np.array_equal(c, ref), 'instance %d' % s


def test_uneven_instances_equal_single_runs_bitwise(lib):
    from festung_gb300 import ensemble as E
    seeds = [0, 1, 2, 3]                          # the workload's own levels: 2048 to 32768 triangles
    ens = E.Ensemble(seeds, precision='fp32', numSteps=8)
    try:
        sizes = sorted({pd.K for pd in ens.problems})
        assert len(sizes) >= 2
        ens.step(8)
        got = ens.states()
    finally:
        ens.close()
    for s, c in zip(seeds, got):
        assert np.array_equal(c, single(s, 'fp32', numSteps=8, tEnd=8 * 5e-4)), 'instance %d' % s


def test_fp64_ensemble_matches_oracle(lib):
    from festung_gb300 import ensemble as E
    from oracle import matfree as MF
    seeds = [3, 4]
    kw = dict(hmax=2 ** -4)
    ens = E.Ensemble(seeds, precision='fp64', numSteps=10, tau=5e-4, **kw)
    try:
        ens.step(10)
        got = ens.states()
    finally:
        ens.close()
    from festung_gb300 import testcases as TC
    for s, c in zip(seeds, got):
        o = MF.main_matfree(testcase='ensemble', instanceSeed=s, hmax=kw['hmax'], p=TC.ensemble_params(s)['p'],
                            numSteps=10, tEnd=10 * 5e-4, isSlopeLim=True).cDisc
        assert np.linalg.norm(c - o) <= 1e-12 * np.linalg.norm(o)


def test_instances_must_fill_whole_blocks(lib):
    from festung_gb300 import _lib as L
    from festung_gb300 import ensemble as E
    with pytest.raises(L.DgadvError) as e:
        E.Ensemble([0, 1], precision='fp32', numSteps=2, hmax=0.1)   # 200 triangles each
    assert e.value.status == L.DGADV_EINVAL


def test_graph_length_and_dependent_launch_leave_results_unchanged(lib):
    from festung_gb300 import _lib as L
    from festung_gb300 import ensemble as E
    ens = E.Ensemble([0, 1, 2], precision='fp32', numSteps=30, hmax=2 ** -4)
    try:
        ens.step(30)
        ref = ens.states()
        for flags, gs in ((0, 1), (0, 7), (L.FLAG_NO_PDL, 24), (L.FLAG_NO_GRAPH, 12)):
            for s in ens.solvers.values():
                s.set_option(L.OPT_FLAGS, flags)
                s.set_option(L.OPT_GRAPH_STEPS, gs)
            ens.reset()
            ens.step(30)
            for a, b in zip(ens.states(), ref):
                assert np.array_equal(a, b), (flags, gs)
    finally:
        ens.close()


def test_autotuner_picks_a_measured_configuration(lib, tmp_path):
    from festung_gb300 import _lib as L
    from festung_gb300 import ensemble as E
    ens = E.Ensemble([0, 1, 2, 3], precision='fp64', numSteps=24, hmax=2 ** -4)
    try:
        cache = str(tmp_path / 'tune.json')
        best = ens.tune(nSteps=12, reps=2, cache=cache)
        sched = best.pop('schedule')
        assert sched['chosen'] in ('linked', 'separate') and (ens.primary is not None) == (sched['chosen'] == 'linked')
        chosen = best['linked'] if sched['chosen'] == 'linked' else best['separate']
        for p, b in (chosen.items() if sched['chosen'] == 'separate' else [('linked', chosen)]):
            s = ens.primary if p == 'linked' else ens.solvers[p]
            assert s.get_option(L.OPT_GRAPH_STEPS) == b['graphSteps']
            assert s.get_option(L.OPT_FLAGS) & (L.FLAG_FUSE | L.FLAG_NO_PDL) == b['flags']
        ens.reset()
        ens.step(24)
        tuned = ens.states()
        # the per-handle configurations come back from the cache (the schedule is timed again)
        again = ens.tune(cache=cache)
        again.pop('schedule', None)
        if sched['chosen'] == 'linked':
            assert again['linked'] == best['linked'] and again['separate'] == best['separate']
        else:
            assert again == best['separate']
    finally:
        ens.close()
    ref = E.Ensemble([0, 1, 2, 3], precision='fp64', numSteps=24, hmax=2 ** -4)
    try:
        ref.step(24)
        for a, b in zip(tuned, ref.states()):
            assert np.linalg.norm(a - b) <= 1e-13 * np.linalg.norm(b)   # the fused pipeline: roundoff
    finally:
        ref.close()


@pytest.mark.parametrize('precision', ['fp32', 'fp64'])
def test_linked_groups_equal_separate_groups_bitwise(lib, precision):
    """dgadv_link: one launch per stage kernel for both degrees (p = 1 with SSP-RK2, p = 2 with
    SSP-RK3) gives bitwise the states of the groups stepped on their own, in fewer launches."""
    from festung_gb300 import ensemble as E
    seeds = list(range(8))
    kw = dict(hmax=2 ** -4)
    runs = {}
    for linked in (True, False):
        ens = E.Ensemble(seeds, precision=precision, numSteps=20, tau=5e-4, linked=linked, **kw)
        try:
            assert len(ens.groups) == 2
            assert (ens.primary is not None) == linked
            ens.step(7)                                   # not a multiple of the graph length
            ens.step(13)
            runs[linked] = (ens.states(), ens.kernels_per_step())
        finally:
            ens.close()
    for a, b in zip(runs[True][0], runs[False][0]):
        assert np.array_equal(a, b)
    assert runs[True][1] == {'linked': 9}                # 3 stages x (operator, cDot limiter, limiter)
    assert runs[False][1] == {1: 2 * 2, 2: 3 * 3}        # p = 1: 2 stages x (operator, limiter)


def test_link_refuses_what_it_does_not_cover(lib):
    from festung_gb300 import _lib as L
    from festung_gb300 import ensemble as E
    ens = E.Ensemble([0, 1, 2, 3], precision='fp32', numSteps=4, hmax=2 ** -4)
    try:
        other = [s for s in ens.solvers.values() if s is not ens.primary][0]
        with pytest.raises(L.DgadvError) as e:
            other.step(1, 0, ens.tau)                     # stepped by its primary only
        assert e.value.status == L.DGADV_EUNSUPPORTED
        ens.primary.link(None)                            # unlinked: steps on its own again
        other.step(1, 0, ens.tau)
        other.sync()
    finally:
        ens.close()
    hier = E.Ensemble([0, 1, 2, 3], precision='fp32', numSteps=4, hmax=2 ** -4, linked=False,
                      typeSlopeLim='hierarch_vert')
    try:
        a, b = list(hier.solvers.values())
        with pytest.raises(L.DgadvError) as e:
            a.link(b)
        assert e.value.status == L.DGADV_EUNSUPPORTED
    finally:
        hier.close()


def test_linked_operator_block_size_leaves_results_unchanged(lib):
    from festung_gb300 import _lib as L
    from festung_gb300 import ensemble as E
    out = []
    for eb in (128, 64):
        ens = E.Ensemble(list(range(6)), precision='fp32', numSteps=12, hmax=2 ** -4)
        try:
            ens.primary.set_option(L.OPT_OP_BLOCK, eb)
            ens.step(12)
            out.append(ens.states())
        finally:
            ens.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)
