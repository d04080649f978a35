"""Solution output through the device solver: nodal values evaluated on the GPU
(dgadv_get_lagrange) against the oracle's projectDataDisc2DataLagr, and the files of the
asynchronous writer (dgadv_output) against the oracle's text of core/visualizeDataLagr.m.

Bars: nodal values within 4 ulp-scale of the oracle (the same sums; the basis values at the nodes
may round differently); file text byte for byte equal to the oracle's text of the values that
dgadv_get_lagrange returns for the same state.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(p, precision='fp64', **kw):
    from festung_gb300 import advection_gpu as G
    args = dict(testcase='solid_body', hmax=2 ** -4, p=p, numSteps=20, precision=precision,
                isSlopeLim=p > 0)
    args.update(kw)
    pd = G.Struct(args)
    pd.problemName = 'advection_gpu'
    for f in G.PRE:
        pd = f(pd)
    return pd


def _bary_e0t(g):
    return g['baryE'][g['E0T']]


@pytest.mark.parametrize('precision', ['fp64', 'fp32', 'df32'])
@pytest.mark.parametrize('p', [0, 1, 2, 3])
def test_nodal_values_match_oracle(lib, p, precision):
    from oracle import output as O
    pd = _setup(p, precision)
    s = pd.solver
    try:
        s.step(7, 0, pd.tau)
        c = s.get_state()
        lag = s.get_lagrange()
    finally:
        s.close()
    ref = O.project_disc_to_lagr(c, p)
    assert lag.shape == ref.shape
    scale = np.abs(c).sum(axis=1, keepdims=True) * 4
    assert np.all(np.abs(lag - ref) <= 4 * np.finfo(np.float64).eps * scale)


def test_async_files_match_oracle_text(lib, tmp_path):
    from oracle import output as O
    pd = _setup(2, 'fp32', numSteps=12)
    s = pd.solver
    base = str(tmp_path / 'out' / 'advection_linear')
    lags = {}
    try:
        for n0, n1, types in [(0, 4, ['vtk', 'tec']), (4, 8, 'vtk'), (8, 12, 'tec')]:
            s.output(base, n0, types)
            lags[n0] = (s.get_lagrange(), types)
            s.step(n1 - n0, n0, pd.tau)         # enqueued while the writer formats the files
        s.output(base, 12, 'vtk')
        lags[12] = (s.get_lagrange(), 'vtk')
        s.output_wait()
    finally:
        s.close()
    g = pd.g
    bE = _bary_e0t(g)
    for t, (lag, types) in lags.items():
        types = [types] if isinstance(types, str) else types
        for ty in ('vtk', 'tec'):
            path = '%s.%d.%s' % (base, t, 'vtu' if ty == 'vtk' else 'plt')
            if ty not in types:
                assert not os.path.exists(path)
                continue
            text = open(path).read()
            ref = O.vtu_text(g['coordV0T'], bE, lag) if ty == 'vtk' else O.tec_text(g['coordV0T'], bE, lag, t)
            assert text == ref, path
    assert not np.array_equal(lags[0][0], lags[12][0])


def test_main_writes_output_every_frequency(lib, tmp_path):
    from festung_gb300 import advection_gpu as G
    base = str(tmp_path / 'run' / 'adv')
    pd = G.main(testcase='solid_body', hmax=2 ** -3, p=1, numSteps=6, isSlopeLim=True, isVisSol=True,
                outputFrequency=2, outputBasename=base, outputTypes=['vtk', 'tec'])
    pd.solver.close()
    for n in (0, 2, 4, 6):
        for ext in ('vtu', 'plt'):
            assert os.path.getsize('%s.%d.%s' % (base, n, ext)) > 0
    assert not os.path.exists(base + '.1.vtu')
    # the final file holds the final state's nodal values (printed to 9 digits)
    from oracle import output as O
    lag = O.project_disc_to_lagr(pd.cDisc, 1)
    lines = open(base + '.6.vtu').read().split('Name="u_h" NumberOfComponents="1" format="ascii">\n')[1]
    vals = np.array(lines.split('</DataArray>')[0].split(), dtype=float).reshape(-1, 3)
    assert np.allclose(vals, lag, rtol=1e-8, atol=1e-12)


def test_ensemble_output_covers_every_instance(lib, tmp_path):
    from festung_gb300 import ensemble as E
    ens = E.Ensemble(range(6), precision='fp32', numSteps=2, hmax=2 ** -4)
    got = {}
    try:
        ens.step(2)
        for p, s in ens.solvers.items():
            base = str(tmp_path / ('ens_p%d' % p))
            s.output(base, 2, 'vtk')
            s.output_wait()
            got[p] = (base, s.get_lagrange().shape[0])
    finally:
        ens.close()
    for p, (base, K) in got.items():
        assert K == sum(ens.problems[i].K for i in ens.groups[p])
        head = open(base + '.2.vtu').read(4096)
        nP = 6 if p >= 2 else 3
        assert 'NumberOfPoints="%d" NumberOfCells="%d"' % (nP * K, K) in head


def test_write_error_is_reported_and_handle_stays_usable(lib, tmp_path):
    from festung_gb300 import _lib as L
    pd = _setup(1, 'fp64')
    s = pd.solver
    blocker = tmp_path / 'file'
    blocker.write_text('')
    try:
        s.output(str(blocker / 'x'), 0, 'vtk')
        with pytest.raises(L.DgadvError) as e:
            s.output_wait()
        assert e.value.status == L.DGADV_EIO
        s.output_wait()                         # the error was reported once
        s.step(2, 0, pd.tau)
        s.output(str(tmp_path / 'ok'), 2, 'vtk')
        s.output_wait()
        assert np.all(np.isfinite(s.get_state()))
    finally:
        s.close()
    assert os.path.exists(str(tmp_path / 'ok') + '.2.vtu')
