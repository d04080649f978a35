"""The transport problem on the GPU (dgadv_transport_*) against the oracle restatement
(oracle/transport.py): masked advection of depth-integrated concentrations, concentration
limiting and mask updates.

Bars: FP64 relative L2 <= 1e-12 for c h and c of every species and identical masks; FP32
within 1e-5 (masks may differ only where the patch range sits at the tolerance).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def run_both(precision, **kw):
    from festung_gb300 import transport_gpu as TG
    from oracle import transport as TR
    g = TG.main(precision=precision, **kw)
    g.solver.close()
    o = TR.main(**kw)
    return g, o


@pytest.mark.parametrize('kw', [
    dict(hmax=2 ** -4, numSteps=10, tEnd=10 * 0.01, numSpecies=2),
    dict(hmax=2 ** -4, numSteps=10, tEnd=10 * 0.01, numSpecies=1, isMask=False),
    dict(hmax=2 ** -4, numSteps=6, tEnd=6 * 0.005, numSpecies=2, p=2),
    dict(hmax=2 ** -3, numSteps=8, tEnd=8 * 0.02, numSpecies=3, ordRK=3),
], ids=['masked', 'unmasked', 'p2', 'rk3'])
def test_fp64_matches_oracle(lib, kw):
    g, o = run_both('fp64', **kw)
    for s in range(kw['numSpecies']):
        assert rel(g.cDisc[s], o.cDisc[s]) <= 1e-12
        assert rel(g.concDisc[s], o.concDisc[s]) <= 1e-12
        assert np.array_equal(g.mask[s], o.mask[s])
    if kw.get('isMask', True):
        assert not g.mask[0].all()          # the masks are in play


def test_fp32_close_to_oracle(lib):
    kw = dict(hmax=2 ** -4, numSteps=10, tEnd=10 * 0.01, numSpecies=2)
    g, o = run_both('fp32', **kw)
    for s in range(2):
        assert rel(g.cDisc[s], o.cDisc[s]) <= 1e-5
        assert np.mean(g.mask[s] != o.mask[s]) < 0.02


def test_transport_needs_the_linear_limiter(lib):
    from festung_gb300 import _lib as L
    from festung_gb300.solver import DeviceSolver
    from festung_gb300 import testcases as TC
    coordV, V0T, _, _ = TC.square_coords(2 ** -3)
    s = DeviceSolver(coordV, V0T, 1, 2)
    try:
        s.set_velocity_function((L.VEL_ROTATION, []))
        with pytest.raises(L.DgadvError) as e:
            s.transport_init(np.zeros((s.K, s.N)), np.zeros((s.K, s.N, 1)))
        assert e.value.status == L.DGADV_EINVAL
    finally:
        s.close()
