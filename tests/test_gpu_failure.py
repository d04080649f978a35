"""GPU failure detection without a fault: a bounded device wait on a flag that nothing sets
runs out, the host reads DGADV_ETIMEOUT, and the handle keeps working (the next run matches the
oracle)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_timeout_and_handle_recovers(lib):
    from festung_gb300 import _lib as L
    from festung_gb300 import advection_gpu as G
    from oracle import matfree as MF
    kw = dict(testcase='gauss_slot', hmax=2 ** -3, p=2, tEnd=0.01, numSteps=5, isSlopeLim=True)
    pd = G.main(precision='fp64', **kw)
    s = pd.solver
    try:
        st = L.load().dgadv_selftest_wait(s._h, 0.05)
        assert st == L.DGADV_ETIMEOUT
        s.sync()                                   # the error was cleared; the context is usable
        s.set_state(G.project(pd.g, pd.tables, pd.c0Cont, pd.qOrd, pd.hatM))
        s.limit_state(0.0)
        s.step(kw['numSteps'], 0, pd.tau)
        c = s.get_state()
    finally:
        s.close()
    o = MF.main_matfree(**kw).cDisc
    assert np.linalg.norm(c - o) <= 1e-12 * np.linalg.norm(o)
