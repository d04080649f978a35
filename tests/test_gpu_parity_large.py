"""GPU parity at production size: the FP64 CUDA path against the oracle's sampled fixtures.

The fixtures (tests/golden/make_golden_large.py) hold, for a run of the matrix-free oracle at
the size the benchmark names, the final coefficients at 32768 seeded positions, the
projections of the whole final state onto 8 sign vectors, its L2 norm, the L2 error and the
oracle's roundoff spread.  The GPU runs the same configuration in FP64 and must match:
  * the sampled coefficients, relative L2 <= tol;
  * each projection within 4 tol ||c|| (the projection of an error e onto a sign vector has the
    size of ||e|| unless e is orthogonal to it, so the 8 of them see every coefficient);
  * the norm and the L2 error within tol (relative / absolute);
with tol = max(1e-12, 10 x spread), the bar of the other FP64 parity tests.
"""
import ast
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), 'golden')
FP64_TOL = 1e-12
CASES = ['gauss_slot_131k_p2_lim', 'gauss_slot_32k_p3_hier_jit']


def _signs(n, j):
    import importlib.util
    spec = importlib.util.spec_from_file_location('mgl', os.path.join(GOLD, 'make_golden_large.py'))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.signs(n, j)


@pytest.mark.parametrize('name', CASES)
def test_fp64_matches_sampled_oracle_at_size(lib, name):
    path = os.path.join(GOLD, name + '.npz')
    if not os.path.exists(path):
        pytest.skip('fixture %s not generated' % name)
    from festung_gb300 import advection_gpu as G
    d = np.load(path)
    kw = ast.literal_eval(str(d['params']))
    pd = G.main(precision='fp64', **kw)
    pd.solver.close()
    c = np.asarray(pd.cDisc)
    assert tuple(c.shape) == tuple(d['shape'])
    tol = max(FP64_TOL, 10 * float(d['spread']))
    flat = c.ravel(order='F')
    sample = d['sample']
    assert np.linalg.norm(flat[d['idx']] - sample) <= tol * np.linalg.norm(sample)
    norm = float(d['norm'])
    assert abs(np.linalg.norm(flat) - norm) <= tol * norm
    for j, pj in enumerate(d['proj']):
        assert abs(_signs(flat.size, j) @ flat - pj) <= 4 * tol * norm, j
    assert abs(pd.error - float(d['error'])) <= tol * max(1.0, float(d['error']))
