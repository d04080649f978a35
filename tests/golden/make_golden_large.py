"""Generates the sampled golden fixtures of the production-size configurations from the oracle.

Run from the repository root:  python tests/golden/make_golden_large.py [name ...]
The oracle here is the matrix-free restatement (oracle.matfree), which runs the 131072-triangle
benchmark case in about 20 minutes on one core; the sparse-operator restatement cannot (the
reference's K x K vertex masks).  A final state of that size (786,432 coefficients) is too large
for a fixture, so each fixture stores:
  * `idx`, `sample`: the final coefficients at 32768 seeded positions of the K x N array in
    column-major order (the reference's cDisc layout), for a relative L2 distance on the sample;
  * `proj`: the projections of the whole final state onto 8 sign vectors (`signs` below, an
    integer hash of the position, no random generator), which see every coefficient;
  * `norm`, `error`: the L2 norm of the whole final state and the oracle's L2 error;
  * `spread`: the oracle's roundoff spread of the configuration (relative L2 distance between
    LU solves and explicit inverses of the same algebra, oracle.matfree.roundoff_spread).
The oracle is test infrastructure (see oracle/__init__.py).
"""
import concurrent.futures as cf
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

CASES = {
    # the production benchmark case: 131072 triangles, p=2, SSP-RK3, tau=1e-4, 500 steps, linear
    # limiter (time-derivative and solution limiting)
    'gauss_slot_131k_p2_lim': dict(testcase='gauss_slot', hmax=2 ** -8, p=2, numSteps=500, tEnd=500 * 1e-4,
                                   isSlopeLim=True, typeSlopeLim='linear', ordRK=3),
    # the large-mesh configuration's shape at 32768 triangles: 10% node jitter, p=3, hierarchical
    # vertex limiter, 100 SSP-RK3 steps of 2e-5
    'gauss_slot_32k_p3_hier_jit': dict(testcase='gauss_slot', hmax=2 ** -7, p=3, numSteps=100, tEnd=100 * 2e-5,
                                       isSlopeLim=True, typeSlopeLim='hierarch_vert', ordRK=3, jitter=0.1,
                                       meshSeed=5),
}
NSAMPLE = 32768
NPROJ = 8


def signs(n, j):
    """Sign vector j (+-1) over n positions: the top bit of a splitmix64 hash of (position, j)."""
    x = np.arange(n, dtype=np.uint64) + np.uint64((j + 1) * 0x9E3779B97F4A7C15 % 2 ** 64)
    x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    x = x ^ (x >> np.uint64(31))
    return np.where((x >> np.uint64(63)) == 1, 1.0, -1.0)


def summarize(c):
    """(norm, projections) of a K x N state taken in column-major order."""
    flat = np.asarray(c).ravel(order='F')
    proj = np.array([signs(flat.size, j) @ flat for j in range(NPROJ)])
    return float(np.linalg.norm(flat)), proj


def _run(kw, rounding):
    import warnings
    warnings.simplefilter('ignore')
    from oracle import matfree as MF
    pd = MF.main_matfree(rounding=rounding, **kw)
    return np.asarray(pd.cDisc), float(pd.error)


def make(name, kw):
    with cf.ProcessPoolExecutor(2, mp_context=mp.get_context('spawn')) as ex:
        fa = ex.submit(_run, kw, 'lu')
        fb = ex.submit(_run, kw, 'inverse')
        (a, err), (b, _) = fa.result(), fb.result()
    spread = float(np.linalg.norm(a - b) / np.linalg.norm(a))
    flat = a.ravel(order='F')
    idx = np.sort(np.random.default_rng(2026).choice(flat.size, size=min(NSAMPLE, flat.size), replace=False))
    norm, proj = summarize(a)
    out = os.path.join(HERE, name + '.npz')
    np.savez_compressed(out, idx=idx.astype(np.int32), sample=flat[idx], proj=proj, norm=norm, error=err,
                        shape=np.array(a.shape), params=repr(kw), spread=spread)
    print(name, a.shape, err, spread, flush=True)


if __name__ == '__main__':
    names = sys.argv[1:] or list(CASES)
    for n in names:
        make(n, CASES[n])
