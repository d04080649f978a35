"""Generates the golden fixtures of tests/golden from the oracle (sparse-operator restatement).

Run from the repository root:  python tests/golden/make_golden.py
Each fixture stores the parameters, the final coefficients cDisc (K x N), the L2 errors and the
roundoff spread of the configuration (relative L2 distance between two roundings of the same
oracle algebra, see oracle.matfree.roundoff_spread), which bounds any parity claim for it.  The oracle is test infrastructure (see oracle/__init__.py); the fixtures let
the GPU tests check the device path without running the slow oracle on the GPU machine.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import advection as adv  # noqa: E402
from oracle import matfree as MF  # noqa: E402

CASES = {
    # the 2048-triangle benchmark case: p=1, RK2, tau=1e-3, 500 steps, linear limiter
    'gauss_slot_2048_p1_lim': dict(testcase='gauss_slot', hmax=2 ** -5, p=1, tEnd=0.5, numSteps=500,
                                   isSlopeLim=True, typeSlopeLim='linear'),
    # p=2 with time-derivative limiting on a smaller mesh
    'p2_lim_h4': dict(testcase='gauss_slot', hmax=2 ** -4, p=2, tEnd=0.05, numSteps=100,
                      isSlopeLim=True, typeSlopeLim='linear'),
    # p=3 with the hierarchical vertex limiter on a jittered mesh
    'p3_hier_jit': dict(testcase='gauss_slot', hmax=2 ** -3, p=3, tEnd=0.02, numSteps=40,
                        isSlopeLim=True, typeSlopeLim='hierarch_vert', jitter=0.1, meshSeed=7),
    # analytical transient case (source and Dirichlet data), no limiter
    'transient_p2': dict(testcase='transient', hmax=2 ** -3, p=2, tEnd=0.1, numSteps=40),
}


def make(name, kw):
    pd = adv.main(oracleCacheOperators=True, **kw)
    # roundoff spread of the configuration: two roundings of the same algebra
    spread = MF.roundoff_spread(**kw)
    out = os.path.join(HERE, name + '.npz')
    np.savez_compressed(out, cDisc=pd.cDisc, error=pd.error, initialError=pd.initialError,
                        params=repr(kw), spread=spread)
    print(name, pd.K, pd.N, pd.error, spread)


if __name__ == '__main__':
    names = sys.argv[1:] or list(CASES)
    for n in names:
        make(n, CASES[n])
