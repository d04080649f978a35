"""CPU oracle for the explicit DG advection step of FESTUNG's ``advection/`` problem.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (``festung_gb300``) imports, links or
executes this package.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs
of ``bench.py`` use it, and only as the checker / the timed CPU baseline.

What it is
    A restatement in numpy/scipy (FP64) of the reference Matlab/Octave solver, function by
    function.  Every function cites the reference file and line range it follows.  The
    default path assembles the same sparse operators as the reference every stage
    (``advection/preprocessSubStep.m:56-99``) and solves with the block mass matrix
    (``advection/solveSubStep.m:62-66``); a matrix-free restatement of the same stage
    (``oracle.matfree``) is kept beside it and checked against it.

Parity status: PARITY UNPINNED.
    The reference is interpreted Matlab/Octave source; no interpreter exists on this machine
    or the GPU machine, and the reference's own tests store no golden vectors or expected
    numbers (its convergence driver only prints EOC tables).  The oracle is therefore pinned
    only by (i) analytic identities (orthonormal basis => hatM ~ I, conservation, p=0 is
    first-order upwind FV), (ii) the theoretical convergence order p+1 on the reference's
    analytical 'transient' test case, and (iii) agreement of its sparse-operator and
    matrix-free restatements.
"""
