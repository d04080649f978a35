"""GB300-native explicit DG advection step (FESTUNG ``advection/`` hot path).

* ``festung_gb300.advection_gpu.main(...)`` -- the ``main('advection_gpu', ...)`` driver with
  the reference's step-function interface.
* ``festung_gb300.solver.DeviceSolver`` -- Python handle over the C-ABI (``include/dgadv.h``).
* ``festung_gb300.build.build()`` -- compiles ``libdgadv.so`` in-tree for sm_103a.
"""

def main(problemName='advection_gpu', problemData=None, **kwargs):
    if problemName != 'advection_gpu':
        raise ValueError('only the advection_gpu problem is provided')
    from .advection_gpu import main as _main
    return _main(problemData, **kwargs)
