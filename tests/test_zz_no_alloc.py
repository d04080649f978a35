"""The no-allocation limiter entry point against the handle-based one.

``dgadv_limit_linear_noalloc`` serves callers that cannot call cudaMalloc (their device memory
comes from another framework's pool, or is capped in advance): it works on device arrays the
caller owns and keeps its scratch in a fixed array inside the library.  Here it is called
through the C-ABI twice in a row, on two different meshes and states, and each result is
compared with one solution-limiter pass of a DeviceSolver handle (``dgadv_limit_state``) on the
same data.  The second call checks that the first call's leftovers in the shared scratch do not
leak into its result.  Bar: the FP64 tolerance of the other GPU parity tests, relative L2
<= 1e-12.  This file is collected last so that it also runs after every other GPU test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def _case(hmax, p, seed, jitter, with_data):
    from festung_gb300 import _lib as L
    from festung_gb300.testcases import jitter_coords, square_coords
    coordV, V0T, _, h = square_coords(hmax)
    coordV = jitter_coords(coordV, h, jitter, seed)
    K, N = V0T.shape[0], (p + 1) * (p + 2) // 2
    rng = np.random.default_rng(seed)
    c = np.asfortranarray(rng.standard_normal((K, N)))
    # vertices of Dirichlet edges (every boundary edge is Dirichlet when no marks are given);
    # edge n of a triangle is opposite its vertex n
    g = L.grid_build(coordV, V0T)
    onBdr = g['T0E'][:, 1] == 0
    vD = np.zeros(coordV.shape[0], dtype=bool)
    vD[g['V0E'][onBdr].ravel()] = True
    markV0TbdrD = np.asfortranarray(vD[V0T].astype(np.uint8))
    data = np.asfortranarray(rng.standard_normal((K, 3))) if with_data else None
    return dict(coordV=coordV, V0T=V0T, p=p, c=c, markV0TbdrD=markV0TbdrD, data=data)


def _with_handle(cs):
    from festung_gb300.solver import DeviceSolver
    K, N = cs['c'].shape
    s = DeviceSolver(cs['coordV'], cs['V0T'], p=cs['p'], ordRK=3, precision='fp64', isSlopeLim=True,
                     typeSlopeLim='linear')
    try:
        if cs['data'] is not None:
            s.set_source_terms([0], [np.zeros((K, N))], [cs['data']])
        s.set_state(cs['c'])
        s.limit_state(0.0)
        return s.get_state()
    finally:
        s.close()


def _no_alloc(cs, in_place=False, V0T=None):
    """Device arrays are made by the test (the caller); the entry point itself allocates none.
    in_place: cOut is cIn.  V0T: vertex ids to pass instead of the case's own."""
    import torch
    from festung_gb300 import _lib as L
    lib = L.load()
    dev = torch.device('cuda:0')
    K, N = cs['c'].shape
    ids = cs['V0T'] if V0T is None else V0T
    V0T = torch.from_numpy(np.asfortranarray(ids, dtype=np.int32).T.copy()).to(dev)          # 3 x K
    mark = torch.from_numpy(cs['markV0TbdrD'].T.copy()).to(dev)
    data = torch.from_numpy(cs['data'].T.copy()).to(dev) if cs['data'] is not None else None
    cin = torch.from_numpy(cs['c'].T.copy()).to(dev)                                          # N x K
    cout = cin if in_place else torch.full_like(cin, float('nan'))
    stream = torch.cuda.current_stream(dev)
    st = lib.dgadv_limit_linear_noalloc(cs['p'], K, cs['coordV'].shape[0], V0T.data_ptr(), mark.data_ptr(),
                                        data.data_ptr() if data is not None else None,
                                        cin.data_ptr(), cout.data_ptr(), stream.cuda_stream)
    L.check(st)
    stream.synchronize()
    return cout.cpu().numpy().T


def test_no_alloc_matches_handle_two_calls():
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('no GPU')
    first = _case(2 ** -5, p=2, seed=11, jitter=0.2, with_data=True)
    second = _case(2 ** -4, p=1, seed=12, jitter=0.1, with_data=False)   # fewer vertices
    for cs in (first, second):
        got = _no_alloc(cs)
        ref = _with_handle(cs)
        assert np.all(np.isfinite(got))
        assert not np.array_equal(ref, cs['c']), 'the limiter changed nothing: the case checks nothing'
        assert rel(got, ref) <= FP64_TOL, rel(got, ref)


def test_no_alloc_in_place():
    """cOut may be cIn: each element reads only its own coefficients after the patch pass."""
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('no GPU')
    cs = _case(2 ** -5, p=2, seed=11, jitter=0.2, with_data=True)
    got = _no_alloc(cs, in_place=True)
    ref = _with_handle(cs)
    assert rel(got, ref) <= FP64_TOL, rel(got, ref)


def test_no_alloc_skips_out_of_range_vertex():
    """A vertex id outside [0, numV) is checked by the kernels: that element enters no patch and
    its output is NaN; the other elements stay finite, and the next call is unaffected."""
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('no GPU')
    from festung_gb300 import _lib as L
    cs = _case(2 ** -4, p=1, seed=12, jitter=0.1, with_data=False)
    numV = cs['coordV'].shape[0]
    bad = np.array(cs['V0T'], dtype=np.int64)
    bad[5, 1] = L.NOALLOC_MAX_VERTICES + 7       # beyond the scratch array's vertex slots
    bad[9, 2] = numV                              # one past the last vertex
    got = _no_alloc(cs, V0T=bad)
    assert np.all(np.isnan(got[[5, 9]]))
    others = np.setdiff1d(np.arange(got.shape[0]), [5, 9])
    assert np.all(np.isfinite(got[others]))
    good = _no_alloc(cs)
    assert rel(good, _with_handle(cs)) <= FP64_TOL


def test_no_alloc_rejects_oversize():
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('no GPU')
    from festung_gb300 import _lib as L
    lib = L.load()
    x = torch.zeros(16, dtype=torch.float64, device='cuda:0')
    v = torch.zeros(3, dtype=torch.int32, device='cuda:0')
    st = lib.dgadv_limit_linear_noalloc(1, 1, L.NOALLOC_MAX_VERTICES + 1, v.data_ptr(), None, None,
                                        x.data_ptr(), x.data_ptr(), None)
    assert st == L.DGADV_ENOMEM
    assert lib.dgadv_limit_linear_noalloc(4, 1, 3, v.data_ptr(), None, None, x.data_ptr(), x.data_ptr(),
                                          None) == L.DGADV_EINVAL
