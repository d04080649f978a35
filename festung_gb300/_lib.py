"""ctypes binding of ``libdgadv.so`` (the C-ABI declared in ``include/dgadv.h``).

There is no fallback: if the shared library is missing or fails to load, every call raises.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libdgadv.so')

DGADV_OK, DGADV_EINVAL, DGADV_ECUDA, DGADV_ENOMEM, DGADV_EMESH = 0, 1, 2, 3, 4
DGADV_ENONFINITE, DGADV_ETIMEOUT, DGADV_EUNSUPPORTED, DGADV_EIO = 5, 6, 7, 8
DGADV_ENOCONV = 9
FP64, FP32, DF32 = 0, 1, 2
LIM_LINEAR, LIM_HIERARCH_VERT, LIM_STRICT = 0, 1, 2
TIME_CONST, TIME_EXP_NEG = 0, 1
FLAG_NO_REORDER, FLAG_NO_SHIFT, FLAG_NO_GRAPH, FLAG_NO_PDL, FLAG_FUSE, FLAG_PERSIST = 1, 2, 4, 8, 16, 32
OPT_GRAPH_STEPS, OPT_FLAGS, OPT_PERSIST_BLOCKS, OPT_ADJ_WARPS, OPT_TAYLOR_MASS, OPT_VOLUME_MMA, OPT_OP_BLOCK, \
    OPT_OPERATOR_FP32, OPT_ADJ_STREAMS, OPT_ELEMENT_OPERATOR, OPT_ADJ_GRAPH = 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11
OUT_VTK, OUT_TEC = 1, 2
FN_CONST, FN_POLY3, FN_SOLID_BODY, FN_GAUSS_SLOT, FN_GAUSS, FN_TRANSIENT, FN_COS7 = 0, 1, 2, 3, 4, 5, 6
VEL_ROTATION, VEL_TRANSIENT, VEL_STREAM, VEL_CONST = 16, 17, 18, 19
FLAG_IMPLICIT = 64
FN_MAX_PARAMS = 64
OUTPUT_TYPES = {'vtk': OUT_VTK, 'tec': OUT_TEC}

LIMITER_TYPES = {'linear': LIM_LINEAR, 'hierarch_vert': LIM_HIERARCH_VERT, 'strict': LIM_STRICT}

_i32p = ctypes.POINTER(ctypes.c_int32)
_dp = ctypes.POINTER(ctypes.c_double)
_u8p = ctypes.POINTER(ctypes.c_uint8)


class DgadvError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__('%s (status %d)' % (msg, status))
        self.status = status


class Grid(ctypes.Structure):
    _fields_ = [('numT', ctypes.c_int32), ('numV', ctypes.c_int32), ('numE', ctypes.c_int32),
                ('V0E', _i32p), ('T0E', _i32p), ('E0T', _i32p), ('E0E', _i32p),
                ('areaE', _dp), ('nuE', _dp), ('baryE', _dp), ('areaT', _dp), ('baryT', _dp),
                ('B', _dp), ('areaE0T', _dp), ('nuE0T', _dp), ('coordV0T', _dp), ('detJ0T', _dp)]


class Mesh(ctypes.Structure):
    _fields_ = [('numT', ctypes.c_int32), ('numV', ctypes.c_int32), ('coordV', _dp),
                ('V0T', _i32p), ('idE0T', _i32p), ('markE0TbdrD', _u8p), ('markE0TbdrN', _u8p)]


class Params(ctypes.Structure):
    _fields_ = [('p', ctypes.c_int32), ('ordRK', ctypes.c_int32), ('precision', ctypes.c_int32),
                ('isSlopeLim', ctypes.c_int32), ('typeSlopeLim', ctypes.c_int32),
                ('device', ctypes.c_int32), ('flags', ctypes.c_int32)]


class Krylov(ctypes.Structure):
    _fields_ = [('tol', ctypes.c_double), ('maxIter', ctypes.c_int32), ('restart', ctypes.c_int32)]


class Function(ctypes.Structure):
    _fields_ = [('kind', ctypes.c_int32), ('nParams', ctypes.c_int32), ('params', _dp)]


def functions(specs):
    """(kind, params) pairs -> a ctypes array of dgadv_function (and the parameter arrays it
    points into, which must stay alive during the call)."""
    arr = (Function * len(specs))()
    keep = []
    for i, (kind, params) in enumerate(specs):
        p = np.ascontiguousarray(np.asarray(params if params is not None else [], dtype=np.float64))
        keep.append(p)
        arr[i].kind = int(kind)
        arr[i].nParams = p.size
        arr[i].params = p.ctypes.data_as(_dp) if p.size else None
    return arr, keep


SYMBOLS = {
    'dgadv_grid_build': (ctypes.c_int, [ctypes.c_int32, _dp, ctypes.c_int32, _i32p,
                                        ctypes.POINTER(ctypes.POINTER(Grid))]),
    'dgadv_grid_free': (None, [ctypes.POINTER(Grid)]),
    'dgadv_quad_rule_1d': (ctypes.c_int, [ctypes.c_int32, _i32p, _dp, _dp]),
    'dgadv_quad_rule_2d': (ctypes.c_int, [ctypes.c_int32, _i32p, _dp, _dp, _dp]),
    'dgadv_basis_eval': (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, _dp, _dp, _dp, _dp]),
    'dgadv_create': (ctypes.c_int, [ctypes.POINTER(Mesh), ctypes.POINTER(Params),
                                    ctypes.POINTER(ctypes.c_void_p)]),
    'dgadv_create_ensemble': (ctypes.c_int, [ctypes.POINTER(Mesh), ctypes.c_int32, ctypes.POINTER(Params),
                                             ctypes.POINTER(ctypes.c_void_p)]),
    'dgadv_set_velocity': (ctypes.c_int, [ctypes.c_void_p, _dp, _dp, _dp]),
    'dgadv_set_source_terms': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _i32p, _dp, _dp]),
    'dgadv_set_state': (ctypes.c_int, [ctypes.c_void_p, _dp]),
    'dgadv_get_state': (ctypes.c_int, [ctypes.c_void_p, _dp]),
    'dgadv_limit_state': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    'dgadv_step': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double]),
    'dgadv_sync': (ctypes.c_int, [ctypes.c_void_p]),
    'dgadv_set_option': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32]),
    'dgadv_get_option': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _i32p]),
    'dgadv_selftest_wait': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    'dgadv_kernels_per_step': (ctypes.c_int, [ctypes.c_void_p, _i32p]),
    'dgadv_link': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    'dgadv_time_steps': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, _dp]),
    'dgadv_profile_kernels': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                             _dp, _i32p]),
    'dgadv_last_error': (ctypes.c_char_p, [ctypes.c_void_p]),
    'dgadv_status_string': (ctypes.c_char_p, [ctypes.c_int]),
    'dgadv_destroy': (None, [ctypes.c_void_p]),
    'dgadv_set_velocity_modes': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _dp, _dp, _dp]),
    'dgadv_set_velocity_theta': (ctypes.c_int, [ctypes.c_void_p, _dp]),
    'dgadv_forward_record': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double, ctypes.c_int32]),
    'dgadv_backward': (ctypes.c_int, [ctypes.c_void_p, _dp, _dp, _dp]),
    'dgadv_checkpoint_schedule': (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, _i32p, _i32p, _i32p]),
    'dgadv_step_implicit': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                           ctypes.c_int32, ctypes.POINTER(Krylov), _i32p, _dp]),
    'dgadv_solve_stationary': (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Krylov), _i32p, _dp]),
    'dgadv_transport_init': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _dp, _dp, ctypes.c_double,
                                            ctypes.c_int32]),
    'dgadv_transport_step': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double]),
    'dgadv_transport_get': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _dp, _dp, _u8p]),
    'dgadv_project_state': (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Function), ctypes.c_int32,
                                           ctypes.c_double, ctypes.c_int32]),
    'dgadv_set_velocity_function': (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Function), ctypes.c_int32]),
    'dgadv_l2_error': (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Function), ctypes.c_int32, ctypes.c_double,
                                      ctypes.c_int32, _dp]),
    'dgadv_get_lagrange': (ctypes.c_int, [ctypes.c_void_p, _dp, _i32p]),
    'dgadv_output': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32,
                                    ctypes.c_int32]),
    'dgadv_output_wait': (ctypes.c_int, [ctypes.c_void_p]),
    'dgadv_write_lagrange': (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, _dp, _i32p, ctypes.c_int32, _dp,
                                            ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32, ctypes.c_int32]),
    'dgadv_limit_linear_noalloc': (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
}

NOALLOC_MAX_VERTICES = 1 << 18

_lib = None


def load(path=LIB_PATH):
    """Load the shared library (raises OSError if it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise OSError('libdgadv.so not built: run festung_gb300.build.build() first (%s)' % path)
        lib = ctypes.CDLL(path)
        for name, (res, args) in SYMBOLS.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def ptr(a, t=_dp):
    return a.ctypes.data_as(t) if a is not None else None


def f64(a):
    return np.require(np.asarray(a, dtype=np.float64), requirements=['F', 'A'])


def check(status, handle=None):
    if status != DGADV_OK:
        lib = load()
        msg = lib.dgadv_status_string(status).decode()
        if handle:
            detail = lib.dgadv_last_error(handle)
            if detail:
                msg += ': ' + detail.decode()
        raise DgadvError(status, msg)


# ---------------------------------------------------------------------------------------------
def grid_build(coordV, V0T):
    """generateGridData(coordV, V0T) through the library; returns a dict of numpy arrays with the
    reference's conventions (V0E, E0T 0-based; T0E, E0E 1-based with 0 = none)."""
    lib = load()
    coordV = f64(coordV)
    V0T = np.require(np.asarray(V0T, dtype=np.int32), requirements=['F', 'A'])
    numV, numT = coordV.shape[0], V0T.shape[0]
    out = ctypes.POINTER(Grid)()
    check(lib.dgadv_grid_build(numV, ptr(coordV), numT, ptr(V0T, _i32p), ctypes.byref(out)))
    g = out.contents
    T, E = g.numT, g.numE

    def arr(p, shape, dt):
        n = int(np.prod(shape))
        ct = p._type_                                # c_double or c_int32
        buf = (ct * n).from_address(ctypes.addressof(p.contents))
        a = np.frombuffer(buf, dtype=np.dtype(ct), count=n).astype(dt, copy=True)
        return a.reshape(shape, order='F')
    res = dict(numT=T, numV=g.numV, numE=E,
               V0E=arr(g.V0E, (E, 2), np.int64), T0E=arr(g.T0E, (E, 2), np.int64),
               E0T=arr(g.E0T, (T, 3), np.int64), E0E=arr(g.E0E, (E, 2), np.int64),
               areaE=arr(g.areaE, (E,), np.float64), nuE=arr(g.nuE, (E, 2), np.float64),
               baryE=arr(g.baryE, (E, 2), np.float64), areaT=arr(g.areaT, (T,), np.float64),
               baryT=arr(g.baryT, (T, 2), np.float64), B=arr(g.B, (T, 2, 2), np.float64),
               areaE0T=arr(g.areaE0T, (T, 3), np.float64), nuE0T=arr(g.nuE0T, (T, 3, 2), np.float64),
               coordV0T=arr(g.coordV0T, (T, 3, 2), np.float64), detJ0T=arr(g.detJ0T, (T,), np.float64))
    lib.dgadv_grid_free(out)
    return res


def output_types(types):
    """'vtk' / 'tec' or a list of them (the reference's outputTypes) -> DGADV_OUT_* bits."""
    if isinstance(types, str):
        types = [types]
    bits = 0
    for t in types:
        if t not in OUTPUT_TYPES:
            raise ValueError('Unknown file type: %s' % t)
        bits |= OUTPUT_TYPES[t]
    return bits


def write_lagrange(coordV, V0T, dataLagr, varName, fileName, tLvl, types='vtk'):
    """Host-only writer (core/visualizeDataLagr.m): coordV numV x 2, V0T numT x 3 (0-based),
    dataLagr numT x numP with numP in {1, 3, 6}."""
    lib = load()
    cV = f64(coordV)
    V = np.require(np.asarray(V0T, dtype=np.int32), requirements=['F', 'A'])
    d = f64(dataLagr)
    check(lib.dgadv_write_lagrange(V.shape[0], cV.shape[0], ptr(cV), ptr(V, _i32p), d.shape[1], ptr(d),
                                   varName.encode(), fileName.encode(), int(tLvl), output_types(types)))


def checkpoint_schedule(nSteps, nSnapshots):
    """The adjoint's checkpointing actions as an (n, 2) array of (action, argument) and the index
    of the first reverse-sweep action (actions: 0 restore slot, 1 advance, 2 store slot,
    3 reverse step)."""
    lib = load()
    n = ctypes.c_int32(0)
    b = ctypes.c_int32(0)
    check(lib.dgadv_checkpoint_schedule(nSteps, nSnapshots, None, ctypes.byref(n), None))
    a = np.zeros(2 * n.value, dtype=np.int32)
    check(lib.dgadv_checkpoint_schedule(nSteps, nSnapshots, ptr(a, _i32p), ctypes.byref(n), ctypes.byref(b)))
    return a.reshape(-1, 2), b.value


def quad_rule_1d(qOrd):
    lib = load()
    R = ctypes.c_int32()
    check(lib.dgadv_quad_rule_1d(qOrd, ctypes.byref(R), None, None))
    Q = np.zeros(R.value); W = np.zeros(R.value)
    check(lib.dgadv_quad_rule_1d(qOrd, ctypes.byref(R), ptr(Q), ptr(W)))
    return Q, W


def quad_rule_2d(qOrd):
    lib = load()
    R = ctypes.c_int32()
    check(lib.dgadv_quad_rule_2d(qOrd, ctypes.byref(R), None, None, None))
    Q1 = np.zeros(R.value); Q2 = np.zeros(R.value); W = np.zeros(R.value)
    check(lib.dgadv_quad_rule_2d(qOrd, ctypes.byref(R), ptr(Q1), ptr(Q2), ptr(W)))
    return Q1, Q2, W


def basis_eval(N, X1, X2, grad=False):
    """phi (nPts x N) and optionally gradPhi (nPts x N x 2) at reference points."""
    lib = load()
    X1 = f64(np.ravel(X1)); X2 = f64(np.ravel(X2))
    n = X1.size
    P = np.zeros((n, N), order='F')
    G = np.zeros((n, N, 2), order='F') if grad else None
    check(lib.dgadv_basis_eval(N, n, ptr(X1), ptr(X2), ptr(P), ptr(G)))
    return (P, G) if grad else P
