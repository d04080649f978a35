"""The C-ABI library on the CPU: it loads, exports every symbol of include/dgadv.h, and its host
helpers (grid incidence maps, quadrature rules, basis) match the oracle.  No GPU work here."""
import ctypes
import os
import re

import numpy as np
import pytest

from festung_gb300 import _lib as L
from oracle import basis as B
from oracle import grid as G
from oracle import testcases as OT

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, 'include', 'dgadv.h')).read()
    return sorted(set(re.findall(r'\b(dgadv_[a-z0-9_]+)\s*\(', src)))


def test_library_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
        assert n in L.SYMBOLS, 'binding missing for ' + n


def declared_constants():
    """NAME -> value of every `DGADV_NAME = value` enumerator in include/dgadv.h."""
    src = open(os.path.join(ROOT, 'include', 'dgadv.h')).read()
    return {m.group(1): int(m.group(2), 0) for m in re.finditer(r'\b(DGADV_[A-Z0-9_]+)\s*=\s*(-?(?:0x[0-9a-fA-F]+|\d+))', src)}


def test_python_constants_match_the_header():
    consts = declared_constants()
    assert len(consts) >= 20 and consts['DGADV_OPT_ADJ_WARPS'] == 4
    checked = 0
    for name, value in consts.items():
        for attr in (name, name[len('DGADV_'):]):
            if hasattr(L, attr):
                assert getattr(L, attr) == value, (attr, getattr(L, attr), value)
                checked += 1
    assert checked >= 15


def test_status_strings(lib):
    assert lib.dgadv_status_string(0) == b'ok'
    assert lib.dgadv_status_string(L.DGADV_EMESH) == b'inconsistent mesh'


@pytest.mark.parametrize('mesh', ['square3', 'square5', 'jitter', 'odd'])
def test_grid_build_is_bit_exact_against_generateGridData(lib, mesh):
    if mesh == 'square3':
        g = G.domainSquare(2 ** -3)
    elif mesh == 'square5':
        g = G.domainSquare(2 ** -5)
    elif mesh == 'jitter':
        g = OT.jittered_square(2 ** -4, 0.2, 11)
    else:
        g = G.domainSquare(1 / 6)
    r = L.grid_build(g.coordV, g.V0T)
    for k in ('V0E', 'E0T', 'T0E', 'E0E'):
        assert np.array_equal(r[k], getattr(g, k)), k
    for k in ('areaE', 'nuE', 'baryE', 'areaT', 'baryT', 'B', 'areaE0T', 'nuE0T', 'coordV0T', 'detJ0T'):
        assert np.array_equal(r[k], getattr(g, k)), k


def test_grid_build_rejects_bad_meshes(lib):
    coordV = np.array([[0., 0.], [1., 0.], [0., 1.], [1., 1.]])
    with pytest.raises(L.DgadvError) as e:
        L.grid_build(coordV, np.array([[0, 2, 1]]))        # clockwise
    assert e.value.status == L.DGADV_EMESH
    with pytest.raises(L.DgadvError):
        L.grid_build(coordV, np.array([[0, 1, 7]]))        # vertex out of range
    with pytest.raises(L.DgadvError):
        L.grid_build(coordV, np.array([[0, 1, 2], [0, 1, 3]]))   # edge with equal orientation


@pytest.mark.parametrize('qOrd', range(0, 10))
def test_quadrature_rules_match(lib, qOrd):
    Q, W = L.quad_rule_1d(qOrd)
    Qo, Wo = B.quadRule1D(qOrd)
    assert np.array_equal(Q, Qo) and np.array_equal(W, Wo)
    a = L.quad_rule_2d(qOrd)
    b = B.quadRule2D(qOrd)
    tol = 0.0 if qOrd < 7 else 4e-16
    for x, y in zip(a, b):
        assert np.abs(x - y).max() <= tol


def test_basis_matches(lib):
    rng = np.random.default_rng(0)
    X = rng.random(50); Y = rng.random(50) * (1 - X)
    P, Gr = L.basis_eval(15, X, Y, grad=True)
    for i in range(15):
        assert np.array_equal(P[:, i], B.phi(i, X, Y))
        for m in range(2):
            assert np.array_equal(Gr[:, i, m], B.gradPhi(i, m, X, Y))


def test_invalid_arguments_are_rejected_without_a_gpu(lib):
    R = ctypes.c_int32()
    assert lib.dgadv_quad_rule_1d(42, ctypes.byref(R), None, None) == L.DGADV_EINVAL
    assert lib.dgadv_create(None, None, None) == L.DGADV_EINVAL
    prm = L.Params(); prm.p = 5; prm.ordRK = 3
    mesh = L.Mesh()
    h = ctypes.c_void_p()
    assert lib.dgadv_create(ctypes.byref(mesh), ctypes.byref(prm), ctypes.byref(h)) == L.DGADV_EINVAL
    prm.p = 4
    assert lib.dgadv_create(ctypes.byref(mesh), ctypes.byref(prm), ctypes.byref(h)) == L.DGADV_EUNSUPPORTED
    prm.p = 2; prm.isSlopeLim = 1; prm.typeSlopeLim = 7
    assert lib.dgadv_create(ctypes.byref(mesh), ctypes.byref(prm), ctypes.byref(h)) == L.DGADV_EINVAL
