"""Solution output on the CPU: the oracle's nodal projection against exact values, and the
library's host writer (dgadv_write_lagrange) against the oracle's text of
core/visualizeDataLagr.m, byte for byte.  The reference's own tests hold no output files, so the
format is pinned by the reference's fprintf formats (restated in oracle/output.py)."""
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from festung_gb300 import _lib as L
from oracle import assembly as A
from oracle import basis as B
from oracle import grid as G
from oracle import output as O
from oracle import testcases as OT


def _mesh(kind):
    if kind == 'square3':
        return G.domainSquare(1 / 3)      # 18 triangles: 54 and 108 points, not multiples of 5
    return OT.jittered_square(2 ** -3, 0.2, 5)


@pytest.mark.parametrize('p', [1, 2, 3])
def test_oracle_nodal_values_of_a_linear_function_are_exact(p):
    """The L2 projection of a linear function is exact for p >= 1, so its values at the Lagrange
    nodes are the function's values at the nodes' physical points."""
    g = _mesh('jitter')
    N = B.N_of_p(p)
    bases = B.computeBasesOnQuad(N)
    hatM = B.integrateRefElemPhiPhi(N, bases)
    f = lambda x, y: 0.3 - 1.7 * x + 2.5 * y
    c = A.projectFuncCont2DataDisc(g, f, 2 * p, hatM, bases)
    lag = O.project_disc_to_lagr(c)
    L1, L2 = O.lagrange_nodes(p)
    X = G.mapRef2Phy(g, 0, L1, L2)
    Y = G.mapRef2Phy(g, 1, L1, L2)
    assert lag.shape == (g.numT, 6 if p >= 2 else 3)
    assert np.abs(lag - f(X, Y)).max() < 1e-13


def test_oracle_nodal_value_at_p0_is_the_mean():
    c = np.array([[2.0], [-1.0]])
    assert np.allclose(O.project_disc_to_lagr(c, 0)[:, 0], c[:, 0] * np.sqrt(2.0))


def _read(path):
    with open(path) as f:
        return f.read()


@pytest.mark.parametrize('kind', ['square3', 'jitter'])
@pytest.mark.parametrize('numP', [1, 3, 6])
def test_host_writer_matches_the_oracle_text(lib, tmp_path, kind, numP):
    g = _mesh(kind)
    rng = np.random.default_rng(numP)
    data = rng.standard_normal((g.numT, numP)) * 10.0 ** rng.integers(-5, 5, (g.numT, numP))
    base = str(tmp_path / 'sub' / 'dir' / 'advection_linear')
    L.write_lagrange(g.coordV, g.V0T, data, 'u_h', base, 7, ['vtk', 'tec'])
    assert _read(base + '.7.vtu') == O.vtu_text(g.coordV0T, g.baryE0T, data, 'u_h')
    assert _read(base + '.7.plt') == O.tec_text(g.coordV0T, g.baryE0T, data, 7, 'u_h')


@pytest.mark.parametrize('numP', [1, 3, 6])
def test_vtu_is_well_formed(lib, tmp_path, numP):
    g = _mesh('jitter')
    data = np.arange(g.numT * numP, dtype=np.float64).reshape(g.numT, numP, order='F')
    base = str(tmp_path / 'out')
    L.write_lagrange(g.coordV, g.V0T, data, 'c', base, 0, 'vtk')
    root = ET.parse(base + '.0.vtu').getroot()
    piece = root.find('UnstructuredGrid/Piece')
    nP = 6 if numP == 6 else 3
    assert int(piece.get('NumberOfPoints')) == nP * g.numT and int(piece.get('NumberOfCells')) == g.numT
    pts = np.array(piece.find('Points/DataArray').text.split(), dtype=float).reshape(-1, 3)
    assert np.array_equal(pts[0:3, :2], g.coordV0T[0])
    if nP == 6:
        assert np.allclose(pts[3, :2], 0.5 * (g.coordV0T[0, 0] + g.coordV0T[0, 1]))
    arrays = {a.get('Name'): a.text.split() for a in piece.iter('DataArray') if a.get('Name')}
    assert len(arrays['connectivity']) == nP * g.numT
    assert set(arrays['types']) == {'22' if nP == 6 else '5'}
    vals = np.array(arrays['c'], dtype=float).reshape(g.numT, nP)
    if numP == 1:
        assert np.array_equal(vals, np.repeat(data, 3, axis=1))
    elif numP == 3:
        assert np.array_equal(vals, data)
    else:
        assert np.array_equal(vals, data[:, [0, 1, 2, 5, 3, 4]])


def test_host_writer_errors(lib, tmp_path):
    g = _mesh('square3')
    data = np.zeros((g.numT, 2))
    with pytest.raises(L.DgadvError) as e:
        L.write_lagrange(g.coordV, g.V0T, data, 'u_h', str(tmp_path / 'x'), 0)
    assert e.value.status == L.DGADV_EINVAL
    with pytest.raises(ValueError):
        L.write_lagrange(g.coordV, g.V0T, np.zeros((g.numT, 3)), 'u_h', str(tmp_path / 'x'), 0, 'png')
    blocker = tmp_path / 'file'
    blocker.write_text('')
    with pytest.raises(L.DgadvError) as e:
        L.write_lagrange(g.coordV, g.V0T, np.zeros((g.numT, 3)), 'u_h', str(blocker / 'x'), 0)
    assert e.value.status == L.DGADV_EIO
    assert not os.path.exists(str(blocker) + '/x.0.vtu')
