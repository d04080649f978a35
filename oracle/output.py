"""Nodal values and the VTK / Tecplot text of the solution output (oracle restatement).

Test infrastructure: see ``oracle/__init__.py``.  Follows core/projectDataDisc2DataLagr.m:43-57
(modal coefficients -> values at the Lagrange nodes) and core/visualizeDataLagr.m:114-260 (the
``.vtu`` and ``.plt`` writers, scalar data only).

The writers return the file text.  The reference prints with MATLAB's ``fprintf``, which cycles
its format over the data in column order and, when the data ends inside the format, prints the
literal text up to the next conversion and stops; ``_cycle`` restates that rule.
"""
import numpy as np

from .basis import phi


def lagrange_nodes(p):
    """Reference-element nodes (L1, L2) of core/projectDataDisc2DataLagr.m:49-53: the centroid
    at p = 0, the vertices at p = 1, vertices and edge midpoints at p >= 2."""
    if p == 0:
        return np.array([1 / 3]), np.array([1 / 3])
    if p == 1:
        return np.array([0.0, 1.0, 0.0]), np.array([0.0, 0.0, 1.0])
    return np.array([0.0, 1.0, 0.0, 0.5, 0.0, 0.5]), np.array([0.0, 0.0, 1.0, 0.5, 0.5, 0.0])


def project_disc_to_lagr(dataDisc, p=None):
    """core/projectDataDisc2DataLagr.m:43-57: K x numP nodal values, summed over the basis in
    order (dataLagr = dataLagr + dataDisc(:, i) * phi(i, L1, L2))."""
    dataDisc = np.asarray(dataDisc, dtype=np.float64)
    K, N = dataDisc.shape
    if p is None:
        p = int(round((np.sqrt(8 * N + 1) - 3) / 2))
    L1, L2 = lagrange_nodes(p)
    out = np.zeros((K, L1.size))
    for i in range(N):
        out = out + dataDisc[:, i:i + 1] * phi(i, L1, L2)[None, :]
    return out


def _cycle(fmt_items, values, sep_after):
    """fprintf(fmt, values) for a format of len(fmt_items) conversions, each conversion
    followed by the literal sep_after[j]: the output stops after the literal that follows the
    last value (core/visualizeDataLagr.m prints its Tecplot blocks this way)."""
    out = []
    n = len(fmt_items)
    for k, v in enumerate(values):
        j = k % n
        out.append(fmt_items[j] % v)
        out.append(sep_after[j])
    return ''.join(out)


def _points(coordV0T, baryE0T, numP):
    """P1, P2 of core/visualizeDataLagr.m:127-138: per element its vertices, then (numP = 6)
    the midpoints of edges 3, 1, 2 (between vertices 1-2, 2-3 and 3-1)."""
    if numP == 3:
        return coordV0T[:, :, 0].reshape(-1), coordV0T[:, :, 1].reshape(-1)
    P1 = np.concatenate([coordV0T[:, :, 0], baryE0T[:, [2, 0, 1], 0]], axis=1).reshape(-1)
    P2 = np.concatenate([coordV0T[:, :, 1], baryE0T[:, [2, 0, 1], 1]], axis=1).reshape(-1)
    return P1, P2


def _point_values(dataLagr):
    """Per-point data in output order (core/visualizeDataLagr.m:209-218): the element value on
    each of its three points (numP = 1), element-major (3), edge nodes permuted [1,2,3,6,4,5]
    for the VTK / Tecplot node order (6)."""
    K, N = dataLagr.shape
    if N == 1:
        return np.repeat(dataLagr[:, 0], 3)
    if N == 3:
        return dataLagr.reshape(-1)
    return dataLagr[:, [0, 1, 2, 5, 3, 4]].reshape(-1)


def vtu_text(coordV0T, baryE0T, dataLagr, varName='u_h'):
    """The .vtu file of core/visualizeDataLagr.m:114-240 for one scalar variable."""
    dataLagr = np.asarray(dataLagr, dtype=np.float64)
    K, N = dataLagr.shape
    numP, cellType = (6, 22) if N == 6 else (3, 5)
    P1, P2 = _points(coordV0T, baryE0T, numP)
    s = ['<?xml version="1.0"?>\n',
         '<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian" '
         'compressor="vtkZLibDataCompressor">\n',
         '  <UnstructuredGrid>\n',
         '    <Piece NumberOfPoints="%d" NumberOfCells="%d">\n' % (K * numP, K),
         '      <Points>\n',
         '        <DataArray type="Float32" NumberOfComponents="3" format="ascii">\n']
    s += ['          %.12e %.12e %.1e\n' % (x, y, 0.0) for x, y in zip(P1, P2)]
    s += ['        </DataArray>\n', '      </Points>\n', '      <Cells>\n',
          '        <DataArray type="Int32" Name="connectivity" format="ascii">\n', '           ']
    s += ['%d ' % i for i in range(K * numP)]
    s += ['\n        </DataArray>\n', '        <DataArray type="Int32" Name="offsets" format="ascii">\n']
    s += ['           %d\n' % o for o in range(numP, numP * K + 1, numP)]
    s += ['        </DataArray>\n', '        <DataArray type="UInt8" Name="types" format="ascii">\n']
    s += ['           %d\n' % cellType] * K
    s += ['        </DataArray>\n', '      </Cells>\n',
          '      <PointData Scalars="%s">\n' % varName,
          '        <DataArray type="Float32" Name="%s" NumberOfComponents="1" format="ascii">\n' % varName]
    s += ['          %.9e\n' % v for v in _point_values(dataLagr)]
    s += ['        </DataArray>\n', '      </PointData>\n', '    </Piece>\n', '  </UnstructuredGrid>\n',
          '</VTKFile>\n']
    return ''.join(s)


def tec_text(coordV0T, baryE0T, dataLagr, tLvl, varName='u_h'):
    """The .plt file of core/visualizeDataLagr.m:242-291 for one scalar variable."""
    dataLagr = np.asarray(dataLagr, dtype=np.float64)
    K, N = dataLagr.shape
    numP = 6 if N == 6 else 3
    P1, P2 = _points(coordV0T, baryE0T, numP)
    if numP == 3:
        V0T = np.arange(1, 3 * K + 1)
        numT = K
    else:
        b = np.arange(0, 6 * K, 6)
        V0T = np.stack([b + 1, b + 4, b + 6, b + 2, b + 5, b + 4, b + 3, b + 6, b + 5,
                        b + 4, b + 5, b + 6], axis=1).reshape(-1)
        numT = 4 * K
    five12 = ['%.12e'] * 5
    five9 = ['%.9e'] * 5
    seps = [' ', ' ', ' ', ' ', '\n']
    s = ['TITLE="FESTUNG output file"\n', 'VARIABLES=X, Y, "%s"\n' % varName,
         'ZONE T="Time=%.3e", ' % tLvl, 'N=%d, E=%d, ' % (P1.size, numT), 'ET=TRIANGLE, F=FEBLOCK, ',
         'SOLUTIONTIME=%.3e\n\n' % tLvl,
         _cycle(five12, P1, seps), '\n\n', _cycle(five12, P2, seps), '\n\n',
         _cycle(five9, _point_values(dataLagr), seps), '\n',
         _cycle(['%d'] * 3, V0T, [' ', ' ', '\n'])]
    return ''.join(s)
