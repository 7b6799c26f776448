"""VTK XML structured-grid (.vts) output of fields and seismograms.

Restates the reference's VTS writers (src/opesciIO.cpp):

  opesci_dump_solution_vts   :68-141   velocity (3 components) and pressure
  opesci_dump_field_vts      :143-194  one array "field"
  opesci_dump_receivers_vts  :196-294  seismograms vss, wss, pss, uss
  opesci_dump_field_vts_3d   :614-667  one field with margins, the generated
                                       code's output_vts step

The reference writes through VTK's vtkXMLStructuredGridWriter with a zlib
compressor.  VTK is not a dependency here: the files are written directly in
the same XML format with the data appended raw (uncompressed; a UInt64 byte
count before each array, little-endian Float32).  Points are inserted in
the reference's loop order with coordinates rounded to float as its
``int * float`` products are.

The reference indexes the solution and receiver arrays as
``k*dims[0]*dims[1] + j*dims[1] + i``, which is the memory order only when
dims[0] == dims[1] (always so for receivers, whose first two dimensions are
both round(sqrt(nrec))); for other solution shapes it leaves tuples
unwritten and reads past the arrays.  These writers keep the memory order,
which equals the reference's output whenever its index is valid.

``ofd_write_field_vts_3d`` in the device runtime's C ABI writes the same
bytes as dump_field_vts_3d for the generated CUDA program.
"""
import struct
import xml.etree.ElementTree as ET

import numpy as np

_HEAD = ('<?xml version="1.0"?>\n'
         '<VTKFile type="StructuredGrid" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n'
         '  <StructuredGrid WholeExtent="0 {ex} 0 {ey} 0 {ez}">\n'
         '    <Piece Extent="0 {ex} 0 {ey} 0 {ez}">\n'
         '      <PointData>\n'
         '{arrays}'
         '      </PointData>\n'
         '      <Points>\n'
         '        <DataArray type="Float32" Name="Points" NumberOfComponents="3" format="appended" offset="{poff}"/>\n'
         '      </Points>\n'
         '    </Piece>\n'
         '  </StructuredGrid>\n'
         '  <AppendedData encoding="raw">\n'
         '_')
_TAIL = b'\n  </AppendedData>\n</VTKFile>\n'
_ARRAY = ('        <DataArray type="Float32" Name="{name}" NumberOfComponents="{nc}" format="appended" '
          'offset="{off}"/>\n')


def _write(path, dims, points, arrays):
    """``arrays``: [(name, components, float32 values in tuple order)]."""
    dims = [int(d) for d in dims]
    n = dims[0] * dims[1] * dims[2]
    blocks, lines, off = [], [], 0
    for name, nc, vals in arrays:
        vals = np.ascontiguousarray(vals, dtype='<f4').reshape(-1)
        if vals.size != n * nc:
            raise ValueError('array %s holds %d values, the grid needs %d' % (name, vals.size, n * nc))
        lines.append(_ARRAY.format(name=name, nc=nc, off=off))
        blocks.append(vals)
        off += 8 + vals.nbytes
    pts = np.ascontiguousarray(points, dtype='<f4').reshape(-1)
    head = _HEAD.format(ex=dims[0] - 1, ey=dims[1] - 1, ez=dims[2] - 1, arrays=''.join(lines), poff=off)
    with open(path, 'wb') as fh:
        fh.write(head.encode('ascii'))
        for b in blocks + [pts]:
            fh.write(struct.pack('<Q', b.nbytes))
            fh.write(b.tobytes())
        fh.write(_TAIL)
    return path


def _points_x_fastest(dims, spacing):
    """(x, y, z) = (i, j, k) * spacing with i fastest (opesciIO.cpp:76-87)."""
    sx, sy, sz = (np.float32(s) for s in spacing)
    k, j, i = np.meshgrid(np.arange(dims[2]), np.arange(dims[1]), np.arange(dims[0]), indexing='ij')
    return np.stack([i.astype(np.float32) * sx, j.astype(np.float32) * sy, k.astype(np.float32) * sz], axis=-1)


def dump_field_vts_3d(name, dims, spacing, margin, field):
    """name.vts of a field laid out [dims[0]][dims[1]][dims[2]] (margins
    included): points ((i - margin) h_x, (j - margin) h_y, (k - margin) h_z)
    inserted x outer, z inner, and the values in memory order
    (opesciIO.cpp:614-667)."""
    sx, sy, sz = (np.float32(s) for s in spacing)
    i, j, k = np.meshgrid(np.arange(dims[0]) - margin, np.arange(dims[1]) - margin, np.arange(dims[2]) - margin,
                          indexing='ij')
    pts = np.stack([i.astype(np.float32) * sx, j.astype(np.float32) * sy, k.astype(np.float32) * sz], axis=-1)
    return _write(name + '.vts', dims, pts, [('field', 1, np.asarray(field, dtype=np.float32))])


def dump_field_vts(name, dims, spacing, field):
    """name.vts of a field with x fastest, one array "field"
    (opesciIO.cpp:143-194)."""
    return _write(name + '.vts', dims, _points_x_fastest(dims, spacing),
                  [('field', 1, np.asarray(field, dtype=np.float32))])


def dump_solution_vts(name, dims, spacing, u, v, w, txx, tyy, tzz):
    """name.vts with point arrays "velocity" (u, v, w) and "pressure"
    (txx + tyy + tzz)/3 in float (opesciIO.cpp:68-141)."""
    f = [np.asarray(a, dtype=np.float32).reshape(-1) for a in (u, v, w, txx, tyy, tzz)]
    vel = np.stack(f[:3], axis=-1)
    pressure = ((f[3] + f[4]) + f[5]) / np.float32(3)
    return _write(name + '.vts', dims, _points_x_fastest(dims, spacing),
                  [('velocity', 3, vel), ('pressure', 1, pressure)])


def dump_receivers_vts(name, dims, spacing, uss, vss, wss, pss):
    """name.vts of seismograms on a (receiver i, receiver j, time) grid,
    arrays in the reference's order vss, wss, pss, uss
    (opesciIO.cpp:196-294)."""
    n = int(dims[0]) * int(dims[1]) * int(dims[2])
    arrs = [('vss', vss), ('wss', wss), ('pss', pss), ('uss', uss)]
    out = []
    for nm, a in arrs:
        a = np.asarray(a, dtype=np.float32).reshape(-1)
        if a.size < n:
            raise ValueError('%s holds %d values, the grid needs %d' % (nm, a.size, n))
        out.append((nm, 1, a[:n]))
    return _write(name + '.vts', dims, _points_x_fastest(dims, spacing), out)


def dump_traces_vts(name, traces, h, dt):
    """Seismograms recorded by ``Simulation.traces()`` ((nt, 4, nrec): U, V,
    W, P) written as the reference driver writes its receivers
    (tests/src/test_ref_iso_elastic.cpp:300-304): dims (round(sqrt(nrec)),
    round(sqrt(nrec)), nt), spacing (h, h, dt)."""
    tr = np.asarray(traces, dtype=np.float32)
    nt, _, nrec = tr.shape
    d = int(np.floor(np.sqrt(nrec) + 0.5))
    if d * d > nrec:
        raise ValueError('%d receivers do not fill a %d x %d grid' % (nrec, d, d))
    chan = [np.ascontiguousarray(tr[:, c, :]).reshape(-1) for c in range(4)]
    return dump_receivers_vts(name, (d, d, nt), (h, h, dt), chan[0], chan[1], chan[2], chan[3])


def read_vts(path):
    """Parse a .vts file with raw appended data (as these writers produce):
    {'extent': (nx, ny, nz), 'points': (n, 3) float32, 'arrays': {name:
    (n,) or (n, components) float32}}."""
    raw = open(path, 'rb').read()
    start = raw.index(b'<AppendedData')
    mark = raw.index(b'_', raw.index(b'>', start)) + 1
    root = ET.fromstring(raw[:start] + b'</VTKFile>')
    if root.get('header_type') != 'UInt64' or root.get('byte_order') != 'LittleEndian':
        raise ValueError('only little-endian files with UInt64 headers are read')
    piece = root.find('StructuredGrid/Piece')
    ext = [int(v) for v in piece.get('Extent').split()]
    dims = (ext[1] - ext[0] + 1, ext[3] - ext[2] + 1, ext[5] - ext[4] + 1)

    def block(el):
        if el.get('format') != 'appended' or el.get('type') != 'Float32':
            raise ValueError('only appended Float32 arrays are read')
        off = mark + int(el.get('offset'))
        nbytes = struct.unpack('<Q', raw[off:off + 8])[0]
        a = np.frombuffer(raw[off + 8:off + 8 + nbytes], dtype='<f4').astype(np.float32)
        nc = int(el.get('NumberOfComponents', '1'))
        return a.reshape(-1, nc) if nc > 1 else a

    arrays = {el.get('Name'): block(el) for el in piece.findall('PointData/DataArray')}
    points = block(piece.find('Points/DataArray'))
    return {'extent': dims, 'points': points, 'arrays': arrays}
