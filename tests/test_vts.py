"""VTS output (CPU): the writers of opesci/vts.py against the reference's
writer loops (src/opesciIO.cpp:68-294,614-667) restated element by element
below, the C ABI writer ofd_write_field_vts_3d (host only, no GPU) against
the Python one byte for byte, and the generated program's output_vts step."""
import ctypes
import os

import numpy as np
import pytest

from opesci import vts


def _ref_points_3d(dims, spacing, margin):
    """opesciIO.cpp:620-633: x outer, z inner, float (i - margin) * h."""
    out = []
    for i in range(dims[0]):
        x = np.float32(i - margin) * np.float32(spacing[0])
        for j in range(dims[1]):
            y = np.float32(j - margin) * np.float32(spacing[1])
            for k in range(dims[2]):
                out.append((x, y, np.float32(k - margin) * np.float32(spacing[2])))
    return np.array(out, dtype=np.float32)


def _ref_points(dims, spacing):
    """opesciIO.cpp:76-87: z outer, x inner, float i * h."""
    out = []
    for k in range(dims[2]):
        z = np.float32(k) * np.float32(spacing[2])
        for j in range(dims[1]):
            y = np.float32(j) * np.float32(spacing[1])
            for i in range(dims[0]):
                out.append((np.float32(i) * np.float32(spacing[0]), y, z))
    return np.array(out, dtype=np.float32)


def test_field_vts_3d_python_and_c_abi_identical(tmp_path):
    from opesci import build, runtime
    build.build()
    lib = runtime.load_library()
    dims, spacing, margin = (7, 5, 6), (12.5, 0.1, 3.0), 2
    rng = np.random.default_rng(3)
    field = rng.standard_normal(int(np.prod(dims))).astype(np.float32)
    py = vts.dump_field_vts_3d(str(tmp_path / 'py'), dims, spacing, margin, field)
    d = (ctypes.c_int * 3)(*dims)
    sp = (ctypes.c_float * 3)(*spacing)
    fp = ctypes.POINTER(ctypes.c_float)
    assert lib.ofd_write_field_vts_3d(str(tmp_path / 'c').encode(), d, sp, margin, field.ctypes.data_as(fp)) == 0
    assert open(py, 'rb').read() == open(str(tmp_path / 'c.vts'), 'rb').read()
    got = vts.read_vts(py)
    assert got['extent'] == dims
    assert np.array_equal(got['arrays']['field'], field)
    assert np.array_equal(got['points'], _ref_points_3d(dims, spacing, margin))
    assert lib.ofd_write_field_vts_3d(str(tmp_path / 'no' / 'dir').encode(), d, sp, margin,
                                      field.ctypes.data_as(fp)) == -1
    assert 'cannot open' in lib.ofd_last_error().decode()


def test_solution_vts_matches_reference_loops(tmp_path):
    dims, spacing = (6, 6, 4), (10.0, 10.0, 2.5)
    n = int(np.prod(dims))
    rng = np.random.default_rng(4)
    u, v, w, txx, tyy, tzz = (rng.standard_normal(n).astype(np.float32) for _ in range(6))
    got = vts.read_vts(vts.dump_solution_vts(str(tmp_path / 'sol'), dims, spacing, u, v, w, txx, tyy, tzz))
    assert np.array_equal(got['points'], _ref_points(dims, spacing))
    vel, pr = got['arrays']['velocity'], got['arrays']['pressure']
    # opesciIO.cpp:95-103 and :113-121, index = k*d0*d1 + j*d1 + i (d0 == d1 here)
    for k in range(dims[2]):
        for j in range(dims[1]):
            for i in range(dims[0]):
                idx = k * dims[0] * dims[1] + j * dims[1] + i
                assert tuple(vel[idx]) == (u[idx], v[idx], w[idx])
                assert pr[idx] == (txx[idx] + tyy[idx] + tzz[idx]) / np.float32(3)


def test_receivers_and_traces_vts(tmp_path):
    nt, nrec, h, dt = 11, 9, 10.0, 1e-3
    tr = np.random.default_rng(5).standard_normal((nt, 4, nrec)).astype(np.float32)
    got = vts.read_vts(vts.dump_traces_vts(str(tmp_path / 'receivers'), tr, h, dt))
    assert got['extent'] == (3, 3, nt)
    # array order of opesciIO.cpp:216-278
    assert list(got['arrays']) == ['vss', 'wss', 'pss', 'uss']
    for c, name in enumerate(('uss', 'vss', 'wss', 'pss')):
        # the driver pushes each step's receivers in turn (test_ref_iso_elastic.cpp:227-270)
        assert np.array_equal(got['arrays'][name], tr[:, c, :].reshape(-1)), name
    assert np.array_equal(got['points'], _ref_points((3, 3, nt), (h, h, dt)))
    with pytest.raises(ValueError):
        vts.dump_traces_vts(str(tmp_path / 'bad'), tr[:, :, :8], h, dt)


def test_program_output_vts_step():
    from opesci.models import eigenwave_grid
    g = eigenwave_grid(grid_size=(12, 12, 12), ntsteps=3)
    assert 'ofd_write_field_vts_3d' not in g.cgen_template.generate()
    g.output_vts = True
    src = g.cgen_template.generate()
    assert 'ofd_write_field_vts_3d(vtkfile.c_str(), vts_dims, vts_spacing, 2, vts_buf.data())' in src
    assert '"U_" + std::to_string(_ti)' in src
