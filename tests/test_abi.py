"""The C ABI library: it loads and exports every entry point include/ofd.h
declares; host-side validation works without a GPU.  No compute calls."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    out = set()
    for name in os.listdir(os.path.join(ROOT, 'include')):
        if name.endswith('.h'):
            txt = open(os.path.join(ROOT, 'include', name)).read()
            out |= set(re.findall(r'\b(ofd_[a-z0-9_]+)\s*\(', txt))
    return out


@pytest.fixture(scope='module')
def lib():
    from opesci import build, runtime
    build.build()
    return runtime.load_library()


def test_library_exports_declared_symbols(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    path = os.path.join(ROOT, 'opesci-fd_gb300', 'lib', 'libofd.so')
    nm = subprocess.run(['nm', '-D', '--defined-only', path], capture_output=True, text=True).stdout
    exported = set(l.split()[-1] for l in nm.splitlines() if ' T ' in l)
    missing = syms - exported
    assert not missing, missing
    for s in syms:
        assert hasattr(lib, s)


def test_footprint_and_validation_without_gpu(lib):
    from opesci import runtime
    cfg = runtime.make_config([68, 68, 68], 4, [0.1] * 3, 1e-3, [9 / 8, -1 / 24])
    n = runtime.Simulation.footprint(cfg)
    # 9 fields x 2 levels + 8 media, padded rows of 128 floats
    assert n >= (9 * 2 + 8) * 68 * 68 * 68 * 4
    bad = runtime.make_config([68, 68, 68], 5, [0.1] * 3, 1e-3, [1.0])
    with pytest.raises(runtime.OFDError, match='space_order'):
        runtime.Simulation.footprint(bad)
    small = runtime.make_config([6, 68, 68], 4, [0.1] * 3, 1e-3, [1.0, 0.0])
    with pytest.raises(runtime.OFDError, match='too small'):
        runtime.Simulation.footprint(small)
    assert 'too small' in lib.ofd_last_error().decode()


def test_null_arguments_rejected_without_gpu(lib):
    """Entry points added for FP64 transfers, three-signal sources and VTS
    output report OFD_EINVAL for null handles and arrays before touching the
    device."""
    import numpy as np
    d = np.zeros(8)
    dp = d.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    assert lib.ofd_upload_field_f64(None, 0, 0, dp) == -1
    assert lib.ofd_download_field_f64(None, 0, 0, dp) == -1
    f = np.zeros(8, dtype=np.float32)
    fp = f.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    assert lib.ofd_set_source_xyz(None, 1, 1, 1, fp, fp, fp, 8) == -1
    assert 'null handle' in lib.ofd_last_error().decode()
    dims = (ctypes.c_int * 3)(2, 2, 2)
    sp = (ctypes.c_float * 3)(1.0, 1.0, 1.0)
    assert lib.ofd_write_field_vts_3d(b'x', dims, sp, 0, None) == -1
    bad = (ctypes.c_int * 3)(2, 0, 2)
    assert lib.ofd_write_field_vts_3d(b'x', bad, sp, 0, fp) == -1
    assert 'positive' in lib.ofd_last_error().decode()


def test_python_binding_covers_every_entry_point(lib):
    """opesci/runtime.py (the ctypes stub of the integration guide) gives
    every function of include/ofd.h an argument signature."""
    syms = declared_symbols()
    for name in syms:
        fn = getattr(lib, name)
        assert fn.argtypes is not None, name
