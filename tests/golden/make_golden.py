"""Regenerate the golden fixtures of this directory from the reference.

Run where the reference checkout is present (argument --reference, the
OPESCI_REFERENCE environment variable, or the directory "reference" beside
this repository):

    python tests/golden/make_golden.py [--reference <dir>]

Writes
  test3d_l2.json          the nine L2 norms printed by the reference's own
                          generated program benchmarks/test3d.cpp (100^3 unit
                          cube, space order 4, dt=0.002, 1000 steps), built by
                          oracle/Makefile with the reference's GNU flags and
                          run on this machine;
  notebook_outputs.json   the text outputs of the known-answer cells of the
                          reference notebooks tests/eigenwave3d.ipynb and
                          tests/eigenwave3d-read.ipynb, verbatim.
  resample.json           inputs and outputs of the reference's own trace
                          resampling opesci_resample_timeseries
                          (src/opesciHandy.cpp:125-195), compiled from where
                          it lies by oracle/Makefile into
                          oracle/_ref/libopescihandy.so, on seeded series
                          (up- and downsampling, odd and even lengths);
  model_be.segy, model_le.segy, segy.json
                          small format-1 SEG-Y models (big- and little-endian,
                          with planted IBM words: negative zero, underflow,
                          overflow, extremes) and what the reference's own
                          opesci_read_model_segy (src/opesciIO.cpp:419-612),
                          compiled into the same library, reads from them.
Nothing at test time reads the reference; tests read only these files.

    python tests/golden/make_golden.py --only resample    # just resample.json
    python tests/golden/make_golden.py --only segy        # just the SEG-Y fixtures
"""
import argparse
import json
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def notebook_cells(path, cells):
    nb = json.load(open(path))
    out = {}
    for i in cells:
        c = nb['cells'][i]
        txt = ''
        for o in c.get('outputs', []):
            if 'text' in o:
                txt += ''.join(o['text'])
            if 'data' in o and 'text/plain' in o['data']:
                txt += ''.join(o['data']['text/plain'])
        out[str(i)] = {'source': ''.join(c.get('source', '')), 'output': txt}
    return out


def resample_fixtures():
    """Run the reference's opesci_resample_timeseries on seeded series."""
    import ctypes
    import numpy as np
    lib = ctypes.CDLL(os.path.join(ROOT, 'oracle', '_ref', 'libopescihandy.so'))
    fp = ctypes.POINTER(ctypes.c_float)
    lib.ref_resample_timeseries.argtypes = [fp, ctypes.c_int, ctypes.c_float, ctypes.c_double, fp, ctypes.c_int]
    rng = np.random.default_rng(20150101)
    cases = []
    for n, dt, sdt, kind in ((100, 1e-3, 2e-3, 'ricker'), (101, 2e-3, 1e-3, 'ricker'), (64, 0.7e-3, 1e-3, 'noise'),
                             (257, 1e-3, 0.9e-3, 'ricker'), (300, 4e-4, 1e-3, 'noise'), (50, 1e-3, 1e-3, 'noise')):
        t = np.arange(n) * sdt
        if kind == 'ricker':
            a = (np.pi * 20.0 * (t - 1.0 / 20.0)) ** 2
            src = ((1 - 2 * a) * np.exp(-a)).astype(np.float32)
        else:
            src = rng.standard_normal(n).astype(np.float32)
        out = np.zeros(4 * n + 16, dtype=np.float32)
        m = lib.ref_resample_timeseries(src.ctypes.data_as(fp), n, dt, sdt, out.ctypes.data_as(fp), len(out))
        cases.append({'dt': dt, 'sdt': sdt, 'src': [float(x) for x in src],
                      'resampled': [float(x) for x in out[:m]]})
    json.dump({'function': 'opesci_resample_timeseries (src/opesciHandy.cpp:125-195)', 'cases': cases},
              open(os.path.join(HERE, 'resample.json'), 'w'))


SEGY_RAW_WORDS = [0x80000000, 0x00000001, 0x7FFFFFFF, 0xFFFFFFFF, 0xC1100000, 0x41100000, 0x00FFFFFF,
                  0x21000001, 0x60FFFFFF, 0x3F7FFFFF]


def segy_fixtures():
    """Small format-1 SEG-Y models (big- and little-endian) read by the
    reference's opesci_read_model_segy; the files are kept as fixtures."""
    import ctypes
    import sys
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, 'opesci-fd_gb300'))
    from opesci import segy
    lib = ctypes.CDLL(os.path.join(ROOT, 'oracle', '_ref', 'libopescihandy.so'))
    fp = ctypes.POINTER(ctypes.c_float)
    lib.ref_read_model_segy.argtypes = [ctypes.c_char_p, fp, ctypes.c_long, ctypes.POINTER(ctypes.c_int), fp]
    rng = np.random.default_rng(1998)
    nz, ny, nx = 11, 5, 7
    model = (1500.0 + 3000.0 * rng.random((nz, ny, nx))).astype(np.float32)
    model[0, 0, :4] = [0.0, -2.5, 1e-30, 3.0e30]
    out = {}
    for name, big in (('model_be.segy', True), ('model_le.segy', False)):
        path = os.path.join(HERE, name)
        segy.write_model_segy(path, model, dx=12.5, dz=10.0, big_endian=big)
        # plant raw IBM words (negative zero, underflow, overflow, extremes)
        data = bytearray(open(path, 'rb').read())
        tracesize = 240 + 4 * nz
        for k, w in enumerate(SEGY_RAW_WORDS):
            tr, iz = 3 + k // nz, k % nz
            off = 3600 + tr * tracesize + 240 + 4 * iz
            data[off:off + 4] = w.to_bytes(4, 'big' if big else 'little')
        open(path, 'wb').write(bytes(data))
        buf = np.zeros(nx * ny * nz, dtype=np.float32)
        dims = (ctypes.c_int * 3)()
        sp = np.zeros(3, dtype=np.float32)
        m = lib.ref_read_model_segy(path.encode(), buf.ctypes.data_as(fp), len(buf), dims, sp.ctypes.data_as(fp))
        assert m == len(buf), m
        out[name] = {'dims': list(dims), 'spacing': [float(x) for x in sp],
                     'values_hex': [format(int(v), '08x') for v in buf.view(np.uint32)]}
    json.dump({'function': 'opesci_read_model_segy (src/opesciIO.cpp:419-612)', 'files': out},
              open(os.path.join(HERE, 'segy.json'), 'w'))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', default=os.environ.get('OPESCI_REFERENCE', os.path.join(os.path.dirname(ROOT), 'reference')),
                    help='reference checkout (default: $OPESCI_REFERENCE, else "reference" beside this repository)')
    ap.add_argument('--threads', type=int, default=os.cpu_count())
    ap.add_argument('--only', choices=['resample', 'segy'], default=None)
    args = ap.parse_args()

    subprocess.check_call(['make', '-C', os.path.join(ROOT, 'oracle'),
                           'REFERENCE=' + args.reference])
    if args.only in (None, 'resample'):
        resample_fixtures()
    if args.only in (None, 'segy'):
        segy_fixtures()
    if args.only is not None:
        return
    env = dict(os.environ, OMP_NUM_THREADS=str(args.threads))
    out = subprocess.check_output([os.path.join(ROOT, 'oracle', '_ref', 'test3d')],
                                  env=env, text=True)
    l2 = {}
    for line in out.splitlines():
        parts = line.split()
        if len(parts) == 2 and parts[0].endswith('_l2'):
            l2[parts[0][:-3]] = float(parts[1])
    json.dump({'program': 'benchmarks/test3d.cpp',
               'grid_size': [100, 100, 100], 'space_order': 4, 'dt': 0.002,
               'ntsteps': 1000, 'rho': 1.0, 'beta': 1.0, 'lambda': 0.5, 'mu': 0.5,
               'l2': l2}, open(os.path.join(HERE, 'test3d_l2.json'), 'w'), indent=1)

    nbs = {
        'eigenwave3d.ipynb': notebook_cells(
            os.path.join(args.reference, 'tests', 'eigenwave3d.ipynb'), [3, 11, 12, 14, 18, 19, 20]),
        'eigenwave3d-read.ipynb': notebook_cells(
            os.path.join(args.reference, 'tests', 'eigenwave3d-read.ipynb'), [14, 15, 24]),
        'eigenwave3d-higher_order.ipynb': notebook_cells(
            os.path.join(args.reference, 'tests', 'eigenwave3d-higher_order.ipynb'), [18]),
    }
    json.dump(nbs, open(os.path.join(HERE, 'notebook_outputs.json'), 'w'), indent=1)
    print('wrote', os.listdir(HERE))


if __name__ == '__main__':
    main()
