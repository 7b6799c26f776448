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
  receivers.txt, sources_xyz.txt, sources_{x,y,z}.raw, io.json
                          point files with edge-case lines (signs, exponents,
                          '.5' and '6.', an incomplete exponent, letters,
                          missing and extra values, lines of blanks, CRLF, no
                          final newline) and raw source signals, with what the
                          reference's opesci_read_receivers and
                          opesci_read_souces (src/opesciIO.cpp:345-396) read
                          from them; and the reference's
                          opesci_calculate_lame_costants and
                          opesci_calculate_dt (src/opesciHandy.cpp:53-89) on
                          seeded models with planted edge values, and the
                          driver's point index (int)round(coor/h) on
                          coordinates at and beside half-way ties.
Nothing at test time reads the reference; tests read only these files.

    python tests/golden/make_golden.py --only resample    # just resample.json
    python tests/golden/make_golden.py --only segy        # just the SEG-Y fixtures
    python tests/golden/make_golden.py --only io          # just the point files and model helpers
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


RECEIVERS_TXT = (
    'x y z receivers\n'
    '100.5 200.25 -3e2\n'
    '  1.5\t2.5   3.5  \n'
    '+4 .5 6.\n'
    '7 8\n'
    '9 abc 10\n'
    '11 12 13 14\n'
    '\n'
    '   \n'
    '1e-3 2E+2 -0.0\n'
    '12e 5 6\n'
    '1.5.3 x\n'
    '3.4028235e38 1e-45 0.1\r\n'
    '\r\n'
    '-.25 +.75e1 8')
SOURCES_TXT = 'sources\n10 20 30\n40.5 50.25 60.125\n'


def io_fixtures():
    import ctypes
    import numpy as np
    lib = ctypes.CDLL(os.path.join(ROOT, 'oracle', '_ref', 'libopescihandy.so'))
    fp = ctypes.POINTER(ctypes.c_float)
    hexs = lambda a: [format(int(v), '08x') for v in np.asarray(a, dtype=np.float32).view(np.uint32)]  # noqa: E731
    out = {}
    rec = os.path.join(HERE, 'receivers.txt')
    with open(rec, 'w', newline='') as fh:
        fh.write(RECEIVERS_TXT)
    buf = np.zeros(300, dtype=np.float32)
    m = lib.ref_read_receivers(rec.encode(), buf.ctypes.data_as(fp), len(buf))
    assert 0 < m < len(buf), m
    out['receivers'] = {'file': 'receivers.txt', 'values_hex': hexs(buf[:m])}
    xyz = os.path.join(HERE, 'sources_xyz.txt')
    with open(xyz, 'w', newline='') as fh:
        fh.write(SOURCES_TXT)
    rng = np.random.default_rng(11)
    paths = []
    for k, c in enumerate('xyz'):
        pth = os.path.join(HERE, 'sources_%s.raw' % c)
        rng.standard_normal(17 + k).astype(np.float32).tofile(pth)
        paths.append(pth)
    pxyz = np.zeros(64, dtype=np.float32)
    sig = np.zeros(256, dtype=np.float32)
    counts = (ctypes.c_int * 4)()
    assert lib.ref_read_sources(xyz.encode(), *[q.encode() for q in paths], pxyz.ctypes.data_as(fp), len(pxyz),
                                sig.ctypes.data_as(fp), len(sig), counts) == 0
    out['sources'] = {'xyz': 'sources_xyz.txt', 'signals': ['sources_x.raw', 'sources_y.raw', 'sources_z.raw'],
                      'counts': list(counts), 'xyz_hex': hexs(pxyz[:counts[0]]),
                      'signals_hex': hexs(sig[:counts[1] + counts[2] + counts[3]])}
    n = 512
    vp = (1500.0 + 3000.0 * rng.random(n)).astype(np.float32)
    vs = (vp / np.float32(1.7) * rng.random(n).astype(np.float32)).astype(np.float32)
    rho = (1000.0 + 2000.0 * rng.random(n)).astype(np.float32)
    vp[:6] = [0.0, 1e-30, 3.0e19, 1.0, 7.0, -2.0]
    vs[:6] = [0.0, 1e-30, 2.0e19, 0.5, 7.0, 1.0]
    rho[:6] = [1.0, 1e30, 1.0, 0.0, 1.0, 3.0]
    mu = np.zeros(n, dtype=np.float32)
    lam = np.zeros(n, dtype=np.float32)
    lib.ref_lame_constants(vp.ctypes.data_as(fp), vs.ctypes.data_as(fp), rho.ctypes.data_as(fp), ctypes.c_long(n),
                           mu.ctypes.data_as(fp), lam.ctypes.data_as(fp))
    out['lame'] = {'vp_hex': hexs(vp), 'vs_hex': hexs(vs), 'rho_hex': hexs(rho), 'mu_hex': hexs(mu),
                   'lam_hex': hexs(lam)}
    lib.ref_calculate_dt.restype = ctypes.c_float
    dts = []
    for h, arr in ((10.0, vp), (12.5, vp[6:]), (1.0, np.array([-1.0, 0.0], dtype=np.float32)),
                   (0.1, np.array([np.nan, 2.0, 3.5], dtype=np.float32))):
        arr = np.ascontiguousarray(arr, dtype=np.float32)
        v = lib.ref_calculate_dt(arr.ctypes.data_as(fp), ctypes.c_long(len(arr)), ctypes.c_float(h))
        dts.append({'h': h, 'vp_hex': hexs(arr), 'dt_hex': hexs([v])[0]})
    out['dt'] = dts
    lib.ref_point_indices.restype = None
    idx = []
    for h in (10.0, 12.5, 7.3, 0.1, 3.0):
        h32 = np.float32(h)
        k = np.arange(-3, 40, dtype=np.float32)
        ties = ((k + np.float32(0.5)) * h32).astype(np.float32)
        near = np.concatenate([np.nextafter(ties, np.float32(-np.inf)), ties, np.nextafter(ties, np.float32(np.inf))])
        coor = np.concatenate([near, (k * h32).astype(np.float32), rng.uniform(-50, 500, 64).astype(np.float32),
                               np.array([0.0, -0.0, 1e-30, 2.0e6], dtype=np.float32)]).astype(np.float32)
        res = np.zeros(len(coor), dtype=np.int32)
        lib.ref_point_indices(coor.ctypes.data_as(fp), ctypes.c_long(len(coor)), ctypes.c_float(h),
                              res.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
        idx.append({'h': h, 'coor_hex': hexs(coor), 'index': res.tolist()})
    out['indices'] = idx
    json.dump({'functions': 'opesci_read_receivers, opesci_read_souces (src/opesciIO.cpp:345-396); '
                            'opesci_calculate_lame_costants, opesci_calculate_dt (src/opesciHandy.cpp:53-89); '
                            'the driver\'s (int)round(coor/h) (tests/src/test_ref_iso_elastic.cpp:230-232)',
               'cases': out}, open(os.path.join(HERE, 'io.json'), 'w'))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', default=os.environ.get('OPESCI_REFERENCE', os.path.join(os.path.dirname(ROOT), 'reference')),
                    help='reference checkout (default: $OPESCI_REFERENCE, else "reference" beside this repository)')
    ap.add_argument('--threads', type=int, default=os.cpu_count())
    ap.add_argument('--only', choices=['resample', 'segy', 'io'], default=None)
    args = ap.parse_args()

    subprocess.check_call(['make', '-C', os.path.join(ROOT, 'oracle'),
                           'REFERENCE=' + args.reference])
    if args.only in (None, 'resample'):
        resample_fixtures()
    if args.only in (None, 'segy'):
        segy_fixtures()
    if args.only in (None, 'io'):
        io_fixtures()
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
