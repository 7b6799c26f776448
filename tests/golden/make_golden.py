"""Regenerate the golden fixtures of this directory from the reference.

Run in a container that has the reference checkout (default /root/reference):

    python tests/golden/make_golden.py [--reference /root/reference]

Writes
  test3d_l2.json          the nine L2 norms printed by the reference's own
                          generated program benchmarks/test3d.cpp (100^3 unit
                          cube, space order 4, dt=0.002, 1000 steps), built by
                          oracle/Makefile with the reference's GNU flags and
                          run on this machine;
  notebook_outputs.json   the text outputs of the known-answer cells of the
                          reference notebooks tests/eigenwave3d.ipynb and
                          tests/eigenwave3d-read.ipynb, verbatim.
Nothing at test time reads the reference; tests read only these files.
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', default='/root/reference')
    ap.add_argument('--threads', type=int, default=os.cpu_count())
    args = ap.parse_args()

    subprocess.check_call(['make', '-C', os.path.join(ROOT, 'oracle'),
                           'REFERENCE=' + args.reference])
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
