"""Raw field files and checkpoints.

The reference writes a field as raw native-endian float32
(opesci_dump_field_raw, src/opesciIO.cpp:60-66: ``<name>.raw``) and reads
media and sources back the same way (opesci_read_simple_binary(_ptr),
opesciIO.cpp:296-342).  A checkpoint of a device-resident simulation is
both time levels of the nine fields in that format, plus the step count, so
that a run resumed from it continues bit for bit (the next step reads the
newest level, and ghost cells that no update rewrites keep their values in
the older one).  Media, coefficients, source and receivers are not part of
a checkpoint: they are set on the new simulation as for the first run.
"""
import json
import os

import numpy as np

from . import runtime


def dump_field_raw(name, field):
    """Write ``field`` to ``name + '.raw'`` as native float32."""
    np.ascontiguousarray(field, dtype=np.float32).tofile(name + '.raw')


def read_simple_binary(path):
    """Every float32 of a raw file."""
    return np.fromfile(path, dtype=np.float32)


def read_simple_binary_ptr(path, size):
    """The first ``size`` float32 of a raw file.  The reference reports a
    file longer than ``size`` and reads its first ``size`` values; a shorter
    file is an error here."""
    a = np.fromfile(path, dtype=np.float32)
    if len(a) < size:
        raise ValueError('%s holds %d floats, %d needed' % (path, len(a), size))
    return a[:size]


def checkpoint(sim, directory):
    """Write both levels of the nine fields and the step count of ``sim``."""
    os.makedirs(directory, exist_ok=True)
    sim.sync()
    for f in runtime.FIELDS:
        for lvl in (0, 1):
            dump_field_raw(os.path.join(directory, '%s_%d' % (f, lvl)), sim.download(f, lvl))
    with open(os.path.join(directory, 'state.json'), 'w') as fh:
        json.dump({'steps': sim.steps, 'dims': list(sim.dims)}, fh)


def restore(sim, directory):
    """Load a checkpoint into ``sim`` (same dims, media and coefficients set
    as for the original run); stepping continues at the saved step."""
    with open(os.path.join(directory, 'state.json')) as fh:
        st = json.load(fh)
    if list(sim.dims) != st['dims']:
        raise ValueError('checkpoint of a %s grid, simulation is %s' % (st['dims'], list(sim.dims)))
    n = int(np.prod(sim.dims))
    for f in runtime.FIELDS:
        for lvl in (0, 1):
            sim.upload(f, lvl, read_simple_binary_ptr(os.path.join(directory, '%s_%d.raw' % (f, lvl)), n))
    sim.steps = st['steps']
