"""Raw field files, checkpoints, source and receiver files, and the
reference's model helpers.

The reference writes a field as raw native-endian float32
(opesci_dump_field_raw, src/opesciIO.cpp:60-66: ``<name>.raw``) and reads
media and sources back the same way (opesci_read_simple_binary(_ptr),
opesciIO.cpp:296-342).  Source and receiver positions come from text files
of one header line and an x y z line per point (opesci_read_souces,
opesci_read_receivers, opesciIO.cpp:345-396); Lame constants and the time
step limit of a model follow opesci_calculate_lame_costants and
opesci_calculate_dt (src/opesciHandy.cpp:53-89).  A checkpoint of a device-resident simulation is
both time levels of the nine fields in that format, plus the step count, so
that a run resumed from it continues bit for bit (the next step reads the
newest level, and ghost cells that no update rewrites keep their values in
the older one).  Media, coefficients, source and receivers are not part of
a checkpoint: they are set on the new simulation as for the first run.
"""
import ctypes
import json
import math
import os
import re

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


# --------------------------------------------------- source / receiver files

_RUN = re.compile(r'[+-]?[0-9]*(?:\.[0-9]*)?(?:[eE][+-]?[0-9]*)?')
_WS = ' \t\n\v\f\r'
_libc = None


def _strtof_whole(run):
    """The float C's strtof makes of ``run``, or None unless it converts the
    whole run (the check std::num_get applies after collecting it)."""
    global _libc
    if not run:
        return None
    if _libc is None:
        _libc = ctypes.CDLL(None)
        _libc.strtof.restype = ctypes.c_float
        _libc.strtof.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p)]
    buf = ctypes.create_string_buffer(run.encode('ascii'))
    end = ctypes.c_char_p()
    v = _libc.strtof(buf, ctypes.byref(end))
    consumed = ctypes.cast(end, ctypes.c_void_p).value - ctypes.addressof(buf)
    return float(np.float32(v)) if consumed == len(run) else None


def three_floats(line):
    """``ss >> x >> y >> z`` on one line, as the reference's readers parse a
    point (std::stringstream in the C locale, values starting at 0): each
    extraction skips white space and collects the longest run of sign,
    digits, decimal point and exponent characters, which must convert
    whole; a failed extraction leaves 0 and every later one on the line
    fails too."""
    vals = [0.0, 0.0, 0.0]
    pos = 0
    for k in range(3):
        while pos < len(line) and line[pos] in _WS:
            pos += 1
        m = _RUN.match(line, pos)
        v = _strtof_whole(m.group() if m else '')
        if v is None:
            break
        vals[k] = v
        pos = m.end()
    return vals


def read_points(path):
    """Point coordinates of a source or receiver text file, shape (n, 3)
    float32 (opesci_read_receivers, src/opesciIO.cpp:374-396): the first
    line is a header; every later line that is not empty (std::getline:
    split at '\n' only, so a line of blanks or a lone '\r' still counts)
    gives one point.  A missing file raises OSError (the reference prints
    an error and returns -1)."""
    with open(path, 'rb') as fh:
        text = fh.read().decode('latin-1')
    pts = [three_floats(line) for line in text.split('\n')[1:] if line != '']
    return np.array(pts, dtype=np.float32).reshape(-1, 3)


def read_receivers(path):
    """opesci_read_receivers (src/opesciIO.cpp:374-396): (n, 3) float32."""
    return read_points(path)


def read_sources(xyz_path, xsrc_path, ysrc_path, zsrc_path):
    """opesci_read_souces (src/opesciIO.cpp:345-372): the source positions
    (n, 3) and the x, y and z source signals as raw float32 files."""
    return (read_points(xyz_path), read_simple_binary(xsrc_path), read_simple_binary(ysrc_path),
            read_simple_binary(zsrc_path))


# ------------------------------------------------------------ model helpers

def lame_constants(vp, vs, rho):
    """(mu, lambda) of a model, float32, as opesci_calculate_lame_costants
    (src/opesciHandy.cpp:53-67) computes them: mu = rho*vs*vs in float, and
    lambda = rho*(vp*vp - 2.0*vs*vs) with vp*vp in float and the rest in
    double (the literal 2.0), rounded to float once at the end."""
    vp = np.ascontiguousarray(vp, dtype=np.float32)
    vs = np.ascontiguousarray(vs, dtype=np.float32)
    rho = np.ascontiguousarray(rho, dtype=np.float32)
    if not (vp.shape == vs.shape == rho.shape):
        raise ValueError('vp, vs and rho must have the same shape')
    mu = (rho * vs) * vs
    vs64 = vs.astype(np.float64)
    lam = (rho.astype(np.float64) * ((vp * vp).astype(np.float64) - (2.0 * vs64) * vs64)).astype(np.float32)
    return mu, lam


def calculate_dt(vp, h):
    """opesci_calculate_dt (src/opesciHandy.cpp:69-89): (6/7)(1/sqrt 3)(h/maxv)
    with maxv the largest positive vp (0 when none), h/maxv in float, the
    product in double, returned as float."""
    vp = np.asarray(vp, dtype=np.float32).ravel()
    pos = vp[vp > 0]
    maxv = np.float32(pos.max()) if pos.size else np.float32(0.0)
    with np.errstate(divide='ignore'):
        q = np.float32(h) / maxv
    return np.float32((6.0 / 7.0) * (1.0 / math.sqrt(3.0)) * float(q))


def checkpoint(sim, directory):
    """Write both levels of the nine fields and the step count of ``sim``."""
    os.makedirs(directory, exist_ok=True)
    sim.sync()
    dtype = np.dtype(sim.host_dtype)
    for f in runtime.FIELDS:
        for lvl in (0, 1):
            # native values of the handle's host type (float64 for FP64 storage)
            np.ascontiguousarray(sim.download(f, lvl), dtype=dtype).tofile(
                os.path.join(directory, '%s_%d.raw' % (f, lvl)))
    with open(os.path.join(directory, 'state.json'), 'w') as fh:
        json.dump({'steps': sim.steps, 'dims': list(sim.dims), 'dtype': dtype.name}, fh)


def restore(sim, directory):
    """Load a checkpoint into ``sim`` (same dims, media and coefficients set
    as for the original run); stepping continues at the saved step."""
    with open(os.path.join(directory, 'state.json')) as fh:
        st = json.load(fh)
    if list(sim.dims) != st['dims']:
        raise ValueError('checkpoint of a %s grid, simulation is %s' % (st['dims'], list(sim.dims)))
    n = int(np.prod(sim.dims))
    dtype = np.dtype(st.get('dtype', 'float32'))
    for f in runtime.FIELDS:
        for lvl in (0, 1):
            a = np.fromfile(os.path.join(directory, '%s_%d.raw' % (f, lvl)), dtype=dtype)
            if len(a) < n:
                raise ValueError('checkpoint field %s_%d holds %d values, %d needed' % (f, lvl, len(a), n))
            sim.upload(f, lvl, a[:n])
    sim.steps = st['steps']
