"""SEG-Y earth models (format code 1, 4-byte IBM floating point).

read_model_segy restates the reference's opesci_read_model_segy
(src/opesciIO.cpp:419-612):

* the 3600-byte file header gives traces per record (Nx, bytes 3213-3214),
  samples per trace (Nz, 3221-3222) and the sample format (3225-3226).  The
  header is first read without byte swapping; if the format code is not
  1..8 it is read again swapped, and only format 1 is decoded;
* each trace is 240 header bytes plus 4*Nz sample bytes.  Ny is the trace
  count / Nx;
* trace i holds column ix = i % Nx, iy = i / Nx.  The output array is
  indexed ix + iy*Nx + iz*Nx*Ny, a C array [Nz][Ny][Nx];
* the horizontal spacing is the larger coordinate step between traces 0
  and 1 (bytes 73-80, scaled by bytes 71-72, a negative scale meaning
  1/|scale|).  The vertical spacing is bytes 117-118 times that scale.

IBM samples are decoded as the reference's real2float does (opesciIO.cpp:
400-417): +-mantissa / 2^24 * 16^(exponent - 64) in double, rounded to
float; the sign is applied to the integer mantissa, so a negative zero
decodes to +0.0.  Decoding runs on the GPU (ofd_segy_decode_ibm) unless
``device=False``.
"""
import ctypes

import numpy as np

_HDR = 3600
_TRH = 240


def _i16(buf, off, swap):
    return int(np.frombuffer(buf, dtype='>i2' if swap else '<i2', count=1, offset=off)[0])


def _i32(buf, off, swap):
    return int(np.frombuffer(buf, dtype='>i4' if swap else '<i4', count=1, offset=off)[0])


def parse_header(data):
    """(nx, ny, nz, swap, tracesize, spacing) of a SEG-Y image (bytes)."""
    if len(data) < _HDR:
        raise ValueError('SEG-Y file shorter than its 3600-byte header')
    swap = False
    for _ in range(2):
        nx = _i16(data, 3212, swap)
        nz = _i16(data, 3220, swap)
        fmt = _i16(data, 3224, swap)
        if fmt < 1 or fmt > 8:
            swap = True
            fmt = _i16(data, 3224, swap)
            if fmt < 1 or fmt > 8:
                raise ValueError('unsupported data sample format code %d' % fmt)
            continue
        break
    if fmt != 1:
        raise ValueError('format code %d not supported (4-byte IBM floating point only)' % fmt)
    if nx <= 0 or nz <= 0:
        raise ValueError('bad SEG-Y header: %d traces per record, %d samples per trace' % (nx, nz))
    tracesize = _TRH + 4 * nz
    ntraces = (len(data) - _HDR) // tracesize
    ny = ntraces // nx
    f32 = np.float32
    spacing = [0.0, 0.0, 0.0]
    if ntraces >= 2:
        t0, t1 = _HDR, _HDR + tracesize
        scale = f32(_i16(data, t0 + 70, swap))
        if scale < 0:
            scale = f32(1.0 / abs(float(scale)))
        x0 = [scale * f32(_i32(data, t0 + 72, swap)), scale * f32(_i32(data, t0 + 76, swap))]
        x1 = [scale * f32(_i32(data, t1 + 72, swap)), scale * f32(_i32(data, t1 + 76, swap))]
        dx = max(abs(f32(x0[0] - x1[0])), abs(f32(x0[1] - x1[1])))
        spacing = [float(dx), float(dx), float(scale * f32(_i16(data, t1 + 116, swap)))]
    return nx, ny, nz, swap, tracesize, spacing


def ibm_to_float(words):
    """Decode IBM floats given as uint32 words (host, numpy)."""
    w = np.asarray(words, dtype=np.uint32).astype(np.int64)
    sign = (w >> 31) & 1
    exp = ((w >> 24) & 0x7F) - 64
    mant = w & 0xFFFFFF
    sm = np.where(sign == 1, -mant, mant).astype(np.float64)
    with np.errstate(over='ignore'):
        return (sm / 16777216.0 * np.ldexp(1.0, 4 * exp)).astype(np.float32)


def _samples(data, nx, ny, nz, swap, tracesize):
    n = nx * ny
    raw = np.frombuffer(data, dtype=np.uint8, count=n * tracesize, offset=_HDR).reshape(n, tracesize)
    return np.ascontiguousarray(raw[:, _TRH:]).view('>u4' if swap else '<u4').reshape(n, nz)


def read_model_segy(path, device=True):
    """(model, dims, spacing): model is float32 of shape (Nz, Ny, Nx) (x
    fastest, as the reference's array), dims = [Nx, Ny, Nz]."""
    with open(path, 'rb') as f:
        data = f.read()
    nx, ny, nz, swap, tracesize, spacing = parse_header(data)
    if device:
        from . import runtime
        lib = runtime.load_library()
        out = np.empty((nz, ny, nx), dtype=np.float32)
        buf = np.frombuffer(data, dtype=np.uint8)
        rc = lib.ofd_segy_decode_ibm(buf.ctypes.data_as(ctypes.c_void_p), len(data), nx, ny, nz,
                                     1 if swap else 0, runtime._fptr(out))
        runtime._check(rc, 'ofd_segy_decode_ibm')
    else:
        words = _samples(data, nx, ny, nz, swap, tracesize)        # (traces, nz)
        vals = ibm_to_float(words.astype(np.uint32))
        out = np.ascontiguousarray(vals.reshape(ny, nx, nz).transpose(2, 0, 1))
    return out, [nx, ny, nz], spacing


def float_to_ibm(values):
    """Encode float32 values as IBM floats (uint32 words), mantissa rounded
    to nearest; zero stays zero."""
    v = np.asarray(values, dtype=np.float64).ravel()
    out = np.zeros(v.shape, dtype=np.uint32)
    nz = v != 0
    a = np.abs(v[nz])
    e = np.floor(np.log2(a) / 4).astype(np.int64) + 1          # a = m * 16^e, m in [1/16, 1)
    m = a / np.ldexp(1.0, 4 * e)
    lo = m < 1.0 / 16
    e[lo] -= 1
    m[lo] *= 16
    hi = m >= 1.0
    e[hi] += 1
    m[hi] /= 16
    mi = np.rint(m * 16777216.0).astype(np.int64)
    over = mi >= 16777216
    mi[over] //= 16
    e[over] += 1
    e = np.clip(e + 64, 0, 127)
    sign = (v[nz] < 0).astype(np.int64)
    out[nz] = ((sign << 31) | (e << 24) | mi).astype(np.uint32)
    return out


def write_model_segy(path, model, dx, dz, scale=-100, big_endian=True):
    """Write a (Nz, Ny, Nx) model as a format-1 SEG-Y file laid out as the
    reference reader expects (coordinates of trace i = (ix*dx, iy*dx) in
    bytes 73-80 with scale ``scale``, dz in bytes 117-118)."""
    model = np.asarray(model, dtype=np.float32)
    nz, ny, nx = model.shape
    e = '>' if big_endian else '<'
    hdr = bytearray(_HDR)
    hdr[3212:3214] = np.array(nx, dtype=e + 'i2').tobytes()
    hdr[3220:3222] = np.array(nz, dtype=e + 'i2').tobytes()
    hdr[3224:3226] = np.array(1, dtype=e + 'i2').tobytes()
    mul = 1.0 / abs(scale) if scale < 0 else float(scale)
    traces = []
    for iy in range(ny):
        for ix in range(nx):
            th = bytearray(_TRH)
            th[70:72] = np.array(scale, dtype=e + 'i2').tobytes()
            th[72:76] = np.array(int(round(ix * dx / mul)), dtype=e + 'i4').tobytes()
            th[76:80] = np.array(int(round(iy * dx / mul)), dtype=e + 'i4').tobytes()
            th[114:116] = np.array(nz, dtype=e + 'i2').tobytes()
            th[116:118] = np.array(int(round(dz / mul)), dtype=e + 'i2').tobytes()
            words = float_to_ibm(model[:, iy, ix])
            traces.append(bytes(th) + words.astype(e + 'u4').tobytes())
    with open(path, 'wb') as f:
        f.write(bytes(hdr) + b''.join(traces))


def model_to_grid(model, margin):
    """A (Nz, Ny, Nx) model as an array of this package's grid layout
    [x][y][z] (z fastest) with ``margin`` points on every side filled with
    the nearest model value."""
    m = np.asarray(model, dtype=np.float32).transpose(2, 1, 0)
    return np.pad(m, margin, mode='edge')
