"""Source and receiver time series on the host: trace resampling and
receiver positions.

The reference resamples a source wavelet given at interval ``sdt`` to the
simulation's time step ``dt`` spectrally (src/opesciHandy.cpp:100-195): a
DFT, zeros inserted into (dt < sdt) or samples removed from (dt > sdt) the
middle of the spectrum, an inverse DFT, each transform normalised by
1/sqrt(n).  resample_timeseries restates it in FP32 as the reference
computes it: the angle 2 pi t k / n formed in double and rounded to float,
the cosine and sine of that float in double, each term added to a float
accumulator.  Receiver positions follow the reference driver
(tests/src/test_ref_iso_elastic.cpp:227-234): index = round(coordinate / h),
plus the margin of this package's arrays.
"""
import math

import numpy as np


def dft(inreal, inimag):
    """Forward DFT of opesciHandy.cpp:100-113 (no normalisation):
    out_k = sum_t in_t exp(-2 pi i t k / n), accumulated in float."""
    xr = np.asarray(inreal, dtype=np.float32)
    xi = np.asarray(inimag, dtype=np.float32)
    n = len(xr)
    k = np.arange(n, dtype=np.float64)
    sr = np.zeros(n, dtype=np.float32)
    si = np.zeros(n, dtype=np.float32)
    for t in range(n):
        ang = (2 * math.pi * t * k / n).astype(np.float32).astype(np.float64)
        c, s = np.cos(ang), np.sin(ang)
        r = float(xr[t])
        i = float(xi[t])
        sr = (sr.astype(np.float64) + (r * c + i * s)).astype(np.float32)
        si = (si.astype(np.float64) + (-r * s + i * c)).astype(np.float32)
    return sr, si


def resample_timeseries(src, dt, sdt):
    """Resample ``src`` (interval sdt) to interval dt without changing its
    frequency content (opesciHandy.cpp:125-195); returns float32."""
    src = np.asarray(src, dtype=np.float32)
    dt32 = float(np.float32(dt))
    if abs(dt32 - sdt) < np.finfo(np.float32).eps * (dt32 + sdt):
        return src.copy()
    snt = len(src)
    snt2 = int(round(snt * sdt / dt32))
    fr, fi = dft(src, np.zeros(snt, dtype=np.float32))
    nrm = np.float32(1.0 / math.sqrt(snt))
    fr = (fr * nrm).astype(np.float32)
    fi = (fi * nrm).astype(np.float32)
    fr2 = np.zeros(snt2, dtype=np.float32)
    fi2 = np.zeros(snt2, dtype=np.float32)
    if dt32 < sdt:
        mid = snt // 2
        fr2[:mid], fi2[:mid] = fr[:mid], fi[:mid]
        off = snt2 - snt
        fr2[off + mid:off + snt], fi2[off + mid:off + snt] = fr[mid:snt], fi[mid:snt]
    else:
        mid = snt2 // 2
        fr2[:mid], fi2[:mid] = fr[:mid], fi[:mid]
        off = snt - snt2
        fr2[mid:snt2], fi2[mid:snt2] = fr[off + mid:off + snt2], fi[off + mid:off + snt2]
    fi2 = -fi2
    out, _ = dft(fr2, fi2)
    nrm2 = np.float32(1.0 / math.sqrt(np.float32(snt2)))
    return (out * nrm2).astype(np.float32)


def point_indices(coords, h, margin=0):
    """Array indices of points at physical coordinates ``coords`` ((n, 3)
    float32 metres from the first interior point), as the reference driver
    forms them for receivers and the source
    (tests/src/test_ref_iso_elastic.cpp:230-232,277-279):
    ``(int)round(coor/h)`` with coor and h floats, so the quotient is rounded
    to float and then rounded half away from zero; plus ``margin``."""
    q = (np.asarray(coords, dtype=np.float32).reshape(-1, 3) / np.float32(h)).astype(np.float64)
    a = np.abs(q)
    r = np.floor(a)
    r = np.where(a - r >= 0.5, r + 1, r)        # a - r is exact: both are the same float
    return (np.copysign(r, q).astype(np.int64) + margin).astype(np.int32)


def receiver_indices(coords, h, margin):
    """Array indices (margins included) of receivers at physical coordinates
    ``coords`` ((n, 3), metres from the first interior point)."""
    return point_indices(coords, h, margin)
