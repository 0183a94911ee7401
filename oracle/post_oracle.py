"""ORACLE / TEST INFRASTRUCTURE ONLY -- the checker, never the product.

numpy restatements of what the reference does around its time step, for
the parity tests of the library's GPU forms (ard_record_neighbourhoods,
ard_render_slice, ard_impulse_response).  Only tests/ import this module.

  neighbourhood  Recorder::RecordField's out_ stream
                 (ARD-simulator-190113/recorder.cpp:40-57)
  slice_colour,  the visualization block of Simulation::Update
  render_slice   (ARD-simulator-190113/simulation.cpp:320-420)
  fir1, rir      matlab/auralization.m:22-32 and matlab/normalizeIR.m, with
                 MATLAB's fir1 (window method, Hamming window, unit DC gain),
                 xcorr and fftfilt restated from their published definitions
  t60            matlab/t60.m (Schroeder integration, line fit), line by line
"""
from __future__ import annotations

import numpy as np


def mround(v):
    """MATLAB round: halves away from zero."""
    v = np.asarray(v, np.float64)
    return np.sign(v) * np.floor(np.abs(v) + 0.5)


def neighbourhood(field, x, y, z):
    """The 1000 values one line of out_<id>.txt holds, in the reference's loop
    order (recorder.cpp:44-52: i over z offsets, j over y, k over x, each
    -5 .. 4); `field` is [z][y][x] of the recorder's partition, (x, y, z) the
    recorder's local cell."""
    out = []
    for i in range(-5, 5):
        for j in range(-5, 5):
            for k in range(-5, 5):
                out.append(field[z + i, y + j, x + k])
    return np.asarray(out)


def slice_colour(p, v_coef=10.0):
    """simulation.cpp:349-367 in float32, every operation rounded on its own,
    as the RGBA8888 word of SDL_MapRGBA(fmt, 255, r, g, b) (R = 255, G = r,
    B = g, A = b).  `p` float32 array; returns uint32 words."""
    f = np.float32
    p = np.asarray(p, np.float32)
    pv = (p * f(v_coef)).astype(np.float32)
    cl = np.maximum(f(-1.0), np.minimum(f(1.0), pv))          # std::max(-1, std::min(1, .))
    cl = np.where(np.isnan(pv), f(1.0), cl)                    # std::min(1.0f, NaN) returns 1.0f
    norm = (f(0.5) * cl + f(0.5)).astype(np.float32)
    hi = norm >= f(0.5)
    v_hi = (f(510.0) * (norm - f(0.5))).astype(np.float32)
    v_lo = (f(255.0) * (f(1.0) - f(2.0) * norm)).astype(np.float32)
    rnd = mround                                               # std::round: halves away from zero
    r = np.where(hi, 255 - rnd(v_hi), 255).astype(np.int64)
    g = np.where(hi, 255 - rnd(v_hi), 255 - rnd(v_lo)).astype(np.int64)
    b = np.where(hi, 255, 255 - rnd(v_lo)).astype(np.int64)
    return (np.uint32(0xFF000000) | (r << 16).astype(np.uint32) | (g << 8).astype(np.uint32)
            | b.astype(np.uint32)).astype(np.uint32)


def _value(field, x, y, z):
    d, h, w = field.shape
    if 0 <= x < w and 0 <= y < h and 0 <= z < d:
        return field[z, y, x]
    return 0.0


def render_slice(partitions, fields, look_from, coord, v_coef=10.0, image=None):
    """simulation.cpp:326-417 with render_pml = false and every partition's
    should_render_ true (dct_partition.cpp:12, pml_partition.cpp:21).
    partitions: [(kind, pml_type, x, y, z, w, h, d)] in list order; fields:
    per partition its pressure [z][y][x].  coord is passed to each partition
    as a local coordinate (get_xy_plane / get_yz_plane receive the global
    pixels_z / pixels_x); outside a partition the value is 0.  Returns
    (pixels uint32, pressure float32) over the scene's bounding box."""
    lo = [min(p[2 + a] for p in partitions) for a in range(3)]
    hi = [max(p[2 + a] + p[5 + a] for p in partitions) for a in range(3)]
    W = hi[0] - lo[0] if look_from == 0 else hi[1] - lo[1]
    H = hi[1] - lo[1] if look_from == 0 else hi[2] - lo[2]
    pix = np.zeros((H, W), np.uint32) if image is None else image.copy()
    pres = np.zeros((H, W), np.float32)
    for q, fld in zip(partitions, fields):
        x0, y0, z0, w, h, d = q[2:8]
        if look_from == 0:
            if z0 > coord or z0 + d < coord:
                continue
            for i in range(h):
                for j in range(w):
                    v = np.float32(_value(fld, j, i, coord))
                    pres[y0 - lo[1] + i, x0 - lo[0] + j] = v
                    pix[y0 - lo[1] + i, x0 - lo[0] + j] = slice_colour(np.array([v]), v_coef)[0]
        else:
            if x0 > coord or x0 + w < coord:
                continue
            for i in range(d):
                for j in range(h):
                    v = np.float32(_value(fld, coord, j, i))
                    pres[z0 - lo[2] + i, y0 - lo[1] + j] = v
                    pix[z0 - lo[2] + i, y0 - lo[1] + j] = slice_colour(np.array([v]), v_coef)[0]
    return pix, pres


def fir1(order, wn):
    """MATLAB fir1(order, wn) for a low-pass: the ideal response
    wn sinc(wn (k - order/2)), k = 0 .. order, times the Hamming window
    0.54 - 0.46 cos(2 pi k / order), scaled to unit gain at DC."""
    k = np.arange(order + 1, dtype=np.float64)
    m = k - 0.5 * order
    h = wn * np.sinc(wn * m)
    w = 0.54 - 0.46 * np.cos(2.0 * np.pi * k / order)
    b = h * w
    return b / b.sum()


def xcorr_first_half(x, y):
    """xcorr(x, y) for equal lengths n, lags -(n-1) .. 0 (the first half that
    auralization.m:30 keeps): c[m] = sum_n x[n + m] y[n]."""
    n = len(x)
    full = np.correlate(np.asarray(x, np.float64), np.asarray(y, np.float64), mode="full")   # lags -(n-1) .. n-1
    return full[:n]


def fftfilt(b, x):
    """fftfilt(b, x): the FIR filter b applied to x, output length len(x)."""
    return np.convolve(x, b)[: len(x)]


def rir(rr, src, truncate=0, fcut=3000.0, sr=16000.0, order=1024):
    """auralization.m:22-32: the response zeroed after `truncate` samples,
    cross-correlated with the reversed source, its first half low-passed
    and normalized (normalizeIR.m)."""
    rr = np.array(rr, np.float64)
    if truncate > 0:
        rr[truncate:] = 0
    x = xcorr_first_half(rr, np.asarray(src, np.float64)[::-1])
    y = fftfilt(fir1(order, fcut / (sr / 2)), x)
    return y / np.abs(y).max()


def t60(impulse, sr):
    """matlab/t60.m, line by line (1-based indices translated).  Returns
    (rt in ms, slope, stop, overrun) where overrun is True where t60.m would
    index past its window (stop is then clamped to it)."""
    imp = np.asarray(impulse, np.float64).ravel()
    n = len(imp)
    begin = int(mround(sr * 0.05))
    T = n if n / sr < 1.5 else int(mround(sr * 1.5))
    iidc = np.cumsum(imp[::-1] ** 2)[::-1]
    y = iidc[:T]
    y = 10 * np.log10(y / np.abs(y).max())
    xtime = np.linspace(1, T / (sr / 1000), T)
    ss = np.arange(1, T + 1, dtype=np.float64)
    exy2 = (np.cumsum(xtime * y) - (np.cumsum(xtime) * np.cumsum(y)) / ss) ** 2
    ex2 = np.cumsum(xtime ** 2) - np.cumsum(xtime) ** 2 / ss
    totss = np.cumsum(y ** 2) - np.cumsum(y) ** 2 / ss
    regss = exy2[begin - 1:T] / ex2[begin - 1:T]
    r2 = regss / totss[begin - 1:T]
    r3 = np.nonzero(r2 == np.nanmax(r2))[0] + 1          # 1-based positions of the maximum
    stop = begin + int(r3[-1])
    overrun = stop > T
    stop = min(stop, T)
    xs, ys = xtime[:stop], y[:stop]
    mx, my = xs.mean(), ys.mean()
    mx2, my2 = (xs ** 2).mean(), (ys ** 2).mean()
    sdx, sdy = np.sqrt(mx2 - mx ** 2), np.sqrt(my2 - my ** 2)
    mxy = (xs * ys).mean()
    r = (mxy - mx * my) / (sdx * sdy)
    slope = r * sdy / sdx
    yint = -(slope * mx) + my
    rt = mround(abs(60 / slope) - yint)
    return float(rt), float(slope), int(stop), bool(overrun)
