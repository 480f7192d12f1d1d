"""CPU restatement (numpy, float32 arithmetic step by step) of crnlib's mip generation, for the
parity tests of the GPU mip generator. TEST INFRASTRUCTURE ONLY.

Follows mipmapped_texture::generate_mipmaps (crnlib/crn_mipmapped_texture.cpp:2140-2215): every
level is resampled from level 0 by image_utils::resample_multithreaded
(crnlib/crn_image_utils.cpp:662-874) over threaded_resampler (crnlib/crn_threaded_resampler.cpp:
66-357): the gamma tables, the contributor lists of Resampler::make_clist
(crnlib/crn_resampler.cpp:119-412), the x pass per source row, the y pass per destination row with
its clamp to [0, 1], and the conversion back to 8 bits. The filters are those of crn_mip_filter
(crnlib/crn_resample_filters.cpp:17-369). Python floats are IEEE doubles, numpy float32 scalars and
arrays single precision, so each expression is evaluated in the precision the reference uses.
"""
from __future__ import annotations

import math

import numpy as np

f32 = np.float32
PI = 3.14159265358979323846


def _box(t):
    return f32(1.0) if (t >= f32(-0.5) and t < f32(0.5)) else f32(0.0)


def _tent(t):
    t = -t if t < f32(0.0) else t
    return f32(f32(1.0) - t) if t < f32(1.0) else f32(0.0)


def _sinc(x: float) -> float:
    x = x * PI
    if x < float(f32(0.01)) and x > -float(f32(0.01)):
        return 1.0 + x * x * (float(f32(-1.0) / f32(6.0)) + x * x * 1.0 / 120.0)
    return math.sin(x) / x


def _clean(t: float):
    if abs(t) < float(f32(0.0000125)):
        return f32(0.0)
    return f32(t)


def _lanczos4(t):
    t = -t if t < f32(0.0) else t
    if t < f32(4.0):
        return _clean(_sinc(float(t)) * _sinc(float(f32(t / f32(4.0)))))
    return f32(0.0)


def _mitchell(t, B, C):
    tt = f32(t * t)
    t = -t if t < f32(0.0) else t
    if t < f32(1.0):
        a = f32(f32(f32(12.0) - f32(f32(9.0) * B)) - f32(f32(6.0) * C))
        b = f32(f32(f32(-18.0) + f32(f32(12.0) * B)) + f32(f32(6.0) * C))
        c = f32(f32(6.0) - f32(f32(2.0) * B))
        t = f32(f32(f32(a * f32(t * tt)) + f32(b * tt)) + c)
        return f32(t / f32(6.0))
    if t < f32(2.0):
        a = f32(f32(f32(-1.0) * B) - f32(f32(6.0) * C))
        b = f32(f32(f32(6.0) * B) + f32(f32(30.0) * C))
        c = f32(f32(f32(-12.0) * B) - f32(f32(48.0) * C))
        d = f32(f32(f32(8.0) * B) + f32(f32(24.0) * C))
        t = f32(f32(f32(f32(a * f32(t * tt)) + f32(b * tt)) + f32(c * t)) + d)
        return f32(t / f32(6.0))
    return f32(0.0)


def _mitchell_f(t):
    third = f32(f32(1.0) / f32(3.0))
    return _mitchell(t, third, third)


def _bessel0(x: float) -> float:
    xh = 0.5 * x
    s, pw, k, ds = 1.0, 1.0, 0, 1.0
    while ds > s * 1e-16:
        k += 1
        pw = pw * (xh / k)
        ds = pw * pw
        s = s + ds
    return s


def _kaiser(t):
    t = -t if t < f32(0.0) else t
    if t < f32(3):
        att = f32(40.0)
        alpha = f32(math.exp(math.log(0.58417 * (float(att) - 20.96)) * 0.4) + 0.07886 * (float(att) - 20.96))
        ratio = float(t) / 3.0
        win = _bessel0(float(alpha) * math.sqrt(1 - ratio * ratio)) / _bessel0(float(alpha))
        return f32(_clean(_sinc(float(t)) * win))
    return f32(0.0)


FILTERS = {"box": (_box, f32(0.5)), "tent": (_tent, f32(1.0)), "lanczos4": (_lanczos4, f32(4.0)),
           "mitchell": (_mitchell_f, f32(2.0)), "kaiser": (_kaiser, f32(3.0))}


def make_clist(src: int, dst: int, filt: str, filter_scale: float, wrap: bool):
    """[(pixels, weights)] per destination sample (Resampler::make_clist with no source offset)."""
    fn, support = FILTERS[filt]
    fs = f32(filter_scale)
    oo = f32(f32(1.0) / fs)
    nudge = f32(0.5)
    xscale = f32(f32(dst) / f32(src))
    down = xscale < f32(1.0)
    half = f32(f32(support / xscale) * fs) if down else f32(support * fs)
    out = []
    for i in range(dst):
        center = f32(f32(f32(i) + nudge) / xscale)
        center = f32(center - nudge)
        left = int(f32(math.floor(f32(center - half))))
        right = int(f32(math.ceil(f32(center + half))))

        def arg(j):
            d = f32(center - f32(j))
            return f32(f32(d * xscale) * oo) if down else f32(d * oo)

        total = f32(0.0)
        for j in range(left, right + 1):
            total = f32(total + fn(arg(j)))
        norm = f32(f32(1.0) / total)
        total = f32(0.0)
        pix, wts = [], []
        max_k, max_w = -1, f32(-1e20)
        for j in range(left, right + 1):
            w = f32(fn(arg(j)) * norm)
            if w == f32(0.0):
                continue
            if j < 0:
                n = (src - ((-j) % src)) % src if wrap else 0
            elif j >= src:
                n = j % src if wrap else src - 1
            else:
                n = j
            pix.append(n)
            wts.append(w)
            total = f32(total + w)
            if w > max_w:
                max_w, max_k = w, len(wts) - 1
        if total != f32(1.0):
            wts[max_k] = f32(wts[max_k] + f32(f32(1.0) - total))
        out.append((np.array(pix, np.int64), np.array(wts, np.float32)))
    return out


def gamma_tables(gamma: float = 2.2):
    g = f32(gamma)
    to_linear = np.array([np.power(f32(f32(f32(i) * f32(1.0)) / f32(255.0)), g) for i in range(256)], np.float32)
    inv_size, inv_g = f32(f32(1.0) / f32(8192)), f32(f32(1.0) / g)
    to_srgb = np.zeros(8192, np.uint8)
    for i in range(8192):
        k = int(f32(f32(f32(255.0) * np.power(f32(f32(i) * inv_size), inv_g)) + f32(0.5)))
        to_srgb[i] = min(max(k, 0), 255)
    return to_linear, to_srgb


def resample(img: np.ndarray, dst_w: int, dst_h: int, filt: str, filter_scale: float, srgb: bool, wrap: bool,
             alpha: bool, tables=None) -> np.ndarray:
    h, w = img.shape[:2]
    to_linear, to_srgb = tables if tables is not None else gamma_tables()
    x = img.astype(np.int64)
    lin = np.empty((h, w, 4), np.float32)
    inv = f32(f32(1.0) / f32(255.0))
    for c in range(4):
        lin[:, :, c] = to_linear[x[:, :, c]] if (srgb and c < 3) else (x[:, :, c].astype(np.float32) * inv)
    cx = make_clist(w, dst_w, filt, filter_scale, wrap)
    cy = make_clist(h, dst_h, filt, filter_scale, wrap)
    tmp = np.empty((h, dst_w, 4), np.float32)
    for i, (pix, wts) in enumerate(cx):
        s = np.zeros((h, 4), np.float32)
        for p, wt in zip(pix, wts):
            s = (s + lin[:, p, :] * wt).astype(np.float32)
        tmp[:, i, :] = s
    out = np.empty((dst_h, dst_w, 4), np.uint8)
    for i, (pix, wts) in enumerate(cy):
        if len(pix) == 1:
            v = tmp[pix[0]].copy()
        else:
            v = (tmp[pix[0]] * wts[0]).astype(np.float32)
            for p, wt in zip(pix[1:], wts[1:]):
                v = (v + tmp[p] * wt).astype(np.float32)
        v = np.minimum(np.maximum(v, f32(0.0)), f32(1.0))
        lin8 = np.clip((v * f32(255.0) + f32(0.5)).astype(np.float32).astype(np.int64), 0, 255)
        if srgb:
            j = np.clip((v[:, :3] * f32(8192.0) + f32(0.5)).astype(np.float32).astype(np.int64), 0, 8191)
            out[i, :, :3] = to_srgb[j]
        else:
            out[i, :, :3] = lin8[:, :3]
        out[i, :, 3] = lin8[:, 3] if alpha else 255
    return out


def generate_mipmaps(img: np.ndarray, filt: str = "kaiser", filter_scale: float = 0.9, srgb: bool = True,
                     wrap: bool = False, alpha: bool = True, levels: int = 0):
    h, w = img.shape[:2]
    full = 1
    while (w >> full) or (h >> full):
        full += 1
    n = levels or full
    tables = gamma_tables()
    out = [np.ascontiguousarray(img)]
    for l in range(1, n):
        out.append(resample(img, max(1, w >> l), max(1, h >> l), filt, filter_scale, srgb, wrap, alpha, tables))
    return out
