"""Reference-rule DXT block decoding and error metrics for parity tests.

Palettes follow dxt1_block::get_block_colors (crnlib/crn_dxt.cpp:291-301: 4-colour when
low > high, else 3-colour + transparent black) and dxt5_block::get_block_values
(crnlib/crn_dxt.cpp:455). Errors use the optimizer's metric (crn_color.h:724-745)."""
from __future__ import annotations

import numpy as np


def _expand565(c):
    c = c.astype(np.int64)
    r, g, b = (c >> 11) & 31, (c >> 5) & 63, c & 31
    return np.stack([(r << 3) | (r >> 2), (g << 2) | (g >> 4), (b << 3) | (b >> 2)], -1)


def dxt1_colours(blocks8: np.ndarray) -> np.ndarray:
    """(n, 8) -> (n, 16, 3) decoded RGB."""
    b = blocks8.astype(np.int64)
    lo = b[:, 0] | (b[:, 1] << 8)
    hi = b[:, 2] | (b[:, 3] << 8)
    c0, c1 = _expand565(lo), _expand565(hi)
    four = (lo > hi)[:, None]
    c2 = np.where(four, (2 * c0 + c1) // 3, (c0 + c1) >> 1)
    c3 = np.where(four, (c0 + 2 * c1) // 3, 0)
    pal = np.stack([c0, c1, c2, c3], 1)  # (n, 4, 3)
    sel = np.stack([(b[:, 4 + (i >> 2)] >> (2 * (i & 3))) & 3 for i in range(16)], 1)
    return np.take_along_axis(pal, sel[:, :, None].repeat(3, 2), 1)


def dxt5a_values(blocks8: np.ndarray) -> np.ndarray:
    """(n, 8) -> (n, 16) decoded alpha."""
    b = blocks8.astype(np.int64)
    l, h = b[:, 0], b[:, 1]
    bits = np.zeros(len(b), np.int64)
    for k in range(6):
        bits |= b[:, 2 + k] << (8 * k)
    eight = l > h
    vals = np.zeros((len(b), 8), np.int64)
    vals[:, 0], vals[:, 1] = l, h
    for j in range(1, 7):
        vals[:, 1 + j] = np.where(eight, ((7 - j) * l + j * h) // 7, 0)
    for j in range(1, 5):
        vals[:, 1 + j] = np.where(eight, vals[:, 1 + j], ((5 - j) * l + j * h) // 5)
    vals[:, 6] = np.where(eight, vals[:, 6], 0)
    vals[:, 7] = np.where(eight, vals[:, 7], 255)
    sel = np.stack([(bits >> (3 * i)) & 7 for i in range(16)], 1)
    return np.take_along_axis(vals, sel, 1)


def dxt1_error(blocks8: np.ndarray, pixels: np.ndarray, perceptual: bool) -> np.ndarray:
    """Per-block weighted squared RGB error of decoded DXT1 vs (n, 64) RGBA pixels."""
    dec = dxt1_colours(blocks8)
    px = pixels.reshape(-1, 16, 4)[:, :, :3].astype(np.int64)
    w = np.array([8, 25, 1] if perceptual else [1, 1, 1])
    return (((dec - px) ** 2) * w).sum((1, 2))


def rgb_rmse(blocks8: np.ndarray, pixels: np.ndarray) -> float:
    """'RGB Average' RMSE (crn_image_utils.cpp:1048-1139): sqrt(sum sq err / (texels * 3))."""
    dec = dxt1_colours(blocks8)
    px = pixels.reshape(-1, 16, 4)[:, :, :3].astype(np.int64)
    return float(np.sqrt(((dec - px) ** 2).sum() / (px.shape[0] * 16 * 3)))
