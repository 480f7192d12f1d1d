"""Error metrics of decoded DXTn blocks against their RGBA8 source blocks, computed on the device:
the 'RGB Average' RMSE of crnlib's image comparison (crnlib/crn_image_utils.cpp:1048-1139) for
DXT1 colour, and the per-channel RMSE of DXT5-style alpha blocks (DXT5 alpha, the two DXN
channels, DXT5A). Decoding follows the block formats (dxt1_block / dxt5_block,
crnlib/crn_dxt.cpp): four- or three-colour DXT1 palettes, eight- or six-value alpha palettes."""
from __future__ import annotations

import torch

CHUNK = 1 << 20  # blocks per decoded chunk (bounds temporary device memory)


def dxt1_colours(b8: torch.Tensor) -> torch.Tensor:
    """(n, 8) uint8 DXT1 blocks -> (n, 16, 3) int64 decoded RGB."""
    b = b8.to(torch.int64)
    lo = b[:, 0] | (b[:, 1] << 8)
    hi = b[:, 2] | (b[:, 3] << 8)

    def expand(c):
        r, g, bl = (c >> 11) & 31, (c >> 5) & 63, c & 31
        return torch.stack([(r << 3) | (r >> 2), (g << 2) | (g >> 4), (bl << 3) | (bl >> 2)], -1)

    c0, c1 = expand(lo), expand(hi)
    four = (lo > hi).unsqueeze(-1)
    c2 = torch.where(four, (2 * c0 + c1) // 3, (c0 + c1) >> 1)
    c3 = torch.where(four, (c0 + 2 * c1) // 3, torch.zeros_like(c0))
    pal = torch.stack([c0, c1, c2, c3], 1)
    sel = torch.stack([(b[:, 4 + (i >> 2)] >> (2 * (i & 3))) & 3 for i in range(16)], 1)
    return torch.gather(pal, 1, sel.unsqueeze(-1).expand(-1, -1, 3))


def alpha_values(b8: torch.Tensor) -> torch.Tensor:
    """(n, 8) uint8 DXT5 alpha blocks -> (n, 16) int64 decoded values."""
    b = b8.to(torch.int64)
    l, h = b[:, :1], b[:, 1:2]
    bits = torch.zeros_like(b[:, 0])
    for k in range(6):
        bits |= b[:, 2 + k] << (8 * k)
    j = torch.arange(1, 7, device=b.device).unsqueeze(0)
    eight = ((7 - j) * l + j * h) // 7
    j4 = torch.arange(1, 5, device=b.device).unsqueeze(0)
    six = torch.cat([((5 - j4) * l + j4 * h) // 5, torch.zeros_like(l), torch.full_like(l, 255)], 1)
    vals = torch.cat([l, h, torch.where(l > h, eight, six)], 1)
    sel = torch.stack([(bits >> (3 * i)) & 7 for i in range(16)], 1)
    return torch.gather(vals, 1, sel)


def block_rmse(dxt: torch.Tensor, src: torch.Tensor, fmt: str) -> dict:
    """dxt: (n, bytes per block) uint8 decoded-format blocks; src: (n, 64) uint8 RGBA8 blocks, on
    the same device. fmt: 'DXT1' -> rmse_color; 'DXT5' -> rmse_color, rmse_alpha (alpha from A);
    'DXN_XY' / 'DXN_YX' -> rmse_xy over R and G (X in the first block for DXN_XY); 'DXT5A' ->
    rmse_alpha."""
    n = int(src.shape[0])
    sums = {"color": 0.0, "alpha": 0.0, "xy": 0.0}
    for c in range(0, n, CHUNK):
        d = dxt[c:c + CHUNK]
        px = src[c:c + CHUNK].view(-1, 16, 4).to(torch.int64)
        if fmt in ("DXT1", "DXT5"):
            col = dxt1_colours(d[:, 8:] if fmt == "DXT5" else d)
            sums["color"] += float(((col - px[:, :, :3]) ** 2).sum())
        if fmt in ("DXT5", "DXT5A"):
            sums["alpha"] += float(((alpha_values(d[:, :8]) - px[:, :, 3]) ** 2).sum())
        if fmt in ("DXN_XY", "DXN_YX"):
            first, second = (0, 1) if fmt == "DXN_XY" else (1, 0)
            sums["xy"] += float(((alpha_values(d[:, :8]) - px[:, :, first]) ** 2).sum() +
                                ((alpha_values(d[:, 8:]) - px[:, :, second]) ** 2).sum())
    out = {}
    if fmt in ("DXT1", "DXT5"):
        out["rmse_color"] = (sums["color"] / (n * 48)) ** 0.5
    if fmt in ("DXT5", "DXT5A"):
        out["rmse_alpha"] = (sums["alpha"] / (n * 16)) ** 0.5
    if fmt in ("DXN_XY", "DXN_YX"):
        out["rmse_xy"] = (sums["xy"] / (n * 32)) ** 0.5
    return out
