"""Seeded synthetic textures for the DXTn path (tests, golden fixtures, bench).

The reference ships no image corpus; the workloads are described by their statistics:

* colour: per-channel 4-octave value noise (base period 64 px, persistence 0.5, scaled to
  0..255) plus 40 axis-aligned flat-colour rectangles (sides 4..64 px, uniform RGB), alpha 255;
* DXT5 alpha: an independent 3-octave value noise with base period 128;
* DXN: a 5-octave fBm height field (period 256), Sobel gradients at strength 4, unit normals,
  X/Y stored in R/G (B = 0, A = 255);
* mip chains: a 2x2 box filter (per channel, linear, rounded) down to 1x1.

Everything is integer hashing plus IEEE float64 add/mul/div/sqrt, so a given seed produces
the same bytes on x86_64 and aarch64 and with any numpy version.
"""
from __future__ import annotations

import numpy as np

_M32 = np.uint64(0xFFFFFFFF)


def _hash32(*keys: np.ndarray | int) -> np.ndarray:
    """32-bit integer hash of a tuple of integer arrays (splitmix-style finaliser)."""
    h = np.uint64(0x9E3779B9)
    for k in keys:
        k = np.asarray(k, dtype=np.int64).astype(np.uint64) & _M32
        h = (h ^ k) & _M32
        h = (h * np.uint64(0x85EBCA6B)) & _M32
        h = h ^ (h >> np.uint64(13))
        h = (h * np.uint64(0xC2B2AE35)) & _M32
        h = h ^ (h >> np.uint64(16))
    return h


def _unit(h: np.ndarray) -> np.ndarray:
    return h.astype(np.float64) / 4294967296.0


def value_noise(w: int, h: int, period: int, octaves: int, seed: int, channel: int,
                persistence: float = 0.5) -> np.ndarray:
    """Sum of `octaves` smoothstep-interpolated lattice noises, normalised to [0, 1]. The lattice
    values are hashed once per lattice point and gathered per pixel; the per-pixel arithmetic is
    the same sequence of float64 operations at every pixel."""
    xs = np.arange(w, dtype=np.int64)
    ys = np.arange(h, dtype=np.int64)
    total = np.zeros((h, w), np.float64)
    amp, norm = 1.0, 0.0
    p = float(period)
    for o in range(octaves):
        fx = xs / p
        fy = ys / p
        ix = np.floor(fx).astype(np.int64)
        iy = np.floor(fy).astype(np.int64)
        tx = fx - ix
        ty = fy - iy
        tx = tx * tx * (3.0 - 2.0 * tx)
        ty = ty * ty * (3.0 - 2.0 * ty)
        gx = np.arange(int(ix[0]), int(ix[-1]) + 2, dtype=np.int64)
        gy = np.arange(int(iy[0]), int(iy[-1]) + 2, dtype=np.int64)
        lat = _unit(_hash32(seed, channel, o, gx[None, :], gy[:, None]))  # lat[y, x]
        cx, cy = ix - gx[0], iy - gy[0]
        v00 = lat[cy][:, cx]
        v10 = lat[cy][:, cx + 1]
        v01 = lat[cy + 1][:, cx]
        v11 = lat[cy + 1][:, cx + 1]
        a = v00 + (v10 - v00) * tx[None, :]
        b = v01 + (v11 - v01) * tx[None, :]
        total += amp * (a + (b - a) * ty[:, None])
        norm += amp
        amp *= persistence
        p = max(p / 2.0, 1.0)
    return total / norm


def _to_u8(v: np.ndarray) -> np.ndarray:
    return np.clip(np.floor(v * 255.0 + 0.5), 0, 255).astype(np.uint8)


def colour_texture(w: int, h: int, seed: int, with_alpha_noise: bool = False) -> np.ndarray:
    """RGBA8 (h, w, 4): value noise + 40 flat rectangles; alpha 255 or noise (period 128)."""
    img = np.empty((h, w, 4), np.uint8)
    for c in range(3):
        img[:, :, c] = _to_u8(value_noise(w, h, 64, 4, seed, c))
    r = _hash32(seed, 1000 + np.arange(40 * 7)).reshape(40, 7)
    for i in range(40):
        rw = 4 + int(r[i, 0] % 61)
        rh = 4 + int(r[i, 1] % 61)
        x0 = int(r[i, 2] % max(w, 1))
        y0 = int(r[i, 3] % max(h, 1))
        img[y0:y0 + rh, x0:x0 + rw, 0] = int(r[i, 4] & 255)
        img[y0:y0 + rh, x0:x0 + rw, 1] = int(r[i, 5] & 255)
        img[y0:y0 + rh, x0:x0 + rw, 2] = int(r[i, 6] & 255)
    if with_alpha_noise:
        img[:, :, 3] = _to_u8(value_noise(w, h, 128, 3, seed, 7))
    else:
        img[:, :, 3] = 255
    return img


def dark_texture(w: int, h: int, seed: int) -> np.ndarray:
    """colour_texture with its darker half pushed to near-black (every channel 0..3): the shadowed
    or outlined content that DXT1's transparent-index-for-black encoding targets."""
    img = colour_texture(w, h, seed)
    rgb = img[:, :, :3].astype(np.int32)
    dark = rgb.sum(2) < 3 * 112
    img[:, :, :3] = np.where(dark[:, :, None], rgb >> 6, rgb).astype(np.uint8)
    return img


def normal_map(w: int, h: int, seed: int, strength: float = 4.0) -> np.ndarray:
    """RGBA8 normal map: fBm height (5 octaves, period 256) -> Sobel -> unit normal, XY in RG."""
    hgt = value_noise(w, h, 256, 5, seed, 11)
    p = np.pad(hgt, 1, mode="edge")
    gx = (p[0:-2, 2:] + 2.0 * p[1:-1, 2:] + p[2:, 2:]) - (p[0:-2, 0:-2] + 2.0 * p[1:-1, 0:-2] + p[2:, 0:-2])
    gy = (p[2:, 0:-2] + 2.0 * p[2:, 1:-1] + p[2:, 2:]) - (p[0:-2, 0:-2] + 2.0 * p[0:-2, 1:-1] + p[0:-2, 2:])
    nx = -gx * strength
    ny = -gy * strength
    inv = 1.0 / np.sqrt(nx * nx + ny * ny + 1.0)
    img = np.zeros((h, w, 4), np.uint8)
    img[:, :, 0] = _to_u8((nx * inv) * 0.5 + 0.5)
    img[:, :, 1] = _to_u8((ny * inv) * 0.5 + 0.5)
    img[:, :, 3] = 255
    return img


def box_mip(img: np.ndarray) -> np.ndarray:
    """One 2x2 box-filter step (edge rows/columns are reused when a dimension is odd or 1)."""
    h, w = img.shape[:2]
    nh, nw = max(1, h >> 1), max(1, w >> 1)
    ys0 = np.minimum(np.arange(nh) * 2, h - 1)
    ys1 = np.minimum(np.arange(nh) * 2 + 1, h - 1)
    xs0 = np.minimum(np.arange(nw) * 2, w - 1)
    xs1 = np.minimum(np.arange(nw) * 2 + 1, w - 1)
    s = (img[ys0][:, xs0].astype(np.uint32) + img[ys0][:, xs1] + img[ys1][:, xs0] + img[ys1][:, xs1])
    return np.ascontiguousarray(((s + 2) >> 2).astype(np.uint8))


def mip_chain(img: np.ndarray, levels: int | None = None) -> list[np.ndarray]:
    """Full (or `levels`-long) box-filtered chain starting with img itself."""
    h, w = img.shape[:2]
    full = 1
    while (w >> full) or (h >> full):
        full += 1
    n = full if levels is None else min(levels, full)
    out = [img]
    for _ in range(n - 1):
        out.append(box_mip(out[-1]))
    return out


def image_blocks(img: np.ndarray) -> np.ndarray:
    """(h, w, 4) -> (blocks_y*blocks_x, 64) uint8 4x4 blocks, edge-clamped, row-major.

    Mirrors the block gather of dxt_image::init_task (crnlib/crn_dxt_image.cpp:334-344):
    pixel (x, y) of block (bx, by) is img[min(4by+y, h-1), min(4bx+x, w-1)].
    """
    h, w = img.shape[:2]
    bx, by = (w + 3) // 4, (h + 3) // 4
    ys = np.minimum(np.arange(by * 4), h - 1)
    xs = np.minimum(np.arange(bx * 4), w - 1)
    full = img[ys][:, xs]
    return np.ascontiguousarray(full.reshape(by, 4, bx, 4, 4).transpose(0, 2, 1, 3, 4).reshape(by * bx, 64))


def _h32_torch(device, *keys):
    """_hash32 on int64 torch tensors (same 32-bit arithmetic)."""
    import torch
    M = 0xFFFFFFFF
    x = torch.full_like(keys[-1], 0x9E3779B9) if torch.is_tensor(keys[-1]) else torch.tensor(0x9E3779B9)
    for k in keys:
        k = k if torch.is_tensor(k) else torch.tensor(k, dtype=torch.int64, device=device)
        x = (x ^ (k & M)) & M
        x = (x * 0x85EBCA6B) & M
        x = x ^ (x >> 13)
        x = (x * 0xC2B2AE35) & M
        x = x ^ (x >> 16)
    return x


def value_noise_torch(w: int, h: int, period: int, octaves: int, seed: int, channel: int, device="cuda"):
    """value_noise in float32 on the GPU: the same lattice hashes, float32 interpolation."""
    import torch
    ys = torch.arange(h, device=device, dtype=torch.int64).view(h, 1).expand(h, w)
    xs = torch.arange(w, device=device, dtype=torch.int64).view(1, w).expand(h, w)
    total = torch.zeros((h, w), dtype=torch.float32, device=device)
    amp, norm, p = 1.0, 0.0, float(period)
    for o in range(octaves):
        fx, fy = xs.float() / p, ys.float() / p
        ix, iy = fx.floor().long(), fy.floor().long()
        tx, ty = fx - ix, fy - iy
        tx = tx * tx * (3 - 2 * tx)
        ty = ty * ty * (3 - 2 * ty)
        u = lambda a, b: _h32_torch(device, seed, channel, o, a, b).float() / 4294967296.0
        v00, v10, v01, v11 = u(ix, iy), u(ix + 1, iy), u(ix, iy + 1), u(ix + 1, iy + 1)
        a = v00 + (v10 - v00) * tx
        b = v01 + (v11 - v01) * tx
        total += amp * (a + (b - a) * ty)
        norm += amp
        amp *= 0.5
        p = max(p / 2, 1.0)
    return total / norm


def colour_texture_torch(w: int, h: int, seed: int, device="cuda", with_alpha_noise: bool = False):
    """Same recipe as colour_texture (4-octave value noise, period 64, + 40 flat rectangles; alpha
    255 or 3-octave noise of period 128) computed on the GPU in float32 for large training,
    evaluation and batch sets. Seeded and deterministic on a given device; not bit-identical to the
    numpy version."""
    import torch
    img = torch.empty((h, w, 4), dtype=torch.uint8, device=device)
    for c in range(3):
        total = value_noise_torch(w, h, 64, 4, seed, c, device)
        img[:, :, c] = (total * 255 + 0.5).floor().clamp(0, 255).to(torch.uint8)
    if with_alpha_noise:
        img[:, :, 3] = (value_noise_torch(w, h, 128, 3, seed, 7, device) * 255 + 0.5).floor().clamp(0, 255).to(torch.uint8)
    else:
        img[:, :, 3] = 255
    r = _h32_torch(device, seed, 1000 + torch.arange(40 * 7, device=device)).view(40, 7).cpu().tolist()
    for i in range(40):
        rw, rh = 4 + r[i][0] % 61, 4 + r[i][1] % 61
        x0, y0 = r[i][2] % w, r[i][3] % h
        img[y0:y0 + rh, x0:x0 + rw, 0] = r[i][4] & 255
        img[y0:y0 + rh, x0:x0 + rw, 1] = r[i][5] & 255
        img[y0:y0 + rh, x0:x0 + rw, 2] = r[i][6] & 255
    return img


def normal_map_torch(w: int, h: int, seed: int, strength: float = 4.0, device="cuda"):
    """normal_map's recipe (fBm height, 5 octaves, period 256, Sobel, unit normal, XY in RG) in
    float32 on the GPU; not bit-identical to the numpy version."""
    import torch
    hgt = value_noise_torch(w, h, 256, 5, seed, 11, device)
    p = torch.nn.functional.pad(hgt[None, None], (1, 1, 1, 1), mode="replicate")[0, 0]
    gx = (p[0:-2, 2:] + 2.0 * p[1:-1, 2:] + p[2:, 2:]) - (p[0:-2, 0:-2] + 2.0 * p[1:-1, 0:-2] + p[2:, 0:-2])
    gy = (p[2:, 0:-2] + 2.0 * p[2:, 1:-1] + p[2:, 2:]) - (p[0:-2, 0:-2] + 2.0 * p[0:-2, 1:-1] + p[0:-2, 2:])
    nx, ny = -gx * strength, -gy * strength
    inv = torch.rsqrt(nx * nx + ny * ny + 1.0)
    img = torch.zeros((h, w, 4), dtype=torch.uint8, device=device)
    img[:, :, 0] = ((nx * inv) * 0.5 + 0.5).mul(255).add(0.5).floor().clamp(0, 255).to(torch.uint8)
    img[:, :, 1] = ((ny * inv) * 0.5 + 0.5).mul(255).add(0.5).floor().clamp(0, 255).to(torch.uint8)
    img[:, :, 3] = 255
    return img


def mip_chain_torch(img, levels: int | None = None):
    """mip_chain on a (h, w, 4) uint8 torch tensor: the same 2x2 box filter with edge reuse for odd
    or unit dimensions."""
    import torch
    h, w = int(img.shape[0]), int(img.shape[1])
    full = 1
    while (w >> full) or (h >> full):
        full += 1
    n = full if levels is None else min(levels, full)
    out = [img]
    for _ in range(n - 1):
        cur = out[-1]
        ch, cw = int(cur.shape[0]), int(cur.shape[1])
        nh, nw = max(1, ch >> 1), max(1, cw >> 1)
        dev = cur.device
        ys0 = torch.clamp(torch.arange(nh, device=dev) * 2, max=ch - 1)
        ys1 = torch.clamp(torch.arange(nh, device=dev) * 2 + 1, max=ch - 1)
        xs0 = torch.clamp(torch.arange(nw, device=dev) * 2, max=cw - 1)
        xs1 = torch.clamp(torch.arange(nw, device=dev) * 2 + 1, max=cw - 1)
        x = cur.to(torch.int32)
        s = x[ys0][:, xs0] + x[ys0][:, xs1] + x[ys1][:, xs0] + x[ys1][:, xs1]
        out.append(((s + 2) >> 2).to(torch.uint8))
    return out


def box_mip_torch(img):
    """box_mip on a (h, w, 4) uint8 torch tensor with even dimensions."""
    x = img.to(dtype=img.new_empty(0, dtype=__import__("torch").int32).dtype)
    s = x[0::2, 0::2] + x[0::2, 1::2] + x[1::2, 0::2] + x[1::2, 1::2]
    return ((s + 2) >> 2).to(img.dtype)


def image_blocks_torch(img):
    """(h, w, 4) uint8 torch tensor (dimensions multiples of 4) -> (n, 64) blocks, row-major."""
    h, w = img.shape[0], img.shape[1]
    return img.view(h // 4, 4, w // 4, 4, 4).permute(0, 2, 1, 3, 4).reshape(-1, 64).contiguous()
