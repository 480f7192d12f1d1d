"""Regenerates the golden fixtures in this folder from the REFERENCE crnlib.

The reference is compiled from its own sources by `make -C oracle ref` (oracle/_ref/libcrnref.so,
x86_64 build container only) and driven through its public API:
  * crn_create_block_compressor / crn_compress_block   (inc/crnlib.h:674-682)
  * crn_compress with source mips                       (inc/crnlib.h:614)
  * crnd_unpack_begin / crnd_unpack_level               (inc/crn_defs.h:174-191)
with cCRNCompFlagDisableEndpointCaching set for block encodes, so the outputs do not depend on
thread count. Inputs come from crunch2_gb300.texgen (seeded, platform-independent) or are stored.

Outputs (all small; committed):
  blocks.npz        edge-case + texture block inputs and the reference DXT1/DXT5/DXN/DXT5A blocks
  blocks_quality.npz  the same below Uber quality, with grayscale sampling, DXT1A transparency and
                    transparent indices for black
  crn/*.crn         reference .crn files; crn/manifest.json holds per-level sha256 of the
                    reference transcode and the generation parameters
Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from crunch2_gb300 import texgen  # noqa: E402
from oracle import ref  # noqa: E402

FLAG_PERCEPTUAL = 1
FLAG_HIERARCHICAL = 2
FLAG_BOTH_BLOCK_TYPES = 8
FLAG_NO_ENDPOINT_CACHING = 32
DXT_UBER = 4
FMT = {"DXT1": 0, "DXT5": 2, "DXN_XY": 7, "DXN_YX": 8, "DXT5A": 9}


def edge_blocks(seed: int = 1) -> np.ndarray:
    """Stress blocks: random 16-colour, 1..5-colour palettes, low-contrast gradients, extremes
    (black/white/primaries, 565 boundary values), with random alpha."""
    rng = np.random.default_rng(seed)
    parts = [rng.integers(0, 256, (400, 64), dtype=np.uint8)]
    for k in (1, 2, 3, 4, 5):
        pal = rng.integers(0, 256, (160, k, 4), dtype=np.uint8)
        idx = rng.integers(0, k, (160, 16))
        parts.append(np.take_along_axis(pal, idx[:, :, None].repeat(4, 2), 1).reshape(160, 64))
    base = rng.integers(0, 256, (200, 1, 4)).astype(int)
    parts.append(np.clip(base + rng.integers(-8, 9, (200, 16, 4)), 0, 255).astype(np.uint8).reshape(200, 64))
    ex = np.array([[0, 0, 0, 255], [255, 255, 255, 255], [255, 0, 0, 255], [0, 255, 0, 255], [0, 0, 255, 255],
                   [8, 4, 8, 255], [247, 251, 247, 255], [4, 4, 4, 255]], np.uint8)
    parts.append(ex[rng.integers(0, 8, (200, 16))].reshape(200, 64))
    solid = rng.integers(0, 256, (100, 1, 4), dtype=np.uint8).repeat(16, 1).reshape(100, 64)
    parts.append(solid)
    b = np.concatenate(parts).reshape(-1, 16, 4)
    b[:, :, 3] = rng.integers(0, 256, (b.shape[0], 16))
    return np.ascontiguousarray(b.reshape(-1, 64))


def sha(a) -> str:
    return hashlib.sha256(bytes(a)).hexdigest()


def make_blocks() -> None:
    edge = edge_blocks()
    c0 = texgen.image_blocks(texgen.colour_texture(256, 256, 0))           # config-0 texture
    dxt5_tex = texgen.image_blocks(texgen.colour_texture(128, 128, 3, with_alpha_noise=True))
    nrm_tex = texgen.image_blocks(texgen.normal_map(128, 128, 4))
    out = {"edge_in": edge, "c0_in_sha": np.frombuffer(sha(c0).encode(), np.uint8),
           "dxt5_tex_sha": np.frombuffer(sha(dxt5_tex).encode(), np.uint8),
           "nrm_tex_sha": np.frombuffer(sha(nrm_tex).encode(), np.uint8)}
    base = FLAG_HIERARCHICAL | FLAG_NO_ENDPOINT_CACHING
    # DXT1, both metrics x both block-type settings, on the edge set; config-0 texture default mode
    for perc in (1, 0):
        for both in (1, 0):
            flags = base | (FLAG_PERCEPTUAL if perc else 0) | (FLAG_BOTH_BLOCK_TYPES if both else 0)
            out[f"edge_dxt1_p{perc}_b{both}"] = ref.compress_blocks(edge, FMT["DXT1"], flags, DXT_UBER)
    out["c0_dxt1"] = ref.compress_blocks(c0, FMT["DXT1"], base | FLAG_PERCEPTUAL | FLAG_BOTH_BLOCK_TYPES, DXT_UBER)
    for name in ("DXT5", "DXN_XY", "DXN_YX", "DXT5A"):
        for both in (1, 0):
            flags = base | FLAG_PERCEPTUAL | (FLAG_BOTH_BLOCK_TYPES if both else 0)
            out[f"edge_{name.lower()}_b{both}"] = ref.compress_blocks(edge, FMT[name], flags, DXT_UBER)
    out["dxt5_tex_dxt5"] = ref.compress_blocks(dxt5_tex, FMT["DXT5"], base | FLAG_PERCEPTUAL | FLAG_BOTH_BLOCK_TYPES,
                                               DXT_UBER)
    out["nrm_tex_dxn_xy"] = ref.compress_blocks(nrm_tex, FMT["DXN_XY"], base | FLAG_BOTH_BLOCK_TYPES, DXT_UBER)
    # Whole-image cross-check: the block API must equal crn_compress's plain .dds output.
    dds = np.frombuffer(ref.compress_texture([[texgen.colour_texture(256, 256, 0)]], FMT["DXT1"], 1, 255,
                                             base | FLAG_PERCEPTUAL | FLAG_BOTH_BLOCK_TYPES, DXT_UBER, 7), np.uint8)
    assert np.array_equal(dds[128:128 + out["c0_dxt1"].size].reshape(-1, 8), out["c0_dxt1"]), "dds != block api"
    np.savez_compressed(os.path.join(HERE, "blocks.npz"), **out)


FLAG_TRANSPARENT_BLACK = 16
FLAG_DXT1A = 128
FLAG_GRAYSCALE = 256
QUALITIES = (0, 1, 2, 3)  # superfast, fast, normal, better (uber is in blocks.npz)


def alpha_blocks(seed: int = 2) -> np.ndarray:
    """DXT1A inputs: the edge blocks with 0..4 texels below the 128 alpha threshold, fully
    transparent blocks, and single-colour blocks with a few transparent texels."""
    rng = np.random.default_rng(seed)
    b = edge_blocks(seed).reshape(-1, 16, 4).copy()
    b[:, :, 3] = 255
    for i in range(b.shape[0]):
        k = int(rng.integers(0, 5))
        b[i, rng.choice(16, k, replace=False), 3] = rng.integers(0, 128, k)
    clear = rng.integers(0, 256, (40, 16, 4), dtype=np.uint8)
    clear[:, :, 3] = rng.integers(0, 128, (40, 16))
    solid = rng.integers(0, 256, (80, 1, 4), dtype=np.uint8).repeat(16, 1)
    solid[:, :, 3] = 255
    for i in range(solid.shape[0]):
        solid[i, rng.choice(16, 1 + i % 6, replace=False), 3] = 0
    return np.ascontiguousarray(np.concatenate([b, clear, solid]).reshape(-1, 64))


def dark_blocks(seed: int = 3) -> np.ndarray:
    """Inputs for the transparent-black trial: blocks mixing near-black texels (every channel
    <= 4) with other colours, plus the edge set."""
    rng = np.random.default_rng(seed)
    n = 600
    b = rng.integers(0, 256, (n, 16, 4), dtype=np.uint8)
    for i in range(n):
        if i % 3 == 0:  # a few colours in the block, as textures with dark outlines have
            pal = rng.integers(0, 256, (3, 4), dtype=np.uint8)
            b[i] = pal[rng.integers(0, 3, 16)]
        k = int(rng.integers(1, 16))
        b[i, rng.choice(16, k, replace=False), :3] = rng.integers(0, 5, (k, 3))
    return np.ascontiguousarray(np.concatenate([b.reshape(n, 64), edge_blocks(seed)]))


def make_quality() -> None:
    """The reference block compressor below Uber quality, with grayscale sampling, DXT1A
    transparency and transparent indices for black: blocks_quality.npz."""
    edge, alpha, dark = edge_blocks(), alpha_blocks(), dark_blocks()
    out = {"alpha_in": alpha, "dark_in": dark}
    base = FLAG_HIERARCHICAL | FLAG_NO_ENDPOINT_CACHING
    for q in QUALITIES:
        for perc in (1, 0):
            for both in (1, 0):
                flags = base | (FLAG_PERCEPTUAL if perc else 0) | (FLAG_BOTH_BLOCK_TYPES if both else 0)
                out[f"dxt1_q{q}_p{perc}_b{both}"] = ref.compress_blocks(edge, FMT["DXT1"], flags, q)
        for name in ("DXT5", "DXN_XY", "DXT5A"):
            for both in (1, 0):
                flags = base | FLAG_PERCEPTUAL | (FLAG_BOTH_BLOCK_TYPES if both else 0)
                out[f"{name.lower()}_q{q}_b{both}"] = ref.compress_blocks(edge, FMT[name], flags, q)
    for q in (4, 3, 1):
        for both in (1, 0):
            flags = base | FLAG_PERCEPTUAL | FLAG_GRAYSCALE | (FLAG_BOTH_BLOCK_TYPES if both else 0)
            out[f"gray_q{q}_b{both}"] = ref.compress_blocks(edge, FMT["DXT1"], flags, q)
        for perc in (1, 0):
            for both in (1, 0):
                flags = base | FLAG_DXT1A | (FLAG_PERCEPTUAL if perc else 0) | (FLAG_BOTH_BLOCK_TYPES if both else 0)
                out[f"dxt1a_q{q}_p{perc}_b{both}"] = ref.compress_blocks(alpha, FMT["DXT1"], flags, q)
            flags = base | FLAG_TRANSPARENT_BLACK | FLAG_BOTH_BLOCK_TYPES | (FLAG_PERCEPTUAL if perc else 0)
            out[f"black_q{q}_p{perc}"] = ref.compress_blocks(dark, FMT["DXT1"], flags, q)
        flags = base | FLAG_TRANSPARENT_BLACK | FLAG_BOTH_BLOCK_TYPES | FLAG_GRAYSCALE
        out[f"black_gray_q{q}"] = ref.compress_blocks(dark, FMT["DXT1"], flags, q)
    np.savez_compressed(os.path.join(HERE, "blocks_quality.npz"), **out)


# (name, width, height, format, faces, content, seed)
CRN_CASES = [
    ("c1_dxt1_1024", 1024, 1024, "DXT1", 1, "colour", 100),   # config-1 texture, 11 levels
    ("dxt1_256", 256, 256, "DXT1", 1, "colour", 10),
    ("dxt1_100x60", 100, 60, "DXT1", 1, "colour", 11),        # odd block counts
    ("dxt1_cube_64", 64, 64, "DXT1", 6, "colour", 12),        # 6 faces share decoder state
    ("dxt5_256", 256, 256, "DXT5", 1, "colour_alpha", 13),
    ("dxt5_cube_64x32", 64, 32, "DXT5", 6, "colour_alpha", 14),
    ("dxn_xy_256", 256, 256, "DXN_XY", 1, "normal", 15),
    ("dxt5a_256", 256, 256, "DXT5A", 1, "colour_alpha", 16),
    ("dxt5_2048", 2048, 2048, "DXT5", 1, "colour_alpha", 200),    # config 2's textures (12 levels)
    ("dxn_xy_2048", 2048, 2048, "DXN_XY", 1, "normal", 201),
]


def texture_levels(w, h, content, seed, faces):
    out = []
    for f in range(faces):
        if content == "normal":
            img = texgen.normal_map(w, h, seed + f)
        elif content == "dark":
            img = texgen.dark_texture(w, h, seed + f)
        else:
            img = texgen.colour_texture(w, h, seed + f, with_alpha_noise=(content == "colour_alpha"))
        out.append(texgen.mip_chain(img))
    return out


def level_bytes(w, h, level, bpb, faces):
    w, h = max(1, w >> level), max(1, h >> level)
    return ((w + 3) // 4) * ((h + 3) // 4) * bpb * faces


def make_crn(only=None) -> None:
    """The reference's .crn files of CRN_CASES (those named in `only`, if given) and the per-level
    SHA-256 of its transcode, into crn/ and crn/manifest.json."""
    os.makedirs(os.path.join(HERE, "crn"), exist_ok=True)
    manifest = {}
    if only:
        with open(os.path.join(HERE, "crn", "manifest.json")) as fh:
            manifest = json.load(fh)
    for name, w, h, fmt, faces, content, seed in CRN_CASES:
        if only and name not in only:
            continue
        fl = texture_levels(w, h, content, seed, faces)
        flags = (0 if content == "normal" else FLAG_PERCEPTUAL) | FLAG_HIERARCHICAL | FLAG_BOTH_BLOCK_TYPES
        crn = ref.compress_texture(fl, FMT[fmt], 0, 128, flags, DXT_UBER, 7)
        with open(os.path.join(HERE, "crn", name + ".crn"), "wb") as fh:
            fh.write(crn)
        bpb = 8 if fmt in ("DXT1", "DXT5A") else 16
        levels = []
        for lvl in range(len(fl[0])):
            out = ref.unpack_level(crn, lvl, level_bytes(w, h, lvl, bpb, faces))
            levels.append({"bytes": int(out.size), "sha256": sha(out)})
        manifest[name] = {"width": w, "height": h, "format": fmt, "faces": faces, "content": content, "seed": seed,
                          "quality": 128, "crn_sha256": sha(crn), "levels": levels,
                          "input_sha256": sha(np.concatenate([im.reshape(-1) for f in fl for im in f]))}
    with open(os.path.join(HERE, "crn", "manifest.json"), "w") as fh:
        json.dump(manifest, fh, indent=1, sort_keys=True)


HC_CASES = [("dxt1_256", 256, 10), ("c1_dxt1_1024", 1024, 100), ("hc_128", 128, 21)]
# (name, format, crn format code, size, seed, content)
HC_ALPHA_CASES = [("dxt5_256", "DXT5", 2, 256, 13, "colour_alpha"), ("dxn_xy_256", "DXN_XY", 7, 256, 15, "normal")]


def make_hc(alpha_only: bool = False) -> None:
    """The reference's clustered DXT1 compressor (crnlib::dxt_hc::compress, run directly on blocks in
    crn_comp's layout at q128 codebook sizes): its tile count, codebook sizes and RGB RMSE, the
    quality bar of the GPU clustered path. alpha_only rewrites only the alpha-format entries."""
    from crunch2_gb300 import hc
    from crunch2_gb300.hc import crn_layout
    sys.path.insert(0, os.path.dirname(HERE))
    from dxt_decode import rgb_rmse
    out = {}
    if alpha_only:
        with open(os.path.join(HERE, "hc_reference.json")) as fh:
            out = {k: v for k, v in json.load(fh).items() if k in dict((c[0], c) for c in HC_CASES)}
    for name, size, seed in ([] if alpha_only else HC_CASES):
        levels = texgen.mip_chain(texgen.colour_texture(size, size, seed))
        blocks, lv, vis = crn_layout([levels])
        ce, cs = hc.codebook_sizes(size, size, 128)[:2]
        dxt, st = ref.dxt_hc_dxt1(blocks, lv, 1, ce, cs, True, threads=8)
        rows = [dxt[fb:fb + nb].reshape(-1, bw, 8)[:by, :bx].reshape(-1, 8) for (fb, nb, bw), (bx, by, _) in zip(lv, vis)]
        src = np.concatenate([texgen.image_blocks(im) for im in levels])
        out[name] = {"size": size, "seed": seed, "quality": 128, "codebook_request": [ce, cs], "tiles": st["tiles"],
                     "endpoints": st["endpoints"], "selectors": st["selectors"],
                     "rmse_visible": rgb_rmse(np.concatenate(rows), src), "rmse_all_blocks": rgb_rmse(dxt, blocks)}
    # alpha-carrying formats: DXT5 (colour + alpha noise, perceptual) and DXN_XY (normal map)
    from dxt_decode import dxt5a_values
    for name, fmt, code, size, seed, content in HC_ALPHA_CASES:
        img = texgen.normal_map(size, size, seed) if content == "normal" else \
            texgen.colour_texture(size, size, seed, with_alpha_noise=True)
        levels = texgen.mip_chain(img)
        blocks, lv, vis = crn_layout([levels])
        sizes = hc.codebook_sizes(size, size, 128, code)
        dxt, st = ref.dxt_hc_alpha(blocks, lv, 1, fmt, sizes, content != "normal", threads=8)
        rows = [dxt[fb:fb + nb].reshape(-1, bw, dxt.shape[1])[:by, :bx].reshape(-1, dxt.shape[1])
                for (fb, nb, bw), (bx, by, _) in zip(lv, vis)]
        dec = np.concatenate(rows)
        src = np.concatenate([texgen.image_blocks(im) for im in levels]).reshape(-1, 16, 4).astype(np.int64)
        rec = {"size": size, "seed": seed, "quality": 128, "format": fmt, "content": content,
               "codebook_request": list(sizes), **st}
        if fmt == "DXT5":
            rec["rmse_color_visible"] = rgb_rmse(dec[:, 8:], src.reshape(-1, 64).astype(np.uint8))
            a = dxt5a_values(dec[:, :8])
            rec["rmse_alpha_visible"] = float(np.sqrt(((a - src[:, :, 3]) ** 2).mean()))
        else:
            x, y = dxt5a_values(dec[:, :8]), dxt5a_values(dec[:, 8:])
            rec["rmse_alpha_visible"] = float(np.sqrt((((x - src[:, :, 0]) ** 2).sum() + ((y - src[:, :, 1]) ** 2).sum())
                                                      / (2 * x.size)))
        out[name] = rec
    with open(os.path.join(HERE, "hc_reference.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)


# clustered DDS (QDXT) cases: (name, size, seed, quality)
QDXT_CASES = [("qdxt_256_q128", 256, 10, 128), ("qdxt_256_q64", 256, 10, 64), ("qdxt_1024_q128", 1024, 100, 128)]
QDXT_ALPHA_CASES = [("qdxt_dxt5_256_q128", "DXT5", 256, 13, "colour_alpha", 128),
                    ("qdxt_dxn_xy_256_q128", "DXN_XY", 256, 15, "normal", 128),
                    ("qdxt_dxt5a_256_q128", "DXT5A", 256, 16, "colour_alpha", 128),
                    ("qdxt_dxt5_256_q64", "DXT5", 256, 13, "colour_alpha", 64)]


def make_qdxt() -> None:
    """The reference's clustered DDS (crn_compress with a DDS file type and quality < 255: its
    QDXT path) on colour mip chains: RGB RMSE of its DXT1 blocks over every level, the bar for the
    GPU path (which is compared on quality, like the .crn clustering)."""
    import time
    sys.path.insert(0, os.path.dirname(HERE))
    from dxt_decode import rgb_rmse
    out = {}
    for name, size, seed, q in QDXT_CASES:
        levels = texgen.mip_chain(texgen.colour_texture(size, size, seed))
        t = time.time()
        dds = ref.compress_texture([levels], FMT["DXT1"], 1, q, FLAG_PERCEPTUAL | FLAG_HIERARCHICAL | FLAG_BOTH_BLOCK_TYPES,
                                   DXT_UBER, 7)
        secs = time.time() - t
        assert dds[:4] == b"DDS ", "not a DDS file"
        blocks = np.frombuffer(dds[128:], np.uint8).reshape(-1, 8)
        src = np.concatenate([texgen.image_blocks(im) for im in levels])
        assert blocks.shape[0] == src.shape[0], (blocks.shape, src.shape)
        out[name] = {"size": size, "seed": seed, "quality": q, "blocks": int(src.shape[0]),
                     "rmse": rgb_rmse(blocks, src), "seconds_8_threads_x86": round(secs, 2),
                     "distinct_endpoints": int(np.unique(blocks[:, :4].copy().view(np.uint32)).size),
                     "distinct_selectors": int(np.unique(blocks[:, 4:].copy().view(np.uint32)).size),
                     "blocks_sha256": sha(blocks)}
        print(name, out[name], flush=True)
    # the alpha-carrying formats (qdxt5 on each alpha / DXN element, qdxt1 on DXT5's colour)
    import torch
    from crunch2_gb300 import quality as Q
    for name, fmt, size, seed, content, q in QDXT_ALPHA_CASES:
        levels = texture_levels(size, size, content, seed, 1)[0]
        flags = (0 if content == "normal" else FLAG_PERCEPTUAL) | FLAG_HIERARCHICAL | FLAG_BOTH_BLOCK_TYPES
        t = time.time()
        dds = ref.compress_texture([levels], FMT[fmt], 1, q, flags, DXT_UBER, 7)
        secs = time.time() - t
        bpb = 8 if fmt == "DXT5A" else 16
        blocks = np.frombuffer(dds[128:], np.uint8).reshape(-1, bpb)
        src = np.concatenate([texgen.image_blocks(im) for im in levels])
        rec = {"size": size, "seed": seed, "quality": q, "format": fmt, "content": content, "flags": flags,
               "blocks": int(src.shape[0]), "seconds_8_threads_x86": round(secs, 2)}
        rec.update(Q.block_rmse(torch.from_numpy(blocks.copy()), torch.from_numpy(src), fmt))
        for k in range(bpb // 8):
            el = blocks[:, 8 * k:8 * k + 8].copy()
            if fmt == "DXT5" and k == 1:
                rec["distinct_colour_endpoints"] = int(np.unique(el[:, :4].view(np.uint32)).size)
                rec["distinct_colour_selectors"] = int(np.unique(el[:, 4:].view(np.uint32)).size)
            else:
                rec[f"distinct_alpha_endpoints_{k}"] = int(np.unique(el[:, :2].view(np.uint16)).size)
                sel = np.concatenate([el[:, 2:], np.zeros((el.shape[0], 2), np.uint8)], axis=1).view(np.uint64)
                rec[f"distinct_alpha_selectors_{k}"] = int(np.unique(sel).size)
        out[name] = rec
        print(name, rec, flush=True)
    with open(os.path.join(HERE, "qdxt_reference.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)


# crnlib-compatible API cases: (name, width, height, format, faces, content, seed, quality). The DDS
# files are written by the reference's crn_compress at quality 255 (plain encode, endpoint caching
# off so the blocks do not depend on encode order) and compared whole; at quality 128 (clustered
# DXT1) only the header and size are pinned.
FMT_ALL = dict(FMT, DXT5_CCxY=3, DXT5_xGxR=4, DXT5_xGBR=5, DXT5_AGBR=6)
COMPAT_DDS_CASES = [
    ("dds_dxt1_256", 256, 256, "DXT1", 1, "colour", 10, 255),
    ("dds_dxt1_100x60", 100, 60, "DXT1", 1, "colour", 11, 255),
    ("dds_dxt1_cube_32", 32, 32, "DXT1", 6, "colour", 12, 255),
    ("dds_dxt5_128", 128, 128, "DXT5", 1, "colour_alpha", 13, 255),
    ("dds_dxn_xy_128", 128, 128, "DXN_XY", 1, "normal", 15, 255),
    ("dds_dxn_yx_64", 64, 64, "DXN_YX", 1, "normal", 17, 255),
    ("dds_dxt5a_128", 128, 128, "DXT5A", 1, "colour_alpha", 16, 255),
    ("dds_ccxy_64", 64, 64, "DXT5_CCxY", 1, "colour_alpha", 18, 255),
    ("dds_xgxr_64", 64, 64, "DXT5_xGxR", 1, "normal", 19, 255),
    ("dds_xgbr_64", 64, 64, "DXT5_xGBR", 1, "colour_alpha", 20, 255),
    ("dds_agbr_64", 64, 64, "DXT5_AGBR", 1, "colour_alpha", 21, 255),
    ("dds_qdxt_dxt1_256", 256, 256, "DXT1", 1, "colour", 10, 128),
]
# rate control: (name, size, format, content, seed, target bits per texel)
BITRATE_CASES = [("dxt1_256_r1.2", 256, "DXT1", "colour", 31, 1.2), ("dxt1_256_r1.6", 256, "DXT1", "colour", 31, 1.6),
                 ("dxt1_256_r2.2", 256, "DXT1", "colour", 31, 2.2), ("dxt5_128_r3.0", 128, "DXT5", "colour_alpha", 32, 3.0),
                 ("dxt1_512_r1.0", 512, "DXT1", "colour", 33, 1.0)]


def make_bitrate() -> None:
    """The reference's crn_compress with m_target_bitrate on seeded mip chains: the quality level its
    search chose and the bitrate it reports (bitrate_reference.json)."""
    out = {}
    for name, size, fmt, content, seed, target in BITRATE_CASES:
        fl = texture_levels(size, size, content, seed, 1)
        flags = FLAG_PERCEPTUAL | FLAG_HIERARCHICAL | FLAG_BOTH_BLOCK_TYPES
        nbytes, q, rate = ref.compress_texture_bitrate(fl[0], FMT[fmt], flags, target, 7)
        out[name] = {"size": size, "format": fmt, "content": content, "seed": seed, "target": target,
                     "quality": q, "bitrate": rate, "bytes": nbytes}
        print(name, out[name], flush=True)
    with open(os.path.join(HERE, "bitrate_reference.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)


# crn_compress to .dds at quality 255 with the block encoder's other parameters: (name, w, h,
# format, content, seed, flags, dxt quality)
FLAG_BASE = FLAG_HIERARCHICAL | FLAG_NO_ENDPOINT_CACHING
COMPAT_DDS_OPTION_CASES = [
    ("dds_dxt1_fast_128", 128, 128, "DXT1", "colour", 30, FLAG_BASE | FLAG_PERCEPTUAL | FLAG_BOTH_BLOCK_TYPES, 1),
    ("dds_dxt1_normal_128", 128, 128, "DXT1", "colour", 31, FLAG_BASE | FLAG_PERCEPTUAL | FLAG_BOTH_BLOCK_TYPES, 2),
    ("dds_dxt1_superfast_uniform_64", 64, 64, "DXT1", "colour", 32, FLAG_BASE, 0),
    ("dds_dxt5_better_128", 128, 128, "DXT5", "colour_alpha", 33, FLAG_BASE | FLAG_PERCEPTUAL | FLAG_BOTH_BLOCK_TYPES, 3),
    ("dds_dxn_fast_64", 64, 64, "DXN_XY", "normal", 34, FLAG_BASE | FLAG_BOTH_BLOCK_TYPES, 1),
    ("dds_dxt1_gray_128", 128, 128, "DXT1", "colour", 35,
     FLAG_BASE | FLAG_PERCEPTUAL | FLAG_BOTH_BLOCK_TYPES | FLAG_GRAYSCALE, 4),
    ("dds_dxt1a_128", 128, 128, "DXT1", "colour_alpha", 36,
     FLAG_BASE | FLAG_PERCEPTUAL | FLAG_BOTH_BLOCK_TYPES | FLAG_DXT1A, 4),
    ("dds_dxt1a_better_64", 64, 64, "DXT1", "colour_alpha", 37,
     FLAG_BASE | FLAG_PERCEPTUAL | FLAG_BOTH_BLOCK_TYPES | FLAG_DXT1A, 3),
    ("dds_dxt1_black_128", 128, 128, "DXT1", "dark", 38,
     FLAG_BASE | FLAG_PERCEPTUAL | FLAG_BOTH_BLOCK_TYPES | FLAG_TRANSPARENT_BLACK, 4),
    ("dds_dxt1_black_normal_64", 64, 64, "DXT1", "dark", 39,
     FLAG_BASE | FLAG_BOTH_BLOCK_TYPES | FLAG_TRANSPARENT_BLACK, 2),
]


def make_compat_dds_options() -> None:
    """Whole .dds files of the reference's crn_compress at quality 255 below Uber dxt quality, with
    grayscale sampling, DXT1A and transparent indices for black: compat_reference.json "dds_opts"."""
    path = os.path.join(HERE, "compat_reference.json")
    with open(path) as fh:
        out = json.load(fh)
    out["dds_opts"] = {}
    for name, w, h, fmt, content, seed, flags, dq in COMPAT_DDS_OPTION_CASES:
        fl = texture_levels(w, h, content, seed, 1)
        dds = ref.compress_texture(fl, FMT_ALL[fmt], 1, 255, flags, dq, 7)
        out["dds_opts"][name] = {"width": w, "height": h, "format": fmt, "content": content, "seed": seed,
                                 "flags": flags, "dxt_quality": dq, "size": len(dds), "header": dds[:128].hex(),
                                 "sha256": sha(np.frombuffer(dds, np.uint8)),
                                 "input_sha256": sha(np.concatenate([im.reshape(-1) for f in fl for im in f]))}
        print(name, len(dds), flush=True)
    with open(path, "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)


# crn_compress with crn_mipmap_params, mips generated from the top level: (name, w, h, format,
# content, seed, file type, quality, mip mode, filter, blurriness, gamma filtering, tiled, max levels,
# min mip size)
COMPAT_MIP_CASES = [
    ("mips_dds_dxt1_kaiser_256", 256, 256, "DXT1", "colour", 30, 1, 255, 2, 4, 0.9, True, False, 16, 1),
    ("mips_dds_dxt5_box_wrap_128x64", 128, 64, "DXT5", "colour_alpha", 31, 1, 255, 0, 0, 1.0, False, True, 5, 1),
    ("mips_dds_dxt1_tent_min8_96", 96, 96, "DXT1", "colour", 32, 1, 255, 0, 1, 0.9, True, False, 16, 8),
    ("mips_crn_dxt1_kaiser_128", 128, 128, "DXT1", "colour", 33, 0, 128, 2, 4, 0.9, True, False, 16, 1),
]


def dds_flags(content: str, quality: int) -> int:
    base = FLAG_HIERARCHICAL | FLAG_BOTH_BLOCK_TYPES | FLAG_NO_ENDPOINT_CACHING
    return base | (0 if content == "normal" else FLAG_PERCEPTUAL)


def make_compat() -> None:
    """Reference outputs for the crnlib-compatible C++ API: whole .dds files of crn_compress (plain
    path, all formats incl. the swizzled DXT5 ones; cube and odd sizes), the clustered DDS header,
    crn_compress with generated mips, crn_decompress_crn_to_dds of every committed .crn, and the
    crnd header API (validate, texture / level info, level data, segmented files) on them."""
    out = {"dds": {}, "mips": {}, "crn_to_dds": {}, "crnd": {}}
    for name, w, h, fmt, faces, content, seed, q in COMPAT_DDS_CASES:
        fl = texture_levels(w, h, content, seed, faces)
        dds = ref.compress_texture(fl, FMT_ALL[fmt], 1, q, dds_flags(content, q), DXT_UBER, 7)
        out["dds"][name] = {"width": w, "height": h, "format": fmt, "faces": faces, "content": content, "seed": seed,
                            "quality": q, "flags": dds_flags(content, q), "size": len(dds),
                            "header": dds[:128].hex(), "sha256": sha(np.frombuffer(dds, np.uint8)),
                            "input_sha256": sha(np.concatenate([im.reshape(-1) for f in fl for im in f]))}
        print(name, len(dds), flush=True)
    for name, w, h, fmt, content, seed, ft, q, mode, filt, blur, gamma, tiled, maxl, minsz in COMPAT_MIP_CASES:
        top = texture_levels(w, h, content, seed, 1)[0][0]
        flags = dds_flags(content, q)
        data = ref.compress_mips([top], FMT_ALL[fmt], ft, q, flags, mode, filt, blur, gamma, tiled, maxl, minsz)
        out["mips"][name] = {"width": w, "height": h, "format": fmt, "content": content, "seed": seed, "file_type": ft,
                             "quality": q, "flags": flags, "mip_mode": mode, "filter": filt, "blurriness": blur,
                             "gamma_filtering": gamma, "tiled": tiled, "max_levels": maxl, "min_mip_size": minsz,
                             "size": len(data), "sha256": sha(np.frombuffer(data, np.uint8)),
                             "header": data[:128].hex() if ft == 1 else None}
        print(name, len(data), flush=True)
    compat_crnd(out, sorted(CASE[0] for CASE in CRN_CASES))
    with open(os.path.join(HERE, "compat_reference.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)


def compat_crnd(out: dict, names) -> None:
    """crn_decompress_crn_to_dds and the crnd header API of the reference on the committed .crn
    files `names`, into out["crn_to_dds"] / out["crnd"]."""
    for name in names:
        with open(os.path.join(HERE, "crn", name + ".crn"), "rb") as fh:
            crn = fh.read()
        dds = ref.crn_to_dds(crn)
        out["crn_to_dds"][name] = {"size": len(dds), "sha256": sha(np.frombuffer(dds, np.uint8)),
                                   "header": dds[:128].hex()}
        values, seg = ref.crnd_probe(crn)
        out["crnd"][name] = {"values": values, "segmented_sha256": sha(np.frombuffer(seg, np.uint8)) if seg else None}


# mip generation cases: (name, width, height, content, seed, filter, filter scale, sRGB, wrap, comps)
MIP_CASES = [("kaiser_64x48_rgba", 64, 48, "colour_alpha", 40, "kaiser", 0.9, True, False, 4),
             ("lanczos4_37x20_rgb", 37, 20, "colour", 41, "lanczos4", 1.0, True, False, 3),
             ("box_32x32_linear", 32, 32, "colour_alpha", 42, "box", 1.0, False, False, 4),
             ("tent_50x64_wrap", 50, 64, "colour_alpha", 43, "tent", 1.0, True, True, 4),
             ("mitchell_16x40_linear_rgb", 16, 40, "colour", 44, "mitchell", 0.9, False, False, 3),
             ("kaiser_1x64", 1, 64, "colour_alpha", 45, "kaiser", 0.9, True, False, 4),
             ("kaiser_128x128_normal", 128, 128, "normal", 46, "kaiser", 0.9, False, True, 3)]


def make_mips() -> None:
    """The reference's mip generation (mipmapped_texture::generate_mipmaps with its resampler) on
    small seeded images: every level for each of the five mip filters, gamma on and off, clamp and
    wrap addressing, 3 and 4 components, a 1-texel-wide image."""
    arrays, meta = {}, {}
    for name, w, h, content, seed, filt, scale, srgb, wrap, comps in MIP_CASES:
        img = texgen.normal_map(w, h, seed) if content == "normal" else \
            texgen.colour_texture(w, h, seed, with_alpha_noise=(content == "colour_alpha"))
        levels = ref.generate_mipmaps(img, filt, scale, srgb, wrap, comps)
        arrays[name + "_base"] = img
        arrays[name + "_levels"] = np.concatenate([l.reshape(-1) for l in levels[1:]])
        meta[name] = {"width": w, "height": h, "filter": filt, "filter_scale": scale, "srgb": srgb, "wrap": wrap,
                      "comps": comps, "levels": len(levels)}
    np.savez_compressed(os.path.join(HERE, "mips.npz"), **arrays)
    with open(os.path.join(HERE, "mips.json"), "w") as fh:
        json.dump(meta, fh, indent=1, sort_keys=True)


# 2048x2048 DXT5 (colour + alpha noise) and DXN_XY (normal map) mip chains at quality 128
CONFIG2_CASES = [("dxt5_2048", "DXT5", 2, 2048, 200, "colour_alpha"), ("dxn_xy_2048", "DXN_XY", 7, 2048, 201, "normal")]


def level_quality(dxt_levels, src_levels, fmt):
    """RMSEs of decoded blocks against the source mip chain (all levels, visible blocks): RGB and
    alpha for DXT5, the two channels together for DXN."""
    sys.path.insert(0, os.path.dirname(HERE))
    from dxt_decode import rgb_rmse, dxt5a_values
    dec = np.concatenate(dxt_levels)
    src = np.concatenate([texgen.image_blocks(im) for im in src_levels]).reshape(-1, 16, 4).astype(np.int64)
    if fmt == "DXT5":
        a = dxt5a_values(dec[:, :8])
        return {"rmse_color": rgb_rmse(dec[:, 8:], src.reshape(-1, 64).astype(np.uint8)),
                "rmse_alpha": float(np.sqrt(((a - src[:, :, 3]) ** 2).mean()))}
    x, y = dxt5a_values(dec[:, :8]), dxt5a_values(dec[:, 8:])
    return {"rmse_xy": float(np.sqrt((((x - src[:, :, 0]) ** 2).sum() + ((y - src[:, :, 1]) ** 2).sum()) / (2 * x.size)))}


def make_config2() -> None:
    """The reference's crn_compress (.crn, q128, its default flags) on the 2048x2048 DXT5 and DXN
    textures: file size and the RMSEs of its crnd-decoded blocks, the bar for the GPU path at that
    size (the .crn files themselves are too large to commit)."""
    import time
    out = {}
    for name, fmt, code, size, seed, content in CONFIG2_CASES:
        fl = texture_levels(size, size, content, seed, 1)
        flags = (0 if content == "normal" else FLAG_PERCEPTUAL) | FLAG_HIERARCHICAL | FLAG_BOTH_BLOCK_TYPES
        t = time.time()
        crn = ref.compress_texture(fl, code, 0, 128, flags, DXT_UBER, 7)
        secs = time.time() - t
        bpb = 16
        dxt = []
        for lvl in range(len(fl[0])):
            w, h = max(1, size >> lvl), max(1, size >> lvl)
            dxt.append(ref.unpack_level(crn, lvl, level_bytes(size, size, lvl, bpb, 1)).reshape(-1, bpb))
        texels = sum(im.shape[0] * im.shape[1] for im in fl[0])
        out[name] = {"size": size, "seed": seed, "format": fmt, "content": content, "quality": 128,
                     "levels": len(fl[0]), "bytes": len(crn), "bits_per_texel": 8 * len(crn) / texels,
                     "crn_sha256": sha(crn), "seconds_8_threads_x86": round(secs, 2),
                     **level_quality(dxt, fl[0], fmt)}
        print(name, out[name], flush=True)
    with open(os.path.join(HERE, "config2_reference.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    if not ref.available():
        sys.exit("oracle/_ref/libcrnref.so missing: run `make -C oracle ref` where the reference tree exists")
    if sys.argv[1:] == ["quality"]:
        make_quality()
        make_compat_dds_options()
        sys.exit(0)
    if sys.argv[1:] == ["bitrate"]:
        make_bitrate()
        sys.exit(0)
    if sys.argv[1:] == ["crn2048"]:
        make_crn(only=("dxt5_2048", "dxn_xy_2048"))
        with open(os.path.join(HERE, "compat_reference.json")) as fh:
            compat = json.load(fh)
        compat_crnd(compat, ("dxt5_2048", "dxn_xy_2048"))
        with open(os.path.join(HERE, "compat_reference.json"), "w") as fh:
            json.dump(compat, fh, indent=1, sort_keys=True)
        sys.exit(0)
    if sys.argv[1:] == ["config2"]:
        make_config2()
        sys.exit(0)
    if sys.argv[1:] == ["mips"]:
        make_mips()
        sys.exit(0)
    if sys.argv[1:] == ["qdxt"]:
        make_qdxt()
        sys.exit(0)
    if sys.argv[1:] == ["compat"]:
        make_compat()
        sys.exit(0)
    if sys.argv[1:] == ["hc_alpha"]:
        make_hc(alpha_only=True)
        sys.exit(0)
    make_blocks()
    make_quality()
    make_crn()
    make_hc()
    make_config2()
    make_mips()
    make_qdxt()
    make_compat()
    make_compat_dds_options()
    make_bitrate()
    print("golden fixtures written to", HERE)
