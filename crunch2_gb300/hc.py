"""Clustered (CRN-style) DXT1 compression through the crngpu C ABI: crn_comp's block layout and
codebook sizes (crnlib/crn_comp.cpp:424-463, 541-577, 713-741) around crngpu_hc_compress_dxt1,
the GPU restatement of dxt_hc::compress (crnlib/crn_dxt_hc.cpp:97-316)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import lib, _check, CrnGpuError, E_PARAM, FMT_DXT1, FMT_DXT5, FMT_DXN_XY, FMT_DXN_YX, FMT_DXT5A


class HcParams(ctypes.Structure):
    class _Level(ctypes.Structure):
        _fields_ = [("first_block", ctypes.c_uint32), ("num_blocks", ctypes.c_uint32),
                    ("block_width", ctypes.c_uint32), ("weight", ctypes.c_float)]
    _fields_ = [("struct_size", ctypes.c_uint32), ("num_blocks", ctypes.c_uint32), ("num_levels", ctypes.c_uint32),
                ("num_faces", ctypes.c_uint32), ("perceptual", ctypes.c_int32),
                ("color_endpoint_codebook_size", ctypes.c_uint32), ("color_selector_codebook_size", ctypes.c_uint32),
                ("adaptive_tile_color_psnr_derating", ctypes.c_float), ("vq_round_fraction", ctypes.c_uint32),
                ("alpha_endpoint_codebook_size", ctypes.c_uint32), ("alpha_selector_codebook_size", ctypes.c_uint32),
                ("adaptive_tile_alpha_psnr_derating", ctypes.c_float), ("color_alpha_weighting_ratio", ctypes.c_float),
                ("alpha_component", ctypes.c_uint32), ("levels", _Level * 16)]


class HcStats(ctypes.Structure):
    _fields_ = [("color_endpoints", ctypes.c_uint32), ("color_selectors", ctypes.c_uint32),
                ("tiles", ctypes.c_uint32), ("reserved", ctypes.c_uint32), ("sse_endpoints", ctypes.c_double),
                ("sse_final", ctypes.c_double), ("alpha_endpoints", ctypes.c_uint32), ("alpha_selectors", ctypes.c_uint32),
                ("sse_alpha", ctypes.c_double)]


def _bind():
    L = lib()
    if getattr(L, "_hc_bound", False):
        return L
    vp = ctypes.c_void_p
    L.crngpu_hc_compress_dxt1.argtypes = [vp, ctypes.POINTER(HcParams), vp, vp, vp, vp, vp, ctypes.POINTER(HcStats), vp]
    L.crngpu_hc_compress_dxt1.restype = ctypes.c_int
    L.crngpu_hc_compress.argtypes = [vp, ctypes.POINTER(HcParams), ctypes.c_uint32, vp, ctypes.POINTER(HcStats), vp]
    L.crngpu_hc_compress.restype = ctypes.c_int
    L.crngpu_hc_codebook_sizes.argtypes = [ctypes.c_uint32] * 4 + [ctypes.POINTER(ctypes.c_uint32)]
    L.crngpu_hc_codebook_sizes.restype = ctypes.c_int
    L._hc_bound = True
    return L


def codebook_sizes(width: int, height: int, quality: int, fmt: int = FMT_DXT1):
    """(colour endpoints, colour selectors, alpha endpoints, alpha selectors) for a quality level."""
    out = (ctypes.c_uint32 * 4)()
    _check(_bind().crngpu_hc_codebook_sizes(width, height, quality, fmt, out), "crngpu_hc_codebook_sizes")
    return tuple(int(v) for v in out)


def crn_layout(faces_levels):
    """faces_levels[face][level] RGBA8 images -> (blocks (n, 64) uint8 in crn_comp's order, per-level
    (first_block, num_blocks, block_width), per-level visible (blocks_x, blocks_y, padded width)).
    Each level is padded to a multiple of 8 texels by edge clamping (crnlib/crn_comp.cpp:454-463,
    717-741); faces of a level are consecutive."""
    from .texgen import image_blocks
    nlev = len(faces_levels[0])
    parts, levels, vis = [], [], []
    first = 0
    for l in range(nlev):
        h, w = faces_levels[0][l].shape[:2]
        pw, ph = (w + 7) & ~7, (h + 7) & ~7
        level_blocks = []
        for f in range(len(faces_levels)):
            img = faces_levels[f][l]
            pad = np.pad(img, ((0, ph - h), (0, pw - w), (0, 0)), mode="edge")
            level_blocks.append(image_blocks(pad))
        lb = np.concatenate(level_blocks)
        parts.append(lb)
        levels.append((first, lb.shape[0], pw // 4))
        vis.append(((w + 3) // 4, (h + 3) // 4, pw // 4))
        first += lb.shape[0]
    return np.ascontiguousarray(np.concatenate(parts)), levels, vis


def compress_dxt1(faces_levels, quality: int = 128, perceptual: bool = True, stream=None, with_indices=False,
                  codebook=None, vq_round_fraction: int = 0):
    """Clustered DXT1 of a mip chain (faces_levels[face][level]): returns (per level, per face, the
    visible DXT1 blocks (by, bx, 8)), stats dict[, index arrays])."""
    import torch
    L = _bind()
    blocks, levels, vis = crn_layout(faces_levels)
    h0, w0 = faces_levels[0][0].shape[:2]
    ce, cs = codebook if codebook else codebook_sizes(w0, h0, quality)[:2]
    p = HcParams()
    p.struct_size = ctypes.sizeof(HcParams)
    p.num_blocks = blocks.shape[0]
    p.num_levels = len(levels)
    p.num_faces = len(faces_levels)
    p.perceptual = int(perceptual)
    p.color_endpoint_codebook_size = ce
    p.color_selector_codebook_size = cs
    p.adaptive_tile_color_psnr_derating = 2.0
    p.vq_round_fraction = vq_round_fraction
    for i, (fb, nb, bw) in enumerate(levels):
        p.levels[i].first_block, p.levels[i].num_blocks, p.levels[i].block_width = fb, nb, bw
        p.levels[i].weight = min(12.0, 1.3 ** i)
    d_blocks = torch.from_numpy(blocks).cuda()
    n = blocks.shape[0]
    out = torch.empty((n, 8), dtype=torch.uint8, device="cuda")
    idx = None
    ptrs = [None] * 4
    if with_indices:
        idx = {"endpoint_index": torch.empty(n, dtype=torch.int16, device="cuda"),
               "selector_index": torch.empty(n, dtype=torch.int16, device="cuda"),
               "endpoints": torch.empty(8192, dtype=torch.int32, device="cuda"),
               "selectors": torch.empty(8192, dtype=torch.int32, device="cuda")}
        ptrs = [v.data_ptr() for v in idx.values()]
    st = HcStats()
    sp = None if stream is None else getattr(stream, "cuda_stream", stream)
    _check(L.crngpu_hc_compress_dxt1(d_blocks.data_ptr(), ctypes.byref(p), out.data_ptr(), *ptrs, ctypes.byref(st), sp),
           "crngpu_hc_compress_dxt1")
    host = out.cpu().numpy()
    res = []
    for (fb, nb, bw), (bx, by, _) in zip(levels, vis):
        faces = []
        per_face = nb // len(faces_levels)
        for f in range(len(faces_levels)):
            g = host[fb + f * per_face: fb + (f + 1) * per_face].reshape(-1, bw, 8)
            faces.append(g[:by, :bx])
        res.append(faces)
    stats = {"color_endpoints": st.color_endpoints, "color_selectors": st.color_selectors, "tiles": st.tiles,
             "codebook_request": (ce, cs), "blocks": n,
             "rmse_endpoints_all_blocks": (st.sse_endpoints / (n * 48)) ** 0.5,
             "rmse_final_all_blocks": (st.sse_final / (n * 48)) ** 0.5}
    if with_indices:
        return res, stats, {k: v.cpu().numpy() for k, v in idx.items()}
    return res, stats


def _params(blocks, levels, nfaces, perceptual, sizes, vq_round_fraction=0, alpha_component=3):
    p = HcParams()
    p.struct_size = ctypes.sizeof(HcParams)
    p.num_blocks = blocks.shape[0]
    p.num_levels = len(levels)
    p.num_faces = nfaces
    p.perceptual = int(perceptual)
    p.color_endpoint_codebook_size, p.color_selector_codebook_size = sizes[0], sizes[1]
    p.alpha_endpoint_codebook_size, p.alpha_selector_codebook_size = sizes[2], sizes[3]
    p.adaptive_tile_color_psnr_derating = 2.0
    p.adaptive_tile_alpha_psnr_derating = 2.0
    p.color_alpha_weighting_ratio = 3.0
    p.alpha_component = alpha_component
    p.vq_round_fraction = vq_round_fraction
    for i, (fb, nb, bw) in enumerate(levels):
        p.levels[i].first_block, p.levels[i].num_blocks, p.levels[i].block_width = fb, nb, bw
        p.levels[i].weight = min(12.0, 1.3 ** i)
    return p


def compress(faces_levels, fmt: int, quality: int = 128, perceptual=None, stream=None, codebook=None,
             vq_round_fraction: int = 0, alpha_component: int = 3):
    """Clustered encode (crn_comp's dxt_hc stage) of a mip chain in DXT1, DXT5, DXN_XY/YX or DXT5A.
    perceptual defaults to crn_comp's choice (on for DXT1/DXT5, off for DXN/DXT5A). Returns (per
    level, per face, the visible blocks (by, bx, bytes per block)), stats dict)."""
    import torch
    L = _bind()
    blocks, levels, vis = crn_layout(faces_levels)
    h0, w0 = faces_levels[0][0].shape[:2]
    sizes = codebook if codebook else codebook_sizes(w0, h0, quality, fmt)
    if perceptual is None:
        perceptual = fmt in (FMT_DXT1, FMT_DXT5)
    p = _params(blocks, levels, len(faces_levels), perceptual, sizes, vq_round_fraction, alpha_component)
    bpb = 8 if fmt in (FMT_DXT1, FMT_DXT5A) else 16
    d_blocks = torch.from_numpy(blocks).cuda()
    n = blocks.shape[0]
    out = torch.empty((n, bpb), dtype=torch.uint8, device="cuda")
    st = HcStats()
    sp = None if stream is None else getattr(stream, "cuda_stream", stream)
    _check(L.crngpu_hc_compress(d_blocks.data_ptr(), ctypes.byref(p), fmt, out.data_ptr(), ctypes.byref(st), sp),
           "crngpu_hc_compress")
    host = out.cpu().numpy()
    res = []
    for (fb, nb, bw), (bx, by, _) in zip(levels, vis):
        per_face = nb // len(faces_levels)
        res.append([host[fb + f * per_face: fb + (f + 1) * per_face].reshape(-1, bw, bpb)[:by, :bx]
                    for f in range(len(faces_levels))])
    stats = {"color_endpoints": st.color_endpoints, "color_selectors": st.color_selectors, "tiles": st.tiles,
             "alpha_endpoints": st.alpha_endpoints, "alpha_selectors": st.alpha_selectors,
             "codebook_request": tuple(sizes), "blocks": n}
    return res, stats
