"""ctypes bindings to oracle/_ref/libcrnref.so: the reference crnlib compiled from its own
sources by oracle/Makefile (target `ref`). Test infrastructure only: used to generate and
re-check the golden fixtures under tests/golden/. The library only exists where the reference
tree is available (the build container); on other hosts `available()` is False."""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_PATH = os.path.join(_HERE, "_ref", "libcrnref.so")
_lib = None

_u8p = ctypes.POINTER(ctypes.c_uint8)
_u32 = ctypes.c_uint32


def available() -> bool:
    return os.path.exists(_PATH)


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(_PATH)
        L.ref_compress_blocks.argtypes = [ctypes.c_void_p, _u32, _u32, _u32, _u32, ctypes.c_void_p]
        L.ref_compress_blocks.restype = ctypes.c_int
        L.ref_compress_blocks_mt.argtypes = [ctypes.c_void_p, _u32, _u32, _u32, _u32, ctypes.c_void_p, _u32,
                                             ctypes.POINTER(ctypes.c_double)]
        L.ref_compress_blocks_mt.restype = ctypes.c_int
        L.ref_compress_texture.argtypes = [ctypes.c_void_p, _u32, _u32, _u32, _u32, _u32, _u32, _u32, _u32, _u32,
                                           _u32, ctypes.c_void_p, _u32]
        L.ref_compress_texture.restype = _u32
        L.ref_compress_texture_bitrate.argtypes = [ctypes.c_void_p, _u32, _u32, _u32, _u32, _u32, ctypes.c_float, _u32,
                                                   ctypes.POINTER(_u32), ctypes.POINTER(ctypes.c_float)]
        L.ref_compress_texture_bitrate.restype = _u32
        L.ref_unpack_level.argtypes = [ctypes.c_void_p, _u32, _u32, ctypes.c_void_p, _u32]
        L.ref_unpack_level.restype = _u32
        L.ref_time_unpack.argtypes = [ctypes.c_void_p, _u32, _u32, ctypes.c_void_p, _u32]
        L.ref_time_unpack.restype = ctypes.c_double
        L.ref_dxt_hc_dxt1.argtypes = [ctypes.c_void_p, _u32, _u32, ctypes.c_void_p, _u32, _u32, _u32, ctypes.c_int,
                                      _u32, ctypes.c_void_p, ctypes.c_void_p]
        L.ref_dxt_hc_dxt1.restype = ctypes.c_int
        L.ref_dxt_hc_alpha.argtypes = [ctypes.c_void_p, _u32, _u32, ctypes.c_void_p, _u32, _u32, ctypes.c_void_p,
                                       ctypes.c_int, _u32, ctypes.c_void_p, ctypes.c_void_p]
        L.ref_dxt_hc_alpha.restype = ctypes.c_int
        L.ref_resample.argtypes = [ctypes.c_void_p, _u32, _u32, _u32, _u32, ctypes.c_char_p, ctypes.c_float,
                                   ctypes.c_int, ctypes.c_int, _u32, ctypes.c_void_p]
        L.ref_resample.restype = ctypes.c_int
        L.ref_compress_mips.argtypes = [ctypes.c_void_p, _u32, _u32, _u32, _u32, _u32, _u32, _u32, _u32, _u32,
                                        ctypes.c_float, _u32, _u32, _u32, _u32, ctypes.c_void_p, _u32]
        L.ref_compress_mips.restype = _u32
        L.ref_crn_to_dds.argtypes = [ctypes.c_void_p, _u32, ctypes.c_void_p, _u32]
        L.ref_crn_to_dds.restype = _u32
        L.ref_crnd_probe.argtypes = [ctypes.c_void_p, _u32, ctypes.c_void_p, ctypes.c_void_p, _u32]
        L.ref_crnd_probe.restype = _u32
        _lib = L
    return _lib


def compress_blocks(blocks: np.ndarray, fmt: int, flags: int, dxt_quality: int = 4, threads: int = 1) -> np.ndarray:
    """blocks: (n, 64) uint8 RGBA 4x4 blocks -> (n, bytes_per_block) uint8 DXT blocks."""
    blocks = np.ascontiguousarray(blocks, dtype=np.uint8)
    n = blocks.shape[0]
    out = np.zeros(n * 16, np.uint8)
    if threads > 1:
        secs = ctypes.c_double()
        bpb = lib().ref_compress_blocks_mt(blocks.ctypes.data, n, fmt, flags, dxt_quality, out.ctypes.data, threads,
                                           ctypes.byref(secs))
    else:
        bpb = lib().ref_compress_blocks(blocks.ctypes.data, n, fmt, flags, dxt_quality, out.ctypes.data)
    if bpb <= 0:
        raise RuntimeError("reference block compressor failed")
    return out[: n * bpb].reshape(n, bpb)


def compress_texture(levels_faces: list[list[np.ndarray]], fmt: int, file_type: int, quality: int, flags: int,
                     dxt_quality: int = 4, helper_threads: int = 0) -> bytes:
    """levels_faces[f][l] = (h, w, 4) uint8 images -> .crn (file_type 0) / .dds (1) bytes."""
    faces = len(levels_faces)
    levels = len(levels_faces[0])
    h, w = levels_faces[0][0].shape[:2]
    flat = np.concatenate([np.ascontiguousarray(im).reshape(-1) for face in levels_faces for im in face])
    cap = max(1 << 20, flat.size * 2)
    out = np.zeros(cap, np.uint8)
    size = lib().ref_compress_texture(flat.ctypes.data, w, h, levels, faces, fmt, file_type, quality, flags,
                                      dxt_quality, helper_threads, out.ctypes.data, cap)
    if size == 0 or size > cap:
        raise RuntimeError("reference crn_compress failed")
    return out[:size].tobytes()


def unpack_level(crn: bytes, level: int, out_size: int) -> np.ndarray:
    src = np.frombuffer(crn, np.uint8)
    out = np.zeros(out_size, np.uint8)
    n = lib().ref_unpack_level(src.ctypes.data, len(crn), level, out.ctypes.data, out_size)
    if n == 0:
        raise RuntimeError("reference crnd_unpack_level failed")
    return out[:n]


def dxt_hc_dxt1(blocks: np.ndarray, levels, faces: int, endpoint_codebook: int, selector_codebook: int,
                perceptual: bool = True, threads: int = 8):
    """The reference's dxt_hc::compress for DXT1 on blocks in crn_comp's layout.
    levels: (first_block, num_blocks, block_width) per level. Returns ((n, 8) DXT1 blocks,
    {tiles, endpoints, selectors})."""
    blocks = np.ascontiguousarray(blocks, dtype=np.uint8)
    n = blocks.shape[0]
    info = np.array([v for lv in levels for v in lv], np.uint32)
    out = np.zeros(n * 8, np.uint8)
    stats = np.zeros(4, np.uint32)
    if not lib().ref_dxt_hc_dxt1(blocks.ctypes.data, n, len(levels), info.ctypes.data, faces, endpoint_codebook,
                                 selector_codebook, int(perceptual), threads, out.ctypes.data, stats.ctypes.data):
        raise RuntimeError("reference dxt_hc failed")
    return out.reshape(n, 8), {"tiles": int(stats[0]), "endpoints": int(stats[1]), "selectors": int(stats[2])}


def dxt_hc_alpha(blocks: np.ndarray, levels, faces: int, fmt: str, codebooks, perceptual: bool = True, threads: int = 8):
    """The reference's dxt_hc::compress for DXT5 (alpha = channel 3), DXN_XY, DXN_YX or DXT5A.
    Returns ((n, 16 or 8) blocks, stats)."""
    code = {"DXT5": 0, "DXN_XY": 1, "DXN_YX": 2, "DXT5A": 3}[fmt]
    blocks = np.ascontiguousarray(blocks, dtype=np.uint8)
    n = blocks.shape[0]
    info = np.array([v for lv in levels for v in lv], np.uint32)
    cb = np.array(codebooks, np.uint32)
    out = np.zeros(n * 16, np.uint8)
    stats = np.zeros(8, np.uint32)
    bpb = lib().ref_dxt_hc_alpha(blocks.ctypes.data, n, len(levels), info.ctypes.data, faces, code, cb.ctypes.data,
                                 int(perceptual), threads, out.ctypes.data, stats.ctypes.data)
    if bpb <= 0:
        raise RuntimeError("reference dxt_hc failed")
    return out[: n * bpb].reshape(n, bpb), {"tiles": int(stats[0]), "color_endpoints": int(stats[1]),
                                            "color_selectors": int(stats[2]), "alpha_endpoints": int(stats[3]),
                                            "alpha_selectors": int(stats[4])}


def resample(rgba: np.ndarray, dst_w: int, dst_h: int, filt: str, filter_scale: float, srgb: bool, wrap: bool,
             num_comps: int) -> np.ndarray:
    """The reference's image_utils::resample_multithreaded: (h, w, 4) uint8 -> (dst_h, dst_w, 4)."""
    src = np.ascontiguousarray(rgba, dtype=np.uint8)
    out = np.zeros((dst_h, dst_w, 4), np.uint8)
    ok = lib().ref_resample(src.ctypes.data, src.shape[1], src.shape[0], dst_w, dst_h, filt.encode(), filter_scale,
                            int(srgb), int(wrap), num_comps, out.ctypes.data)
    if not ok:
        raise RuntimeError("reference resample failed")
    return out


def generate_mipmaps(rgba: np.ndarray, filt: str, filter_scale: float, srgb: bool, wrap: bool, num_comps: int):
    """mipmapped_texture::generate_mipmaps (crnlib/crn_mipmapped_texture.cpp:2140-2215): every level
    resampled from the level-0 image down to 1x1 (min mip size 1)."""
    h, w = rgba.shape[:2]
    levels = [np.ascontiguousarray(rgba)]
    l = 1
    while (w >> (l - 1)) > 1 or (h >> (l - 1)) > 1:
        levels.append(resample(rgba, max(1, w >> l), max(1, h >> l), filt, filter_scale, srgb, wrap, num_comps))
        l += 1
    return levels


def compress_mips(faces_top: list[np.ndarray], fmt: int, file_type: int, quality: int, flags: int, mip_mode: int = 2,
                  filt: int = 4, blurriness: float = 0.9, gamma_filtering: bool = True, tiled: bool = False,
                  max_levels: int = 16, min_mip_size: int = 1) -> bytes:
    """crn_compress with crn_mipmap_params from the top level of each face -> .crn / .dds bytes."""
    h, w = faces_top[0].shape[:2]
    flat = np.concatenate([np.ascontiguousarray(im, dtype=np.uint8).reshape(-1) for im in faces_top])
    cap = max(1 << 20, flat.size * 2)
    out = np.zeros(cap, np.uint8)
    size = lib().ref_compress_mips(flat.ctypes.data, w, h, len(faces_top), fmt, file_type, quality, flags, mip_mode,
                                   filt, blurriness, int(gamma_filtering), int(tiled), max_levels, min_mip_size,
                                   out.ctypes.data, cap)
    if size == 0 or size > cap:
        raise RuntimeError("reference crn_compress (mip params) failed")
    return out[:size].tobytes()


def crn_to_dds(crn: bytes) -> bytes:
    buf = np.frombuffer(crn, np.uint8)
    cap = 64 << 20
    out = np.zeros(cap, np.uint8)
    size = lib().ref_crn_to_dds(buf.ctypes.data, len(crn), out.ctypes.data, cap)
    if size == 0 or size > cap:
        raise RuntimeError("reference crn_decompress_crn_to_dds failed")
    return out[:size].tobytes()


def crnd_probe(crn: bytes):
    """(values, segmented base file) from the reference's crnd header API (ref_crnd_probe)."""
    buf = np.frombuffer(crn, np.uint8)
    info = np.zeros(4096, np.uint32)
    seg = np.zeros(len(crn), np.uint8)
    n = lib().ref_crnd_probe(buf.ctypes.data, len(crn), info.ctypes.data, seg.ctypes.data, len(crn))
    values = [int(v) for v in info[:n]]
    base = values[-2]
    return values, seg[:base].tobytes() if values[-1] else b""


def compress_texture_bitrate(levels: list[np.ndarray], fmt: int, flags: int, target: float,
                             helper_threads: int = 0) -> tuple[int, int, float]:
    """crn_compress (.crn) of one face's mip chain with m_target_bitrate: (file size, chosen quality
    level, reported bitrate)."""
    flat = np.ascontiguousarray(np.concatenate([np.ascontiguousarray(l, dtype=np.uint8).reshape(-1) for l in levels]))
    h, w = levels[0].shape[:2]
    q, rate = _u32(0), ctypes.c_float(0)
    size = lib().ref_compress_texture_bitrate(flat.ctypes.data, w, h, len(levels), fmt, flags, target, helper_threads,
                                              ctypes.byref(q), ctypes.byref(rate))
    if not size:
        raise RuntimeError("reference crn_compress with a target bitrate failed")
    return int(size), int(q.value), float(rate.value)
