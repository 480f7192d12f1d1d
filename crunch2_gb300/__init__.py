"""crunch2_gb300: GB300-native crnlib DXTn hot path (DXT1/DXT5A block encode, CRN -> DXTn transcode).

The compute lives in libcrngpu.so (C ABI, include/crngpu.h; CUDA kernels for sm_103a). This module
is a thin ctypes host mirror of the reference's interfaces for the path:

  crnlib (inc/crnlib.h)                      this module
  ---------------------------------------    ----------------------------------------------
  dxt1_endpoint_optimizer::compute           dxt1_optimize(blocks, perceptual, use_alpha_blocks)
  dxt5_endpoint_optimizer::compute           dxt5a_optimize(blocks, comp_index, use_both_block_types)
  crn_compress_block (batched)               compress_blocks(blocks, fmt, flags)
  crn_compress, quality 255 (.dds blocks)    compress_image(rgba, fmt, flags)
  crnd_unpack_begin / _level / _end          unpack_begin / unpack_level / unpack_end
  crn_decompress (emscripten wrapper)        crn_decompress(src, first_level, level_count)

There is no CPU fallback: if the library is missing or a call fails, an exception is raised.
Arrays may be numpy arrays (host) or torch CUDA tensors (device; the call is then asynchronous on
the given stream).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import texgen  # noqa: F401  (seeded synthetic inputs)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libcrngpu.so")

OK, E_PARAM, E_CORRUPT, E_DEVICE, E_UNSUPPORTED, E_NOMEM = 0, -1, -2, -3, -4, -5
MEM_HOST, MEM_DEVICE = 0, 1
FMT_DXT1, FMT_DXT5, FMT_DXN_XY, FMT_DXN_YX, FMT_DXT5A = 0, 2, 7, 8, 9
FLAG_PERCEPTUAL, FLAG_USE_BOTH_BLOCK_TYPES = 1, 8
FLAG_TRANSPARENT_BLACK, FLAG_DXT1A, FLAG_GRAYSCALE = 16, 128, 256
# crn_dxt_quality
DXT_SUPERFAST, DXT_FAST, DXT_NORMAL, DXT_BETTER, DXT_UBER = 0, 1, 2, 3, 4


class CrnGpuError(RuntimeError):
    def __init__(self, code: int, where: str):
        super().__init__(f"{where} failed ({code}): {last_error()}")
        self.code = code


class _Dxt1Params(ctypes.Structure):
    """crngpu_dxt1_params"""
    _fields_ = [("struct_size", ctypes.c_uint32), ("perceptual", ctypes.c_int32),
                ("use_alpha_blocks", ctypes.c_int32), ("reserved", ctypes.c_int32), ("dxt_quality", ctypes.c_uint32),
                ("grayscale_sampling", ctypes.c_int32), ("dxt1a", ctypes.c_int32),
                ("dxt1a_alpha_threshold", ctypes.c_uint32), ("use_transparent_indices_for_black", ctypes.c_int32)]


class _BlockOptions(ctypes.Structure):
    """crngpu_block_options"""
    _fields_ = [("struct_size", ctypes.c_uint32), ("dxt_quality", ctypes.c_uint32),
                ("dxt1a_alpha_threshold", ctypes.c_uint32)]


_lib = None


class _BatchItem(ctypes.Structure):
    """crngpu_unpack_batch_item"""
    _fields_ = [("ctx", ctypes.c_void_p), ("first_level", ctypes.c_uint32), ("level_count", ctypes.c_uint32),
                ("dst", ctypes.c_void_p), ("dst_size", ctypes.c_uint64)]


class _CrnBatchItem(ctypes.Structure):
    _fields_ = [("rgba_levels", ctypes.c_void_p), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("levels", ctypes.c_uint32), ("faces", ctypes.c_uint32), ("format", ctypes.c_uint32),
                ("quality_level", ctypes.c_uint32), ("flags", ctypes.c_uint32), ("out", ctypes.c_void_p),
                ("out_capacity", ctypes.c_uint64), ("result", ctypes.c_int64)]


class _WaitStats(ctypes.Structure):
    """crngpu_wait_stats"""
    _fields_ = [("encode_stage_timeouts", ctypes.c_uint32), ("encode_drain_failures", ctypes.c_uint32),
                ("expand_stage_timeouts", ctypes.c_uint32), ("expand_drain_failures", ctypes.c_uint32),
                ("mma_wait_timeouts", ctypes.c_uint32)]


class _EncodeItem(ctypes.Structure):
    _fields_ = [("rgba", ctypes.c_void_p), ("out", ctypes.c_void_p), ("width", ctypes.c_uint32),
                ("height", ctypes.c_uint32), ("levels", ctypes.c_uint32), ("format", ctypes.c_uint32)]


def lib():
    """Loads libcrngpu.so (building it first if it is missing). Raises if that fails."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from .build import build
        build()
    L = ctypes.CDLL(LIB_PATH)
    vp, u32, i32, i64, u64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_int64, ctypes.c_uint64
    L.crngpu_version.restype = ctypes.c_char_p
    L.crngpu_last_error.restype = ctypes.c_char_p
    L.crngpu_dxt1_optimize_batch.argtypes = [vp, u32, ctypes.POINTER(_Dxt1Params), vp, vp, i32, vp]
    L.crngpu_dxt1_optimize_batch.restype = i32
    L.crngpu_dxt5a_optimize_batch.argtypes = [vp, u32, u32, ctypes.c_int32, vp, i32, vp]
    L.crngpu_dxt5a_optimize_batch.restype = i32
    L.crngpu_compress_blocks.argtypes = [vp, u32, u32, u32, vp, i32, vp]
    L.crngpu_compress_blocks.restype = i32
    L.crngpu_compress_image.argtypes = [vp, u32, u32, u32, u32, u32, vp, u64, i32, vp]
    L.crngpu_compress_image.restype = i64
    L.crngpu_compress_blocks_ex.argtypes = [vp, u32, u32, u32, ctypes.POINTER(_BlockOptions), vp, i32, vp]
    L.crngpu_compress_blocks_ex.restype = i32
    L.crngpu_compress_image_ex.argtypes = [vp, u32, u32, u32, u32, u32, ctypes.POINTER(_BlockOptions), vp, u64, i32,
                                           vp]
    L.crngpu_compress_image_ex.restype = i64
    L.crngpu_unpack_begin.argtypes = [vp, u32]
    L.crngpu_unpack_begin.restype = vp
    L.crngpu_get_info.argtypes = [vp] + [ctypes.POINTER(u32)] * 6
    L.crngpu_get_info.restype = i32
    L.crngpu_unpack_level.argtypes = [vp, ctypes.POINTER(vp), u32, u32, u32, i32, vp]
    L.crngpu_unpack_level.restype = i32
    L.crngpu_unpack_level_segmented.argtypes = [vp, vp, u32, ctypes.POINTER(vp), u32, u32, u32, i32, vp]
    L.crngpu_unpack_level_segmented.restype = i32
    L.crngpu_unpack_levels.argtypes = [vp, u32, u32, vp, u64, i32, vp]
    L.crngpu_unpack_levels.restype = i64
    L.crngpu_unpack_end.argtypes = [vp]
    L.crngpu_unpack_end.restype = i32
    L.crngpu_unpack_batch_create.argtypes = [ctypes.POINTER(_BatchItem), u32]
    L.crngpu_unpack_batch_create.restype = vp
    L.crngpu_unpack_batch_launch.argtypes = [vp, u32, vp]
    L.crngpu_unpack_batch_launch.restype = i32
    L.crngpu_unpack_batch_status.argtypes = [vp, vp]
    L.crngpu_unpack_batch_status.restype = i32
    L.crngpu_unpack_batch_bytes.argtypes = [vp]
    L.crngpu_unpack_batch_bytes.restype = i64
    L.crngpu_unpack_batch_tuning.argtypes = [vp, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_float), u32]
    L.crngpu_unpack_batch_tuning.restype = i32
    L.crngpu_unpack_batch_set_variant.argtypes = [vp, i32]
    L.crngpu_unpack_batch_set_variant.restype = i32
    L.crngpu_unpack_batch_destroy.argtypes = [vp]
    L.crngpu_unpack_batch_destroy.restype = i32
    L.crngpu_crn_decompress.argtypes = [vp, ctypes.c_uint, vp, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint]
    L.crngpu_crn_decompress.restype = None
    L.crngpu_compress_crn.argtypes = [vp, u32, u32, u32, u32, u32, u32, u32, vp, u64]
    L.crngpu_compress_crn.restype = i64
    L.crngpu_compress_dds_clustered.argtypes = [vp, u32, u32, u32, u32, u32, u32, u32, vp, u64]
    L.crngpu_compress_dds_clustered.restype = i64
    L.crngpu_compress_crn_batch.argtypes = [ctypes.POINTER(_CrnBatchItem), u32, u32]
    L.crngpu_compress_crn_batch.restype = i32
    L.crngpu_compress_crn_bitrate.argtypes = [vp, u32, u32, u32, u32, u32, ctypes.c_float, u32, vp, u64,
                                              ctypes.POINTER(u32), ctypes.POINTER(ctypes.c_float)]
    L.crngpu_compress_crn_bitrate.restype = i64
    L.crngpu_crn_pack.argtypes = [vp, u32, u32, u32, u32, u32, vp, u64]
    L.crngpu_crn_pack.restype = i64
    L.crngpu_encode_batch_create.argtypes = [ctypes.POINTER(_EncodeItem), u32, u32]
    L.crngpu_encode_batch_create.restype = vp
    L.crngpu_encode_batch_launch.argtypes = [vp, u32, vp]
    L.crngpu_encode_batch_launch.restype = i32
    L.crngpu_encode_batch_tuning.argtypes = [vp, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_float), u32]
    L.crngpu_encode_batch_tuning.restype = i32
    L.crngpu_encode_batch_size.argtypes = [vp, ctypes.POINTER(ctypes.c_uint64)]
    L.crngpu_encode_batch_size.restype = i64
    L.crngpu_encode_batch_destroy.argtypes = [vp]
    L.crngpu_encode_batch_destroy.restype = i32
    L.crngpu_generate_mipmaps.argtypes = [vp, u32, u32, u32, u32, ctypes.c_float, u32, vp, u64, i32, vp]
    L.crngpu_generate_mipmaps.restype = i64
    L.crngpu_profile_counters.argtypes = [i32, ctypes.POINTER(ctypes.c_uint64), vp]
    L.crngpu_profile_counters.restype = i32
    L.crngpu_wait_counters.argtypes = [ctypes.POINTER(_WaitStats), i32]
    L.crngpu_wait_counters.restype = i32
    L.crngpu_force_wait_timeouts.argtypes = [i32]
    L.crngpu_force_wait_timeouts.restype = i32
    L.crngpu_set_decode_split.argtypes = [u32]
    L.crngpu_set_decode_split.restype = i32
    _lib = L
    return L


def version() -> str:
    return lib().crngpu_version().decode()


def last_error() -> str:
    return (lib().crngpu_last_error() or b"").decode(errors="replace")


def profile_counters(enable: bool, stream=None) -> int:
    """Returns the DXT1 candidate x colour evaluations counted since the last call and turns
    counting on or off (profiling hook; counting is off by default)."""
    v = ctypes.c_uint64(0)
    _check(lib().crngpu_profile_counters(int(enable), ctypes.byref(v), _stream_ptr(stream)), "crngpu_profile_counters")
    return int(v.value)


def wait_counters(reset: bool = False) -> dict:
    """How often the kernels' bounded waits ran out on the current device (crngpu_wait_counters):
    staging waits fall back to global memory, MMA waits make the call fail, drains that ran out
    mean a CTA exited with a copy in flight."""
    st = _WaitStats()
    _check(lib().crngpu_wait_counters(ctypes.byref(st), int(reset)), "crngpu_wait_counters")
    return {name: int(getattr(st, name)) for name, _ in _WaitStats._fields_}


def force_wait_timeouts(on: bool) -> None:
    """Test hook: every first bounded wait gives up at once (on) or the normal bounds apply (off)."""
    _check(lib().crngpu_force_wait_timeouts(int(on)), "crngpu_force_wait_timeouts")


DECODE_SPLIT_DEFAULT, DECODE_LANE_ONLY, DECODE_WIDE_ONLY = 0, 0xFFFFFFFF, 1


def set_decode_split(min_blocks: int) -> None:
    """Which levels run on the wide (CTA-per-level) decoder and which on the lane decoder
    (crngpu_set_decode_split): DECODE_SPLIT_DEFAULT lets each plan pick the split with the shortest
    decode; a block count sends levels at least that large to the wide decoder; DECODE_LANE_ONLY /
    DECODE_WIDE_ONLY force one decoder for every level. Both give the same bytes."""
    _check(lib().crngpu_set_decode_split(int(min_blocks) & 0xFFFFFFFF), "crngpu_set_decode_split")


def _check(rc: int, where: str) -> int:
    if rc < 0:
        raise CrnGpuError(rc, where)
    return rc


def _is_torch_cuda(x) -> bool:
    return hasattr(x, "is_cuda") and getattr(x, "is_cuda")


def _ptr_mem(x):
    """(pointer, mem kind) of a C-contiguous numpy array or torch tensor (CUDA = device, CPU = host)."""
    if hasattr(x, "data_ptr"):
        if not x.is_contiguous():
            raise CrnGpuError(E_PARAM, "tensor must be contiguous")
        return x.data_ptr(), (MEM_DEVICE if x.is_cuda else MEM_HOST)
    if not x.flags["C_CONTIGUOUS"]:
        raise CrnGpuError(E_PARAM, "array must be C-contiguous")
    return x.ctypes.data, MEM_HOST


def _contiguous(x):
    """x itself when already C-contiguous, else a C-contiguous copy (numpy or torch)."""
    if hasattr(x, "data_ptr"):
        return x.contiguous()
    return np.ascontiguousarray(x)


def _stream_ptr(stream):
    if stream is None:
        return None
    return getattr(stream, "cuda_stream", stream)


def _out_like(inp, shape, dtype=np.uint8):
    if hasattr(inp, "data_ptr"):
        import torch
        tdt = {np.uint8: torch.uint8, np.uint64: torch.int64}[dtype]
        if inp.is_cuda:
            return torch.empty(shape, dtype=tdt, device=inp.device)
        return torch.empty(shape, dtype=tdt, pin_memory=inp.is_pinned())
    return np.zeros(shape, dtype)


# ------------------------------------------------------------------------------------------
# Block encoders

def dxt1_optimize(blocks, perceptual: bool = True, use_alpha_blocks: bool = True, with_error: bool = False,
                  stream=None, quality: int = DXT_UBER, grayscale: bool = False, dxt1a: bool = False,
                  alpha_threshold: int = 128, transparent_black: bool = False):
    """(n, 64) RGBA8 blocks -> (n, 8) dxt1 blocks [, (n,) squared errors]: dxt1_endpoint_optimizer
    at crn_dxt_quality `quality`, optionally with grayscale sampling, DXT1A transparency (texels
    with alpha below alpha_threshold) and transparent indices for black."""
    blocks = _contiguous(blocks)
    n = int(blocks.shape[0])
    out = _out_like(blocks, (n, 8))
    err = _out_like(blocks, (n,), np.uint64) if with_error else None
    p = _Dxt1Params(ctypes.sizeof(_Dxt1Params), int(perceptual), int(use_alpha_blocks), 0, int(quality),
                    int(grayscale), int(dxt1a), int(alpha_threshold), int(transparent_black))
    ip, mem = _ptr_mem(blocks)
    op, _ = _ptr_mem(out)
    ep = _ptr_mem(err)[0] if err is not None else None
    _check(lib().crngpu_dxt1_optimize_batch(ip, n, ctypes.byref(p), op, ep, mem, _stream_ptr(stream)),
           "crngpu_dxt1_optimize_batch")
    return (out, err) if with_error else out


def dxt5a_optimize(blocks, comp_index: int = 3, use_both_block_types: bool = True, stream=None):
    """(n, 64) RGBA8 blocks -> (n, 8) dxt5 alpha blocks of channel comp_index."""
    blocks = _contiguous(blocks)
    n = int(blocks.shape[0])
    out = _out_like(blocks, (n, 8))
    ip, mem = _ptr_mem(blocks)
    _check(lib().crngpu_dxt5a_optimize_batch(ip, n, comp_index, int(use_both_block_types), _ptr_mem(out)[0], mem,
                                             _stream_ptr(stream)), "crngpu_dxt5a_optimize_batch")
    return out


def bytes_per_block(fmt: int) -> int:
    return 8 if fmt in (FMT_DXT1, FMT_DXT5A) else 16


def compress_blocks(blocks, fmt: int, flags: int = FLAG_PERCEPTUAL | FLAG_USE_BOTH_BLOCK_TYPES, stream=None,
                    quality: int = DXT_UBER, alpha_threshold: int = 128):
    """Batched crn_compress_block: (n, 64) RGBA8 -> (n, 8|16) DXTn blocks (crn_comp_flags `flags`,
    crn_dxt_quality `quality`, m_dxt1a_alpha_threshold `alpha_threshold`)."""
    blocks = _contiguous(blocks)
    n = int(blocks.shape[0])
    out = _out_like(blocks, (n, bytes_per_block(fmt)))
    ip, mem = _ptr_mem(blocks)
    o = _BlockOptions(ctypes.sizeof(_BlockOptions), int(quality), int(alpha_threshold))
    _check(lib().crngpu_compress_blocks_ex(ip, n, fmt, flags, ctypes.byref(o), _ptr_mem(out)[0], mem,
                                           _stream_ptr(stream)), "crngpu_compress_blocks_ex")
    return out


def compress_image(rgba, fmt: int = FMT_DXT1, flags: int = FLAG_PERCEPTUAL | FLAG_USE_BOTH_BLOCK_TYPES,
                   out=None, stream=None, quality: int = DXT_UBER, alpha_threshold: int = 128):
    """Plain DXTn encode of an (h, w, 4) RGBA8 image -> (blocks_y * blocks_x, 8|16) blocks."""
    rgba = _contiguous(rgba)
    h, w = int(rgba.shape[0]), int(rgba.shape[1])
    n = ((w + 3) // 4) * ((h + 3) // 4)
    if out is None:
        out = _out_like(rgba, (n, bytes_per_block(fmt)))
    ip, mem = _ptr_mem(rgba)
    o = _BlockOptions(ctypes.sizeof(_BlockOptions), int(quality), int(alpha_threshold))
    _check(lib().crngpu_compress_image_ex(ip, w, h, 0, fmt, flags, ctypes.byref(o), _ptr_mem(out)[0],
                                          n * bytes_per_block(fmt), mem, _stream_ptr(stream)),
           "crngpu_compress_image_ex")
    return out


MIP_FILTERS = {"box": 0, "tent": 1, "lanczos4": 2, "mitchell": 3, "kaiser": 4}
MIP_SRGB, MIP_WRAP, MIP_ALPHA = 1, 2, 4


def generate_mipmaps(rgba, filt: str = "kaiser", filter_scale: float = 0.9, srgb: bool = True, wrap: bool = False,
                     alpha: bool = True, levels: int = 0, stream=None):
    """crnlib's mip generation on the GPU (crngpu_generate_mipmaps): (h, w, 4) RGBA8 level 0, numpy
    or torch (CUDA tensors stay on the device) -> the list of levels, level 0 first. Defaults are
    crunch's: Kaiser filter, blurriness 0.9, gamma filtering."""
    rgba = _contiguous(rgba)
    h, w = int(rgba.shape[0]), int(rgba.shape[1])
    full = 1
    while (w >> full) or (h >> full):
        full += 1
    n = levels or full
    dims = [(max(1, h >> l), max(1, w >> l)) for l in range(n)]
    need = sum(a * b * 4 for a, b in dims)
    out = _out_like(rgba, (need,))
    ip, mem = _ptr_mem(rgba)
    flags = (MIP_SRGB if srgb else 0) | (MIP_WRAP if wrap else 0) | (MIP_ALPHA if alpha else 0)
    _check(int(lib().crngpu_generate_mipmaps(ip, w, h, n, MIP_FILTERS[filt], filter_scale, flags, _ptr_mem(out)[0],
                                              need, mem, _stream_ptr(stream))), "crngpu_generate_mipmaps")
    res, ofs = [], 0
    for a, b in dims:
        res.append(out[ofs:ofs + a * b * 4].reshape(a, b, 4))
        ofs += a * b * 4
    return res


def mip_chain_blocks(width: int, height: int, levels: int) -> int:
    """Blocks of a mip chain's levels (each level max(1, w >> l) x max(1, h >> l))."""
    return sum(((max(1, width >> l) + 3) // 4) * ((max(1, height >> l) + 3) // 4) for l in range(levels))


class EncodeBatch:
    """Plain DXTn encode of many textures' mip chains, mixed sizes and formats, in one gather
    launch and two persistent encoder launches (crngpu_encode_batch_*). items: (rgba, out, width,
    height, levels, fmt) with rgba a CUDA uint8 tensor holding the levels' texels back to back and
    out a CUDA uint8 tensor receiving every level's blocks back to back."""

    def __init__(self, items, flags: int = FLAG_PERCEPTUAL | FLAG_USE_BOTH_BLOCK_TYPES):
        self._keep = [(rgba, out) for rgba, out, *_ in items]  # buffers outlive the batch
        arr = (_EncodeItem * len(items))()
        for i, (rgba, out, w, h, levels, fmt) in enumerate(items):
            need = mip_chain_blocks(w, h, levels) * bytes_per_block(fmt)
            if out.numel() * out.element_size() < need:
                raise CrnGpuError(E_PARAM, f"EncodeBatch: item {i} output smaller than {need} bytes")
            arr[i] = _EncodeItem(rgba.data_ptr(), out.data_ptr(), w, h, levels, fmt)
        self.handle = lib().crngpu_encode_batch_create(arr, len(items), flags)
        if not self.handle:
            raise CrnGpuError(E_PARAM, "crngpu_encode_batch_create: " + last_error())
        tex = ctypes.c_uint64(0)
        self.blocks = int(lib().crngpu_encode_batch_size(self.handle, ctypes.byref(tex)))
        self.texels = int(tex.value)

    def launch(self, use_graph: bool = False, stream=None):
        _check(lib().crngpu_encode_batch_launch(self.handle, 1 if use_graph else 0, _stream_ptr(stream)),
               "crngpu_encode_batch_launch")

    def tuning(self):
        """((colour grid, alpha grid), measured ms of the colour then the alpha variants)."""
        g = (ctypes.c_int32 * 2)()
        ms = (ctypes.c_float * 16)()
        n = lib().crngpu_encode_batch_tuning(self.handle, g, ms, 16)
        return (int(g[0]), int(g[1])), [round(float(ms[i]), 4) for i in range(max(n, 0))]

    def close(self):
        if self.handle:
            lib().crngpu_encode_batch_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------------------------------
# Transcoder

class UnpackContext:
    """crnd_unpack_begin .. crnd_unpack_end for one .crn file (context lives on the device)."""

    def __init__(self, crn: bytes):
        self._buf = np.frombuffer(crn, np.uint8)
        self.handle = lib().crngpu_unpack_begin(self._buf.ctypes.data, len(crn))
        if not self.handle:
            raise CrnGpuError(E_CORRUPT, "crngpu_unpack_begin")
        vals = [ctypes.c_uint32() for _ in range(6)]
        _check(lib().crngpu_get_info(self.handle, *[ctypes.byref(v) for v in vals]), "crngpu_get_info")
        self.width, self.height, self.levels, self.faces, self.format, self.bytes_per_block = [v.value for v in vals]

    def level_dims(self, level: int):
        w, h = max(1, self.width >> level), max(1, self.height >> level)
        return (w + 3) // 4, (h + 3) // 4

    def level_bytes(self, level: int) -> int:
        bx, by = self.level_dims(level)
        return bx * by * self.bytes_per_block * self.faces

    def unpack_level(self, level: int, row_pitch: int = 0, out=None, stream=None):
        """All faces of one level; returns a (faces, blocks_y * pitch) uint8 array/tensor."""
        bx, by = self.level_dims(level)
        pitch = row_pitch or bx * self.bytes_per_block
        if out is None:
            out = np.zeros((self.faces, by * pitch), np.uint8)
        ptr, mem = _ptr_mem(out)
        stride = by * pitch
        faces = (ctypes.c_void_p * self.faces)(*[ptr + f * stride for f in range(self.faces)])
        _check(lib().crngpu_unpack_level(self.handle, faces, stride, row_pitch, level, mem, _stream_ptr(stream)),
               "crngpu_unpack_level")
        return out

    def unpack_levels(self, first: int = 0, count: int | None = None, out=None, stream=None):
        """Levels first..first+count-1 back to back (minimal pitch); one launch pair."""
        count = self.levels - first if count is None else count
        total = sum(self.level_bytes(l) for l in range(first, first + count))
        if out is None:
            out = np.zeros(total, np.uint8)
        ptr, mem = _ptr_mem(out)
        _check(lib().crngpu_unpack_levels(self.handle, first, count, ptr, total, mem, _stream_ptr(stream)),
               "crngpu_unpack_levels")
        return out

    def close(self):
        if self.handle:
            lib().crngpu_unpack_end(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class UnpackBatch:
    """Many levels of many open contexts transcoded by one persistent decode launch and one
    expansion launch (crngpu_unpack_batch_*). items: (context, first_level, level_count, dst)
    with dst a CUDA uint8 tensor receiving the levels back to back (minimal pitch)."""

    def __init__(self, items):
        self._keep = [(ctx, dst) for ctx, _, _, dst in items]  # contexts and outputs outlive the batch
        arr = (_BatchItem * len(items))()
        for i, (ctx, first, count, dst) in enumerate(items):
            arr[i] = _BatchItem(ctx.handle, first, count, dst.data_ptr(), dst.numel() * dst.element_size())
        self.handle = lib().crngpu_unpack_batch_create(arr, len(items))
        if not self.handle:
            raise CrnGpuError(E_PARAM, "crngpu_unpack_batch_create")
        self.bytes = int(lib().crngpu_unpack_batch_bytes(self.handle))

    def launch(self, use_graph: bool = False, expand_only: bool = False, stream=None):
        flags = (1 if use_graph else 0) | (2 if expand_only else 0)
        _check(lib().crngpu_unpack_batch_launch(self.handle, flags, _stream_ptr(stream)),
               "crngpu_unpack_batch_launch")

    def status(self, stream=None):
        _check(lib().crngpu_unpack_batch_status(self.handle, _stream_ptr(stream)), "crngpu_unpack_batch_status")

    def set_variant(self, variant: int):
        """Forces the expansion variant of later launches (-1: autotune again)."""
        _check(lib().crngpu_unpack_batch_set_variant(self.handle, variant), "crngpu_unpack_batch_set_variant")

    def tuning(self):
        """(chosen expansion variant, measured ms per variant) of the autotuner (first launch)."""
        v = ctypes.c_int32(-1)
        ms = (ctypes.c_float * 32)()
        n = lib().crngpu_unpack_batch_tuning(self.handle, ctypes.byref(v), ms, 32)
        return int(v.value), [round(float(ms[i]), 4) for i in range(max(n, 0))]

    def close(self):
        if self.handle:
            lib().crngpu_unpack_batch_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def unpack_begin(crn: bytes) -> UnpackContext:
    return UnpackContext(crn)


def crn_decompress(src: bytes, first_level: int, level_count: int, dst_size: int) -> np.ndarray:
    """emscripten crn_decompress contract: levels back to back into one host buffer."""
    s = np.frombuffer(src, np.uint8)
    out = np.zeros(dst_size, np.uint8)
    lib().crngpu_crn_decompress(s.ctypes.data, len(src), out.ctypes.data, dst_size, first_level, level_count)
    return out


def crn_pack(blocks, width: int, height: int, levels: int, faces: int, fmt: int) -> bytes:
    """DXTn blocks in crn_comp's layout (numpy, host) -> .crn bytes (crngpu_crn_pack)."""
    b = np.ascontiguousarray(blocks, dtype=np.uint8)
    size = _check(int(lib().crngpu_crn_pack(b.ctypes.data, width, height, levels, faces, fmt, None, 0)),
                  "crngpu_crn_pack")
    out = np.zeros(size, np.uint8)
    _check(int(lib().crngpu_crn_pack(b.ctypes.data, width, height, levels, faces, fmt, out.ctypes.data, size)),
           "crngpu_crn_pack")
    return out.tobytes()


def crn_layout_from_levels(level_blocks, width: int, height: int, faces: int, bpb: int):
    """Visible blocks per level ([level][face] -> (by, bx, bpb)) -> crn_comp's padded layout, the
    blocks outside the image filled with the nearest edge block."""
    parts = []
    for l, fl in enumerate(level_blocks):
        w, h = max(1, width >> l), max(1, height >> l)
        W, H = ((w + 7) & ~7) >> 2, ((h + 7) & ~7) >> 2
        for f in range(faces):
            v = np.asarray(fl[f]).reshape((h + 3) // 4, (w + 3) // 4, bpb)
            parts.append(np.pad(v, ((0, H - v.shape[0]), (0, W - v.shape[1]), (0, 0)), mode="edge").reshape(-1, bpb))
    return np.concatenate(parts)


def compress_crn_bitrate(faces_levels, target_bitrate: float, fmt: int = FMT_DXT1, flags: int = FLAG_PERCEPTUAL):
    """crn_compress with m_target_bitrate: (.crn bytes, chosen quality level, its bitrate in bits
    per texel over all faces and levels)."""
    h, w = faces_levels[0][0].shape[:2]
    flat = np.concatenate([np.ascontiguousarray(im, dtype=np.uint8).reshape(-1) for face in faces_levels for im in face])
    L = lib()
    q, br = ctypes.c_uint32(0), ctypes.c_float(0)
    args = (flat.ctypes.data, w, h, len(faces_levels[0]), len(faces_levels), fmt, ctypes.c_float(target_bitrate), flags)
    bpb = 8 if fmt in (FMT_DXT1, FMT_DXT5A) else 16
    cap = sum(((max(1, w >> l) + 7) // 8 * 2) * ((max(1, h >> l) + 7) // 8 * 2) * bpb
              for l in range(len(faces_levels[0]))) * len(faces_levels) + (1 << 20)
    out = np.zeros(cap, np.uint8)
    size = _check(int(L.crngpu_compress_crn_bitrate(*args, out.ctypes.data, cap, ctypes.byref(q), ctypes.byref(br))),
                  "crngpu_compress_crn_bitrate")
    if size > cap:
        raise CrnGpuError(E_PARAM, "crngpu_compress_crn_bitrate: output larger than expected")
    out = out[:size]
    return out.tobytes(), int(q.value), float(br.value)


def compress_dds_clustered(faces_levels, quality: int = 128, flags: int = FLAG_PERCEPTUAL | FLAG_USE_BOTH_BLOCK_TYPES,
                           fmt: int = FMT_DXT1):
    """The block data of a DDS written by crn_compress (crngpu_compress_dds_clustered): clustered
    (the reference's QDXT path: qdxt1 on colour, qdxt5 on alpha / DXN channels) below quality 255,
    the plain encoder at 255; every face's mip chain, per level its visible blocks (numpy (n, bytes
    per block))."""
    h, w = faces_levels[0][0].shape[:2]
    flat = np.concatenate([np.ascontiguousarray(im, dtype=np.uint8).reshape(-1) for face in faces_levels for im in face])
    L = lib()
    bpb = bytes_per_block(fmt)
    args = (flat.ctypes.data, w, h, len(faces_levels[0]), len(faces_levels), fmt, quality, flags)
    need = len(faces_levels) * sum(((max(1, w >> l) + 3) // 4) * ((max(1, h >> l) + 3) // 4) * bpb
                                   for l in range(len(faces_levels[0])))
    out = np.zeros(need, np.uint8)
    _check(int(L.crngpu_compress_dds_clustered(*args, out.ctypes.data, need)), "crngpu_compress_dds_clustered")
    return out.reshape(-1, bpb)


def compress_crn_batch(items, threads: int = 4):
    """Many compress_crn calls at once (crngpu_compress_crn_batch): items are (faces_levels, fmt,
    quality, flags); returns the .crn bytes of each, in order."""
    arr = (_CrnBatchItem * len(items))()
    keep = []
    for i, (faces_levels, fmt, quality, flags) in enumerate(items):
        h, w = faces_levels[0][0].shape[:2]
        flat = np.concatenate([np.ascontiguousarray(im, dtype=np.uint8).reshape(-1) for face in faces_levels
                               for im in face])
        bpb = 8 if fmt in (FMT_DXT1, FMT_DXT5A) else 16
        cap = sum(((max(1, w >> l) + 7) // 8 * 2) * ((max(1, h >> l) + 7) // 8 * 2) * bpb
                  for l in range(len(faces_levels[0]))) * len(faces_levels) + (1 << 20)
        out = np.zeros(cap, np.uint8)
        keep.append((flat, out))
        arr[i] = _CrnBatchItem(flat.ctypes.data, w, h, len(faces_levels[0]), len(faces_levels), fmt, quality, flags,
                               out.ctypes.data, cap, 0)
    rc = int(lib().crngpu_compress_crn_batch(arr, len(items), threads))
    res = []
    for i, (flat, out) in enumerate(keep):
        r = int(arr[i].result)
        if r < 0:
            raise CrnGpuError(r, f"crngpu_compress_crn_batch item {i}: " + last_error())
        if r > out.size:
            raise CrnGpuError(E_PARAM, "crngpu_compress_crn_batch: output larger than expected")
        res.append(out[:r].tobytes())
    _check(rc, "crngpu_compress_crn_batch")
    return res


def compress_crn(faces_levels, fmt: int = FMT_DXT1, quality: int = 128, flags: int = FLAG_PERCEPTUAL) -> bytes:
    """crn_compress to a .crn with source mips: faces_levels[face][level] RGBA8 images."""
    h, w = faces_levels[0][0].shape[:2]
    flat = np.concatenate([np.ascontiguousarray(im, dtype=np.uint8).reshape(-1) for face in faces_levels for im in face])
    L = lib()
    args = (flat.ctypes.data, w, h, len(faces_levels[0]), len(faces_levels), fmt, quality, flags)
    # a .crn is smaller than its DXT blocks (at most ~3 prefix codes of <= 16 bits per block)
    # plus palettes (<= 8192 entries x 12 bytes) and models
    bpb = 8 if fmt in (FMT_DXT1, FMT_DXT5A) else 16
    cap = sum(((max(1, w >> l) + 7) // 8 * 2) * ((max(1, h >> l) + 7) // 8 * 2) * bpb
              for l in range(len(faces_levels[0]))) * len(faces_levels) + (1 << 20)
    out = np.zeros(cap, np.uint8)
    size = _check(int(L.crngpu_compress_crn(*args, out.ctypes.data, cap)), "crngpu_compress_crn")
    if size > cap:
        raise CrnGpuError(E_PARAM, "crngpu_compress_crn: output larger than expected")
    return out[:size].tobytes()
