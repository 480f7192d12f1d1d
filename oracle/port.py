"""ctypes bindings to oracle/_build/libcrnoracle.so, this project's CPU restatement of the
reference DXTn path (see crn_oracle.h). Test infrastructure and CPU baseline only."""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_PATH = os.path.join(_HERE, "_build", "libcrnoracle.so")
_lib = None


class Dxt1Opts(ctypes.Structure):
    """oracle_dxt1_opts (crn_oracle.h)"""
    _fields_ = [(n, ctypes.c_int) for n in ("perceptual", "use_alpha_blocks", "quality", "grayscale", "dxt1a",
                                            "alpha_threshold", "transparent_black")]


def build() -> str:
    """Compiles the restatement (make port); returns the library path."""
    subprocess.run(["make", "-s", "-C", _HERE, "port"], check=True)
    return _PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_PATH):
            build()
        L = ctypes.CDLL(_PATH)
        vp, u32, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int
        L.oracle_dxt1_blocks.argtypes = [vp, u32, i32, i32, vp, vp, i32]
        L.oracle_dxt1_blocks.restype = i32
        L.oracle_dxt5a_blocks.argtypes = [vp, u32, i32, i32, vp, i32]
        L.oracle_dxt5a_blocks.restype = i32
        L.oracle_dxt1_blocks_ex.argtypes = [vp, u32, ctypes.POINTER(Dxt1Opts), vp, vp, i32]
        L.oracle_dxt1_blocks_ex.restype = i32
        L.oracle_dxt5a_blocks_q.argtypes = [vp, u32, i32, i32, i32, vp]
        L.oracle_dxt5a_blocks_q.restype = i32
        L.oracle_dxt1_count_evaluations.argtypes = [vp, u32, i32, i32, i32]
        L.oracle_dxt1_count_evaluations.restype = ctypes.c_uint64
        L.oracle_encode_blocks.argtypes = [vp, u32, i32, i32, i32, vp, i32]
        L.oracle_encode_blocks.restype = i32
        L.oracle_unpack_level.argtypes = [vp, u32, u32, vp, u32, u32]
        L.oracle_unpack_level.restype = i32
        L.oracle_time_unpack.argtypes = [vp, u32, u32, i32]
        L.oracle_time_unpack.restype = ctypes.c_double
        _lib = L
    return _lib


def dxt1_blocks(blocks: np.ndarray, perceptual: bool = True, use_alpha_blocks: bool = True, threads: int = 1):
    blocks = np.ascontiguousarray(blocks, dtype=np.uint8)
    n = blocks.shape[0]
    out = np.zeros((n, 8), np.uint8)
    err = np.zeros(n, np.uint64)
    lib().oracle_dxt1_blocks(blocks.ctypes.data, n, int(perceptual), int(use_alpha_blocks), out.ctypes.data,
                             err.ctypes.data, threads)
    return out, err


def dxt1_blocks_ex(blocks: np.ndarray, perceptual: bool = True, use_alpha_blocks: bool = True, quality: int = 4,
                   grayscale: bool = False, dxt1a: bool = False, alpha_threshold: int = 128,
                   transparent_black: bool = False, threads: int = 1):
    """DXT1 blocks with every block-compressor parameter (quality 0 superfast .. 4 uber)."""
    blocks = np.ascontiguousarray(blocks, dtype=np.uint8)
    n = blocks.shape[0]
    out = np.zeros((n, 8), np.uint8)
    err = np.zeros(n, np.uint64)
    o = Dxt1Opts(int(perceptual), int(use_alpha_blocks), int(quality), int(grayscale), int(dxt1a),
                 int(alpha_threshold), int(transparent_black))
    if lib().oracle_dxt1_blocks_ex(blocks.ctypes.data, n, ctypes.byref(o), out.ctypes.data, err.ctypes.data,
                                   threads) != 0:
        raise ValueError("bad DXT1 options")
    return out, err


def dxt5a_blocks(blocks: np.ndarray, comp: int, use_both_block_types: bool = True, quality: int = 4) -> np.ndarray:
    blocks = np.ascontiguousarray(blocks, dtype=np.uint8)
    n = blocks.shape[0]
    out = np.zeros((n, 8), np.uint8)
    if lib().oracle_dxt5a_blocks_q(blocks.ctypes.data, n, comp, int(use_both_block_types), quality,
                                   out.ctypes.data) != 0:
        raise ValueError("bad quality")
    return out


def dxt1_count_evaluations(blocks: np.ndarray, perceptual: bool = True, use_alpha_blocks: bool = True,
                           threads: int = 1) -> int:
    """Candidate x unique-colour evaluations of the reference's Uber DXT1 search on the blocks."""
    blocks = np.ascontiguousarray(blocks, dtype=np.uint8)
    return int(lib().oracle_dxt1_count_evaluations(blocks.ctypes.data, blocks.shape[0], int(perceptual),
                                                   int(use_alpha_blocks), threads))


def encode_blocks(blocks: np.ndarray, fmt: int, perceptual: bool = True, use_both_block_types: bool = True,
                  threads: int = 1) -> np.ndarray:
    blocks = np.ascontiguousarray(blocks, dtype=np.uint8)
    n = blocks.shape[0]
    out = np.zeros(n * 16, np.uint8)
    bpb = lib().oracle_encode_blocks(blocks.ctypes.data, n, fmt, int(perceptual), int(use_both_block_types),
                                     out.ctypes.data, threads)
    if bpb <= 0:
        raise ValueError("unsupported format %d" % fmt)
    return out[: n * bpb].reshape(n, bpb)


def unpack_level(crn: bytes, level: int, out_size: int, row_pitch: int = 0):
    src = np.frombuffer(crn, np.uint8)
    out = np.zeros(out_size, np.uint8)
    ok = lib().oracle_unpack_level(src.ctypes.data, len(crn), level, out.ctypes.data, out_size, row_pitch)
    return (out if ok else None)


def time_unpack(crn: bytes, reps: int, threads: int) -> float:
    src = np.frombuffer(crn, np.uint8)
    return lib().oracle_time_unpack(src.ctypes.data, len(crn), reps, threads)
