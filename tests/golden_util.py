"""Shared loaders for the committed golden fixtures (produced by the reference crnlib)."""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def blocks() -> dict:
    with np.load(os.path.join(GOLDEN, "blocks.npz")) as z:
        return {k: z[k] for k in z.files}


def blocks_quality() -> dict:
    """The reference block compressor below Uber, with grayscale sampling, DXT1A transparency and
    transparent indices for black (tests/golden/make_golden.py quality)."""
    with np.load(os.path.join(GOLDEN, "blocks_quality.npz")) as z:
        return {k: z[k] for k in z.files}


def manifest() -> dict:
    with open(os.path.join(GOLDEN, "crn", "manifest.json")) as fh:
        return json.load(fh)


def crn_bytes(name: str) -> bytes:
    with open(os.path.join(GOLDEN, "crn", name + ".crn"), "rb") as fh:
        return fh.read()


def sha(a) -> str:
    return hashlib.sha256(bytes(a)).hexdigest()


def c0_blocks() -> np.ndarray:
    from crunch2_gb300 import texgen
    return texgen.image_blocks(texgen.colour_texture(256, 256, 0))


def dxt5_tex_blocks() -> np.ndarray:
    from crunch2_gb300 import texgen
    return texgen.image_blocks(texgen.colour_texture(128, 128, 3, with_alpha_noise=True))


def nrm_tex_blocks() -> np.ndarray:
    from crunch2_gb300 import texgen
    return texgen.image_blocks(texgen.normal_map(128, 128, 4))


def level_bytes(w, h, level, bpb, faces):
    w, h = max(1, w >> level), max(1, h >> level)
    return ((w + 3) // 4) * ((h + 3) // 4) * bpb * faces


def bytes_per_block(fmt: str) -> int:
    return 8 if fmt in ("DXT1", "DXT5A") else 16
