"""Learned DXT1 endpoint proposal: training and inference through the crngpu C ABI.

The network (48 -> 256 -> 256 -> 8, GELU, BF16 tensor-core GEMMs with FP32 accumulation) is
trained on blocks the plain GPU optimizer labels (its endpoints and its error); the learned
encode keeps a prediction after one selector refit unless its error is above 1.5x the
predicted bound, and sends the rest to the exact optimizer.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import lib, _check, CrnGpuError, E_PARAM, dxt1_optimize

PARAM_SHAPES = [(256, 48), (256,), (256, 256), (256,), (16, 256), (16,)]
PARAM_NAMES = ["W1", "b1", "W2", "b2", "W3", "b3"]


def _bind():
    L = lib()
    if getattr(L, "_mlp_bound", False):
        return L
    vp, u32, i32, f32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_float
    L.crngpu_mlp_create.argtypes = [ctypes.c_uint64]
    L.crngpu_mlp_create.restype = vp
    L.crngpu_mlp_destroy.argtypes = [vp]
    L.crngpu_mlp_param.argtypes = [vp, i32, i32, vp, u32, i32]
    L.crngpu_mlp_forward.argtypes = [vp, vp, u32, vp, vp]
    L.crngpu_mlp_make_targets.argtypes = [vp, vp, u32, vp, vp]
    L.crngpu_mlp_gradients.argtypes = [vp, vp, vp, u32, ctypes.POINTER(f32), vp]
    L.crngpu_mlp_train_step.argtypes = [vp, vp, vp, u32, f32, f32, ctypes.POINTER(f32), vp]
    L.crngpu_dxt1_learned.argtypes = [vp, vp, u32, i32, f32, vp, ctypes.POINTER(u32), vp]
    for fn in ("crngpu_mlp_destroy", "crngpu_mlp_param", "crngpu_mlp_forward", "crngpu_mlp_make_targets",
               "crngpu_mlp_gradients", "crngpu_mlp_train_step", "crngpu_dxt1_learned"):
        getattr(L, fn).restype = i32
    L._mlp_bound = True
    return L


def _sp(stream):
    return None if stream is None else getattr(stream, "cuda_stream", stream)


class EndpointNet:
    def __init__(self, seed: int = 0):
        self.L = _bind()
        self.h = self.L.crngpu_mlp_create(seed)
        if not self.h:
            raise CrnGpuError(E_PARAM, "crngpu_mlp_create")

    def close(self):
        if self.h:
            self.L.crngpu_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # parameters ------------------------------------------------------------------------------
    def get(self, which: int, grad: bool = False) -> np.ndarray:
        a = np.zeros(PARAM_SHAPES[which], np.float32)
        _check(self.L.crngpu_mlp_param(self.h, which, int(grad), a.ctypes.data, a.size, 0), "crngpu_mlp_param")
        return a

    def set(self, which: int, value: np.ndarray):
        a = np.ascontiguousarray(value, np.float32).reshape(PARAM_SHAPES[which])
        _check(self.L.crngpu_mlp_param(self.h, which, 0, a.ctypes.data, a.size, 1), "crngpu_mlp_param")

    def state(self) -> dict:
        return {nm: self.get(i) for i, nm in enumerate(PARAM_NAMES)}

    def load(self, state: dict):
        for i, nm in enumerate(PARAM_NAMES):
            self.set(i, state[nm])

    # compute ---------------------------------------------------------------------------------
    def forward(self, d_blocks, stream=None):
        import torch
        n = int(d_blocks.shape[0])
        y = torch.empty((n, 16), dtype=torch.float32, device=d_blocks.device)
        _check(self.L.crngpu_mlp_forward(self.h, d_blocks.data_ptr(), n, y.data_ptr(), _sp(stream)),
               "crngpu_mlp_forward")
        return y

    def gradients(self, d_blocks, d_targets, stream=None) -> float:
        loss = ctypes.c_float(0)
        _check(self.L.crngpu_mlp_gradients(self.h, d_blocks.data_ptr(), d_targets.data_ptr(), int(d_blocks.shape[0]),
                                           ctypes.byref(loss), _sp(stream)), "crngpu_mlp_gradients")
        return float(loss.value)

    def train_step(self, d_blocks, d_targets, lr: float = 1e-3, weight_decay: float = 0.01, stream=None) -> float:
        loss = ctypes.c_float(0)
        _check(self.L.crngpu_mlp_train_step(self.h, d_blocks.data_ptr(), d_targets.data_ptr(), int(d_blocks.shape[0]),
                                            lr, weight_decay, ctypes.byref(loss), _sp(stream)),
               "crngpu_mlp_train_step")
        return float(loss.value)

    def encode(self, d_blocks, perceptual: bool = True, threshold: float = 1.5, out=None, stream=None):
        """Learned DXT1 encode; returns (blocks (n, 8) uint8 device tensor, fallback count)."""
        import torch
        n = int(d_blocks.shape[0])
        if out is None:
            out = torch.empty((n, 8), dtype=torch.uint8, device=d_blocks.device)
        fb = ctypes.c_uint32(0)
        _check(self.L.crngpu_dxt1_learned(self.h, d_blocks.data_ptr(), n, int(perceptual), threshold, out.data_ptr(),
                                          ctypes.byref(fb), _sp(stream)), "crngpu_dxt1_learned")
        return out, int(fb.value)


def make_targets(d_blocks, perceptual: bool = True, stream=None):
    """Labels from the plain GPU optimizer: (targets (n, 8) fp32, plain blocks (n, 8) uint8)."""
    import torch
    n = int(d_blocks.shape[0])
    plain, err = dxt1_optimize(d_blocks, perceptual, True, with_error=True, stream=stream)
    t = torch.empty((n, 8), dtype=torch.float32, device=d_blocks.device)
    L = _bind()
    _check(L.crngpu_mlp_make_targets(plain.data_ptr(), err.data_ptr(), n, t.data_ptr(), _sp(stream)),
           "crngpu_mlp_make_targets")
    return t, plain


def training_blocks(n_textures: int, size: int, seed0: int, device="cuda"):
    """Blocks of seeded config-0-style textures generated on the GPU."""
    import torch
    from .texgen import colour_texture_torch, image_blocks_torch
    parts = [image_blocks_torch(colour_texture_torch(size, size, seed0 + i, device)) for i in range(n_textures)]
    return torch.cat(parts)


def train(net: EndpointNet, d_blocks, d_targets, steps: int, batch: int = 8192, lr: float = 1e-3,
          weight_decay: float = 0.01, seed: int = 0, log_every: int = 0):
    """AdamW over random batches drawn without replacement, epoch by epoch."""
    import torch
    n = int(d_blocks.shape[0])
    g = torch.Generator(device=d_blocks.device)
    g.manual_seed(seed)
    losses = []
    perm = torch.randperm(n, generator=g, device=d_blocks.device)
    pos = 0
    for step in range(steps):
        if pos + batch > n:
            perm = torch.randperm(n, generator=g, device=d_blocks.device)
            pos = 0
        idx = perm[pos:pos + batch]
        pos += batch
        loss = net.train_step(d_blocks[idx].contiguous(), d_targets[idx].contiguous(), lr, weight_decay)
        losses.append(loss)
        if log_every and step % log_every == 0:
            print(f"step {step} loss {loss:.6f}")
    return losses
