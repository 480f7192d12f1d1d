"""Learned DXT1 endpoint proposal: training and inference through the crngpu C ABI.

The network (48 -> 256 -> 256 -> 8, GELU, BF16 tensor-core GEMMs with FP32 accumulation) is
trained on blocks the plain GPU optimizer labels (its endpoints and its error); the learned
encode keeps a refined prediction (selector fit, least-squares refit, +-1 search, 3-colour check)
unless its error is above a threshold (1.5x by default) times the predicted bound -- the
network's 0.75-quantile estimate of the error the plain optimizer reaches -- and sends the rest
to the exact optimizer.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import lib, _check, CrnGpuError, E_PARAM, dxt1_optimize

import os

PARAM_SHAPES = [(256, 48), (256,), (256, 256), (256,), (16, 256), (16,)]
# Trained network shipped with the package:
#   python -m crunch2_gb300.learned steps=16384 tau=0.75 bound_weight=0.25 mips=1 out=<this path>
# (22,369,600 training blocks: 64 seeded 2048x2048 colour textures and their box-filtered mip
# levels, labels from the plain GPU optimizer, 16384 AdamW steps of 8192 blocks, lr 1e-3, weight
# decay 0.01, init seed 0; endpoint outputs trained on squared error, the error-bound output on
# the 0.75-quantile pinball loss so that it is an upper bound of the plain optimizer's error for
# 75% of blocks).
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "dxt1_endpoint_net.npz")
DEFAULT_THRESHOLD = 1.5
# crn_dxt_quality of the exact optimizer on the blocks that fall back: Better (3). The fallback
# blocks are the ones the network proposes badly; on the 1024x1024 mip chain (seed 100) Better
# instead of Uber there costs +0.002 RGB RMSE and takes the encode from 0.69 to 0.50 ms (GB300).
DEFAULT_FALLBACK_QUALITY = 3
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
    L.crngpu_dxt1_learned_ex.argtypes = [vp, vp, u32, i32, f32, u32, vp, ctypes.POINTER(u32), vp]
    L.crngpu_mlp_set_bound_loss.argtypes = [vp, f32, f32]
    for fn in ("crngpu_mlp_destroy", "crngpu_mlp_param", "crngpu_mlp_forward", "crngpu_mlp_make_targets",
               "crngpu_mlp_gradients", "crngpu_mlp_train_step", "crngpu_dxt1_learned", "crngpu_dxt1_learned_ex", "crngpu_mlp_set_bound_loss"):
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

    def set_bound_loss(self, tau: float, weight: float = 1.0):
        """tau <= 0: squared error on the bound output; 0 < tau < 1: tau-quantile (pinball) loss."""
        _check(self.L.crngpu_mlp_set_bound_loss(self.h, tau, weight), "crngpu_mlp_set_bound_loss")

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

    def encode(self, d_blocks, perceptual: bool = True, threshold: float = DEFAULT_THRESHOLD, out=None, stream=None,
               fallback_quality: int = DEFAULT_FALLBACK_QUALITY):
        """Learned DXT1 encode; returns (blocks (n, 8) uint8 device tensor, fallback count).
        fallback_quality: the exact optimizer's crn_dxt_quality (0 superfast .. 4 uber) on the
        blocks that fall back."""
        import torch
        n = int(d_blocks.shape[0])
        if out is None:
            out = torch.empty((n, 8), dtype=torch.uint8, device=d_blocks.device)
        fb = ctypes.c_uint32(0)
        _check(self.L.crngpu_dxt1_learned_ex(self.h, d_blocks.data_ptr(), n, int(perceptual), threshold,
                                             int(fallback_quality), out.data_ptr(), ctypes.byref(fb), _sp(stream)),
               "crngpu_dxt1_learned_ex")
        return out, int(fb.value)


def default_net(path: str = WEIGHTS) -> EndpointNet:
    """The shipped trained network on the current device."""
    net = EndpointNet(seed=0)
    net.load(dict(np.load(path)))
    return net


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


def training_blocks(n_textures: int, size: int, seed0: int, device="cuda", mips: bool = False):
    """Blocks of seeded config-0-style textures generated on the GPU; with mips, also the blocks of
    every box-filtered mip level down to 4x4 (mip chains are what real textures are encoded as)."""
    import torch
    from .texgen import colour_texture_torch, image_blocks_torch, box_mip_torch
    parts = []
    for i in range(n_textures):
        img = colour_texture_torch(size, size, seed0 + i, device)
        parts.append(image_blocks_torch(img))
        while mips and img.shape[0] >= 8 and img.shape[1] >= 8:
            img = box_mip_torch(img)
            parts.append(image_blocks_torch(img))
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


def rgb_rmse_torch(blocks8, pixels):
    """'RGB Average' RMSE (crnlib/crn_image_utils.cpp:1048-1139) of DXT1 blocks vs RGBA8 blocks,
    computed on the device in chunks."""
    import torch
    total = 0.0
    n = int(pixels.shape[0])
    for c0 in range(0, n, 1 << 21):
        b = blocks8[c0:c0 + (1 << 21)].to(torch.int64)
        px = pixels[c0:c0 + (1 << 21)].view(-1, 16, 4)[:, :, :3].to(torch.int64)
        lo = b[:, 0] | (b[:, 1] << 8)
        hi = b[:, 2] | (b[:, 3] << 8)

        def exp565(c):
            r, g, bb = (c >> 11) & 31, (c >> 5) & 63, c & 31
            return torch.stack([(r << 3) | (r >> 2), (g << 2) | (g >> 4), (bb << 3) | (bb >> 2)], -1)
        c0_, c1_ = exp565(lo), exp565(hi)
        four = (lo > hi).unsqueeze(-1)
        c2 = torch.where(four, (2 * c0_ + c1_) // 3, (c0_ + c1_) >> 1)
        c3 = torch.where(four, (c0_ + 2 * c1_) // 3, torch.zeros_like(c0_))
        pal = torch.stack([c0_, c1_, c2, c3], 1)
        sel = torch.stack([(b[:, 4 + (i >> 2)] >> (2 * (i & 3))) & 3 for i in range(16)], 1)
        dec = torch.gather(pal, 1, sel.unsqueeze(-1).expand(-1, -1, 3))
        total += float(((dec - px) ** 2).sum())
    return (total / (n * 16 * 3)) ** 0.5


def config4(train_textures=64, train_size=2048, eval_textures=32, eval_size=4096, steps=2048, batch=8192,
            lr=1e-3, threshold=1.5, log_every=256, seed=0, weights=None, tau=0.0, bound_weight=1.0, mips=0,
            fallback_quality=DEFAULT_FALLBACK_QUALITY):
    """Learned endpoint proposal end to end: GPU-labelled training set, GPU training, and learned
    vs plain DXT1 encode on held-out textures (different seed range). `threshold` may be a list
    (or a comma-separated string) to report several fallback thresholds from one trained net;
    `weights` loads a saved state instead of training; tau > 0 trains the error-bound output as
    the tau-quantile of the plain optimizer's error (pinball loss, scaled by bound_weight);
    fallback_quality is the exact optimizer's crn_dxt_quality on the blocks that fall back.
    Returns a metrics dict."""
    import time
    import torch
    ev = lambda: torch.cuda.Event(enable_timing=True)
    net = EndpointNet(seed=seed)
    fallback_quality = int(fallback_quality)
    res = {"tau": tau, "bound_weight": bound_weight, "fallback_quality": fallback_quality}
    if tau > 0:
        net.set_bound_loss(tau, bound_weight)
    if weights:
        net.load(dict(np.load(weights)))
        res["weights"] = str(weights)
    else:
        t0 = time.perf_counter()
        train_blocks = training_blocks(train_textures, train_size, seed0=1000, mips=bool(mips))
        n_train = int(train_blocks.shape[0])
        targets, _ = make_targets(train_blocks)
        torch.cuda.synchronize()
        t_label = time.perf_counter() - t0
        t1 = time.perf_counter()
        losses = train(net, train_blocks, targets, steps=steps, batch=batch, lr=lr, log_every=log_every)
        torch.cuda.synchronize()
        t_train = time.perf_counter() - t1
        del train_blocks, targets
        res.update({"train_blocks": n_train, "train_mips": bool(mips), "train_steps": steps,
                    "batch": batch,
                    "label_s": round(t_label, 3), "train_s": round(t_train, 3), "loss_first": losses[0],
                    "loss_last": float(np.mean(losses[-32:]))})
    if isinstance(threshold, str):
        threshold = [float(t) for t in threshold.split(",")]
    ths = list(threshold) if isinstance(threshold, (list, tuple)) else [float(threshold)]
    tot = {"plain_ms": 0.0, "forward_ms": 0.0, "blocks": 0, "se_plain": 0.0}
    per = [{"learned_ms": 0.0, "fallbacks": 0, "se": 0.0} for _ in ths]
    from .texgen import colour_texture_torch, image_blocks_torch
    from . import dxt1_optimize
    for i in range(eval_textures):
        blocks = image_blocks_torch(colour_texture_torch(eval_size, eval_size, 50000 + i))
        n = int(blocks.shape[0])
        out_p = torch.empty((n, 8), dtype=torch.uint8, device=blocks.device)
        out_l = torch.empty_like(out_p)
        dxt1_optimize(blocks)  # warm
        a, b = ev(), ev()
        a.record(); out_p = dxt1_optimize(blocks); b.record(); torch.cuda.synchronize()
        tot["plain_ms"] += a.elapsed_time(b)
        net.forward(blocks)
        a, b = ev(), ev()
        a.record(); net.forward(blocks); b.record(); torch.cuda.synchronize()
        tot["forward_ms"] += a.elapsed_time(b)
        tot["blocks"] += n
        tot["se_plain"] += rgb_rmse_torch(out_p, blocks) ** 2 * n
        for th, acc in zip(ths, per):
            a, b = ev(), ev()
            a.record()
            out_l, fb = net.encode(blocks, threshold=th, out=out_l, fallback_quality=fallback_quality)
            b.record()
            torch.cuda.synchronize()
            acc["learned_ms"] += a.elapsed_time(b)
            acc["fallbacks"] += fb
            acc["se"] += rgb_rmse_torch(out_l, blocks) ** 2 * n
    texels = tot["blocks"] * 16
    res.update({"eval_textures": eval_textures, "eval_size": eval_size, "eval_blocks": tot["blocks"],
                "plain_mtexel_s": texels / (tot["plain_ms"] / 1e3) / 1e6,
                "rmse_plain": (tot["se_plain"] / tot["blocks"]) ** 0.5,
                "forward_ms_per_mblock": tot["forward_ms"] / (tot["blocks"] / 1e6)})
    # the mip chain of a 1024x1024 texture (seed 100, box-filtered levels): plain vs learned
    from .texgen import colour_texture, mip_chain, image_blocks
    chain = torch.from_numpy(np.concatenate([image_blocks(l) for l in mip_chain(colour_texture(1024, 1024, 100))])).cuda()
    out_p = dxt1_optimize(chain)
    res["mip_chain_1024"] = {"rmse_plain": rgb_rmse_torch(out_p, chain)}
    for th in ths:
        out_l, fb = net.encode(chain, threshold=th, fallback_quality=fallback_quality)
        res["mip_chain_1024"][f"rmse_learned@{th}"] = rgb_rmse_torch(out_l, chain)
        res["mip_chain_1024"][f"fallback@{th}"] = fb / chain.shape[0]
    res["learned"] = [{"threshold": th,
                       "learned_mtexel_s": texels / (acc["learned_ms"] / 1e3) / 1e6,
                       "speedup": tot["plain_ms"] / acc["learned_ms"],
                       "rmse_learned": (acc["se"] / tot["blocks"]) ** 0.5,
                       "fallback_frac": acc["fallbacks"] / tot["blocks"]} for th, acc in zip(ths, per)]
    res["state"] = net.state()
    return res


if __name__ == "__main__":
    # python -m crunch2_gb300.learned [key=value ...] [out=weights.npz]
    import json
    import sys
    kw, out = {}, None
    for a in sys.argv[1:]:
        k, v = a.split("=", 1)
        if k == "out":
            out = v
        else:
            try:
                kw[k] = int(v)
            except ValueError:
                try:
                    kw[k] = float(v)
                except ValueError:
                    kw[k] = v
    r = config4(**kw)
    st = r.pop("state")
    if out:
        np.savez(out, **st)
    print(json.dumps(r))
