"""Benchmark: plain DXT1 (uber) encode and CRN -> DXT1 transcode of the 1024x1024 mip-chained
synthetic texture (value noise + 40 flat rectangles, seed 100; 11 box-filtered levels,
1,398,101 texels, 87,383 4x4 blocks), on GB300.

One JSON line on stdout (rank 0):
  value      whole-job DXT1 encode Mtexel/s, inputs resident in HBM, device time of K steps
  learned    the learned-proposal encode of the same blocks (shipped weights): Mtexel/s, RGB
             RMSE beside the plain encode's, fallback fraction; the fallback blocks through the
             exact optimizer at Better quality, and at Uber (uber_fallback)
  e2e        the same encode through the reference-facing C-ABI call with host buffers:
             crngpu_compress_dds_clustered at quality 255 (what crn_compress to DDS runs), the host
             mip chain in and the DDS blocks out, one call per step, wall time; e2e_batch_launch
             the same chain from pinned host memory through crngpu_encode_batch_launch (CUDA
             graph) with the copies around it; e2e_per_level through crngpu_compress_image per level
  clustered_dds  clustered DDS (the reference's QDXT1 path) of the same chain at quality 128
  clustered  crn_compress of the same mip chain to .crn at quality 128 (DXT1): Mtexel/s, bits per
             texel and RGB RMSE beside the reference's own .crn of the texture
  clustered_2048  the same for 2048x2048 DXT5 (colour + alpha noise) and DXN_XY (normal map) mip
             chains: colour / alpha / XY RMSE and bits per texel beside the reference's
  mixed_batch  512 textures of uneven sizes and mixed formats: batched plain encode (CUDA graph),
             their .crn through crn_compress, and the batched transcode of those files
  mips       crunch's default mip generation (Kaiser, gamma filtering) of a 4096x4096 texture
  transcode  CRN -> DXT1 transcode GB/s: a batch of 1024 textures (each with its own context holding
             the reference-encoded .crn of the same texture, q128) in one persistent decode launch
             and one expansion launch (CUDA graph); the expansion kernel's HBM roofline; the
             single-texture latency; the oracle on all host cores over the same .crn
  roofline   the encoder kernel: ALU issue roofline (the reference's candidate x colour evaluations
             on this workload, counted by the oracle, x lane-ops per evaluation, over the peak
             lane-op rate); the evaluations the device executed are reported beside them
  cpu_baseline  the oracle (CPU restatement of the reference, bit-identical outputs) on all
             host cores over a bounded sample of the same blocks
Multi-GPU: replicas only (every rank encodes its own copy; value = all ranks' texels / max time).
`--impl reference` times the reference's CPU implementation of the path (the oracle port,
since the compiled reference cannot run on this host's architecture) with all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

TEXTURE_SIZE = 1024
TEXTURE_SEED = 100
CRN_FIXTURE = os.path.join(ROOT, "tests", "golden", "crn", "c1_dxt1_1024.crn")
METRIC = "DXT1 encode Mtexel/s at matched RMSE, learned vs plain; CRN→DXT1 transcode GB/s"
L2_FLUSH_BYTES = 256 << 20
TX_BATCH = 1024  # textures per transcode batch
QUALITY_NAMES = ["superfast", "fast", "normal", "better", "uber"]  # crn_dxt_quality 0..4
# DRAM bytes (read, written) per launch of the two plain-encode kernels on this workload, from one
# ncu capture (dram__bytes_read.sum, dram__bytes_write.sum)
DXT1_ENCODE_DRAM = {"k_dxt1_seeds": (6.28e6, 0.91e6), "k_dxt1_encode": (13.8e6, 32.7e6)}
LANE_OPS_PER_EVAL = 27  # uber inner loop per candidate x colour: 15 FFMA, 4 FMNMX, 4 FADD, 2 IADD, 2 IMAD


def workload():
    from crunch2_gb300 import texgen
    img = texgen.colour_texture(TEXTURE_SIZE, TEXTURE_SIZE, TEXTURE_SEED)
    levels = texgen.mip_chain(img)
    blocks = np.concatenate([texgen.image_blocks(l) for l in levels])
    texels = sum(l.shape[0] * l.shape[1] for l in levels)
    return levels, blocks, texels


def clustered_leg(cg, dev, levels, blocks, texels, steps: int) -> dict:
    """crn_compress of the 1024x1024 mip chain at q128 (DXT1), median wall time of up to 5 calls;
    RMSE and bits per texel beside the reference's own .crn of the texture (committed fixture),
    both decoded by the GPU transcoder."""
    import torch
    from crunch2_gb300 import learned as LR
    cg.compress_crn([levels], cg.FMT_DXT1, quality=128)  # warm-up (allocations, tables)
    crn_times = []
    for _ in range(max(1, min(steps, 5))):
        t0 = time.perf_counter()
        our_crn = cg.compress_crn([levels], cg.FMT_DXT1, quality=128)
        crn_times.append(time.perf_counter() - t0)
    crn_s = statistics.median(crn_times)

    def crn_rmse(data):
        with cg.unpack_begin(data) as c:
            dec = c.unpack_levels()
        return LR.rgb_rmse_torch(torch.from_numpy(dec.reshape(-1, 8)).to(dev), torch.from_numpy(blocks).to(dev))

    with open(CRN_FIXTURE, "rb") as fh:
        ref_crn = fh.read()
    return {"value": round(texels / crn_s / 1e6, 3), "unit": "Mtexel/s", "s_per_texture": round(crn_s, 4),
            "quality": 128, "rmse": round(crn_rmse(our_crn), 4), "rmse_reference_crn": round(crn_rmse(ref_crn), 4),
            "bits_per_texel": round(len(our_crn) * 8 / texels, 4),
            "bits_per_texel_reference": round(len(ref_crn) * 8 / texels, 4),
            "path": "crngpu_compress_crn: host RGBA8 mip chain -> H2D -> crn_comp block gather and clustered "
                    "encode (every dxt_hc stage) on the GPU -> D2H -> .crn writer (host); wall time"}


QDXT_REFERENCE = os.path.join(ROOT, "tests", "golden", "qdxt_reference.json")
ENCODE_WORK = os.path.join(ROOT, "tests", "golden", "encode_work.json")


def qdxt_leg(cg, dev, levels, blocks, texels, steps: int) -> dict:
    """Clustered DDS of the 1024x1024 mip chain at q128 (crn_compress to DDS below quality 255,
    the reference's QDXT1 path), median wall time of up to 5 calls; RMSE and distinct endpoint and
    selector words beside the reference's output on the same chain (committed with the fixtures)."""
    import torch
    from crunch2_gb300 import learned as LR
    with open(QDXT_REFERENCE) as fh:
        ref = json.load(fh)["qdxt_1024_q128"]
    cg.compress_dds_clustered([levels], quality=128)  # warm-up
    times = []
    for _ in range(max(1, min(steps, 5))):
        t0 = time.perf_counter()
        out = cg.compress_dds_clustered([levels], quality=128)
        times.append(time.perf_counter() - t0)
    s = statistics.median(times)
    return {"value": round(texels / s / 1e6, 3), "unit": "Mtexel/s", "s_per_texture": round(s, 4), "quality": 128,
            "rmse": round(LR.rgb_rmse_torch(torch.from_numpy(out).to(dev), torch.from_numpy(blocks).to(dev)), 4),
            "rmse_reference": round(ref["rmse"], 4),
            "distinct_endpoints": int(np.unique(out[:, :4].copy().view(np.uint32)).size),
            "distinct_selectors": int(np.unique(out[:, 4:].copy().view(np.uint32)).size),
            "distinct_endpoints_reference": ref["distinct_endpoints"],
            "distinct_selectors_reference": ref["distinct_selectors"],
            "reference_s_8_threads_x86": ref["seconds_8_threads_x86"],
            "path": "crngpu_compress_dds_clustered: host RGBA8 mip chain -> H2D -> qdxt1 tiling, clustering and "
                    "block refit on the GPU -> D2H of the DDS blocks; wall time"}


CONFIG2_REFERENCE = os.path.join(ROOT, "tests", "golden", "config2_reference.json")


def clustered_2048_leg(cg, dev, steps: int) -> dict:
    """crn_compress of 2048x2048 DXT5 and DXN_XY mip chains (12 levels) at q128; quality of the
    GPU-decoded blocks against the source, beside the reference's own .crn of each texture."""
    import torch
    from crunch2_gb300 import quality as Q
    from crunch2_gb300 import texgen
    with open(CONFIG2_REFERENCE) as fh:
        refs = json.load(fh)
    out = {}
    for name, fmt_name, fmt in (("dxt5_2048", "DXT5", cg.FMT_DXT5), ("dxn_xy_2048", "DXN_XY", cg.FMT_DXN_XY)):
        r = refs[name]
        size = r["size"]
        img = texgen.normal_map(size, size, r["seed"]) if r["content"] == "normal" else \
            texgen.colour_texture(size, size, r["seed"], with_alpha_noise=True)
        levels = texgen.mip_chain(img)
        texels = sum(l.shape[0] * l.shape[1] for l in levels)
        flags = 0 if r["content"] == "normal" else cg.FLAG_PERCEPTUAL
        cg.compress_crn([levels], fmt, quality=128, flags=flags)  # warm-up
        times = []
        for _ in range(steps):
            t0 = time.perf_counter()
            crn = cg.compress_crn([levels], fmt, quality=128, flags=flags)
            times.append(time.perf_counter() - t0)
        secs = statistics.median(times)
        with cg.unpack_begin(crn) as c:
            dec = c.unpack_levels()
        src = torch.from_numpy(np.concatenate([texgen.image_blocks(l) for l in levels])).to(dev)
        q = Q.block_rmse(torch.from_numpy(dec.reshape(-1, 16)).to(dev), src, fmt_name)
        rec = {"mtexel_s": round(texels / secs / 1e6, 3), "s_per_texture": round(secs, 4), "texels": texels,
               "bits_per_texel": round(8 * len(crn) / texels, 4),
               "bits_per_texel_reference": round(r["bits_per_texel"], 4)}
        for k, v in q.items():
            rec[k] = round(v, 4)
            rec[k + "_reference"] = round(r[k], 4)
        rec["reference_seconds_8_threads_x86"] = r["seconds_8_threads_x86"]
        out[name] = rec
    out["path"] = ("crngpu_compress_crn (host RGBA8 mip chain -> .crn), decoded by the GPU transcoder; the "
                   "reference's figures are its own crn_compress output of the same texture, decoded by crnd")
    return out


MIXED_TEXTURES = 512
MIXED_SEED = 3000


def mixed_batch_workload(cg, dev):
    """512 textures: width and height drawn independently and log-uniformly from the powers of two
    32..2048, full mip chains, formats 60% DXT1 / 25% DXT5 / 15% DXN_XY, content as the colour
    recipe (DXT5 with alpha noise) or the normal-map recipe, per-texture seeds; generated on the
    GPU. Returns [(levels (device tensors), width, height, format)]."""
    from crunch2_gb300 import texgen
    rng = np.random.default_rng(MIXED_SEED)
    out = []
    for i in range(MIXED_TEXTURES):
        w, h = 1 << int(rng.integers(5, 12)), 1 << int(rng.integers(5, 12))
        u = float(rng.random())
        fmt = cg.FMT_DXT1 if u < 0.60 else cg.FMT_DXT5 if u < 0.85 else cg.FMT_DXN_XY
        seed = MIXED_SEED + i
        img = texgen.normal_map_torch(w, h, seed, device=dev) if fmt == cg.FMT_DXN_XY else \
            texgen.colour_texture_torch(w, h, seed, device=dev, with_alpha_noise=(fmt == cg.FMT_DXT5))
        out.append((texgen.mip_chain_torch(img), w, h, fmt))
    return out


def mixed_batch_leg(cg, dev, stream, timed, steps: int, warmup: int) -> dict:
    import torch
    tex = mixed_batch_workload(cg, dev)
    names = {cg.FMT_DXT1: "DXT1", cg.FMT_DXT5: "DXT5", cg.FMT_DXN_XY: "DXN_XY"}
    items = []
    for levels, w, h, fmt in tex:
        rgba = torch.cat([l.reshape(-1) for l in levels])
        out = torch.empty(cg.mip_chain_blocks(w, h, len(levels)) * cg.bytes_per_block(fmt), dtype=torch.uint8,
                          device=dev)
        items.append((rgba, out, w, h, len(levels), fmt))
    flags = cg.FLAG_PERCEPTUAL | cg.FLAG_USE_BOTH_BLOCK_TYPES
    enc = cg.EncodeBatch(items, flags)
    for _ in range(warmup):
        enc.launch(use_graph=True, stream=stream)
    torch.cuda.synchronize()
    grids, tune_ms = enc.tuning()
    # parity: every 64th texture against the single-image path, level by level
    parity = True
    for (rgba, out, w, h, n, fmt), (levels, *_) in list(zip(items, tex))[::64]:
        got, ofs = out.cpu().numpy(), 0
        for l in levels:
            ref = cg.compress_image(l.cpu().numpy(), fmt, flags).reshape(-1)
            parity &= bool(np.array_equal(got[ofs:ofs + ref.size], ref))
            ofs += ref.size
    enc_ms = timed(lambda: enc.launch(use_graph=True, stream=stream), steps)
    texels, blocks = enc.texels, enc.blocks
    enc.close()
    counts = {names[f]: sum(1 for *_, f2 in tex if f2 == f) for f in names}
    # .crn of every texture (clustered, q128) through crn_compress, one texture after another
    host = [([l.cpu().numpy() for l in levels], w, h, fmt) for levels, w, h, fmt in tex]
    del items
    crn_threads = min(8, cpu_threads())
    t0 = time.perf_counter()
    crns = cg.compress_crn_batch([([lv], fmt, 128, 0 if fmt == cg.FMT_DXN_XY else cg.FLAG_PERCEPTUAL)
                                  for lv, w, h, fmt in host], threads=crn_threads)
    crn_s = time.perf_counter() - t0
    # batched transcode of those files
    ctxs = [cg.unpack_begin(c) for c in crns]
    outs = [torch.empty(sum(c.level_bytes(l) for l in range(c.levels)), dtype=torch.uint8, device=dev) for c in ctxs]
    tb = cg.UnpackBatch([(c, 0, c.levels, o) for c, o in zip(ctxs, outs)])
    for _ in range(warmup):
        tb.launch(use_graph=True, stream=stream)
    tb.status(stream=stream)
    tx_parity = all(bool((outs[i].cpu().numpy() == ctxs[i].unpack_levels()).all()) for i in range(0, len(ctxs), 64))
    tx_ms = timed(lambda: tb.launch(use_graph=True, stream=stream), steps)
    tb.status(stream=stream)
    exp_ms = timed(lambda: tb.launch(expand_only=True, stream=stream), steps)
    tx_bytes = tb.bytes
    variant, _ = tb.tuning()
    tb.close()
    for c in ctxs:
        c.close()
    return {"textures": MIXED_TEXTURES, "formats": counts, "texels": texels, "blocks": blocks,
            "workload": "512 textures, W and H log-uniform over 32..2048 (powers of two), full mip chains, "
                        "60/25/15% DXT1/DXT5/DXN_XY, generated on the GPU (seeded)",
            "encode": {"value": round(texels / (enc_ms / 1e3) / 1e6, 1), "unit": "Mtexel/s",
                       "ms_per_batch": round(enc_ms, 3), "parity_vs_single_image": parity,
                       "grids": {"colour": grids[0], "alpha": grids[1]}, "tuning_ms": tune_ms,
                       "path": "crngpu_encode_batch (CUDA graph: gather + persistent colour and alpha encoders "
                               "on two streams), uber, perceptual, inputs resident in HBM (larger than L2)"},
            "crn_encode": {"value": round(texels / crn_s / 1e6, 2), "unit": "Mtexel/s", "s_total": round(crn_s, 3),
                           "bytes": sum(len(c) for c in crns), "host_threads": crn_threads,
                           "path": "crngpu_compress_crn_batch (host RGBA8 in, .crn out, q128): host threads with "
                                   "a CUDA stream each, one texture's gather and .crn writer overlapping other "
                                   "textures' GPU encodes"},
            "transcode": {"value": round(tx_bytes / (tx_ms / 1e3) / 1e9, 3), "unit": "GB/s", "ms_per_batch": round(tx_ms, 3),
                          "output_bytes": tx_bytes, "expand_ms": round(exp_ms, 4),
                          "expand_gb_s_output": round(tx_bytes / (exp_ms / 1e3) / 1e9, 1),
                          "parity_vs_single_context": tx_parity, "expand_variant": variant,
                          "path": "crngpu_unpack_batch (CUDA graph) over the 512 .crn files"}}


def mips_leg(cg, dev, stream, timed, steps: int, warmup: int) -> dict:
    import torch
    from crunch2_gb300 import texgen
    size = 4096
    img = texgen.colour_texture_torch(size, size, 4096, device=dev, with_alpha_noise=True)
    out_texels = sum(max(1, size >> l) ** 2 for l in range(1, 13))
    for _ in range(warmup):
        cg.generate_mipmaps(img, stream=stream)
    ms = timed(lambda: cg.generate_mipmaps(img, stream=stream), steps)
    return {"value": round(out_texels / (ms / 1e3) / 1e6, 1), "unit": "Mtexel/s (generated levels)",
            "ms_per_chain": round(ms, 3), "levels": 13, "size": size,
            "path": "crngpu_generate_mipmaps (Kaiser, blurriness 0.9, gamma 2.2, alpha), device buffers; "
                    "bit-identical to crnlib's generate_mipmaps on the committed fixtures"}


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("CRNGPU_BENCH_BACKEND", "nccl") == "nccl" else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, value: float) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu, self.rows, self.proc = gpu, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, nm in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def cpu_encode_baseline(blocks: np.ndarray, texels_per_block: float, budget_s: float = 3.0):
    """Oracle port (bit-identical to the reference's encoder) on all host threads, repeated over
    the workload's blocks for about budget_s seconds."""
    from oracle import port
    threads = cpu_threads()
    t0 = time.perf_counter()
    done = 0
    while True:
        port.dxt1_blocks(blocks, True, True, threads=threads)
        done += blocks.shape[0]
        if time.perf_counter() - t0 >= budget_s:
            break
    secs = time.perf_counter() - t0
    return {"value": done * texels_per_block / secs / 1e6, "unit": "Mtexel/s", "cores": threads, "kind": "port",
            "sample": f"{done} blocks ({done // blocks.shape[0]} passes over the 87,383-block mip chain), "
                      f"{secs:.1f} s on {threads} threads"}


def cpu_transcode_baseline(crn: bytes, out_bytes: int, budget_s: float = 1.0):
    from oracle import port
    threads = cpu_threads()
    reps = 1
    while True:
        secs = port.time_unpack(crn, reps, threads)
        if secs >= budget_s or reps >= 4096:
            break
        reps *= 2
    return {"value": out_bytes * reps / secs / 1e9, "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": f"{reps} transcodes of the 11-level .crn ({threads} threads, levels in parallel)"}


def run_reference(args, world, rank):
    """CPU arm: the reference's DXT1 encode path (oracle port) on all host threads."""
    if rank != 0:
        return
    levels, blocks, texels = workload()
    # bounded per-step sample: the whole mip chain is only ~0.1 s of work on a many-core host
    from oracle import port
    threads = cpu_threads()
    for _ in range(args.warmup):
        port.dxt1_blocks(blocks[:4096], True, True, threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        port.dxt1_blocks(blocks, True, True, threads=threads)
    secs = time.perf_counter() - t0
    value = texels * args.steps / secs / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "Mtexel/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(secs * 1e3 / args.steps, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": "DXT1 uber encode, 1024x1024 RGBA8 + full box mip chain (11 levels, "
                                   "1,398,101 texels, 87,383 blocks)", "quality": "uber",
                       "endpoint_caching": False},
            "cpu_baseline": {"value": round(value, 3), "unit": "Mtexel/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} passes over the 87,383-block mip chain"},
            "e2e": {"value": round(value, 3), "unit": "Mtexel/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--skip", default="", help="comma-separated legs to leave out of the run (their keys are "
                                               "null): clustered, clustered_2048, mixed, mips, config4")
    args = ap.parse_args()
    skip = set(x for x in args.skip.split(",") if x)
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return

    import torch
    import crunch2_gb300 as cg
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    levels, blocks, texels = workload()
    n_blocks = blocks.shape[0]
    d_blocks = torch.from_numpy(blocks).to(dev)
    d_out = torch.empty((n_blocks, 8), dtype=torch.uint8, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    params = cg._Dxt1Params(16, 1, 1, 0)
    L = cg.lib()

    def encode():
        rc = L.crngpu_dxt1_optimize_batch(d_blocks.data_ptr(), n_blocks, cg.ctypes.byref(params), d_out.data_ptr(),
                                          None, cg.MEM_DEVICE, stream.cuda_stream)
        if rc < 0:
            raise cg.CrnGpuError(rc, "crngpu_dxt1_optimize_batch")

    # parity of this exact workload against the oracle on a sample (cheap guard against a stale build)
    encode()
    torch.cuda.synchronize()
    from oracle import port
    sample = slice(0, 4096)
    ref_sample, _ = port.dxt1_blocks(blocks[sample], True, True, threads=cpu_threads())
    parity = float((d_out[sample].cpu().numpy() == ref_sample).all(1).mean())
    # work count (outside the timed region): candidate x colour evaluations per launch
    cg.profile_counters(True, stream)
    encode()
    evals = cg.profile_counters(False, stream)

    for _ in range(args.warmup):
        flush.fill_(1)
        encode()
    torch.cuda.synchronize()
    barrier(world)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        barrier(world)
        wall0 = time.perf_counter()
        for i in range(args.steps):
            flush.fill_(i & 0xFF)  # L2 flush between steps, outside the events
            starts[i].record(stream)
            encode()
            ends[i].record(stream)
        torch.cuda.synchronize()
        barrier(world)
        wall = time.perf_counter() - wall0
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    dev_s = sum(step_ms) / 1e3
    dev_s = max_over_ranks(world, dev_s)
    value = world * texels * args.steps / dev_s / 1e6
    kernel_ms = sum(step_ms) / len(step_ms)

    # ---- end to end through the public API with pinned host buffers (per level, image path)
    host_levels = [torch.from_numpy(np.ascontiguousarray(l)).pin_memory() for l in levels]
    host_outs = [torch.empty((((l.shape[1] + 3) // 4) * ((l.shape[0] + 3) // 4), 8), dtype=torch.uint8).pin_memory()
                 for l in levels]
    h2d = sum(int(l.numel()) for l in host_levels)
    d2h = sum(int(o.numel()) for o in host_outs)

    def per_level_step():
        for lv, out in zip(host_levels, host_outs):
            cg.compress_image(lv, cg.FMT_DXT1, out=out, stream=stream)

    for _ in range(args.warmup):
        per_level_step()
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        per_level_step()
    torch.cuda.synchronize()
    per_level_s = max_over_ranks(world, time.perf_counter() - t0)
    per_level_value = world * texels * args.steps / per_level_s / 1e6
    e2e_parity = float((host_outs[0].numpy() == d_out[:host_outs[0].shape[0]].cpu().numpy()).all())

    # the whole chain in one call: pinned host levels back to back -> H2D -> crngpu_encode_batch
    # (CUDA graph: gather + persistent encoder) -> D2H of every level's blocks -> host sync
    host_chain = torch.cat([l.reshape(-1) for l in host_levels]).pin_memory()
    host_chain_out = torch.empty((n_blocks, 8), dtype=torch.uint8).pin_memory()
    d_chain = torch.empty_like(host_chain, device=dev)
    d_chain_out = torch.empty((n_blocks, 8), dtype=torch.uint8, device=dev)
    w0, h0 = levels[0].shape[1], levels[0].shape[0]
    chain_batch = cg.EncodeBatch([(d_chain, d_chain_out, w0, h0, len(levels), cg.FMT_DXT1)])
    d_chain.copy_(host_chain)
    chain_batch.launch(use_graph=True, stream=stream)  # first launch: autotune + graph capture
    torch.cuda.synchronize()

    def e2e_step():
        with torch.cuda.stream(stream):
            d_chain.copy_(host_chain, non_blocking=True)
            chain_batch.launch(use_graph=True, stream=stream)
            host_chain_out.copy_(d_chain_out, non_blocking=True)
        stream.synchronize()

    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(world, time.perf_counter() - t0)
    e2e_value = world * texels * args.steps / e2e_s / 1e6
    chain_parity = bool(np.array_equal(host_chain_out.numpy(), d_out.cpu().numpy()))
    chain_grids = chain_batch.tuning()[0]
    chain_batch.close()
    h2d_chain, d2h_chain = int(host_chain.numel()), int(host_chain_out.numel())

    # the drop-in path: crn_compress to DDS at quality 255 calls crngpu_compress_dds_clustered with
    # the host mip chain (upload, GPU gather of every level, one encoder launch, one download)
    host_chain_np = host_chain.numpy()
    dds_out = np.zeros(n_blocks * 8, np.uint8)
    L = cg.lib()

    def drop_in_step():
        rc = L.crngpu_compress_dds_clustered(host_chain_np.ctypes.data, w0, h0, len(levels), 1, cg.FMT_DXT1, 255,
                                             cg.FLAG_PERCEPTUAL | cg.FLAG_USE_BOTH_BLOCK_TYPES,
                                             dds_out.ctypes.data, dds_out.size)
        if rc < 0:
            raise cg.CrnGpuError(rc, "crngpu_compress_dds_clustered")

    for _ in range(args.warmup):
        drop_in_step()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        drop_in_step()
    drop_in_s = max_over_ranks(world, time.perf_counter() - t0)
    drop_in_value = world * texels * args.steps / drop_in_s / 1e6
    drop_in_parity = bool(np.array_equal(dds_out.reshape(-1, 8), d_out.cpu().numpy()))

    # ---- learned endpoint proposal (shipped weights) on the same blocks, against the plain result
    from crunch2_gb300 import learned as LR
    net = LR.default_net()
    d_learned = torch.empty_like(d_out)
    rmse_plain = LR.rgb_rmse_torch(d_out, d_blocks)

    def learned_run(quality):
        for _ in range(args.warmup):
            flush.fill_(1)
            net.encode(d_blocks, threshold=LR.DEFAULT_THRESHOLD, out=d_learned, stream=stream, fallback_quality=quality)
        torch.cuda.synchronize()
        ln_start = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ln_end = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        fallbacks = 0
        for i in range(args.steps):
            flush.fill_(i & 0xFF)
            ln_start[i].record(stream)
            _, fallbacks = net.encode(d_blocks, threshold=LR.DEFAULT_THRESHOLD, out=d_learned, stream=stream,
                                      fallback_quality=quality)
            ln_end[i].record(stream)
        torch.cuda.synchronize()
        ln_ms = sum(s.elapsed_time(e) for s, e in zip(ln_start, ln_end)) / args.steps
        rmse_learned = LR.rgb_rmse_torch(d_learned, d_blocks)
        return {"value": round(texels / (ln_ms / 1e3) / 1e6, 3), "unit": "Mtexel/s", "ms_per_step": round(ln_ms, 4),
                "speedup_vs_plain": round(kernel_ms / ln_ms, 3), "rmse_plain": round(rmse_plain, 4),
                "rmse_learned": round(rmse_learned, 4), "rmse_delta": round(rmse_learned - rmse_plain, 4),
                "fallback_frac": round(fallbacks / n_blocks, 4), "threshold": LR.DEFAULT_THRESHOLD,
                "fallback_quality": QUALITY_NAMES[quality]}

    learned = learned_run(LR.DEFAULT_FALLBACK_QUALITY)
    learned.update({"weights": "crunch2_gb300/weights/dxt1_endpoint_net.npz",
                    "path": "crngpu_dxt1_learned_ex: fused MLP (k_mlp_infer) + refit (k_learned_refit) + exact "
                            "optimizer on the fallback blocks at the stated crn_dxt_quality; one host sync per call"})
    if LR.DEFAULT_FALLBACK_QUALITY != 4:
        learned["uber_fallback"] = learned_run(4)
    del net

    # ---- config 4's evaluation: the shipped weights on 32 held-out 4096x4096 textures (a seed
    # range the training never saw), learned vs plain encode time and RGB RMSE per texture
    config4_eval = None
    if "config4" not in skip:
        r4 = LR.config4(weights=LR.WEIGHTS, eval_textures=32, eval_size=4096, threshold=LR.DEFAULT_THRESHOLD,
                        fallback_quality=LR.DEFAULT_FALLBACK_QUALITY)
        g4 = r4["learned"][0]
        config4_eval = {"textures": r4["eval_textures"], "size": r4["eval_size"], "blocks": r4["eval_blocks"],
                        "plain_mtexel_s": round(r4["plain_mtexel_s"], 1),
                        "learned_mtexel_s": round(g4["learned_mtexel_s"], 1), "speedup": round(g4["speedup"], 3),
                        "rmse_plain": round(r4["rmse_plain"], 4), "rmse_learned": round(g4["rmse_learned"], 4),
                        "rmse_delta": round(g4["rmse_learned"] - r4["rmse_plain"], 4),
                        "fallback_frac": round(g4["fallback_frac"], 4), "threshold": LR.DEFAULT_THRESHOLD,
                        "fallback_quality": QUALITY_NAMES[LR.DEFAULT_FALLBACK_QUALITY],
                        "path": "learned.config4(weights=shipped): per texture, crngpu_dxt1_optimize_batch and "
                                "crngpu_dxt1_learned_ex on device blocks, CUDA events"}
        learned["config4_eval"] = config4_eval

    # ---- CRN -> DXT1 transcode: a batch of TX_BATCH textures (each its own context, i.e. its own
    # tables and palettes, holding the reference-encoded .crn of the same texture, q128, 11 levels)
    # in one persistent decode launch + one expansion launch, replayed as a CUDA graph
    with open(CRN_FIXTURE, "rb") as fh:
        crn = fh.read()
    ctx0 = cg.unpack_begin(crn)
    tx_bytes = sum(ctx0.level_bytes(l) for l in range(ctx0.levels))
    tx_blocks = tx_bytes // 8
    d_tx = torch.empty(tx_bytes, dtype=torch.uint8, device=dev)

    def timed(fn, steps):
        st = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        en = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        for i in range(steps):
            flush.fill_(i & 0xFF)
            st[i].record(stream)
            fn()
            en[i].record(stream)
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in zip(st, en)) / steps

    for _ in range(args.warmup):
        ctx0.unpack_levels(out=d_tx, stream=stream)
    single_ms = timed(lambda: ctx0.unpack_levels(out=d_tx, stream=stream), args.steps)
    # the same texture with every level on the lane decoder (one lane per level stream)
    cg.set_decode_split(cg.DECODE_LANE_ONLY)
    ctx0.unpack_levels(out=d_tx, stream=stream)
    single_lane_ms = timed(lambda: ctx0.unpack_levels(out=d_tx, stream=stream), max(3, args.steps // 4))
    cg.set_decode_split(cg.DECODE_SPLIT_DEFAULT)
    # a crnlib caller's sequence for one file: crnd_unpack_begin, crnd_unpack_level for every level
    # in turn, crnd_unpack_end (the C ABI's calls, device destinations), wall time per file
    lvl_views, o = [], 0
    for lv in range(ctx0.levels):
        nb = ctx0.level_bytes(lv)
        lvl_views.append(d_tx[o:o + nb].view(ctx0.faces, -1))
        o += nb

    def per_level_file():
        with cg.unpack_begin(crn) as c:
            for lv in range(c.levels):
                c.unpack_level(lv, out=lvl_views[lv], stream=stream)

    for _ in range(args.warmup):
        per_level_file()
    torch.cuda.synchronize()
    reps = max(5, args.steps)
    t0 = time.perf_counter()
    for _ in range(reps):
        per_level_file()
    torch.cuda.synchronize()
    per_level_ms = (time.perf_counter() - t0) / reps * 1e3
    per_level_parity = bool((d_tx.cpu().numpy() == ctx0.unpack_levels()).all())
    # the reference's own 2048x2048 DXT5 .crn (12 levels), one texture
    with open(os.path.join(ROOT, "tests", "golden", "crn", "dxt5_2048.crn"), "rb") as fh:
        crn5 = fh.read()
    with cg.unpack_begin(crn5) as ctx5:
        d5 = torch.empty(sum(ctx5.level_bytes(l) for l in range(ctx5.levels)), dtype=torch.uint8, device=dev)
        ctx5.unpack_levels(out=d5, stream=stream)
        single5_ms = timed(lambda: ctx5.unpack_levels(out=d5, stream=stream), max(3, args.steps // 4))
        single5_bytes = d5.numel()
    del d5
    ctxs = [cg.unpack_begin(crn) for _ in range(TX_BATCH)]
    outs = [torch.empty(tx_bytes, dtype=torch.uint8, device=dev) for _ in range(TX_BATCH)]
    batch = cg.UnpackBatch([(c, 0, c.levels, o) for c, o in zip(ctxs, outs)])
    for _ in range(args.warmup):
        batch.launch(use_graph=True, stream=stream)
    batch.status(stream=stream)
    tune_variant, tune_ms = batch.tuning()
    tx_parity = bool((outs[-1].cpu().numpy() == ctx0.unpack_levels()).all())
    batch_ms = timed(lambda: batch.launch(use_graph=True, stream=stream), args.steps)
    batch.status(stream=stream)
    with torch.cuda.nvtx.range("expand_only"):  # lets a profiler select these launches
        expand_ms = timed(lambda: batch.launch(expand_only=True, stream=stream), args.steps)
    # end to end through the C ABI: the batch plus the copy of every texture's DXT1 levels to
    # pinned host memory (the .crn files are uploaded once, by crngpu_unpack_begin)
    host_tx = torch.empty((TX_BATCH, tx_bytes), dtype=torch.uint8).pin_memory()

    def tx_e2e():
        batch.launch(use_graph=True, stream=stream)
        for i, o in enumerate(outs):
            host_tx[i].copy_(o, non_blocking=True)
        batch.status(stream=stream)

    tx_e2e()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        tx_e2e()
    tx_e2e_s = (time.perf_counter() - t0) / args.steps
    batch.close()
    for c in ctxs:
        c.close()
    del outs
    ctx0.close()
    exp_bytes = TX_BATCH * tx_blocks * 12  # 4-byte index record read + 8-byte DXT1 block written
    transcode = {"value": round(TX_BATCH * tx_bytes / (batch_ms / 1e3) / 1e9, 3), "unit": "GB/s",
                 "mtexel_s": round(TX_BATCH * texels / (batch_ms / 1e3) / 1e6, 1),
                 "ms_per_batch": round(batch_ms, 4), "textures_per_batch": TX_BATCH,
                 "output_bytes_per_batch": TX_BATCH * tx_bytes, "crn_bytes_per_texture": len(crn),
                 "parity_vs_single_context": tx_parity,
                 "e2e": {"value": round(TX_BATCH * tx_bytes / tx_e2e_s / 1e9, 3), "unit": "GB/s",
                         "h2d_bytes_per_step": 0, "d2h_bytes_per_step": TX_BATCH * tx_bytes,
                         "path": "crngpu_unpack_batch_launch (graph) + D2H of every level to pinned host memory"},
                 "single_texture": {"ms": round(single_ms, 4), "GB/s": round(tx_bytes / (single_ms / 1e3) / 1e9, 4),
                                    "lane_decoder_ms": round(single_lane_ms, 4),
                                    "per_level_calls_ms": round(per_level_ms, 4),
                                    "per_level_calls_parity": per_level_parity,
                                    "dxt5_2048_ms": round(single5_ms, 4),
                                    "dxt5_2048_GB/s": round(single5_bytes / (single5_ms / 1e3) / 1e9, 4),
                                    "path": "ctx.unpack_levels (crngpu_unpack_levels), device destination: levels of "
                                            ">= 256 blocks on k_crn_decode_wide (a CTA per level), the rest on the "
                                            "lane decoder; lane_decoder_ms: every level on the lane decoder; per_level_calls_ms: "
                                            "unpack_begin + crngpu_unpack_level per level + unpack_end, wall time "
                                            "per file (the crnd_unpack_level pattern)"},
                 "expand_roofline": None,
                 "expand_autotune": {"variant": tune_variant, "ms_per_variant": tune_ms,
                                     "variants": "0-11: tile of 1024 << (v >> 1) blocks, DXT1 palettes staged "
                                                 "in shared memory when v is odd; 12-15: 8192/16384-block tiles "
                                                 "with the next pass's records loaded ahead (staged when odd); "
                                                 "16, 17: 16384/32768-block tiles, pipelined, 4096-block passes; "
                                                 "18-20: 16384/32768-block tiles, records staged by TMA bulk "
                                                 "copies (palettes staged when v = 19), 2048-block passes"},
                 "workload": f"{TX_BATCH} contexts of the 1024x1024 q128 DXT1 .crn (11 levels, {len(crn)} bytes)"}
    expand = {"kernel": "k_crn_expand_tiles", "bound": "hbm", "unit": "GB/s",
              "ms": round(expand_ms, 4), "bytes_algorithmic": exp_bytes,
              "achieved": round(exp_bytes / (expand_ms / 1e3) / 1e9, 1)}

    # ---- crn_compress of the same mip chain at quality 128 (DXT1): clustered encode on the GPU
    # (crngpu_hc_compress) + the .crn writer (host); quality and size beside the reference's own
    # .crn of this texture (committed fixture), both decoded by the GPU transcoder
    clustered = None if "clustered" in skip else clustered_leg(cg, dev, levels, blocks, texels, args.steps)

    # ---- clustered DDS (the reference's QDXT1 path) of the same mip chain at quality 128
    qdxt = None if "qdxt" in skip else qdxt_leg(cg, dev, levels, blocks, texels, args.steps)

    # ---- the 2048x2048 DXT5 (colour + alpha noise) and DXN_XY (normal map) mip chains at quality
    # 128: crn_compress wall time, and the RMSEs of the GPU-decoded result beside those of the
    # reference's own .crn of the same textures (reference numbers committed with the fixtures)
    clustered_2048 = None if "clustered_2048" in skip else \
        clustered_2048_leg(cg, dev, steps=max(1, min(args.steps, 3)))

    # ---- 512 textures of uneven sizes and mixed formats: batched plain encode (one gather + two
    # persistent encoder launches, CUDA graph), their .crn through crn_compress, and the batched
    # transcode of those .crn files (one persistent decode + one expansion launch, CUDA graph)
    mixed_batch = None if "mixed" in skip else \
        mixed_batch_leg(cg, dev, stream, timed, steps=args.steps, warmup=args.warmup)

    # ---- mip generation (crunch's defaults: Kaiser, blurriness 0.9, gamma filtering, alpha) of a
    # 4096x4096 RGBA8 texture on the device: every level resampled from level 0
    mips = None if "mips" in skip else mips_leg(cg, dev, stream, timed, steps=args.steps, warmup=args.warmup)

    peaks, peak_kind = measured_peaks()
    clk = clocks.summary()
    sm_max = clk.get("sm_max_mhz") or peaks.get("sm_max_mhz", 2070.0)
    props = torch.cuda.get_device_properties(dev)
    peak_ops = props.multi_processor_count * 128 * sm_max * 1e6  # lane-ops/s: 4 SMSPs x 32 lanes per SM
    # algorithmic units: the reference's candidate x colour evaluations on this workload (a fixed
    # count, tests/golden/encode_work.json); the device's own executed count is reported beside it
    with open(ENCODE_WORK) as fh:
        work = json.load(fh)
    alg_evals = int(work["candidate_colour_evaluations"]) if work["blocks"] == n_blocks else evals
    achieved = alg_evals * LANE_OPS_PER_EVAL / (kernel_ms / 1e3)
    executed = evals * LANE_OPS_PER_EVAL / (kernel_ms / 1e3)
    roofline = {"bound": "alu", "kernel": "k_dxt1_encode", "achieved": round(achieved / 1e12, 3),
                "peak": round(peak_ops / 1e12, 3), "unit": "Tops/s", "frac": round(achieved / peak_ops, 4),
                "traffic": DXT1_ENCODE_DRAM["k_dxt1_encode"][0] + DXT1_ENCODE_DRAM["k_dxt1_encode"][1],
                "traffic_detail": {"read_write_bytes_per_launch": DXT1_ENCODE_DRAM,
                                   "source": "one ncu capture of the first timed step: dram__bytes_read.sum, "
                                             "dram__bytes_write.sum; the writes are mostly the L2 write-back of "
                                             "the 256 MiB flush before the step"},
                "peak_source": f"SMs x 128 lanes x max SM clock ({peak_kind} clock)",
                "evals_per_launch": alg_evals, "evals_source": "the reference's evaluate_solution loops on this "
                "workload, counted by the oracle (tests/golden/encode_work.json)",
                "evals_executed": evals, "frac_executed": round(executed / peak_ops, 4),
                "lane_ops_per_eval": LANE_OPS_PER_EVAL,
                "kernel_ms": round(kernel_ms, 4), "hbm_bytes_algorithmic": n_blocks * 72}
    expand["peak"] = peaks["hbm_gbs"]
    expand["frac"] = round(expand["achieved"] / peaks["hbm_gbs"], 4)
    expand["peak_source"] = f"{peak_kind} HBM copy bandwidth"
    transcode["expand_roofline"] = expand

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_encode_baseline(blocks, texels / n_blocks)
        transcode["cpu_baseline"] = cpu_transcode_baseline(crn, tx_bytes)
        transcode["vs_cpu"] = round(transcode["value"] / transcode["cpu_baseline"]["value"], 2)
        # one host thread transcoding the same single file (the reference's use case, one file per call)
        from oracle import port
        reps = 8
        secs = port.time_unpack(crn, reps, 1)
        transcode["single_texture"]["cpu_1_thread_ms"] = round(secs / reps * 1e3, 4)

    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 3), "unit": "Mtexel/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dev_s * 1e3 / args.steps, 4),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
                "data": "synthetic",
                "config": {"workload": "DXT1 uber encode, 1024x1024 RGBA8 + full box mip chain (11 levels, "
                                       "1,398,101 texels, 87,383 blocks), inputs resident in HBM",
                           "quality": "uber", "perceptual": True, "endpoint_caching": False,
                           "l2": "flushed between timed steps (256 MiB write)", "parallelism": f"replicas x{world}"},
                "parity_vs_oracle_sample": parity, "e2e_parity": e2e_parity,
                "e2e": {"value": round(drop_in_value, 3), "unit": "Mtexel/s",
                        "h2d_bytes_per_step": h2d_chain, "d2h_bytes_per_step": d2h_chain,
                        "parity_vs_device_encode": drop_in_parity,
                        "path": "crngpu_compress_dds_clustered at quality 255 (what crn_compress to DDS calls): "
                                "pageable host mip chain in, DDS block data out, one call per step; wall time"},
                "e2e_batch_launch": {"value": round(e2e_value, 3), "unit": "Mtexel/s", "h2d_bytes_per_step": h2d_chain,
                                     "d2h_bytes_per_step": d2h_chain, "parity_vs_device_encode": chain_parity,
                                     "grid": chain_grids[0],
                                     "path": "pinned host mip chain -> H2D -> crngpu_encode_batch_launch (CUDA graph) "
                                             "-> D2H -> host sync, every step; wall time"},
                "e2e_per_level": {"value": round(per_level_value, 3), "unit": "Mtexel/s", "h2d_bytes_per_step": h2d,
                                  "d2h_bytes_per_step": d2h,
                                  "path": "crngpu_compress_image per level (11 calls, each synchronous), "
                                          "pinned host buffers; wall time"},
                "learned": learned, "transcode": transcode, "clustered": clustered, "clustered_dds": qdxt,
                "clustered_2048": clustered_2048, "mixed_batch": mixed_batch, "mips": mips, "roofline": roofline,
                "cpu_baseline": cpu,
                "gpu_launches": args.steps * 2, "clocks": clk, "wall_s_timed": round(wall, 4)}
        # compact figures of every leg, last, so that a truncated log still carries them
        def pick(d, *keys):
            for k in keys:
                d = d.get(k) if isinstance(d, dict) else None
            return d
        line["summary"] = {
            "encode_mtexel_s": round(value, 1), "e2e_mtexel_s": round(drop_in_value, 1),
            "e2e_batch_launch_mtexel_s": round(e2e_value, 1),
            "encode_roofline_frac": roofline["frac"],
            "learned_mtexel_s": pick(learned, "value"), "learned_speedup": pick(learned, "speedup_vs_plain"),
            "learned_rmse_delta": pick(learned, "rmse_delta"),
            "learned_uber_fallback_speedup": pick(learned, "uber_fallback", "speedup_vs_plain"),
            "config4_learned_speedup": pick(learned, "config4_eval", "speedup"),
            "config4_rmse_delta": pick(learned, "config4_eval", "rmse_delta"),
            "transcode_batch_gb_s": transcode["value"], "transcode_single_ms": transcode["single_texture"]["ms"],
            "transcode_single_cpu_1_thread_ms": pick(transcode, "single_texture", "cpu_1_thread_ms"),
            "transcode_single_per_level_calls_ms": pick(transcode, "single_texture", "per_level_calls_ms"),
            "transcode_dxt5_2048_ms": transcode["single_texture"]["dxt5_2048_ms"],
            "expand_hbm_frac": expand["frac"],
            "mixed_encode_mtexel_s": pick(mixed_batch, "encode", "value"),
            "mixed_transcode_gb_s": pick(mixed_batch, "transcode", "value"),
            "crn_encode_mtexel_s": pick(clustered, "value"),
            "cpu_encode_mtexel_s": round(cpu["value"], 3) if cpu else None}
        print(json.dumps(line))


if __name__ == "__main__":
    main()
