"""Clustered (CRN-style) DXT1 on the GPU against the reference's own clustered compressor:
tests/golden/hc_reference.json holds what crnlib::dxt_hc::compress produced on the same blocks
(tile count, codebook sizes, RGB RMSE; generated by tests/golden/make_golden.py), and the
reference's q128 .crn of the 256 and 1024 textures (committed fixtures) gives the same RMSE.
The adaptive tiling is deterministic and restated bit-exactly (same tile count); the clusterizer
of the reference depends on its thread count, so codebooks are compared on quality."""
import json
import os
import numpy as np
import pytest

import golden_util as G
from dxt_decode import rgb_rmse

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def hc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crunch2_gb300 import hc
    hc._bind()
    return hc


def reference_rmse(name, levels):
    """RMSE of the reference's clustered encode: its .crn transcoded by the oracle, all levels."""
    from oracle import port
    from crunch2_gb300 import texgen
    crn = G.crn_bytes(name)
    m = G.manifest()[name]
    dec, src = [], []
    for l, img in enumerate(levels):
        dec.append(port.unpack_level(crn, l, m["levels"][l]["bytes"]).reshape(-1, 8))
        src.append(texgen.image_blocks(img))
    return rgb_rmse(np.concatenate(dec), np.concatenate(src))


def gpu_rmse(out, levels):
    from crunch2_gb300 import texgen
    dec = np.concatenate([out[l][0].reshape(-1, 8) for l in range(len(levels))])
    src = np.concatenate([texgen.image_blocks(img) for img in levels])
    return rgb_rmse(dec, src)


def hc_reference():
    with open(os.path.join(G.GOLDEN, "hc_reference.json")) as fh:
        return json.load(fh)


@pytest.mark.parametrize("name", ["hc_128", "dxt1_256", "c1_dxt1_1024"])
def test_clustered_dxt1_matches_reference_quality(hc, name):
    from crunch2_gb300 import texgen
    R = hc_reference()[name]
    size, seed = R["size"], R["seed"]
    levels = texgen.mip_chain(texgen.colour_texture(size, size, seed))
    out, stats = hc.compress_dxt1([levels], quality=128)
    ce, cs = stats["codebook_request"]
    assert [ce, cs] == R["codebook_request"] == list(hc.codebook_sizes(size, size, 128)[:2])
    assert stats["tiles"] == R["tiles"]  # determine_tiles_task restated exactly
    assert 0 < stats["color_endpoints"] <= ce
    assert 0 < stats["color_selectors"] <= cs
    ours = gpu_rmse(out, levels)
    if name in G.manifest():  # the committed .crn agrees with the reference run
        assert abs(reference_rmse(name, levels) - R["rmse_visible"]) < 1e-9
    print(f"{name}: GPU clustered RMSE {ours:.4f}, reference dxt_hc {R['rmse_visible']:.4f}, stats {stats}")
    assert ours <= 1.02 * R["rmse_visible"], (ours, R["rmse_visible"])


def test_clustered_dxt1_indices_reproduce_blocks(hc):
    """The endpoint/selector codebooks and per-block indices (what a .crn stores) rebuild exactly
    the DXT1 blocks the call returned."""
    from crunch2_gb300 import texgen
    levels = texgen.mip_chain(texgen.colour_texture(128, 128, 21))
    out, stats, idx = hc.compress_dxt1([levels], quality=128, with_indices=True)
    blocks, lv, vis = hc.crn_layout([levels])
    ei = idx["endpoint_index"].astype(np.uint16).astype(np.int64)
    si = idx["selector_index"].astype(np.uint16).astype(np.int64)
    eps = idx["endpoints"].astype(np.uint32)[:stats["color_endpoints"]]
    sels = idx["selectors"].astype(np.uint32)[:stats["color_selectors"]]
    assert ei.max() < len(eps) and si.max() < len(sels)
    first, second = eps & 0xFFFF, eps >> 16
    assert (first > second).all()  # 4-colour order
    from_linear = np.array([0, 2, 3, 1], np.uint32)
    lin = sels[si]
    dxt = np.zeros_like(lin)
    for p in range(16):
        dxt |= from_linear[(lin >> (2 * p)) & 3] << (2 * p)
    rebuilt = np.stack([eps[ei], dxt], 1).astype("<u4").view(np.uint8).reshape(-1, 8)
    fb, nb, bw = lv[0]
    bx, by, _ = vis[0]
    assert (rebuilt[fb:fb + nb].reshape(-1, bw, 8)[:by, :bx] == out[0][0]).all()


def test_codebook_sizes_follow_quality(hc):
    # crn_comp::quantize_images: 1024x1024 at q128 (the config-1 sizes) and the clamps at 0 / 255
    ce, cs, ae, as_ = hc.codebook_sizes(1024, 1024, 128)
    assert (ce, cs) == (2415, 2692)
    lo = hc.codebook_sizes(1024, 1024, 0)
    assert lo[0] == 64 and lo[1] == 96
    hi = hc.codebook_sizes(64, 64, 255)
    assert hi[0] == 256 and hi[1] == 256
    # the clamps use cCRNMinPaletteSize = 8: alpha endpoints reach 24 at quality 0, and an 8x8
    # texture (4 blocks) gets the minimum of 8 entries everywhere at full quality
    assert hc.codebook_sizes(1024, 1024, 0, hc.FMT_DXT5)[2:] == (24, 48)
    assert hc.codebook_sizes(8, 8, 255) == (8, 8, 8, 8)


@pytest.mark.parametrize("name", ["dxt5_256", "dxn_xy_256"])
def test_clustered_alpha_formats_match_reference_quality(hc, name):
    """DXT5 (colour + alpha) and DXN (two alpha channels) through crngpu_hc_compress against the
    reference dxt_hc on the same blocks: same tile count (the alpha tile errors are restated
    exactly), RGB and alpha RMSE within a few percent."""
    from crunch2_gb300 import texgen
    import crunch2_gb300 as cg
    from dxt_decode import dxt5a_values
    R = hc_reference()[name]
    size, seed = R["size"], R["seed"]
    img = texgen.normal_map(size, size, seed) if R["content"] == "normal" else \
        texgen.colour_texture(size, size, seed, with_alpha_noise=True)
    levels = texgen.mip_chain(img)
    fmt = cg.FMT_DXT5 if R["format"] == "DXT5" else cg.FMT_DXN_XY
    out, stats = hc.compress([levels], fmt, quality=128)
    assert list(stats["codebook_request"]) == R["codebook_request"]
    assert stats["tiles"] == R["tiles"]
    assert 0 < stats["alpha_endpoints"] <= R["codebook_request"][2]
    assert 0 < stats["alpha_selectors"] <= R["codebook_request"][3]
    dec = np.concatenate([out[l][0].reshape(-1, 16) for l in range(len(levels))])
    src = np.concatenate([texgen.image_blocks(im) for im in levels]).reshape(-1, 16, 4).astype(np.int64)
    if fmt == cg.FMT_DXT5:
        rc = rgb_rmse(dec[:, 8:], src.reshape(-1, 64).astype(np.uint8))
        a = dxt5a_values(dec[:, :8])
        ra = float(np.sqrt(((a - src[:, :, 3]) ** 2).mean()))
        print(f"{name}: colour RMSE {rc:.4f} (reference {R['rmse_color_visible']:.4f}), alpha {ra:.4f} "
              f"(reference {R['rmse_alpha_visible']:.4f}), stats {stats}")
        assert rc <= 1.03 * R["rmse_color_visible"]
    else:
        x, y = dxt5a_values(dec[:, :8]), dxt5a_values(dec[:, 8:])
        ra = float(np.sqrt((((x - src[:, :, 0]) ** 2).sum() + ((y - src[:, :, 1]) ** 2).sum()) / (2 * x.size)))
        print(f"{name}: alpha RMSE {ra:.4f} (reference {R['rmse_alpha_visible']:.4f}), stats {stats}")
    assert ra <= max(1.05 * R["rmse_alpha_visible"], R["rmse_alpha_visible"] + 0.02)


@pytest.mark.parametrize("name", ["c1_dxt1_1024", "dxt5_256", "dxn_xy_256", "dxt1_cube_64"])
def test_compress_crn_round_trip(hc, name):
    """crngpu_compress_crn (crn_compress with source mips -> .crn): the file transcodes on the GPU
    and in the oracle to the same blocks, at the reference's quality and a comparable size."""
    import crunch2_gb300 as cg
    from crunch2_gb300 import texgen
    from oracle import port
    from dxt_decode import dxt5a_values
    m = G.manifest()[name]
    w, h, faces = m["width"], m["height"], m["faces"]
    fmt = {"DXT1": cg.FMT_DXT1, "DXT5": cg.FMT_DXT5, "DXN_XY": cg.FMT_DXN_XY}[m["format"]]
    fl = []
    for f in range(faces):
        img = texgen.normal_map(w, h, m["seed"] + f) if m["content"] == "normal" else \
            texgen.colour_texture(w, h, m["seed"] + f, with_alpha_noise=(m["content"] == "colour_alpha"))
        fl.append(texgen.mip_chain(img))
    flags = 0 if m["content"] == "normal" else cg.FLAG_PERCEPTUAL
    crn = cg.compress_crn(fl, fmt, quality=128, flags=flags)
    ref_crn = G.crn_bytes(name)
    bpb = G.bytes_per_block(m["format"])
    ours_se = ref_se = 0.0
    with cg.unpack_begin(crn) as ctx:
        assert (ctx.width, ctx.height, ctx.levels, ctx.faces) == (w, h, len(fl[0]), faces)
        for l, info in enumerate(m["levels"]):
            gpu = ctx.unpack_level(l).reshape(-1)
            assert np.array_equal(gpu, port.unpack_level(crn, l, info["bytes"])), (name, l)
            ref = port.unpack_level(ref_crn, l, info["bytes"])
            src = np.concatenate([texgen.image_blocks(fl[f][l]) for f in range(faces)]).reshape(-1, 16, 4).astype(np.int64)
            for dec, acc in ((gpu, "ours"), (ref, "ref")):
                d = dec.reshape(-1, bpb)
                if m["format"] == "DXT1":
                    from dxt_decode import dxt1_colours
                    se = float(((dxt1_colours(d) - src[:, :, :3]) ** 2).sum())
                elif m["format"] == "DXT5":
                    from dxt_decode import dxt1_colours
                    se = float(((dxt1_colours(d[:, 8:]) - src[:, :, :3]) ** 2).sum() +
                               ((dxt5a_values(d[:, :8]) - src[:, :, 3]) ** 2).sum())
                else:
                    se = float(((dxt5a_values(d[:, :8]) - src[:, :, 0]) ** 2).sum() +
                               ((dxt5a_values(d[:, 8:]) - src[:, :, 1]) ** 2).sum())
                if acc == "ours":
                    ours_se += se
                else:
                    ref_se += se
    print(f"{name}: .crn {len(crn)} bytes (reference {len(ref_crn)}), squared error {ours_se:.0f} "
          f"(reference {ref_se:.0f})")
    assert ours_se <= 1.06 * ref_se
    assert len(crn) <= 1.4 * len(ref_crn)


def test_compress_crn_bitrate_search(hc):
    """Rate control (crn_comp_params::m_target_bitrate): the chosen file decodes, its bitrate is the
    one reported, it is at or below the target when some level reaches that, and the next quality
    level's file is above the target (the search found the boundary)."""
    import crunch2_gb300 as cg
    from crunch2_gb300 import texgen
    levels = texgen.mip_chain(texgen.colour_texture(256, 256, 31))
    texels = sum(l.shape[0] * l.shape[1] for l in levels)
    target = 1.6
    crn, q, rate = cg.compress_crn_bitrate([levels], target, cg.FMT_DXT1)
    assert abs(len(crn) * 8 / texels - rate) < 1e-4
    assert 0 <= q <= 255
    with cg.unpack_begin(crn) as c:
        assert c.levels == len(levels)
    same = cg.compress_crn([levels], cg.FMT_DXT1, quality=q)
    assert same == crn  # the search's file is the plain compress at the chosen level
    lowest = len(cg.compress_crn([levels], cg.FMT_DXT1, quality=0)) * 8 / texels
    if lowest <= target:
        assert rate <= target
        if q < 255:
            above = len(cg.compress_crn([levels], cg.FMT_DXT1, quality=q + 1)) * 8 / texels
            assert above > target or abs(above - target) < abs(rate - target) + 0.05
    print(f"target {target}: quality {q}, {rate:.4f} bpp (quality 0: {lowest:.4f})")


def test_compress_crn_batch_equals_single_calls(hc):
    """crngpu_compress_crn_batch (several host threads, one stream each) writes, for every item,
    exactly the file crngpu_compress_crn writes for it alone."""
    import crunch2_gb300 as cg
    from crunch2_gb300 import texgen
    items = []
    for i, (w, h, fmt, content) in enumerate([(64, 64, cg.FMT_DXT1, "colour"), (128, 32, cg.FMT_DXT5, "colour_alpha"),
                                              (48, 80, cg.FMT_DXN_XY, "normal"), (256, 256, cg.FMT_DXT1, "colour"),
                                              (16, 16, cg.FMT_DXT5A, "colour_alpha"), (100, 60, cg.FMT_DXT1, "colour")]):
        img = texgen.normal_map(w, h, 70 + i) if content == "normal" else \
            texgen.colour_texture(w, h, 70 + i, with_alpha_noise=content == "colour_alpha")
        items.append(([texgen.mip_chain(img)], fmt, 100 + 20 * i, 0 if content == "normal" else cg.FLAG_PERCEPTUAL))
    batch = cg.compress_crn_batch(items, threads=3)
    for it, got in zip(items, batch):
        assert got == cg.compress_crn(*it)


def qdxt_reference():
    with open(os.path.join(G.GOLDEN, "qdxt_reference.json")) as fh:
        return json.load(fh)


@pytest.mark.parametrize("name", ["qdxt_256_q128", "qdxt_256_q64", "qdxt_1024_q128"])
def test_clustered_dds_matches_reference_quality(hc, name):
    """Clustered DDS (crnlib's QDXT1 path: crn_compress to DDS below quality 255) against the
    reference's own output on the same mip chain (tests/golden/qdxt_reference.json): RGB RMSE within
    5% of the reference's, and the block data clustered like the reference's (distinct endpoint
    and selector words of the same order, far fewer than the blocks)."""
    import crunch2_gb300 as cg
    from crunch2_gb300 import texgen
    R = qdxt_reference()[name]
    levels = texgen.mip_chain(texgen.colour_texture(R["size"], R["size"], R["seed"]))
    blocks = cg.compress_dds_clustered([levels], quality=R["quality"])
    src = np.concatenate([texgen.image_blocks(im) for im in levels])
    assert blocks.shape == (R["blocks"], 8) == src.shape[:1] + (8,)
    ours = rgb_rmse(blocks, src)
    de = np.unique(blocks[:, :4].copy().view(np.uint32)).size
    ds = np.unique(blocks[:, 4:].copy().view(np.uint32)).size
    print(f"{name}: GPU RMSE {ours:.4f} (reference {R['rmse']:.4f}); distinct endpoints {de} "
          f"(reference {R['distinct_endpoints']}), selectors {ds} (reference {R['distinct_selectors']})")
    assert ours <= 1.05 * R["rmse"], (ours, R["rmse"])
    assert de <= 1.5 * R["distinct_endpoints"] and ds <= 1.5 * R["distinct_selectors"], (de, ds)


def test_clustered_dds_full_quality_is_the_block_encoder(hc):
    """At quality 255 the clustered DDS path is the plain block encoder on every level."""
    import crunch2_gb300 as cg
    from crunch2_gb300 import texgen
    levels = texgen.mip_chain(texgen.colour_texture(64, 48, 5))
    got = cg.compress_dds_clustered([levels], quality=255)
    want = np.concatenate([cg.compress_image(im, cg.FMT_DXT1, cg.FLAG_PERCEPTUAL | cg.FLAG_USE_BOTH_BLOCK_TYPES)
                           .reshape(-1, 8) for im in levels])
    assert np.array_equal(got, want)


@pytest.mark.parametrize("name", ["qdxt_dxt5_256_q128", "qdxt_dxn_xy_256_q128", "qdxt_dxt5a_256_q128",
                                  "qdxt_dxt5_256_q64"])
def test_clustered_dds_alpha_formats_match_reference_quality(hc, name):
    """Clustered DDS for DXT5 (qdxt1 on the colour element, qdxt5 on alpha), DXN (qdxt5 on each
    channel) and DXT5A against the reference's output on the same chain: per-element RMSE within
    5% (+0.02 for the near-lossless alpha channels) and codebook sizes of the same order."""
    import crunch2_gb300 as cg
    from crunch2_gb300 import texgen
    from crunch2_gb300 import quality as Q
    R = qdxt_reference()[name]
    img = texgen.normal_map(R["size"], R["size"], R["seed"]) if R["content"] == "normal" else \
        texgen.colour_texture(R["size"], R["size"], R["seed"], with_alpha_noise=True)
    levels = texgen.mip_chain(img)
    fmt = {"DXT5": cg.FMT_DXT5, "DXN_XY": cg.FMT_DXN_XY, "DXT5A": cg.FMT_DXT5A}[R["format"]]
    blocks = cg.compress_dds_clustered([levels], quality=R["quality"], flags=R["flags"] & 9, fmt=fmt)
    src = np.concatenate([texgen.image_blocks(im) for im in levels])
    assert blocks.shape[0] == R["blocks"] == src.shape[0]
    ours = Q.block_rmse(torch.from_numpy(blocks.copy()), torch.from_numpy(src), R["format"])
    stats = {}
    for k in range(blocks.shape[1] // 8):
        el = blocks[:, 8 * k:8 * k + 8].copy()
        if R["format"] == "DXT5" and k == 1:
            stats["distinct_colour_endpoints"] = int(np.unique(el[:, :4].view(np.uint32)).size)
            stats["distinct_colour_selectors"] = int(np.unique(el[:, 4:].view(np.uint32)).size)
        else:
            stats[f"distinct_alpha_endpoints_{k}"] = int(np.unique(el[:, :2].view(np.uint16)).size)
            sel = np.concatenate([el[:, 2:], np.zeros((el.shape[0], 2), np.uint8)], axis=1).view(np.uint64)
            stats[f"distinct_alpha_selectors_{k}"] = int(np.unique(sel).size)
    print(f"{name}: GPU {ours} {stats}; reference", {k: R[k] for k in list(ours) + list(stats)})
    for key, v in ours.items():
        assert v <= 1.05 * R[key] + (0.02 if key != "rmse_color" else 0.0), (key, v, R[key])
    for key, v in stats.items():
        assert v <= 2 * R[key] + 16, (key, v, R[key])


@pytest.mark.parametrize("name", ["dxt5_2048", "dxn_xy_2048"])
def test_config2_2048_crn_matches_reference_quality(hc, name):
    """Config 2: crn_compress (.crn, q128) of the 2048 x 2048 DXT5 and DXN_XY 12-level mip chains
    through crngpu_compress_crn, decoded by the GPU transcoder, against the reference's own .crn of
    the same textures (tests/golden/config2_reference.json): every RMSE within 2% and the bitrate
    within 3% of the reference's."""
    import crunch2_gb300 as cg
    from crunch2_gb300 import quality as Q
    from crunch2_gb300 import texgen
    with open(os.path.join(G.GOLDEN, "config2_reference.json")) as fh:
        r = json.load(fh)[name]
    size = r["size"]
    img = texgen.normal_map(size, size, r["seed"]) if r["content"] == "normal" else \
        texgen.colour_texture(size, size, r["seed"], with_alpha_noise=True)
    levels = texgen.mip_chain(img)
    assert len(levels) == r["levels"]
    fmt = {"DXT5": cg.FMT_DXT5, "DXN_XY": cg.FMT_DXN_XY}[r["format"]]
    crn = cg.compress_crn([levels], fmt, quality=128, flags=0 if r["content"] == "normal" else cg.FLAG_PERCEPTUAL)
    texels = sum(l.shape[0] * l.shape[1] for l in levels)
    with cg.unpack_begin(crn) as c:
        dec = c.unpack_levels()
    src = torch.from_numpy(np.concatenate([texgen.image_blocks(l) for l in levels])).cuda()
    q = Q.block_rmse(torch.from_numpy(dec.reshape(-1, 16)).cuda(), src, r["format"])
    bpt = 8 * len(crn) / texels
    print(name, {k: round(v, 4) for k, v in q.items()}, "bpt", round(bpt, 4), "reference",
          {k: round(r[k], 4) for k in q}, round(r["bits_per_texel"], 4))
    for k, v in q.items():
        assert v <= 1.02 * r[k], (k, v, r[k])
    assert bpt <= 1.03 * r["bits_per_texel"], (bpt, r["bits_per_texel"])


def bitrate_reference():
    with open(os.path.join(G.GOLDEN, "bitrate_reference.json")) as fh:
        return json.load(fh)


@pytest.mark.parametrize("name", sorted(bitrate_reference()))
def test_compress_crn_bitrate_matches_reference(hc, name):
    """Rate control against the reference: crn_compress with m_target_bitrate on the same seeded mip
    chain (tests/golden/bitrate_reference.json, crnlib/crn_texture_comp.cpp:143-260). The search runs
    on this library's own file sizes, which are within about 1% of the reference's, so it lands on
    the reference's quality level or one near it where the size barely changes with the level: the
    achieved bitrate within 1.5% of the reference's, the chosen level within 12 of it, and the
    bitrate at or below the target whenever the reference's is."""
    import crunch2_gb300 as cg
    from crunch2_gb300 import texgen
    r = bitrate_reference()[name]
    img = texgen.colour_texture(r["size"], r["size"], r["seed"], with_alpha_noise=(r["content"] == "colour_alpha"))
    levels = texgen.mip_chain(img)
    fmt = {"DXT1": cg.FMT_DXT1, "DXT5": cg.FMT_DXT5}[r["format"]]
    crn, q, rate = cg.compress_crn_bitrate([levels], r["target"], fmt)
    print(f"{name}: quality {q} (reference {r['quality']}), {rate:.4f} bpt (reference {r['bitrate']:.4f})")
    assert abs(q - r["quality"]) <= 12
    assert abs(rate - r["bitrate"]) <= 0.015 * r["bitrate"]
    if r["bitrate"] <= r["target"]:
        assert rate <= r["target"]
