"""GPU parity: the CUDA path through the C ABI against the reference's golden vectors and the
oracle (CPU restatement pinned to those vectors)."""
import numpy as np
import pytest

import golden_util as G
from dxt_decode import dxt1_error, rgb_rmse

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def cg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import crunch2_gb300
    crunch2_gb300.lib()
    return crunch2_gb300


@pytest.fixture(scope="module")
def gold():
    return G.blocks()


def check_dxt1(out, ref, pixels, perceptual, exact_min=0.999):
    """>= 99.9% identical blocks, no differing block with a higher error, RMSE within 0.01."""
    same = (out == ref).all(1)
    frac = same.mean()
    if not same.all():
        e_out = dxt1_error(out[~same], pixels[~same], perceptual)
        e_ref = dxt1_error(ref[~same], pixels[~same], perceptual)
        assert (e_out <= e_ref).all(), "a differing block has a higher error than the reference"
    assert abs(rgb_rmse(out, pixels) - rgb_rmse(ref, pixels)) <= 0.01
    assert frac >= exact_min, f"only {frac:.5f} of blocks identical"
    return frac


@pytest.mark.parametrize("perc", [1, 0])
@pytest.mark.parametrize("both", [1, 0])
@pytest.mark.parametrize("device", [True, False])
def test_dxt1_edge_blocks(cg, gold, perc, both, device):
    blocks = gold["edge_in"]
    inp = torch.from_numpy(blocks).cuda() if device else blocks
    out = cg.dxt1_optimize(inp, bool(perc), bool(both))
    out = out.cpu().numpy() if device else out
    frac = check_dxt1(out, gold[f"edge_dxt1_p{perc}_b{both}"], blocks, bool(perc))
    print(f"edge dxt1 p{perc} b{both}: identical {frac:.5f}")


def test_dxt1_config0_texture(cg, gold):
    blocks = G.c0_blocks()
    out = cg.dxt1_optimize(torch.from_numpy(blocks).cuda()).cpu().numpy()
    check_dxt1(out, gold["c0_dxt1"], blocks, True)


def test_dxt1_error_output_matches_oracle(cg, gold):
    from oracle import port
    blocks = gold["edge_in"][:512]
    out, err = cg.dxt1_optimize(blocks, True, True, with_error=True)
    ref, ref_err = port.dxt1_blocks(blocks, True, True)
    same = (out == ref).all(1)
    assert (err[same] == ref_err[same]).all()


@pytest.mark.parametrize("name,fmt", [("dxt5", 2), ("dxn_xy", 7), ("dxn_yx", 8), ("dxt5a", 9)])
@pytest.mark.parametrize("both", [1, 0])
def test_alpha_formats(cg, gold, name, fmt, both):
    flags = cg.FLAG_PERCEPTUAL | (cg.FLAG_USE_BOTH_BLOCK_TYPES if both else 0)
    out = cg.compress_blocks(gold["edge_in"], fmt, flags)
    ref = gold[f"edge_{name}_b{both}"]
    same = (out == ref).all(1)
    if fmt == 2:  # colour half goes through the float optimizer: same bar as DXT1
        assert (out[:, :8] == ref[:, :8]).all(), "DXT5 alpha half must be bit-exact"
        check_dxt1(out[:, 8:], ref[:, 8:], gold["edge_in"], True)
    else:
        assert same.all(), np.nonzero(~same)[0][:10]


def test_dxt5_dxn_textures(cg, gold):
    out = cg.compress_blocks(G.dxt5_tex_blocks(), 2, cg.FLAG_PERCEPTUAL | cg.FLAG_USE_BOTH_BLOCK_TYPES)
    ref = gold["dxt5_tex_dxt5"]
    assert (out[:, :8] == ref[:, :8]).all()
    check_dxt1(out[:, 8:], ref[:, 8:], G.dxt5_tex_blocks(), True)
    nrm = cg.compress_blocks(G.nrm_tex_blocks(), 7, cg.FLAG_USE_BOTH_BLOCK_TYPES)
    assert (nrm == gold["nrm_tex_dxn_xy"]).all()


def test_compress_image_edge_clamp(cg):
    from crunch2_gb300 import texgen
    from oracle import port
    img = texgen.colour_texture(37, 22, 5)  # ragged: 10 x 6 blocks with clamped edges
    out = cg.compress_image(img, cg.FMT_DXT1)
    ref, _ = port.dxt1_blocks(texgen.image_blocks(img), True, True)
    assert (out == ref).all(1).mean() >= 0.999
    dev = cg.compress_image(torch.from_numpy(img).cuda(), cg.FMT_DXT1).cpu().numpy()
    assert (dev == out).all()


def test_empty_batch(cg):
    out = cg.dxt1_optimize(np.zeros((0, 64), np.uint8))
    assert out.shape == (0, 8)


# ------------------------------------------------------------------------------------------
# transcoder

@pytest.mark.parametrize("name", sorted(G.manifest().keys()))
def test_transcode_levels_bit_exact(cg, name):
    m = G.manifest()[name]
    crn = G.crn_bytes(name)
    with cg.unpack_begin(crn) as ctx:
        assert (ctx.width, ctx.height, ctx.faces) == (m["width"], m["height"], m["faces"])
        for lvl, info in enumerate(m["levels"]):
            out = ctx.unpack_level(lvl)
            assert G.sha(out.reshape(-1)) == info["sha256"], (name, lvl)
            dev = torch.zeros(out.size, dtype=torch.uint8, device="cuda")
            ctx.unpack_level(lvl, out=dev.view(ctx.faces, -1))
            assert G.sha(dev.cpu().numpy()) == info["sha256"], (name, lvl, "device")
        allv = ctx.unpack_levels()
        pos = 0
        for lvl, info in enumerate(m["levels"]):
            assert G.sha(allv[pos:pos + info["bytes"]]) == info["sha256"]
            pos += info["bytes"]


@pytest.fixture
def decode_split(cg):
    """Sets crngpu_set_decode_split for one test and restores the default after it."""
    def set_split(mode):
        cg.set_decode_split({"wide": cg.DECODE_WIDE_ONLY, "lane": cg.DECODE_LANE_ONLY}[mode])
    yield set_split
    cg.set_decode_split(cg.DECODE_SPLIT_DEFAULT)


@pytest.mark.parametrize("mode", ["wide", "lane"])
@pytest.mark.parametrize("name", sorted(G.manifest().keys()))
def test_transcode_each_decoder_bit_exact(cg, decode_split, name, mode):
    """Every level of every fixture through one decoder alone: the wide decoder (a CTA per level,
    1x1 mip levels and cube faces included) or the lane decoder (a lane per level stream), against
    the reference's per-level SHA-256, one level per call and all levels in one call."""
    decode_split(mode)
    m = G.manifest()[name]
    with cg.unpack_begin(G.crn_bytes(name)) as ctx:
        for lvl, info in enumerate(m["levels"]):
            assert G.sha(ctx.unpack_level(lvl).reshape(-1)) == info["sha256"], (name, lvl, mode)
        allv = ctx.unpack_levels()
        pos = 0
        for lvl, info in enumerate(m["levels"]):
            assert G.sha(allv[pos:pos + info["bytes"]]) == info["sha256"], (name, lvl, mode, "all levels")
            pos += info["bytes"]


@pytest.mark.parametrize("name", ["dxt1_256", "dxt5_256", "dxn_xy_256", "dxt5a_256", "dxt5_cube_64x32"])
def test_transcode_decoders_agree_on_corrupt_streams(cg, decode_split, name):
    """Random bytes written over a level's stream: the wide and the lane decoder return the same
    outcome -- the same error code, or the same bytes when the stream still decodes."""
    import struct
    crn = bytes(G.crn_bytes(name))
    nlev = len(G.manifest()[name]["levels"])
    ofs = [struct.unpack(">I", crn[70 + 4 * l:74 + 4 * l])[0] for l in range(nlev)] + [len(crn)]
    rng = np.random.default_rng(11)
    for trial in range(12):
        lvl = trial % 2
        bad = bytearray(crn)
        span = ofs[lvl + 1] - ofs[lvl]
        pos = ofs[lvl] + int(rng.integers(0, max(1, span - 16)))
        n = int(min(32, ofs[lvl + 1] - pos))
        bad[pos:pos + n] = rng.integers(0, 256, n, dtype=np.uint8).tobytes()
        outcome = {}
        for mode in ("wide", "lane"):
            decode_split(mode)
            with cg.unpack_begin(bytes(bad)) as ctx:
                try:
                    outcome[mode] = ("ok", G.sha(ctx.unpack_level(lvl).reshape(-1)))
                except cg.CrnGpuError as e:
                    outcome[mode] = ("error", e.code)
        assert outcome["wide"] == outcome["lane"], (name, trial, outcome)


@pytest.mark.parametrize("name", ["dxt1_256", "dxt5_256", "dxt5_cube_64x32"])
def test_per_level_calls_with_a_corrupt_level(cg, name):
    """crngpu_unpack_level decodes every level on its first call and serves later calls from
    that decode; a level the decoder rejects must not take the others with it: with one level's
    stream overwritten, every other level, asked for in any order, is still bit-exact."""
    import struct
    crn = bytearray(G.crn_bytes(name))
    levels = G.manifest()[name]["levels"]
    ofs = [struct.unpack(">I", bytes(crn[70 + 4 * l:74 + 4 * l]))[0] for l in range(len(levels))] + [len(crn)]
    bad = 1
    crn[ofs[bad]:ofs[bad + 1]] = bytes([0xFF]) * (ofs[bad + 1] - ofs[bad])
    order = list(range(len(levels)))[::-1]
    with cg.unpack_begin(bytes(crn)) as ctx:
        for lvl in order:
            if lvl == bad:
                try:
                    ctx.unpack_level(lvl)
                except cg.CrnGpuError:
                    pass
                continue
            assert G.sha(ctx.unpack_level(lvl).reshape(-1)) == levels[lvl]["sha256"], (name, lvl)
    # intact file, levels in a shuffled order, twice over the same context
    with cg.unpack_begin(G.crn_bytes(name)) as ctx:
        for lvl in [2, 0, 1] + list(range(len(levels))):
            assert G.sha(ctx.unpack_level(lvl).reshape(-1)) == levels[lvl]["sha256"], (name, lvl)


@pytest.mark.parametrize("use_graph", [False, True])
def test_transcode_batch_mixed_formats(cg, use_graph):
    """Every fixture (DXT1, DXT5, DXN, DXT5A, cube maps, NPOT) in one batch, each twice with its
    own context: one persistent decode launch + one expansion, replayed; bit-exact per level."""
    man = G.manifest()
    names = sorted(man) * 2
    ctxs = [cg.unpack_begin(G.crn_bytes(n)) for n in names]
    outs = [torch.full((sum(l["bytes"] for l in man[n]["levels"]),), 0xCD, dtype=torch.uint8, device="cuda")
            for n in names]
    with cg.UnpackBatch([(c, 0, c.levels, o) for c, o in zip(ctxs, outs)]) as batch:
        assert batch.bytes == sum(o.numel() for o in outs)
        for rep in range(3):
            for o in outs:
                o.fill_(0xCD)
            batch.launch(use_graph=use_graph)
            batch.status()
            for n, o in zip(names, outs):
                host = o.cpu().numpy()
                pos = 0
                for lvl, info in enumerate(man[n]["levels"]):
                    assert G.sha(host[pos:pos + info["bytes"]]) == info["sha256"], (n, lvl, rep)
                    pos += info["bytes"]
    for c in ctxs:
        c.close()


def test_transcode_batch_every_expansion_variant(cg):
    """Every expansion variant (tile sizes, staged palettes, pipelined passes, TMA-staged records)
    writes the golden levels of every fixture, cube faces whose records start mid-line included."""
    man = G.manifest()
    names = sorted(man)
    ctxs = [cg.unpack_begin(G.crn_bytes(n)) for n in names]
    outs = [torch.full((sum(l["bytes"] for l in man[n]["levels"]),), 0xCD, dtype=torch.uint8, device="cuda")
            for n in names]
    with cg.UnpackBatch([(c, 0, c.levels, o) for c, o in zip(ctxs, outs)]) as batch:
        batch.launch()
        batch.status()
        nvar = len(batch.tuning()[1])
        assert nvar == 21
        for v in range(nvar):
            batch.set_variant(v)
            for o in outs:
                o.fill_(0xCD)
            batch.launch(use_graph=(v % 2 == 1))
            batch.status()
            for n, o in zip(names, outs):
                host = o.cpu().numpy()
                pos = 0
                for lvl, info in enumerate(man[n]["levels"]):
                    assert G.sha(host[pos:pos + info["bytes"]]) == info["sha256"], (v, n, lvl)
                    pos += info["bytes"]
        with pytest.raises(cg.CrnGpuError):
            batch.set_variant(nvar)
    for c in ctxs:
        c.close()


def test_transcode_batch_level_subset(cg):
    man = G.manifest()
    crn = G.crn_bytes("c1_dxt1_1024")
    with cg.unpack_begin(crn) as ctx:
        lv = man["c1_dxt1_1024"]["levels"]
        out = torch.zeros(sum(l["bytes"] for l in lv[3:7]), dtype=torch.uint8, device="cuda")
        with cg.UnpackBatch([(ctx, 3, 4, out)]) as batch:
            batch.launch()
            batch.status()
        host = out.cpu().numpy()
        pos = 0
        for info in lv[3:7]:
            assert G.sha(host[pos:pos + info["bytes"]]) == info["sha256"]
            pos += info["bytes"]
        small = torch.zeros(10, dtype=torch.uint8, device="cuda")
        with pytest.raises(cg.CrnGpuError):
            cg.UnpackBatch([(ctx, 0, 2, small)])


def test_transcode_row_pitch_padding(cg):
    crn = G.crn_bytes("dxt5_256")
    with cg.unpack_begin(crn) as ctx:
        bx, by = ctx.level_dims(1)
        pitch = bx * 16 + 20  # multiple of 4, not 16: exercises the scalar store path
        out = np.full((1, by * pitch), 0xAB, np.uint8)
        ctx.unpack_level(1, row_pitch=pitch, out=out)
        tight = ctx.unpack_level(1).reshape(by, bx * 16)
        rows = out.reshape(by, pitch)
        assert (rows[:, :bx * 16] == tight).all()
        assert (rows[:, bx * 16:] == 0xAB).all()


def test_transcode_segmented(cg):
    import struct
    crn = G.crn_bytes("dxt1_256")
    ofs = [struct.unpack(">I", crn[70 + 4 * l:74 + 4 * l])[0] for l in range(9)]
    with cg.unpack_begin(crn) as ctx:
        for lvl in (0, 3, 8):
            end = ofs[lvl + 1] if lvl + 1 < 9 else len(crn)
            seg = np.frombuffer(crn[ofs[lvl]:end], np.uint8).copy()
            bx, by = ctx.level_dims(lvl)
            out = np.zeros(bx * by * 8, np.uint8)
            faces = (cg.ctypes.c_void_p * 1)(out.ctypes.data)
            rc = cg.lib().crngpu_unpack_level_segmented(ctx.handle, seg.ctypes.data, seg.size, faces, out.size, 0,
                                                        lvl, cg.MEM_HOST, None)
            assert rc == 0
            assert (out == ctx.unpack_level(lvl).reshape(-1)).all()


def test_crn_decompress_contract(cg):
    crn = G.crn_bytes("c1_dxt1_1024")
    m = G.manifest()["c1_dxt1_1024"]
    total = sum(l["bytes"] for l in m["levels"][2:6])
    out = cg.crn_decompress(crn, 2, 4, total)
    pos = 0
    for info in m["levels"][2:6]:
        assert G.sha(out[pos:pos + info["bytes"]]) == info["sha256"]
        pos += info["bytes"]


def test_transcode_rejects_bad_input(cg):
    crn = bytearray(G.crn_bytes("dxt1_256"))
    with pytest.raises(cg.CrnGpuError):
        cg.unpack_begin(bytes(crn[:60]))
    bad = bytearray(crn)
    bad[0] ^= 0xFF
    with pytest.raises(cg.CrnGpuError):
        cg.unpack_begin(bytes(bad))
    with cg.unpack_begin(bytes(crn)) as ctx:
        with pytest.raises(cg.CrnGpuError):
            ctx.unpack_level(0, row_pitch=6)
        with pytest.raises(cg.CrnGpuError):
            ctx.unpack_level(99)


def test_transcode_corrupt_stream_reports_error(cg):
    """Random garbage in a level's block stream must come back as an error or as some output,
    never as a hang or a fault; the device decoder bounds every table and palette index."""
    import struct
    crn = bytearray(G.crn_bytes("dxt5_256"))
    lvl0 = struct.unpack(">I", bytes(crn[70:74]))[0]
    rng = np.random.default_rng(7)
    for trial in range(8):
        bad = bytearray(crn)
        pos = lvl0 + int(rng.integers(0, 64))
        bad[pos:pos + 64] = rng.integers(0, 256, 64, dtype=np.uint8).tobytes()
        with cg.unpack_begin(bytes(bad)) as ctx:
            try:
                ctx.unpack_level(0)
            except cg.CrnGpuError as e:
                assert e.code == cg.E_CORRUPT


def test_dxt1_full_1024_mip_chain_against_oracle(cg):
    """Every block of the 1024 x 1024 texture's 11-level box mip chain (87,383 blocks, the encode
    workload timed by the benchmark), perceptual with 3-colour blocks, through the batched encoder
    (one launch for the whole chain), against the oracle on all host threads: >= 99.9% of blocks
    identical, no differing block with a higher error, RGB RMSE within 0.01 -- per level and over
    the chain."""
    import os
    from crunch2_gb300 import texgen
    from oracle import port
    levels = texgen.mip_chain(texgen.colour_texture(1024, 1024, 100))
    rgba = torch.from_numpy(np.concatenate([l.reshape(-1) for l in levels])).cuda()
    out = torch.zeros(cg.mip_chain_blocks(1024, 1024, len(levels)) * 8, dtype=torch.uint8, device="cuda")
    with cg.EncodeBatch([(rgba, out, 1024, 1024, len(levels), cg.FMT_DXT1)]) as b:
        b.launch()
    got = out.cpu().numpy().reshape(-1, 8)
    blocks = np.concatenate([texgen.image_blocks(l) for l in levels])
    assert got.shape[0] == blocks.shape[0] == 87383
    ref, _ = port.dxt1_blocks(blocks, True, True, threads=os.cpu_count() or 4)
    ofs = 0
    for l in levels:
        n = texgen.image_blocks(l).shape[0]
        check_dxt1(got[ofs:ofs + n], ref[ofs:ofs + n], blocks[ofs:ofs + n], True)
        ofs += n
    frac = check_dxt1(got, ref, blocks, True)
    print(f"1024 chain: {frac:.5f} of {got.shape[0]} blocks identical to the oracle")


def test_transcode_batch_of_own_files_matches_oracle(cg):
    """Files this library writes (crngpu_compress_crn) in the shapes of config 3's mixed batch --
    non-square sizes from 32 to 512, full mip chains, DXT1 / DXT5 / DXN_XY / DXT5A -- decoded in one
    batch (the plan's split sends the larger levels to the wide decoder), every level against the
    oracle's CPU restatement of crnd's unpacker (pinned to the reference's transcodes)."""
    from crunch2_gb300 import texgen
    from oracle import port
    shapes = [(512, 256, cg.FMT_DXT1), (256, 512, cg.FMT_DXT5), (512, 512, cg.FMT_DXN_XY), (128, 32, cg.FMT_DXT1),
              (32, 256, cg.FMT_DXT5A), (512, 128, cg.FMT_DXT5)]
    files = []
    for i, (w, h, fmt) in enumerate(shapes):
        img = texgen.normal_map(w, h, 700 + i) if fmt == cg.FMT_DXN_XY else \
            texgen.colour_texture(w, h, 700 + i, with_alpha_noise=fmt in (cg.FMT_DXT5, cg.FMT_DXT5A))
        files.append(cg.compress_crn([texgen.mip_chain(img)], fmt=fmt, quality=128))
    ctxs = [cg.unpack_begin(f) for f in files]
    outs = [torch.zeros(sum(c.level_bytes(l) for l in range(c.levels)), dtype=torch.uint8, device="cuda") for c in ctxs]
    with cg.UnpackBatch([(c, 0, c.levels, o) for c, o in zip(ctxs, outs)]) as batch:
        batch.launch()
        batch.status()
    for f, c, o in zip(files, ctxs, outs):
        host = o.cpu().numpy()
        pos = 0
        for lvl in range(c.levels):
            n = c.level_bytes(lvl)
            want = port.unpack_level(f, lvl, n)
            assert want is not None and np.array_equal(host[pos:pos + n], want), (c.width, c.height, lvl)
            pos += n
        c.close()


@pytest.mark.parametrize("mode", ["wide", "lane"])
def test_transcode_widest_rows_match_oracle(cg, decode_split, mode):
    """The widest rows a .crn holds: a 4096 x 32 DXT1 and a 4096 x 64 DXT5 texture (rows of 1024
    blocks, the wide decoder's largest row buffer), written by this library, every level through
    one decoder against the oracle's crnd restatement."""
    from crunch2_gb300 import texgen
    from oracle import port
    decode_split(mode)
    for w, h, fmt, seed in ((4096, 32, cg.FMT_DXT1, 900), (4096, 64, cg.FMT_DXT5, 901)):
        img = texgen.colour_texture(w, h, seed, with_alpha_noise=fmt == cg.FMT_DXT5)
        crn = cg.compress_crn([texgen.mip_chain(img)], fmt=fmt, quality=96)
        with cg.unpack_begin(crn) as ctx:
            for lvl in range(ctx.levels):
                n = ctx.level_bytes(lvl)
                want = port.unpack_level(crn, lvl, n)
                assert want is not None and np.array_equal(ctx.unpack_level(lvl).reshape(-1), want), (w, h, lvl, mode)
