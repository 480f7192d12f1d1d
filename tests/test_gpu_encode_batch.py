"""Batched plain encode (crngpu_encode_batch_*): the mip chains of textures of mixed sizes and
formats, encoded by one gather launch and two persistent encoder launches, must give exactly the
blocks crngpu_compress_image gives on each level -- directly and replayed from the CUDA graph --
and the oracle's on a sample of them."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def cg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import crunch2_gb300
    crunch2_gb300.lib()
    return crunch2_gb300


# (width, height, format, content, seed): NPOT, 1-texel and tall/wide chains, every format family
CASES = [(32, 32, "DXT1", "colour", 1), (64, 128, "DXT5", "colour_alpha", 2), (100, 60, "DXN_XY", "normal", 3),
         (256, 32, "DXT1", "colour", 4), (48, 48, "DXT5A", "colour_alpha", 5), (1, 1, "DXT1", "colour", 6),
         (128, 64, "DXN_YX", "normal", 7), (512, 512, "DXT1", "colour", 8), (8, 200, "DXT5", "colour_alpha", 9),
         (300, 5, "DXT5A", "colour_alpha", 10)]


def make_items(cg, cases):
    from crunch2_gb300 import texgen
    fmts = {"DXT1": cg.FMT_DXT1, "DXT5": cg.FMT_DXT5, "DXN_XY": cg.FMT_DXN_XY, "DXN_YX": cg.FMT_DXN_YX,
            "DXT5A": cg.FMT_DXT5A}
    items, chains = [], []
    for w, h, fmt, content, seed in cases:
        img = texgen.normal_map(w, h, seed) if content == "normal" else \
            texgen.colour_texture(w, h, seed, with_alpha_noise=(content == "colour_alpha"))
        levels = texgen.mip_chain(img)
        rgba = torch.from_numpy(np.concatenate([l.reshape(-1) for l in levels])).cuda()
        f = fmts[fmt]
        out = torch.zeros(cg.mip_chain_blocks(w, h, len(levels)) * cg.bytes_per_block(f), dtype=torch.uint8,
                          device="cuda")
        items.append((rgba, out, w, h, len(levels), f))
        chains.append(levels)
    return items, chains


@pytest.mark.parametrize("flags", ["perceptual_both", "uniform"])
def test_batch_equals_per_image(cg, flags):
    fl = cg.FLAG_PERCEPTUAL | cg.FLAG_USE_BOTH_BLOCK_TYPES if flags == "perceptual_both" else 0
    items, chains = make_items(cg, CASES)
    with cg.EncodeBatch(items, fl) as b:
        assert b.blocks == sum(cg.mip_chain_blocks(w, h, n) for _, _, w, h, n, _ in items)
        for use_graph in (False, True, True):
            for _, out, *_ in items:
                out.zero_()
            b.launch(use_graph=use_graph)
            torch.cuda.synchronize()
            for (rgba, out, w, h, n, f), levels in zip(items, chains):
                got = out.cpu().numpy()
                ofs = 0
                for l in levels:
                    ref = np.asarray(cg.compress_image(l, f, fl)).reshape(-1)
                    assert np.array_equal(got[ofs:ofs + ref.size], ref), (w, h, f, l.shape, use_graph)
                    ofs += ref.size
                assert ofs == got.size
        grids, ms = b.tuning()
        assert grids[0] > 0 and grids[1] > 0 and len(ms) == 8


def test_batch_rejects_bad_items(cg):
    items, _ = make_items(cg, CASES[:2])
    rgba, out, w, h, n, f = items[0]
    with pytest.raises(cg.CrnGpuError):
        cg.EncodeBatch([(rgba, out, w, h, n + 5, f)])  # more levels than the chain has
    with pytest.raises(cg.CrnGpuError):
        cg.EncodeBatch([(rgba, out, w, h, n, 4)])  # a format this encoder does not write (DXT3)
    with pytest.raises(cg.CrnGpuError):
        cg.EncodeBatch([(rgba, out[:8], w, h, n, f)])  # output too small
