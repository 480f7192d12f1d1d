"""GPU parity below Uber quality and for the block compressor's other DXT1 parameters.

The reference block compressor's outputs (tests/golden/blocks_quality.npz, made by
crn_compress_block with endpoint caching off) at superfast / fast / normal / better quality, with
grayscale sampling, with DXT1A transparency and with transparent indices for black, against the
CUDA encoders through the C ABI. The bar is the encoder's: at least 99.9% of blocks identical and
no differing block with a higher error than the reference's under the optimizer's own metric.
"""
import numpy as np
import pytest

import golden_util as G
from dxt_decode import dxt1_colours

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


@pytest.fixture(scope="module")
def goldq():
    return G.blocks_quality()


def luma(c):
    return (c[..., 0] * 19595 + c[..., 1] * 38470 + c[..., 2] * 7471 + 32768) >> 16


def block_error(blocks8, pixels, perceptual=True, gray=False, threshold=None):
    """The optimizer's metric of decoded DXT1 against the texels: perceptual (8, 25, 1), uniform, or
    squared luma difference; with a DXT1A threshold, transparent texels count only when they are
    not decoded as transparent."""
    dec = dxt1_colours(blocks8)
    px = pixels.reshape(-1, 16, 4).astype(np.int64)
    if gray:
        e = (luma(dec) - luma(px[:, :, :3])) ** 2
    else:
        w = np.array([8, 25, 1] if perceptual else [1, 1, 1])
        e = (((dec - px[:, :, :3]) ** 2) * w).sum(2)
    if threshold is not None:
        b = blocks8.astype(np.int64)
        sel = np.stack([(b[:, 4 + (i >> 2)] >> (2 * (i & 3))) & 3 for i in range(16)], 1)
        three = (b[:, 0] | (b[:, 1] << 8)) <= (b[:, 2] | (b[:, 3] << 8))
        clear = (px[:, :, 3] < threshold)
        e = np.where(clear, np.where(three[:, None] & (sel == 3), 0, 1 << 20), e)
    return e.sum(1)


def check(out, ref, pixels, **metric):
    same = (out == ref).all(1)
    if not same.all():
        e_out = block_error(out[~same], pixels[~same], **metric)
        e_ref = block_error(ref[~same], pixels[~same], **metric)
        assert (e_out <= e_ref).all(), "a differing block has a higher error than the reference"
    assert same.mean() >= 0.999, f"only {same.mean():.5f} of blocks identical"
    return same.mean()


@pytest.mark.parametrize("q", [0, 1, 2, 3])
@pytest.mark.parametrize("perc", [1, 0])
@pytest.mark.parametrize("both", [1, 0])
def test_dxt1_quality_levels(cg, gold, goldq, q, perc, both):
    blocks = gold["edge_in"]
    out = cg.dxt1_optimize(torch.from_numpy(blocks).cuda(), bool(perc), bool(both), quality=q).cpu().numpy()
    frac = check(out, goldq[f"dxt1_q{q}_p{perc}_b{both}"], blocks, perceptual=bool(perc))
    print(f"dxt1 q{q} p{perc} b{both}: identical {frac:.5f}")


@pytest.mark.parametrize("q", [0, 1, 2, 3])
@pytest.mark.parametrize("name,fmt", [("dxt5", 2), ("dxn_xy", 7), ("dxt5a", 9)])
@pytest.mark.parametrize("both", [1, 0])
def test_alpha_formats_quality_levels(cg, gold, goldq, q, name, fmt, both):
    flags = (cg.FLAG_PERCEPTUAL if name != "dxn_xy" else cg.FLAG_PERCEPTUAL) | (cg.FLAG_USE_BOTH_BLOCK_TYPES * both)
    out = cg.compress_blocks(gold["edge_in"], fmt, flags, quality=q)
    ref = goldq[f"{name}_q{q}_b{both}"]
    same = (out == ref).all(1).mean()
    assert same >= 0.999, same


@pytest.mark.parametrize("q", [4, 3, 1])
@pytest.mark.parametrize("both", [1, 0])
def test_dxt1_grayscale_sampling(cg, gold, goldq, q, both):
    blocks = gold["edge_in"]
    flags = cg.FLAG_PERCEPTUAL | cg.FLAG_GRAYSCALE | (cg.FLAG_USE_BOTH_BLOCK_TYPES * both)
    out = cg.compress_blocks(blocks, cg.FMT_DXT1, flags, quality=q)
    check(out, goldq[f"gray_q{q}_b{both}"], blocks, gray=True)


@pytest.mark.parametrize("q", [4, 3, 1])
@pytest.mark.parametrize("perc", [1, 0])
@pytest.mark.parametrize("both", [1, 0])
def test_dxt1a_transparency(cg, goldq, q, perc, both):
    blocks = goldq["alpha_in"]
    flags = cg.FLAG_DXT1A | (cg.FLAG_PERCEPTUAL * perc) | (cg.FLAG_USE_BOTH_BLOCK_TYPES * both)
    out = cg.compress_blocks(torch.from_numpy(blocks).cuda(), cg.FMT_DXT1, flags, quality=q).cpu().numpy()
    check(out, goldq[f"dxt1a_q{q}_p{perc}_b{both}"], blocks, perceptual=bool(perc), threshold=128)


@pytest.mark.parametrize("q", [4, 3, 1])
@pytest.mark.parametrize("mode", ["p1", "p0", "gray"])
def test_dxt1_transparent_indices_for_black(cg, goldq, q, mode):
    blocks = goldq["dark_in"]
    flags = cg.FLAG_TRANSPARENT_BLACK | cg.FLAG_USE_BOTH_BLOCK_TYPES | (cg.FLAG_PERCEPTUAL if mode == "p1" else 0) | \
        (cg.FLAG_GRAYSCALE if mode == "gray" else 0)
    out = cg.compress_blocks(blocks, cg.FMT_DXT1, flags, quality=q)
    ref = goldq[f"black_q{q}_{mode}" if mode != "gray" else f"black_gray_q{q}"]
    check(out, ref, blocks, perceptual=(mode == "p1"), gray=(mode == "gray"))
    # the trial changed blocks: some outputs are 3-colour blocks that decode near-black texels to black
    lo = out[:, 0].astype(np.int64) | (out[:, 1].astype(np.int64) << 8)
    hi = out[:, 2].astype(np.int64) | (out[:, 3].astype(np.int64) << 8)
    assert (lo <= hi).any()


def test_optimize_batch_error_output_with_black_trial(cg, goldq):
    """results::m_error after try_alpha_as_black_optimization: the lower of the two errors."""
    from oracle import port
    blocks = goldq["dark_in"][:512]
    out, err = cg.dxt1_optimize(blocks, True, True, with_error=True, transparent_black=True)
    ref, ref_err = port.dxt1_blocks_ex(blocks, True, True, transparent_black=True, threads=4)
    same = (out == ref).all(1)
    assert same.mean() >= 0.999
    assert np.array_equal(err[same], ref_err[same])


def test_legacy_params_layout_is_uber(cg, gold):
    """A crngpu_dxt1_params of the earlier four-field layout (struct_size 16) encodes at Uber."""
    import ctypes
    blocks = np.ascontiguousarray(gold["edge_in"][:256])
    out = np.zeros((256, 8), np.uint8)
    p = cg._Dxt1Params(16, 1, 1, 0)
    rc = cg.lib().crngpu_dxt1_optimize_batch(blocks.ctypes.data, 256, ctypes.byref(p), out.ctypes.data, None,
                                             cg.MEM_HOST, None)
    assert rc == 0
    assert np.array_equal(out, gold["edge_dxt1_p1_b1"][:256])


def test_rejects_bad_options(cg, gold):
    with pytest.raises(cg.CrnGpuError):
        cg.compress_blocks(gold["edge_in"][:4], cg.FMT_DXT1, quality=5)
    with pytest.raises(cg.CrnGpuError):
        cg.dxt1_optimize(gold["edge_in"][:4], quality=7)
