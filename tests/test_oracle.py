"""Pins the CPU restatement (oracle/) against the golden vectors made by the reference crnlib."""
import numpy as np
import pytest

import golden_util as G
from oracle import port

FMT = {"dxt5": 2, "dxn_xy": 7, "dxn_yx": 8, "dxt5a": 9}


@pytest.fixture(scope="module")
def gold():
    return G.blocks()


def test_texture_inputs_are_stable(gold):
    # the seeded generator must reproduce the exact inputs the fixtures were made from
    assert G.sha(G.c0_blocks()) == bytes(gold["c0_in_sha"]).decode()
    assert G.sha(G.dxt5_tex_blocks()) == bytes(gold["dxt5_tex_sha"]).decode()
    assert G.sha(G.nrm_tex_blocks()) == bytes(gold["nrm_tex_sha"]).decode()


@pytest.mark.parametrize("perc", [1, 0])
@pytest.mark.parametrize("both", [1, 0])
def test_dxt1_edge_blocks(gold, perc, both):
    out, _ = port.dxt1_blocks(gold["edge_in"], bool(perc), bool(both), threads=4)
    ref = gold[f"edge_dxt1_p{perc}_b{both}"]
    assert np.array_equal(out, ref), np.nonzero((out != ref).any(1))[0][:10]


def test_dxt1_config0_texture(gold):
    out, _ = port.dxt1_blocks(G.c0_blocks(), True, True, threads=4)
    assert np.array_equal(out, gold["c0_dxt1"])


@pytest.mark.parametrize("name", ["dxt5", "dxn_xy", "dxn_yx", "dxt5a"])
@pytest.mark.parametrize("both", [1, 0])
def test_alpha_formats_edge_blocks(gold, name, both):
    out = port.encode_blocks(gold["edge_in"], FMT[name], True, bool(both), threads=4)
    ref = gold[f"edge_{name}_b{both}"]
    assert np.array_equal(out, ref), np.nonzero((out != ref).any(1))[0][:10]


def test_dxt5_and_dxn_textures(gold):
    assert np.array_equal(port.encode_blocks(G.dxt5_tex_blocks(), 2, True, True, threads=4), gold["dxt5_tex_dxt5"])
    assert np.array_equal(port.encode_blocks(G.nrm_tex_blocks(), 7, False, True, threads=4), gold["nrm_tex_dxn_xy"])


@pytest.mark.parametrize("name", sorted(G.manifest().keys()))
def test_transcode_matches_reference(name):
    m = G.manifest()[name]
    crn = G.crn_bytes(name)
    assert G.sha(crn) == m["crn_sha256"]
    bpb = G.bytes_per_block(m["format"])
    for lvl, info in enumerate(m["levels"]):
        size = G.level_bytes(m["width"], m["height"], lvl, bpb, m["faces"])
        assert size == info["bytes"]
        out = port.unpack_level(crn, lvl, size)
        assert out is not None
        assert G.sha(out) == info["sha256"], (name, lvl)


def test_transcode_rejects_bad_input():
    crn = G.crn_bytes("dxt1_256")
    size = G.level_bytes(256, 256, 0, 8, 1)
    assert port.unpack_level(crn[:60], 0, size) is None          # truncated header
    bad = bytearray(crn)
    bad[0] ^= 0xFF                                               # signature
    assert port.unpack_level(bytes(bad), 0, size) is None
    assert port.unpack_level(crn, 0, size - 8) is None           # destination too small
    assert port.unpack_level(crn, 0, size, row_pitch=6) is None  # pitch not a multiple of 4
    assert port.unpack_level(crn, 99, size) is None              # level out of range


# ------------------------------------------------------------------------------------------
# below Uber quality, grayscale sampling, DXT1A transparency, transparent indices for black
# (tests/golden/blocks_quality.npz, made by the reference block compressor)

@pytest.fixture(scope="module")
def goldq():
    return G.blocks_quality()


@pytest.mark.parametrize("q", [0, 1, 2, 3])
@pytest.mark.parametrize("perc", [1, 0])
@pytest.mark.parametrize("both", [1, 0])
def test_dxt1_quality_levels(gold, goldq, q, perc, both):
    out, _ = port.dxt1_blocks_ex(gold["edge_in"], bool(perc), bool(both), quality=q, threads=4)
    ref = goldq[f"dxt1_q{q}_p{perc}_b{both}"]
    assert np.array_equal(out, ref), np.nonzero((out != ref).any(1))[0][:10]


@pytest.mark.parametrize("q", [0, 1, 2, 3])
@pytest.mark.parametrize("name", ["dxt5", "dxn_xy", "dxt5a"])
@pytest.mark.parametrize("both", [1, 0])
def test_alpha_formats_quality_levels(gold, goldq, q, name, both):
    edge = gold["edge_in"]
    ref = goldq[f"{name}_q{q}_b{both}"]
    if name == "dxt5":
        alpha = port.dxt5a_blocks(edge, 3, bool(both), q)
        colour, _ = port.dxt1_blocks_ex(edge, True, False, quality=q, threads=4)
        out = np.concatenate([alpha, colour], 1)
    elif name == "dxn_xy":
        out = np.concatenate([port.dxt5a_blocks(edge, 0, bool(both), q), port.dxt5a_blocks(edge, 1, bool(both), q)], 1)
    else:
        out = port.dxt5a_blocks(edge, 3, bool(both), q)
    assert np.array_equal(out, ref), np.nonzero((out != ref).any(1))[0][:10]


@pytest.mark.parametrize("q", [4, 3, 1])
@pytest.mark.parametrize("both", [1, 0])
def test_dxt1_grayscale_sampling(gold, goldq, q, both):
    out, _ = port.dxt1_blocks_ex(gold["edge_in"], True, bool(both), quality=q, grayscale=True, threads=4)
    ref = goldq[f"gray_q{q}_b{both}"]
    assert np.array_equal(out, ref), np.nonzero((out != ref).any(1))[0][:10]


@pytest.mark.parametrize("q", [4, 3, 1])
@pytest.mark.parametrize("perc", [1, 0])
@pytest.mark.parametrize("both", [1, 0])
def test_dxt1a_transparency(goldq, q, perc, both):
    out, _ = port.dxt1_blocks_ex(goldq["alpha_in"], bool(perc), bool(both), quality=q, dxt1a=True, threads=4)
    ref = goldq[f"dxt1a_q{q}_p{perc}_b{both}"]
    assert np.array_equal(out, ref), np.nonzero((out != ref).any(1))[0][:10]


@pytest.mark.parametrize("q", [4, 3, 1])
@pytest.mark.parametrize("mode", ["p1", "p0", "gray"])
def test_dxt1_transparent_indices_for_black(goldq, q, mode):
    out, _ = port.dxt1_blocks_ex(goldq["dark_in"], mode == "p1", True, quality=q, grayscale=(mode == "gray"),
                                 transparent_black=True, threads=4)
    ref = goldq[f"black_q{q}_{mode}" if mode != "gray" else f"black_gray_q{q}"]
    assert np.array_equal(out, ref), np.nonzero((out != ref).any(1))[0][:10]
