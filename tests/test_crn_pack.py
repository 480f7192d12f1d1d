"""The .crn writer (crngpu_crn_pack, host code) against the decoders: every committed fixture is
decoded, repacked by this library and decoded again -- by the oracle (the CPU restatement pinned
to the reference) and, where it is built, by the reference's own crnd -- and must give back
exactly the same DXTn blocks, in a file no more than 1% larger than the reference's. No GPU
needed."""
import numpy as np
import pytest

import golden_util as G


@pytest.fixture(scope="module")
def cg():
    import crunch2_gb300
    crunch2_gb300.lib()
    return crunch2_gb300


FMT = {"DXT1": 0, "DXT5": 2, "DXN_XY": 7, "DXN_YX": 8, "DXT5A": 9}


def decode_all(crn, m, port):
    bpb = G.bytes_per_block(m["format"])
    out = []
    for l, info in enumerate(m["levels"]):
        w, h = max(1, m["width"] >> l), max(1, m["height"] >> l)
        by, bx = (h + 3) // 4, (w + 3) // 4
        raw = port.unpack_level(crn, l, info["bytes"])
        assert raw is not None
        out.append(list(raw.reshape(m["faces"], by, bx, bpb)))
    return out


@pytest.mark.parametrize("name", sorted(G.manifest().keys()))
def test_repacked_fixture_decodes_to_the_same_blocks(cg, name):
    from oracle import port, ref
    m = G.manifest()[name]
    crn = G.crn_bytes(name)
    levels = decode_all(crn, m, port)
    bpb = G.bytes_per_block(m["format"])
    blocks = cg.crn_layout_from_levels(levels, m["width"], m["height"], m["faces"], bpb)
    packed = cg.crn_pack(blocks, m["width"], m["height"], len(levels), m["faces"], FMT[m["format"]])
    again = decode_all(packed, m, port)
    for l in range(len(levels)):
        for f in range(m["faces"]):
            assert np.array_equal(again[l][f], levels[l][f]), (name, l, f)
    if ref.available():  # the reference decoder accepts the file and agrees
        for l, info in enumerate(m["levels"]):
            assert np.array_equal(ref.unpack_level(packed, l, info["bytes"]),
                                  np.concatenate([x.reshape(-1) for x in levels[l]])), (name, l, "reference crnd")
    print(f"{name}: reference .crn {len(crn)} bytes, repacked {len(packed)} bytes")
    # palette ordering as crn_comp's: the same blocks code in about the reference's size
    assert len(packed) <= 1.01 * len(crn), (name, len(packed), len(crn))


def test_pack_rejects_unclusterable_and_bad_input(cg):
    rng = np.random.default_rng(0)
    blocks = rng.integers(0, 256, size=(64 * 64, 8), dtype=np.uint8)  # 4096 distinct random DXT1 blocks
    with pytest.raises(cg.CrnGpuError):
        cg.crn_pack(np.zeros((10, 8), np.uint8), 0, 4, 1, 1, 0)
    with pytest.raises(cg.CrnGpuError):
        cg.crn_pack(np.zeros((8, 8), np.uint8), 16, 16, 1, 3, 0)
    big = rng.integers(0, 256, size=(256 * 256 // 16 * 4, 8), dtype=np.uint8)  # > 8192 distinct selectors
    with pytest.raises(cg.CrnGpuError):
        cg.crn_pack(big, 512, 512, 1, 1, 0)
    assert cg.crn_pack(blocks, 256, 256, 1, 1, 0)[:2] == b"Hx"
