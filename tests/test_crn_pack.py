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


# sha256 of each fixture's repacked file: the bytes the straightforward writer (full chain scans,
# a sorted pair list, heap-built Huffman trees, a bit-at-a-time writer) made; the 2048 x 2048
# files take the writer's threaded per-block passes.
REPACK_SHA = {
    "c1_dxt1_1024": "8785e5dbdbb1736bb0eb17faabd36827f7d0b106c239681165024d911f227bc4",
    "dxn_xy_2048": "845b938e86a585d14022436505ef6569e08bdc99dc5ee44036435075b96682e8",
    "dxn_xy_256": "dc625e843abb266b383bb951ffb09627506167f494cb68a8b749995eb17b0d52",
    "dxt1_100x60": "7f6dc1bca24d403a43bda5b6322171cf94e13ce8db5abfe0648c82e0003c751a",
    "dxt1_256": "4841a1c0fc306943c725e7244e69ecb6a84d22fc126db61bd708d7a19cf3186e",
    "dxt1_cube_64": "199b6a3e9ecb619d4aee06f834f82745bb069e4541cd3c4042e503cfcc31baeb",
    "dxt5_2048": "dbacca76cfc674157a50643a00b728d15adb87c39e9346e26ffdb651920dfb78",
    "dxt5_256": "612bef535d8160c3cc293aa6093f1ae017d0828f606495b5bd3b00a541a5ebaa",
    "dxt5_cube_64x32": "2c70b0ff2e7176735e7bcfab53aa69bfed9efa4582419f99fdb5c57a48da1bc3",
    "dxt5a_256": "2cf8da5070b63919fa29e572f79cc2566633aef6dced07245d4f6fec1b2de0bc",
}


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
    import hashlib
    assert hashlib.sha256(packed).hexdigest() == REPACK_SHA[name], name
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


def synthetic_levels(rng, w, h, faces, bpb, colour, nalpha):
    """Visible blocks per level and face drawn from small pools, with runs of repeated endpoints,
    as a clustered encode leaves them."""
    levels = []
    l = 0
    while True:
        lw, lh = max(1, w >> l), max(1, h >> l)
        by, bx = (lh + 3) // 4, (lw + 3) // 4
        fl = []
        for _ in range(faces):
            n = by * bx
            blk = np.zeros((n, bpb), np.uint8)
            pick = rng.integers(0, 40, n)
            runs = rng.random(n) < 0.4
            for i in range(1, n):
                if runs[i]:
                    pick[i] = pick[i - 1]
            for a in range(nalpha):
                blk[:, 8 * a:8 * a + 2] = rng.integers(0, 256, (40, 2), dtype=np.uint8)[pick]
                blk[:, 8 * a + 2:8 * a + 8] = rng.integers(0, 256, (25, 6), dtype=np.uint8)[rng.integers(0, 25, n)]
            if colour:
                c = 8 if bpb == 16 else 0
                blk[:, c:c + 4] = rng.integers(0, 256, (40, 4), dtype=np.uint8)[pick]
                blk[:, c + 4:c + 8] = rng.integers(0, 256, (30, 4), dtype=np.uint8)[rng.integers(0, 30, n)]
            fl.append(blk.reshape(by, bx, bpb))
        levels.append(fl)
        if lw == 1 and lh == 1:
            return levels
        l += 1


# (format, bytes per block, colour block, alpha blocks, width, height, faces) -> sha256 of the file.
# The writer's bytes are pinned (the hashes are of the files the straightforward form of the
# writer made: full chain scans, a sorted pair list, heap-built Huffman trees, a bit-at-a-time
# writer); its restatements for speed must leave them unchanged.
WRITER_CASES = {
    ("DXT1", 8, True, 0, 100, 60, 1):
        "58421731e4e3c2976369a3007a665dcd472b04a1157043bf279cafdb719832e2",
    ("DXT1", 8, True, 0, 64, 64, 6):
        "053ba262df93808a4b95584ad7e8b5c4483e2ced4a68875d2f775c9675bb604c",
    ("DXT5", 16, True, 1, 256, 128, 1):
        "9c5dd8cd4ec5cd65824df5d616a037522a99ee00a698e93c5fb86751b9add5bc",
    ("DXN_XY", 16, False, 2, 96, 200, 1):
        "715c9aa169dcae8d58ebb0de222cef4a672440e0fcef82d2a04e3b8e1deffe36",
    ("DXT5A", 8, False, 1, 128, 128, 6):
        "595c03e7c0856c7b5cb0bc4f9f336426a5686fc398c47e249a99e5a4a4926074",
}


@pytest.mark.parametrize("case", sorted(WRITER_CASES))
def test_writer_bytes_are_pinned(cg, case):
    import hashlib
    from oracle import port
    name, bpb, colour, nalpha, w, h, faces = case
    rng = np.random.default_rng(1000 + sorted(WRITER_CASES).index(case))
    levels = synthetic_levels(rng, w, h, faces, bpb, colour, nalpha)
    blocks = cg.crn_layout_from_levels(levels, w, h, faces, bpb)
    packed = cg.crn_pack(blocks, w, h, len(levels), faces, FMT[name])
    for l, fl in enumerate(levels):
        raw = port.unpack_level(packed, l, sum(x.size for x in fl))
        assert np.array_equal(raw, np.concatenate([x.reshape(-1) for x in fl])), (case, l)
    digest = hashlib.sha256(packed).hexdigest()
    print(case, len(packed), digest)
    assert digest == WRITER_CASES[case], (case, digest)
