"""The crnlib-compatible C++ API on the GPU, called through its C++ link names exactly as a program
built against the reference's headers calls it, against the reference's own outputs
(tests/golden/compat_reference.json, written by tests/golden/make_golden.py compat):

- crn_compress to DDS at quality 255 (plain path): whole files bit-identical for DXT1, DXT5, DXN,
  DXT5A, the swizzled DXT5 formats (source conversions), cube maps and odd sizes;
- crn_compress to DDS below 255 (clustered DXT1): the reference's header, this library's blocks;
- crn_compress with crn_mipmap_params (mips generated on the GPU): whole DDS files bit-identical;
- crn_decompress_crn_to_dds of every committed .crn: bit-identical;
- crnd_unpack_begin / _level / _level_segmented / _end: the committed golden levels, into host
  and device memory;
- crn_compress to .crn: the same file as the C ABI's crngpu_compress_crn; memory hooks, progress
  callback and cancellation; the block compressor."""
import ctypes
import json
import os

import numpy as np
import pytest

import golden_util as G
import crnlib_abi as A

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

FMT = {"DXT1": 0, "DXT5": 2, "DXT5_CCxY": 3, "DXT5_xGxR": 4, "DXT5_xGBR": 5, "DXT5_AGBR": 6, "DXN_XY": 7,
       "DXN_YX": 8, "DXT5A": 9}


@pytest.fixture(scope="module")
def api():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import crunch2_gb300 as cg
    return A.Api(cg.lib())


def compat():
    with open(os.path.join(G.GOLDEN, "compat_reference.json")) as fh:
        return json.load(fh)


def texture_levels(w, h, content, seed, faces):
    from crunch2_gb300 import texgen
    out = []
    for f in range(faces):
        if content == "normal":
            img = texgen.normal_map(w, h, seed + f)
        elif content == "dark":
            img = texgen.dark_texture(w, h, seed + f)
        else:
            img = texgen.colour_texture(w, h, seed + f, with_alpha_noise=(content == "colour_alpha"))
        out.append(texgen.mip_chain(img))
    return out


def params_for(faces_levels, fmt, file_type, quality, flags):
    p = A.CrnCompParams()
    h, w = faces_levels[0][0].shape[:2]
    p.m_file_type, p.m_width, p.m_height = file_type, w, h
    p.m_faces, p.m_levels = len(faces_levels), len(faces_levels[0])
    p.m_format, p.m_flags, p.m_quality_level = fmt, flags, quality
    keep = []
    for f, face in enumerate(faces_levels):
        for l, im in enumerate(face):
            a = np.ascontiguousarray(im, dtype=np.uint8)
            keep.append(a)
            p.m_pImages[f][l] = a.ctypes.data
    return p, keep


def call_compress(api, p, mip=None):
    size, q, rate = ctypes.c_uint32(0), ctypes.c_uint32(0), ctypes.c_float(0)
    if mip is None:
        ptr = api.crn_compress(ctypes.byref(p), ctypes.byref(size), ctypes.byref(q), ctypes.byref(rate))
    else:
        ptr = api.crn_compress_mips(ctypes.byref(p), ctypes.byref(mip), ctypes.byref(size), ctypes.byref(q),
                                    ctypes.byref(rate))
    if not ptr:
        return None, size.value, q.value, rate.value
    data = ctypes.string_at(ptr, size.value)
    api.crn_free_block(ptr)
    return data, size.value, q.value, rate.value


def sha(b: bytes) -> str:
    return G.sha(np.frombuffer(b, np.uint8))


@pytest.mark.parametrize("name", sorted(compat()["dds"]))
def test_crn_compress_dds_matches_reference(api, name):
    R = compat()["dds"][name]
    fl = texture_levels(R["width"], R["height"], R["content"], R["seed"], R["faces"])
    assert G.sha(np.concatenate([im.reshape(-1) for f in fl for im in f])) == R["input_sha256"]
    p, keep = params_for(fl, FMT[R["format"]], 1, R["quality"], R["flags"])
    data, size, q, _ = call_compress(api, p)
    assert data is not None, name
    assert size == R["size"] and q == R["quality"]
    assert data[:128].hex() == R["header"]
    if R["quality"] == 255:
        assert sha(data) == R["sha256"], name  # the whole file: header and every block
    else:
        import crunch2_gb300 as cg
        blocks = cg.compress_dds_clustered(fl, quality=R["quality"], flags=R["flags"] & 9, fmt=FMT[R["format"]])
        assert data[128:] == blocks.tobytes()


@pytest.mark.parametrize("name", sorted(compat()["dds_opts"]))
def test_crn_compress_dds_block_options_match_reference(api, name):
    """crn_compress to .dds at quality 255 below Uber dxt quality, with grayscale sampling, DXT1A
    transparency and transparent indices for black: the reference's whole file, byte for byte."""
    R = compat()["dds_opts"][name]
    fl = texture_levels(R["width"], R["height"], R["content"], R["seed"], 1)
    assert G.sha(np.concatenate([im.reshape(-1) for f in fl for im in f])) == R["input_sha256"]
    p, keep = params_for(fl, FMT[R["format"]], 1, 255, R["flags"])
    p.m_dxt_quality = R["dxt_quality"]
    data, size, q, _ = call_compress(api, p)
    assert data is not None, name
    assert size == R["size"] and data[:128].hex() == R["header"]
    assert sha(data) == R["sha256"], name


def test_block_compressor_options(api):
    """crn_create_block_compressor honours m_dxt_quality, DXT1A, grayscale sampling and transparent
    indices for black like the batched entry point."""
    import crunch2_gb300 as cg
    goldq = G.blocks_quality()
    blocks = goldq["alpha_in"][:12]
    for flags, dq in ((1 | 8, 1), (1 | 8 | 128, 4), (1 | 8 | 256, 3), (1 | 8 | 16, 4)):
        p = A.CrnCompParams()
        p.m_format, p.m_flags, p.m_width, p.m_height, p.m_dxt_quality = 0, flags, 4, 4, dq
        ctx = api.crn_create_block_compressor(ctypes.byref(p))
        assert ctx
        out = np.zeros((len(blocks), 8), np.uint8)
        for i, b in enumerate(blocks):
            src = np.ascontiguousarray(b, dtype=np.uint8)
            api.crn_compress_block(ctx, src.ctypes.data, out[i].ctypes.data)
        api.crn_free_block_compressor(ctx)
        assert np.array_equal(out, cg.compress_blocks(blocks, 0, flags, quality=dq)), (flags, dq)


@pytest.mark.parametrize("name", sorted(compat()["mips"]))
def test_crn_compress_with_generated_mips(api, name):
    R = compat()["mips"][name]
    top = texture_levels(R["width"], R["height"], R["content"], R["seed"], 1)[0][0]
    p, keep = params_for([[top]], FMT[R["format"]], R["file_type"], R["quality"], R["flags"])
    m = A.CrnMipmapParams()
    m.m_mode, m.m_filter, m.m_blurriness = R["mip_mode"], R["filter"], R["blurriness"]
    m.m_gamma_filtering, m.m_tiled = int(R["gamma_filtering"]), int(R["tiled"])
    m.m_max_levels, m.m_min_mip_size = R["max_levels"], R["min_mip_size"]
    data, size, q, rate = call_compress(api, p, m)
    assert data is not None
    if R["file_type"] == 1:
        assert data[:128].hex() == R["header"]
        assert size == R["size"] and sha(data) == R["sha256"]
    else:
        # .crn: the clusterizer is compared on quality elsewhere; here the level chain and the file
        # must be exactly those of the C ABI fed with the GPU-generated chain
        import crunch2_gb300 as cg
        ti = A.CrnTextureInfo()
        ti.m_struct_size = ctypes.sizeof(ti)
        assert api.crnd_get_texture_info(data, len(data), ctypes.byref(ti))
        levels = cg.generate_mipmaps(top, filt="kaiser", filter_scale=R["blurriness"], srgb=True, wrap=False,
                                     alpha=False)
        assert ti.m_levels == len(levels) == 8
        assert data == cg.compress_crn([levels], FMT[R["format"]], quality=R["quality"], flags=R["flags"] & 9)


@pytest.mark.parametrize("name", sorted(G.manifest()))
def test_crn_decompress_crn_to_dds_matches_reference(api, name):
    R = compat()["crn_to_dds"][name]
    crn = G.crn_bytes(name)
    size = ctypes.c_uint32(len(crn))
    ptr = api.crn_decompress_crn_to_dds(crn, ctypes.byref(size))
    assert ptr and size.value == R["size"]
    data = ctypes.string_at(ptr, size.value)
    api.crn_free_block(ptr)
    assert data[:128].hex() == R["header"]
    assert sha(data) == R["sha256"]


@pytest.mark.parametrize("name", sorted(G.manifest()))
def test_crnd_unpack_matches_golden_host_and_device(api, name):
    m = G.manifest()[name]
    crn = G.crn_bytes(name)
    buf = ctypes.create_string_buffer(crn, len(crn))
    ctx = api.crnd_unpack_begin(buf, len(crn))
    assert ctx
    data, dsize = ctypes.c_void_p(), ctypes.c_uint32()
    assert api.crnd_get_data(ctx, ctypes.byref(data), ctypes.byref(dsize))
    assert data.value == ctypes.addressof(buf) and dsize.value == len(crn)
    bpb, faces = G.bytes_per_block(m["format"]), m["faces"]
    base = ctypes.create_string_buffer(len(crn))
    assert api.crnd_create_segmented_file(buf, len(crn), base, len(crn))
    base_size = api.crnd_get_segmented_file_size(buf, len(crn))
    seg_ctx = api.crnd_unpack_begin(base, base_size)
    assert seg_ctx
    try:
        for l, L in enumerate(m["levels"]):
            w, h = max(1, m["width"] >> l), max(1, m["height"] >> l)
            pitch = ((w + 3) // 4) * bpb
            face_bytes = pitch * ((h + 3) // 4)
            host = [np.zeros(face_bytes, np.uint8) for _ in range(faces)]
            ptrs = (ctypes.c_void_p * 6)(*[a.ctypes.data for a in host])
            assert api.crnd_unpack_level(ctx, ptrs, face_bytes, 0, l)
            got = np.concatenate(host)
            assert got.size == L["bytes"] and G.sha(got) == L["sha256"], (name, l)
            dev = [torch.zeros(face_bytes, dtype=torch.uint8, device="cuda") for _ in range(faces)]
            dptrs = (ctypes.c_void_p * 6)(*[t.data_ptr() for t in dev])
            assert api.crnd_unpack_level(ctx, dptrs, face_bytes, 0, l)
            assert np.array_equal(torch.cat(dev).cpu().numpy(), got)
            # the segmented base file plus this level's data from the full file
            lsize = ctypes.c_uint32()
            lptr = api.crnd_get_level_data(buf, len(crn), l, ctypes.byref(lsize))
            seg = [np.zeros(face_bytes, np.uint8) for _ in range(faces)]
            sptrs = (ctypes.c_void_p * 6)(*[a.ctypes.data for a in seg])
            assert api.crnd_unpack_level_segmented(seg_ctx, lptr, lsize.value, sptrs, face_bytes, 0, l)
            assert np.array_equal(np.concatenate(seg), got)
            # a segmented base file carries no level data of its own
            assert not api.crnd_unpack_level(seg_ctx, sptrs, face_bytes, 0, l)
    finally:
        assert api.crnd_unpack_end(ctx) and api.crnd_unpack_end(seg_ctx)
    assert not api.crnd_unpack_level(None, None, 0, 0, 0)


def test_crnd_memory_hooks_carry_the_transcoder_state(api):
    """crnd_set_memory_callbacks: the transcoder's host state -- context, parsed header, models,
    palettes, launch plans -- is allocated through the caller's hooks, as crnd's is; crnd_unpack_end
    returns all of it, and the output does not change."""
    name = "dxt5_256"
    m = G.manifest()[name]
    crn = G.crn_bytes(name)
    live, calls = {}, {"alloc": 0, "free": 0, "bytes": 0}

    @A.REALLOC
    def realloc(ptr, size, actual, movable, user):
        if not ptr:
            b = ctypes.create_string_buffer(size)
            live[ctypes.addressof(b)] = b
            calls["alloc"] += 1
            calls["bytes"] += size
            if actual:
                actual[0] = size
            return ctypes.addressof(b)
        if size == 0:
            calls["free"] += 1
            live.pop(ptr, None)
        return None

    @A.MSIZE
    def msize(ptr, user):
        return ctypes.sizeof(live[ptr]) if ptr in live else 0

    buf = ctypes.create_string_buffer(crn, len(crn))
    api.crnd_set_memory_callbacks(realloc, msize, None)
    try:
        ctx = api.crnd_unpack_begin(buf, len(crn))
        assert ctx and calls["alloc"] > 0
        begun = calls["alloc"]
        bpb = G.bytes_per_block(m["format"])
        for l, L in enumerate(m["levels"]):
            w, h = max(1, m["width"] >> l), max(1, m["height"] >> l)
            face_bytes = ((w + 3) // 4) * bpb * ((h + 3) // 4)
            out = np.zeros(face_bytes, np.uint8)
            ptrs = (ctypes.c_void_p * 6)(out.ctypes.data)
            assert api.crnd_unpack_level(ctx, ptrs, face_bytes, 0, l)
            assert G.sha(out) == L["sha256"], l
        assert calls["alloc"] > begun  # each call's launch plan too
        assert api.crnd_unpack_end(ctx)
    finally:
        api.crnd_set_memory_callbacks(A.REALLOC(0), A.MSIZE(0), None)
    print(calls)
    assert calls["alloc"] == calls["free"] and not live


def test_crn_compress_crn_is_the_c_abi_file(api):
    import crunch2_gb300 as cg
    fl = texture_levels(128, 128, "colour", 21, 1)
    p, keep = params_for(fl, 0, 0, 128, 1 | 2 | 8)
    data, size, q, rate = call_compress(api, p)
    texels = sum(im.shape[0] * im.shape[1] for im in fl[0])
    assert data == cg.compress_crn(fl, cg.FMT_DXT1, quality=128, flags=cg.FLAG_PERCEPTUAL)
    assert q == 128 and abs(rate - size * 8 / texels) < 1e-5
    # target bitrate: the C ABI's search; manual palette sizes turn it off
    p.m_target_bitrate = 1.5
    data_b, size_b, q_b, rate_b = call_compress(api, p)
    want, wq, wrate = cg.compress_crn_bitrate(fl, 1.5, cg.FMT_DXT1)
    assert data_b == want and q_b == wq and abs(rate_b - wrate) < 1e-6
    p.m_flags |= 64
    p.m_crn_color_endpoint_palette_size, p.m_crn_color_selector_palette_size = 64, 96
    data_m, _, q_m, _ = call_compress(api, p)
    assert data_m is not None and q_m == 0
    ti = A.CrnFileInfo()
    ti.m_struct_size = ctypes.sizeof(ti)
    assert api.crnd_validate_file(data_m, len(data_m), ctypes.byref(ti))
    assert ti.m_color_endpoint_palette_entries <= 64 and ti.m_color_selector_palette_entries <= 96


def test_memory_hooks_progress_and_cancel(api):
    fl = texture_levels(32, 32, "colour", 5, 1)
    p, keep = params_for(fl, 0, 1, 255, 1 | 8)
    calls = {"alloc": 0, "free": 0}
    live = {}

    @A.REALLOC
    def realloc(ptr, size, actual, movable, user):
        if not ptr:
            buf = ctypes.create_string_buffer(size)
            live[ctypes.addressof(buf)] = buf
            calls["alloc"] += 1
            if actual:
                actual[0] = size
            return ctypes.addressof(buf)
        if size == 0:
            calls["free"] += 1
            live.pop(ptr, None)
        return None

    @A.MSIZE
    def msize(ptr, user):
        return ctypes.sizeof(live[ptr]) if ptr in live else 0

    seen = []

    @A.PROGRESS
    def progress(phase, total, sub, total_sub, user):
        seen.append((phase, total))
        return 1

    api.crn_set_memory_callbacks(realloc, msize, None)
    try:
        p.m_pProgress_func = ctypes.cast(progress, ctypes.c_void_p)
        data, size, _, _ = call_compress(api, p)
        assert data is not None and calls == {"alloc": 1, "free": 1} and seen == [(0, 2), (1, 2)]

        @A.PROGRESS
        def cancel(phase, total, sub, total_sub, user):
            return 0

        p.m_pProgress_func = ctypes.cast(cancel, ctypes.c_void_p)
        data, size, _, _ = call_compress(api, p)
        assert data is None and size == 0
    finally:
        api.crn_set_memory_callbacks(A.REALLOC(0), A.MSIZE(0), None)
    # parameters outside crn_comp_params::check and formats not built give NULL
    p.m_pProgress_func = None
    p.m_quality_level = 300
    assert call_compress(api, p)[0] is None
    p.m_quality_level, p.m_format = 255, 10  # ETC1
    assert call_compress(api, p)[0] is None


def test_block_compressor(api):
    import crunch2_gb300 as cg
    blocks = G.c0_blocks()[:24]
    for fmt, flags in ((0, 1 | 8), (2, 1), (7, 0), (9, 8)):
        p = A.CrnCompParams()
        p.m_format, p.m_flags, p.m_width, p.m_height = fmt, flags, 4, 4
        ctx = api.crn_create_block_compressor(ctypes.byref(p))
        assert ctx
        bpb = 8 if fmt in (0, 9) else 16
        out = np.zeros((len(blocks), bpb), np.uint8)
        for i, b in enumerate(blocks):
            src = np.ascontiguousarray(b, dtype=np.uint8)
            api.crn_compress_block(ctx, src.ctypes.data, out[i].ctypes.data)
        api.crn_free_block_compressor(ctx)
        assert np.array_equal(out, cg.compress_blocks(blocks, fmt, flags).reshape(len(blocks), bpb))


@pytest.mark.parametrize("name", ["c1_dxt1_1024", "dxt5_256", "dxn_xy_256", "dxt1_100x60"])
def test_emscripten_crn_decompress(api, name):
    """crn_decompress (the emscripten wrapper's transcode entry, by its own C name): levels of face
    0 back to back, each the committed golden level."""
    m = G.manifest()[name]
    crn = G.crn_bytes(name)
    first, count = 1, len(m["levels"]) - 1
    sizes = [api.crn_get_uncompressed_size(crn, len(crn), l) for l in range(first, first + count)]
    dst = np.zeros(sum(sizes), np.uint8)
    api.crn_decompress(crn, len(crn), dst.ctypes.data, dst.size, first, count)
    ofs = 0
    for l, n in zip(range(first, first + count), sizes):
        L = m["levels"][l]
        if n:
            assert n == L["bytes"] and G.sha(dst[ofs:ofs + n]) == L["sha256"], (name, l)
        ofs += n
