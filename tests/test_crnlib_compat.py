"""CPU checks of the crnlib-compatible C++ API (include/crnlib_compat.h): the library exports the
reference's functions under their C++ link names, a program written against the reference's own
headers links against it, the struct layouts are the reference's, and the host-only crnd header
functions return what the reference returns on the committed .crn files
(tests/golden/compat_reference.json, written by tests/golden/make_golden.py compat). Nothing here
launches GPU work."""
import ctypes
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

import golden_util as G
import crnlib_abi as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# the reference's headers (CRN_REFERENCE_DIR, else the container's copy); tests that compile
# against them skip where the tree is absent
REF_INC = os.path.join(os.environ.get("CRN_REFERENCE_DIR", "/root/reference"), "inc")


def compat():
    with open(os.path.join(G.GOLDEN, "compat_reference.json")) as fh:
        return json.load(fh)


@pytest.fixture(scope="module")
def api():
    if not (shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
        pytest.skip("no CUDA toolkit to build libcrngpu.so")
    import crunch2_gb300 as cg
    return A.Api(cg.lib())


@pytest.fixture(scope="module")
def libpath(api):
    import crunch2_gb300 as cg
    return cg._lib._name


def _gxx():
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    return gxx


LAYOUT_PROGRAM = r"""
#include <cstddef>
#include <cstdio>
%s
#define F(T, m) std::printf(#T "." #m " %%zu %%zu\n", offsetof(T, m), sizeof(((T*)0)->m));
int main() {
  std::printf("sizes %%zu %%zu %%zu %%zu %%zu %%zu %%zu\n", sizeof(crn_comp_params), sizeof(crn_mipmap_params),
              sizeof(crn_texture_desc), sizeof(crnd::crn_file_info), sizeof(crnd::crn_texture_info),
              sizeof(crnd::crn_level_info), sizeof(crn_format));
  F(crn_comp_params, m_file_type) F(crn_comp_params, m_levels) F(crn_comp_params, m_format)
  F(crn_comp_params, m_flags) F(crn_comp_params, m_pImages) F(crn_comp_params, m_target_bitrate)
  F(crn_comp_params, m_quality_level) F(crn_comp_params, m_dxt_quality) F(crn_comp_params, m_alpha_component)
  F(crn_comp_params, m_crn_adaptive_tile_color_psnr_derating) F(crn_comp_params, m_crn_alpha_selector_palette_size)
  F(crn_comp_params, m_num_helper_threads) F(crn_comp_params, m_userdata1) F(crn_comp_params, m_pProgress_func)
  F(crn_comp_params, m_pProgress_func_data)
  F(crn_mipmap_params, m_mode) F(crn_mipmap_params, m_gamma) F(crn_mipmap_params, m_max_levels)
  F(crn_mipmap_params, m_renormalize) F(crn_mipmap_params, m_scale_mode) F(crn_mipmap_params, m_window_bottom)
  F(crn_mipmap_params, m_clamp_height)
  F(crnd::crn_file_info, m_level_compressed_size) F(crnd::crn_file_info, m_alpha_selector_palette_entries)
  F(crnd::crn_texture_info, m_format) F(crnd::crn_level_info, m_format)
  crn_comp_params p; crn_mipmap_params m;
  std::printf("defaults %%u %%u %%u %%u %%g %%g %%u %%u %%g %%g\n", p.m_size_of_obj, p.m_flags, p.m_quality_level,
              p.m_dxt1a_alpha_threshold, p.m_crn_adaptive_tile_color_psnr_derating,
              p.m_crn_adaptive_tile_alpha_psnr_derating, m.m_mode, m.m_filter, m.m_gamma, m.m_blurriness);
  return 0;
}
"""


def _run_layout(tmp_path, includes, incdirs, tag):
    src = tmp_path / f"layout_{tag}.cpp"
    exe = tmp_path / f"layout_{tag}"
    src.write_text(LAYOUT_PROGRAM % includes)
    cmd = [_gxx(), "-std=c++14", "-w", str(src), "-o", str(exe)] + [f"-I{d}" for d in incdirs]
    subprocess.run(cmd, check=True, capture_output=True)
    return subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout


def test_struct_layouts_and_defaults_match_the_reference_headers(tmp_path):
    if not os.path.isdir(REF_INC):
        pytest.skip("reference headers not present on this machine")
    ours = _run_layout(tmp_path, '#include "crnlib_compat.h"', [os.path.join(ROOT, "include")], "ours")
    theirs = _run_layout(tmp_path, '#include "crnlib.h"\n#include "crn_defs.h"',
                         [REF_INC, os.path.join(ROOT, "oracle", "refbuild")], "ref")
    assert ours == theirs
    assert "sizes 888 84 20 104 40 40 8" in ours


def test_program_written_against_reference_headers_links(tmp_path, libpath):
    """Every crnlib / crnd function this library exports resolves, under the reference's own
    declarations, against libcrngpu.so alone (the link fails on any unresolved C++ name)."""
    if not os.path.isdir(REF_INC):
        pytest.skip("reference headers not present on this machine")
    src = tmp_path / "user.cpp"
    src.write_text(r"""
#include "crnlib.h"
#include "crn_defs.h"
extern "C" {  // emscripten/crunch_lib.cpp:32-41
unsigned int crn_get_width(void* src, unsigned int src_size);
unsigned int crn_get_height(void* src, unsigned int src_size);
unsigned int crn_get_levels(void* src, unsigned int src_size);
unsigned int crn_get_dxt_format(void* src, unsigned int src_size);
unsigned int crn_get_bytes_per_block(void* src, unsigned int src_size);
unsigned int crn_get_uncompressed_size(void* p, unsigned int size, unsigned int level);
void crn_decompress(void* src, unsigned int src_size, void* dst, unsigned int dst_size, unsigned int firstLevel,
                    unsigned int levelCount);
}
typedef void* (*compress_a)(const crn_comp_params&, crn_uint32&, crn_uint32*, float*);
typedef void* (*compress_b)(const crn_comp_params&, const crn_mipmap_params&, crn_uint32&, crn_uint32*, float*);
void* volatile sink;
int main() {
  sink = (void*)(compress_a)&crn_compress; sink = (void*)(compress_b)&crn_compress;
  sink = (void*)&crn_free_block; sink = (void*)&crn_set_memory_callbacks; sink = (void*)&crn_decompress_crn_to_dds;
  sink = (void*)&crn_get_format_fourcc; sink = (void*)&crn_get_format_bits_per_texel;
  sink = (void*)&crn_get_bytes_per_dxt_block; sink = (void*)&crn_get_fundamental_dxt_format;
  sink = (void*)&crn_get_file_type_ext; sink = (void*)&crn_get_format_string; sink = (void*)&crn_get_dxt_quality_string;
  sink = (void*)&crn_get_mip_mode_desc; sink = (void*)&crn_get_mip_mode_name; sink = (void*)&crn_get_mip_filter_name;
  sink = (void*)&crn_get_scale_mode_desc; sink = (void*)&crn_create_block_compressor; sink = (void*)&crn_compress_block;
  sink = (void*)&crn_free_block_compressor; sink = (void*)&crn_get_version; sink = (void*)&crn_get_version_number;
  sink = (void*)&crn_get_version_major; sink = (void*)&crn_get_version_minor; sink = (void*)&crn_get_version_patch;
  sink = (void*)&crnd::crnd_set_memory_callbacks; sink = (void*)&crnd::crnd_crn_format_to_fourcc;
  sink = (void*)&crnd::crnd_get_fundamental_dxt_format; sink = (void*)&crnd::crnd_get_crn_format_bits_per_texel;
  sink = (void*)&crnd::crnd_get_bytes_per_dxt_block; sink = (void*)&crnd::crnd_validate_file;
  sink = (void*)&crnd::crnd_get_texture_info; sink = (void*)&crnd::crnd_get_level_info;
  sink = (void*)&crnd::crnd_unpack_begin; sink = (void*)&crnd::crnd_get_data; sink = (void*)&crnd::crnd_unpack_level;
  sink = (void*)&crnd::crnd_unpack_level_segmented; sink = (void*)&crnd::crnd_unpack_end;
  sink = (void*)&crnd::crnd_get_level_data; sink = (void*)&crnd::crnd_get_segmented_file_size;
  sink = (void*)&crnd::crnd_create_segmented_file;
  sink = (void*)&crn_get_width; sink = (void*)&crn_get_height; sink = (void*)&crn_get_levels;
  sink = (void*)&crn_get_dxt_format; sink = (void*)&crn_get_bytes_per_block; sink = (void*)&crn_get_uncompressed_size;
  sink = (void*)&crn_decompress;
  return 0;
}
""")
    exe = tmp_path / "user"
    cmd = [_gxx(), "-std=c++14", "-w", str(src), "-o", str(exe), f"-I{REF_INC}",
           f"-I{os.path.join(ROOT, 'oracle', 'refbuild')}", libpath, "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


def test_format_helpers_and_strings(api):
    assert api.crn_get_format_fourcc(0) == int.from_bytes(b"DXT1", "little")
    assert api.crnd_crn_format_to_fourcc(7) == int.from_bytes(b"A2XY", "little")
    assert [api.crn_get_bytes_per_dxt_block(f) for f in (0, 2, 7, 8, 9)] == [8, 16, 16, 16, 8]
    assert [api.crn_get_format_bits_per_texel(f) for f in (0, 3, 9)] == [4, 8, 4]
    assert [api.crn_get_fundamental_dxt_format(f) for f in (3, 4, 5, 6, 7)] == [2, 2, 2, 2, 7]
    assert api.crn_get_format_string(5) == b"DXT5_xGBR" and api.crn_get_format_string(99) == b"?"
    assert api.crn_get_file_type_ext(1) == b"dds" and api.crn_get_dxt_quality_string(4) == b"Uber"
    assert api.crn_get_mip_mode_name(2) == b"Generate" and api.crn_get_mip_filter_name(4) == b"kaiser"
    assert api.crn_get_scale_mode_desc(4) == b"nearestpow2"
    assert api.crn_get_version_number() == 104


@pytest.mark.parametrize("name", sorted(G.manifest()))
def test_crnd_header_api_matches_reference(api, name):
    """crnd_validate_file, crnd_get_texture_info, crnd_get_level_info, crnd_get_level_data,
    crnd_get_segmented_file_size and crnd_create_segmented_file return exactly the reference's
    values (and the same segmented base file) on every committed .crn."""
    R = compat()["crnd"][name]
    crn = G.crn_bytes(name)
    values, seg = A.probe(api, crn)
    assert values == R["values"]
    assert (G.sha(np.frombuffer(seg, np.uint8)) if seg else None) == R["segmented_sha256"]
    # the segmented base file validates on its own and refuses a second segmentation
    v2, seg2 = A.probe(api, seg)
    assert v2[0] == 1 and seg2 == b""


def test_crnd_validate_rejects_corruption(api):
    crn = bytearray(G.crn_bytes("dxt1_256"))
    fi = A.CrnFileInfo()
    fi.m_struct_size = ctypes.sizeof(fi)
    buf = (ctypes.c_uint8 * len(crn)).from_buffer(crn)
    assert api.crnd_validate_file(buf, len(crn), ctypes.byref(fi))
    crn[len(crn) // 2] ^= 0x40  # data CRC
    assert not api.crnd_validate_file(buf, len(crn), None)
    crn[len(crn) // 2] ^= 0x40
    crn[13] ^= 1  # width: header CRC
    assert not api.crnd_validate_file(buf, len(crn), None)
    fi.m_struct_size = 12  # wrong struct size is refused before any read
    assert not api.crnd_validate_file(buf, len(crn), ctypes.byref(fi))


@pytest.mark.parametrize("name", sorted(G.manifest()))
def test_emscripten_wrapper_geometry(api, name):
    """emscripten/crunch_lib.cpp's C exports report the committed files' geometry."""
    m = G.manifest()[name]
    crn = G.crn_bytes(name)
    fmt = {"DXT1": 0, "DXT5": 2, "DXN_XY": 7, "DXT5A": 9}[m["format"]]
    assert api.crn_get_width(crn, len(crn)) == m["width"] and api.crn_get_height(crn, len(crn)) == m["height"]
    assert api.crn_get_levels(crn, len(crn)) == len(m["levels"]) and api.crn_get_dxt_format(crn, len(crn)) == fmt
    bpb = G.bytes_per_block(m["format"])
    assert api.crn_get_bytes_per_block(crn, len(crn)) == bpb
    for l, L in enumerate(m["levels"]):
        w, h = m["width"] >> l, m["height"] >> l
        assert api.crn_get_uncompressed_size(crn, len(crn), l) == ((w + 3) // 4) * ((h + 3) // 4) * bpb
    assert api.crn_get_width(b"not a crn file at all, just bytes" * 4, 136) == 0


def test_refused_allocations_end_the_call_without_leaks(api):
    """crnd_set_memory_callbacks hooks that refuse an allocation (after 0, 1, 2, ... granted ones):
    crnd_unpack_begin returns NULL as crnd does -- no exception crosses the C++ and C interfaces --
    the last error names the refusal, and everything granted before it is given back. Only host
    parsing runs before the first refusal, so no GPU work is involved."""
    import crunch2_gb300 as cg
    crn = G.crn_bytes("dxt5_256")
    buf = ctypes.create_string_buffer(crn, len(crn))
    seen_limits = 0
    for limit in range(0, 64):
        live, calls = {}, {"alloc": 0, "free": 0, "refused": 0}

        @A.REALLOC
        def realloc(ptr, size, actual, movable, user):
            if not ptr:
                if calls["alloc"] >= limit:
                    calls["refused"] += 1
                    return None
                b = ctypes.create_string_buffer(size)
                live[ctypes.addressof(b)] = b
                calls["alloc"] += 1
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

        api.crnd_set_memory_callbacks(realloc, msize, None)
        try:
            ctx = api.crnd_unpack_begin(buf, len(crn))
        finally:
            api.crnd_set_memory_callbacks(A.REALLOC(0), A.MSIZE(0), None)
        if not calls["refused"]:
            if ctx:  # a GPU is present and the whole context fitted within the limit
                assert api.crnd_unpack_end(ctx)
            break  # the parse needs fewer allocations than this limit
        seen_limits += 1
        assert not ctx, limit
        assert cg.last_error() == "out of host memory", (limit, cg.last_error())
        assert calls["alloc"] == calls["free"] and not live, (limit, calls)
    assert seen_limits >= 3  # the context, the parsed file and its tables each met a refusal
