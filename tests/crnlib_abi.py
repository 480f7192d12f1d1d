"""ctypes view of libcrngpu.so's crnlib-compatible C++ API (include/crnlib_compat.h): the structs
with the reference's layouts and the functions under their C++ link names, as a program built
against the reference's inc/crnlib.h and inc/crn_defs.h would call them."""
import ctypes

u32 = ctypes.c_uint32
vp = ctypes.c_void_p


class CrnCompParams(ctypes.Structure):
    """crn_comp_params (inc/crnlib.h:231-414); crn_format is a 64-bit enum (its range holds -1 and
    0xFFFFFFFF), so m_format sits at offset 24 and the struct is 888 bytes."""
    _fields_ = [("m_size_of_obj", u32), ("m_file_type", u32), ("m_faces", u32), ("m_width", u32),
                ("m_height", u32), ("m_levels", u32), ("m_format", ctypes.c_int64), ("m_flags", u32),
                ("m_pImages", (vp * 16) * 6), ("m_target_bitrate", ctypes.c_float), ("m_quality_level", u32),
                ("m_dxt1a_alpha_threshold", u32), ("m_dxt_quality", u32), ("m_dxt_compressor_type", u32),
                ("m_alpha_component", u32), ("m_crn_adaptive_tile_color_psnr_derating", ctypes.c_float),
                ("m_crn_adaptive_tile_alpha_psnr_derating", ctypes.c_float),
                ("m_crn_color_endpoint_palette_size", u32), ("m_crn_color_selector_palette_size", u32),
                ("m_crn_alpha_endpoint_palette_size", u32), ("m_crn_alpha_selector_palette_size", u32),
                ("m_num_helper_threads", u32), ("m_userdata0", u32), ("m_userdata1", u32),
                ("m_pProgress_func", vp), ("m_pProgress_func_data", vp)]

    def __init__(self):
        super().__init__()
        self.m_size_of_obj = ctypes.sizeof(self)
        self.m_faces, self.m_levels, self.m_format = 1, 1, 0
        self.m_flags = 1 | 2 | 8
        self.m_quality_level, self.m_dxt1a_alpha_threshold, self.m_dxt_quality = 255, 128, 4
        self.m_alpha_component = 3
        self.m_crn_adaptive_tile_color_psnr_derating = 2.0
        self.m_crn_adaptive_tile_alpha_psnr_derating = 2.0


class CrnMipmapParams(ctypes.Structure):
    """crn_mipmap_params (inc/crnlib.h:471-574)."""
    _fields_ = [("m_size_of_obj", u32), ("m_mode", u32), ("m_filter", u32), ("m_gamma_filtering", u32),
                ("m_gamma", ctypes.c_float), ("m_blurriness", ctypes.c_float), ("m_max_levels", u32),
                ("m_min_mip_size", u32), ("m_renormalize", u32), ("m_rtopmip", u32), ("m_tiled", u32),
                ("m_scale_mode", u32), ("m_scale_x", ctypes.c_float), ("m_scale_y", ctypes.c_float),
                ("m_window_left", u32), ("m_window_top", u32), ("m_window_right", u32), ("m_window_bottom", u32),
                ("m_clamp_scale", u32), ("m_clamp_width", u32), ("m_clamp_height", u32)]

    def __init__(self):
        super().__init__()
        self.m_size_of_obj = ctypes.sizeof(self)
        self.m_filter, self.m_gamma_filtering, self.m_gamma, self.m_blurriness = 4, 1, 2.2, 0.9
        self.m_max_levels, self.m_min_mip_size = 16, 1
        self.m_scale_x = self.m_scale_y = 1.0


class CrnFileInfo(ctypes.Structure):
    _fields_ = [("m_struct_size", u32), ("m_actual_data_size", u32), ("m_header_size", u32),
                ("m_total_palette_size", u32), ("m_tables_size", u32), ("m_levels", u32),
                ("m_level_compressed_size", u32 * 16), ("m_color_endpoint_palette_entries", u32),
                ("m_color_selector_palette_entries", u32), ("m_alpha_endpoint_palette_entries", u32),
                ("m_alpha_selector_palette_entries", u32)]


class CrnTextureInfo(ctypes.Structure):
    _fields_ = [("m_struct_size", u32), ("m_width", u32), ("m_height", u32), ("m_levels", u32), ("m_faces", u32),
                ("m_bytes_per_block", u32), ("m_userdata0", u32), ("m_userdata1", u32),
                ("m_format", ctypes.c_int64)]


class CrnLevelInfo(ctypes.Structure):
    _fields_ = [("m_struct_size", u32), ("m_width", u32), ("m_height", u32), ("m_faces", u32), ("m_blocks_x", u32),
                ("m_blocks_y", u32), ("m_bytes_per_block", u32), ("m_format", ctypes.c_int64)]


PROGRESS = ctypes.CFUNCTYPE(u32, u32, u32, u32, u32, vp)
REALLOC = ctypes.CFUNCTYPE(vp, vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t), ctypes.c_bool, vp)
MSIZE = ctypes.CFUNCTYPE(ctypes.c_size_t, vp, vp)

# C++ (Itanium ABI) link names of the reference's declarations
SYMBOLS = {
    "crn_compress": ("_Z12crn_compressRK15crn_comp_paramsRjPjPf", vp, [vp, vp, vp, vp]),
    "crn_compress_mips": ("_Z12crn_compressRK15crn_comp_paramsRK17crn_mipmap_paramsRjPjPf", vp, [vp, vp, vp, vp, vp]),
    "crn_free_block": ("_Z14crn_free_blockPv", None, [vp]),
    "crn_set_memory_callbacks": ("_Z24crn_set_memory_callbacksPFPvS_mPmbS_EPFmS_S_ES_", None, [REALLOC, MSIZE, vp]),
    "crnd_set_memory_callbacks": ("_ZN4crnd25crnd_set_memory_callbacksEPFPvS0_mPmbS0_EPFmS0_S0_ES0_", None,
                                  [REALLOC, MSIZE, vp]),
    "crn_decompress_crn_to_dds": ("_Z25crn_decompress_crn_to_ddsPKvRj", vp, [vp, vp]),
    "crn_create_block_compressor": ("_Z27crn_create_block_compressorRK15crn_comp_params", vp, [vp]),
    "crn_compress_block": ("_Z18crn_compress_blockPvPKjS_", None, [vp, vp, vp]),
    "crn_free_block_compressor": ("_Z25crn_free_block_compressorPv", None, [vp]),
    "crn_get_format_fourcc": ("_Z21crn_get_format_fourcc10crn_format", u32, [ctypes.c_int64]),
    "crn_get_format_bits_per_texel": ("_Z29crn_get_format_bits_per_texel10crn_format", u32, [ctypes.c_int64]),
    "crn_get_bytes_per_dxt_block": ("_Z27crn_get_bytes_per_dxt_block10crn_format", u32, [ctypes.c_int64]),
    "crn_get_fundamental_dxt_format": ("_Z30crn_get_fundamental_dxt_format10crn_format", ctypes.c_int64,
                                       [ctypes.c_int64]),
    "crn_get_format_string": ("_Z21crn_get_format_string10crn_format", ctypes.c_char_p, [ctypes.c_int64]),
    "crn_get_file_type_ext": ("_Z21crn_get_file_type_ext13crn_file_type", ctypes.c_char_p, [u32]),
    "crn_get_dxt_quality_string": ("_Z26crn_get_dxt_quality_string15crn_dxt_quality", ctypes.c_char_p, [u32]),
    "crn_get_mip_mode_name": ("_Z21crn_get_mip_mode_name12crn_mip_mode", ctypes.c_char_p, [u32]),
    "crn_get_mip_mode_desc": ("_Z21crn_get_mip_mode_desc12crn_mip_mode", ctypes.c_char_p, [u32]),
    "crn_get_mip_filter_name": ("_Z23crn_get_mip_filter_name14crn_mip_filter", ctypes.c_char_p, [u32]),
    "crn_get_scale_mode_desc": ("_Z23crn_get_scale_mode_desc14crn_scale_mode", ctypes.c_char_p, [u32]),
    "crn_get_version_number": ("_Z22crn_get_version_numberv", ctypes.c_int, []),
    "crnd_validate_file": ("_ZN4crnd18crnd_validate_fileEPKvjPNS_13crn_file_infoE", ctypes.c_bool, [vp, u32, vp]),
    "crnd_get_texture_info": ("_ZN4crnd21crnd_get_texture_infoEPKvjPNS_16crn_texture_infoE", ctypes.c_bool,
                              [vp, u32, vp]),
    "crnd_get_level_info": ("_ZN4crnd19crnd_get_level_infoEPKvjjPNS_14crn_level_infoE", ctypes.c_bool,
                            [vp, u32, u32, vp]),
    "crnd_get_level_data": ("_ZN4crnd19crnd_get_level_dataEPKvjjPj", vp, [vp, u32, u32, vp]),
    "crnd_get_segmented_file_size": ("_ZN4crnd28crnd_get_segmented_file_sizeEPKvj", u32, [vp, u32]),
    "crnd_create_segmented_file": ("_ZN4crnd26crnd_create_segmented_fileEPKvjPvj", ctypes.c_bool, [vp, u32, vp, u32]),
    "crnd_unpack_begin": ("_ZN4crnd17crnd_unpack_beginEPKvj", vp, [vp, u32]),
    "crnd_get_data": ("_ZN4crnd13crnd_get_dataEPvPPKvPj", ctypes.c_bool, [vp, vp, vp]),
    "crnd_unpack_level": ("_ZN4crnd17crnd_unpack_levelEPvPS0_jjj", ctypes.c_bool, [vp, vp, u32, u32, u32]),
    "crnd_unpack_level_segmented": ("_ZN4crnd27crnd_unpack_level_segmentedEPvPKvjPS0_jjj", ctypes.c_bool,
                                    [vp, vp, u32, vp, u32, u32, u32]),
    "crnd_unpack_end": ("_ZN4crnd15crnd_unpack_endEPv", ctypes.c_bool, [vp]),
    "crnd_crn_format_to_fourcc": ("_ZN4crnd25crnd_crn_format_to_fourccE10crn_format", u32, [ctypes.c_int64]),
    # emscripten/crunch_lib.cpp's extern "C" exports
    "crn_get_width": ("crn_get_width", u32, [vp, u32]),
    "crn_get_height": ("crn_get_height", u32, [vp, u32]),
    "crn_get_levels": ("crn_get_levels", u32, [vp, u32]),
    "crn_get_dxt_format": ("crn_get_dxt_format", u32, [vp, u32]),
    "crn_get_bytes_per_block": ("crn_get_bytes_per_block", u32, [vp, u32]),
    "crn_get_uncompressed_size": ("crn_get_uncompressed_size", u32, [vp, u32, u32]),
    "crn_decompress": ("crn_decompress", None, [vp, u32, vp, u32, u32, u32]),
}


class Api:
    """The functions of SYMBOLS bound on a loaded libcrngpu.so."""

    def __init__(self, lib):
        for name, (sym, restype, argtypes) in SYMBOLS.items():
            fn = getattr(lib, sym)
            fn.restype = restype
            fn.argtypes = argtypes
            setattr(self, name, fn)


def probe(api, crn: bytes):
    """The same values, in the same order, as the reference harness's ref_crnd_probe."""
    buf = ctypes.create_string_buffer(crn, len(crn))
    n = len(crn)
    out = []
    fi = CrnFileInfo()
    fi.m_struct_size = ctypes.sizeof(fi)
    out.append(int(api.crnd_validate_file(buf, n, ctypes.byref(fi))))
    out += list(memoryview(fi).cast("B").cast("I"))
    ti = CrnTextureInfo()
    ti.m_struct_size = ctypes.sizeof(ti)
    out.append(int(api.crnd_get_texture_info(buf, n, ctypes.byref(ti))))
    out += [ti.m_width, ti.m_height, ti.m_levels, ti.m_faces, ti.m_bytes_per_block, ti.m_userdata0, ti.m_userdata1,
            ti.m_format & 0xFFFFFFFF]
    for l in range(ti.m_levels):
        li = CrnLevelInfo()
        li.m_struct_size = ctypes.sizeof(li)
        out.append(int(api.crnd_get_level_info(buf, n, l, ctypes.byref(li))))
        out += [li.m_width, li.m_height, li.m_faces, li.m_blocks_x, li.m_blocks_y, li.m_bytes_per_block,
                li.m_format & 0xFFFFFFFF]
        size = u32(0)
        p = api.crnd_get_level_data(buf, n, l, ctypes.byref(size))
        out += [p - ctypes.addressof(buf) if p else 0xFFFFFFFF, size.value]
    base = int(api.crnd_get_segmented_file_size(buf, n))
    seg = ctypes.create_string_buffer(max(base, 1))
    ok = bool(base) and base <= n and api.crnd_create_segmented_file(buf, n, seg, base)
    out += [base, int(ok)]
    return out, (seg.raw[:base] if ok else b"")
