"""CPU checks of the drop-in boundary: the C-ABI library builds, loads and exports every
entry point include/crngpu.h declares (no GPU calls here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    with open(os.path.join(ROOT, "include", "crngpu.h")) as fh:
        text = fh.read()
    return sorted(set(re.findall(r"CRNGPU_API\s+[\w\s\*]+?\b(crngpu_\w+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("crngpu_dxt1_optimize_batch", "crngpu_dxt5a_optimize_batch", "crngpu_compress_blocks",
                 "crngpu_compress_image", "crngpu_unpack_begin", "crngpu_unpack_level",
                 "crngpu_unpack_level_segmented", "crngpu_unpack_levels", "crngpu_unpack_end",
                 "crngpu_crn_decompress"):
        assert must in names


def test_library_exports_every_declared_symbol():
    import shutil
    if not (shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
        pytest.skip("no CUDA toolkit to build libcrngpu.so")
    import crunch2_gb300 as cg
    lib = cg.lib()
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert "sm_103a" in cg.version()


def test_host_mirror_names_follow_the_reference():
    import crunch2_gb300 as cg
    for name in ("dxt1_optimize", "dxt5a_optimize", "compress_blocks", "compress_image", "unpack_begin",
                 "crn_decompress", "UnpackContext"):
        assert hasattr(cg, name)


def test_pointer_helpers_refuse_strided_buffers():
    """The C ABI takes plain pointers: a strided numpy view (such as a transposed mip level) must
    be copied to C order by the wrappers, never passed as is."""
    import numpy as np
    import crunch2_gb300 as cg
    a = np.arange(4 * 6 * 4, dtype=np.uint8).reshape(4, 6, 4).transpose(1, 0, 2)
    with pytest.raises(cg.CrnGpuError):
        cg._ptr_mem(a)
    c = cg._contiguous(a)
    assert c.flags["C_CONTIGUOUS"] and np.array_equal(c, a)
    assert cg._ptr_mem(c)[1] == cg.MEM_HOST
