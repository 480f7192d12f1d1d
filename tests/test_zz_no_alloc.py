"""The allocation-free transcode entry point, called through the C ABI.

crngpu_unpack_level_noalloc serves callers that cannot allocate GPU memory while they run
(engines that reserve their VRAM budget up front and forbid untracked allocations, real-time
loops that cannot afford cudaMalloc/cudaFree waiting for the device to go idle). It keeps its
scratch in one fixed device array shared by every call. This test checks its output on two
calls in a row (the second call sees the array as the first call left it): against the
reference's own per-level SHA-256 for every level of every fixture, and against the regular
crngpu_unpack_level on a 2048 x 2048 level and a 1024 x 1024 cube-map level, whose launch
descriptors are larger than the small fixtures'. It lives in its own file, collected last, and
passes alone or after the other tests.
"""
import ctypes

import numpy as np
import pytest

import golden_util as G

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def cg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import crunch2_gb300
    crunch2_gb300.lib()
    return crunch2_gb300


def noalloc_fn(cg):
    fn = cg.lib().crngpu_unpack_level_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_void_p), ctypes.c_uint32, ctypes.c_uint32,
                   ctypes.c_uint32, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def noalloc_level(cg, crn: bytes, level: int, faces: int, face_bytes: int):
    src = np.frombuffer(crn, np.uint8)
    out = torch.full((faces, face_bytes), 0x5A, dtype=torch.uint8, device="cuda")
    ptrs = (ctypes.c_void_p * faces)(*[out[f].data_ptr() for f in range(faces)])
    rc = noalloc_fn(cg)(src.ctypes.data, len(crn), ptrs, face_bytes, 0, level, None)
    assert rc == 0, cg.last_error()
    return out.cpu().numpy()


@pytest.mark.parametrize("name", sorted(G.manifest().keys()))
def test_noalloc_matches_reference_twice(cg, name):
    m = G.manifest()[name]
    crn = G.crn_bytes(name)
    for lvl, info in enumerate(m["levels"]):
        face_bytes = info["bytes"] // m["faces"]
        first = noalloc_level(cg, crn, lvl, m["faces"], face_bytes)
        second = noalloc_level(cg, crn, lvl, m["faces"], face_bytes)
        assert G.sha(first.reshape(-1)) == info["sha256"], (name, lvl, "first call")
        assert G.sha(second.reshape(-1)) == info["sha256"], (name, lvl, "second call")


@pytest.mark.parametrize("size,faces", [(2048, 1), (1024, 6)])
def test_noalloc_large_levels_match_unpack_level(cg, size, faces):
    from crunch2_gb300 import texgen
    face_levels = [[texgen.colour_texture(size, size, 40 + f)] for f in range(faces)]
    crn = cg.compress_crn(face_levels, cg.FMT_DXT1, 128)
    with cg.unpack_begin(crn) as ctx:
        want = ctx.unpack_level(0)
    for call in ("first", "second"):
        got = noalloc_level(cg, crn, 0, faces, want.shape[1])
        assert np.array_equal(got, want), (size, faces, call)


def test_noalloc_rejects_bad_arguments(cg):
    crn = G.crn_bytes("dxt1_256")
    fn = noalloc_fn(cg)
    out = torch.zeros(64 * 64 * 8, dtype=torch.uint8, device="cuda")
    ptrs = (ctypes.c_void_p * 1)(out.data_ptr())
    src = np.frombuffer(crn, np.uint8)
    assert fn(src.ctypes.data, len(crn), ptrs, out.numel(), 6, 0, None) == cg.E_PARAM      # pitch
    assert fn(src.ctypes.data, len(crn), ptrs, 16, 0, 0, None) == cg.E_PARAM               # too small
    assert fn(src.ctypes.data, 60, ptrs, out.numel(), 0, 0, None) == cg.E_CORRUPT         # truncated
    assert fn(src.ctypes.data, len(crn), ptrs, out.numel(), 0, 0, None) == 0               # still usable
