"""The allocation-free transcode entry point, called through the C ABI.

crngpu_unpack_level_noalloc serves callers that cannot allocate GPU memory while they run
(engines that reserve their VRAM budget up front and forbid untracked allocations, real-time
loops that cannot afford cudaMalloc/cudaFree waiting for the device to go idle). It keeps its
scratch in one fixed device array shared by every call, so this test checks its output against
the regular crngpu_unpack_level on two calls in a row for every level of every fixture (the
second call sees the array as the first call left it), bit for bit as all transcode tests are.
It lives in its own file, collected last, and passes alone or after the other tests.
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


def noalloc_level(cg, crn: bytes, level: int, faces: int, face_bytes: int):
    L = cg.lib()
    fn = L.crngpu_unpack_level_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_void_p), ctypes.c_uint32, ctypes.c_uint32,
                   ctypes.c_uint32, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    src = np.frombuffer(crn, np.uint8)
    out = torch.full((faces, face_bytes), 0x5A, dtype=torch.uint8, device="cuda")
    ptrs = (ctypes.c_void_p * faces)(*[out[f].data_ptr() for f in range(faces)])
    rc = fn(src.ctypes.data, len(crn), ptrs, face_bytes, 0, level, None)
    assert rc == 0, cg.last_error()
    return out.cpu().numpy()


@pytest.mark.parametrize("name", sorted(G.manifest().keys()))
def test_noalloc_matches_unpack_level_twice(cg, name):
    crn = G.crn_bytes(name)
    with cg.unpack_begin(crn) as ctx:
        for lvl in range(ctx.levels):
            want = ctx.unpack_level(lvl)
            face_bytes = want.shape[1]
            first = noalloc_level(cg, crn, lvl, ctx.faces, face_bytes)
            second = noalloc_level(cg, crn, lvl, ctx.faces, face_bytes)
            assert np.array_equal(first, want), (name, lvl, "first call")
            assert np.array_equal(second, want), (name, lvl, "second call")


def test_noalloc_rejects_bad_arguments(cg):
    crn = G.crn_bytes("dxt1_256")
    fn = cg.lib().crngpu_unpack_level_noalloc
    out = torch.zeros(64 * 64 * 8, dtype=torch.uint8, device="cuda")
    ptrs = (ctypes.c_void_p * 1)(out.data_ptr())
    src = np.frombuffer(crn, np.uint8)
    assert fn(src.ctypes.data, len(crn), ptrs, out.numel(), 6, 0, None) == cg.E_PARAM      # pitch
    assert fn(src.ctypes.data, len(crn), ptrs, 16, 0, 0, None) == cg.E_PARAM               # too small
    assert fn(src.ctypes.data, 60, ptrs, out.numel(), 0, 0, None) == cg.E_CORRUPT         # truncated
    assert fn(src.ctypes.data, len(crn), ptrs, out.numel(), 0, 0, None) == 0               # still usable
