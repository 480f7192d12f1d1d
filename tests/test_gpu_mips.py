"""GPU mip generation (crngpu_generate_mipmaps) against the reference's own mip levels (golden
fixtures from crnlib's generate_mipmaps resampler) and, at sizes beyond the fixtures, against the
oracle (the CPU restatement pinned to those fixtures): bit-exact, host and device buffers."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def cg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import crunch2_gb300
    crunch2_gb300.lib()
    return crunch2_gb300


def cases():
    with open(os.path.join(HERE, "golden", "mips.json")) as fh:
        return json.load(fh)


@pytest.mark.parametrize("name", sorted(cases().keys()))
def test_gpu_mips_match_reference(cg, name):
    m = cases()[name]
    z = np.load(os.path.join(HERE, "golden", "mips.npz"))
    base = z[name + "_base"]
    levels = cg.generate_mipmaps(base, m["filter"], m["filter_scale"], m["srgb"], m["wrap"], alpha=m["comps"] == 4)
    assert len(levels) == m["levels"]
    assert np.array_equal(levels[0], base)
    got = np.concatenate([l.reshape(-1) for l in levels[1:]])
    ref = z[name + "_levels"]
    assert np.array_equal(got, ref), (name, int((got != ref).sum()), got.size)


@pytest.mark.parametrize("filt,srgb,wrap", [("kaiser", True, False), ("lanczos4", False, True), ("box", True, True)])
def test_gpu_mips_match_oracle_device_buffers(cg, filt, srgb, wrap):
    from oracle import mip_oracle
    from crunch2_gb300 import texgen
    img = texgen.colour_texture(203, 130, 77, with_alpha_noise=True)
    want = mip_oracle.generate_mipmaps(img, filt, 0.9, srgb, wrap, alpha=True, levels=4)
    got = cg.generate_mipmaps(torch.from_numpy(img).cuda(), filt, 0.9, srgb, wrap, alpha=True, levels=4)
    for l, (a, b) in enumerate(zip(got, want)):
        assert np.array_equal(a.cpu().numpy(), b), (filt, l)
