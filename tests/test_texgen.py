"""The synthetic texture generator reproduces, byte for byte, the inputs the reference was run on
when the golden fixtures were made (their SHA-256 is in the fixture manifest): the fixtures'
quality bars only hold for those exact textures. No GPU needed."""
import numpy as np
import pytest

import golden_util as G


def texture_levels(w, h, content, seed, faces):
    from crunch2_gb300 import texgen
    out = []
    for f in range(faces):
        img = texgen.normal_map(w, h, seed + f) if content == "normal" else \
            texgen.colour_texture(w, h, seed + f, with_alpha_noise=(content == "colour_alpha"))
        out.append(texgen.mip_chain(img))
    return out


@pytest.mark.parametrize("name", sorted(G.manifest().keys()))
def test_fixture_inputs_reproduce(name):
    m = G.manifest()[name]
    fl = texture_levels(m["width"], m["height"], m["content"], m["seed"], m["faces"])
    assert G.sha(np.concatenate([im.reshape(-1) for f in fl for im in f])) == m["input_sha256"], name
