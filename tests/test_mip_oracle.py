"""The mip-generation oracle (CPU restatement, oracle/mip_oracle.py) against the reference's own
mip levels (tests/golden/mips.npz, written by crnlib's generate_mipmaps resampler): every level of
every case, each of the five mip filters, gamma on and off, clamp and wrap, 3 and 4 components.
No GPU needed."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def cases():
    with open(os.path.join(HERE, "golden", "mips.json")) as fh:
        return json.load(fh)


@pytest.mark.parametrize("name", sorted(cases().keys()))
def test_oracle_mips_match_reference(name):
    from oracle import mip_oracle
    m = cases()[name]
    z = np.load(os.path.join(HERE, "golden", "mips.npz"))
    base = z[name + "_base"]
    levels = mip_oracle.generate_mipmaps(base, m["filter"], m["filter_scale"], m["srgb"], m["wrap"],
                                         alpha=m["comps"] == 4)
    assert len(levels) == m["levels"]
    got = np.concatenate([l.reshape(-1) for l in levels[1:]])
    ref = z[name + "_levels"]
    assert np.array_equal(got, ref), (name, int((got != ref).sum()), got.size)
