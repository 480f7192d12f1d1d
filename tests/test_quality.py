"""The device-side quality metrics (crunch2_gb300.quality, torch) against the numpy block decoders
of the tests, on random blocks in every mode (four/three-colour DXT1, eight/six-value alpha).
Runs on the CPU."""
import numpy as np
import torch

from dxt_decode import dxt1_colours, dxt5a_values


def test_decoders_match_numpy():
    from crunch2_gb300 import quality as Q
    rng = np.random.default_rng(3)
    b = rng.integers(0, 256, size=(4096, 8), dtype=np.uint8)
    b[::2, 0], b[::2, 1] = 0, 255  # alpha: l < h (six-value mode) on half the blocks
    b[1::4, :4] = b[1::4, [2, 3, 0, 1]]  # DXT1: swap endpoints on a quarter (mode flip where distinct)
    assert np.array_equal(Q.dxt1_colours(torch.from_numpy(b)).numpy(), dxt1_colours(b))
    assert np.array_equal(Q.alpha_values(torch.from_numpy(b)).numpy(), dxt5a_values(b))


def test_block_rmse_formats():
    from crunch2_gb300 import quality as Q
    rng = np.random.default_rng(4)
    d = rng.integers(0, 256, size=(1000, 16), dtype=np.uint8)
    src = rng.integers(0, 256, size=(1000, 64), dtype=np.uint8)
    px = src.reshape(-1, 16, 4).astype(np.int64)
    r = Q.block_rmse(torch.from_numpy(d), torch.from_numpy(src), "DXT5")
    col = dxt1_colours(d[:, 8:])
    assert abs(r["rmse_color"] - np.sqrt(((col - px[:, :, :3]) ** 2).mean())) < 1e-9
    assert abs(r["rmse_alpha"] - np.sqrt(((dxt5a_values(d[:, :8]) - px[:, :, 3]) ** 2).mean())) < 1e-9
    r = Q.block_rmse(torch.from_numpy(d), torch.from_numpy(src), "DXN_XY")
    x, y = dxt5a_values(d[:, :8]), dxt5a_values(d[:, 8:])
    ref = np.sqrt((((x - px[:, :, 0]) ** 2).sum() + ((y - px[:, :, 1]) ** 2).sum()) / (2 * x.size))
    assert abs(r["rmse_xy"] - ref) < 1e-9
