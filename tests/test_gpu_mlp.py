"""Learned endpoint proposal on GB300: tensor-core forward/backward against the CPU oracle
(oracle/mlp_oracle.py), training, and the learned encode with its exact-optimizer fallback."""
import numpy as np
import pytest

import golden_util as G

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def L():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crunch2_gb300 import learned
    learned._bind()
    return learned


def rel_err(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12))


@pytest.fixture(scope="module")
def batch():
    blocks = np.concatenate([G.c0_blocks()[:384], G.blocks()["edge_in"][:256]])
    rng = np.random.default_rng(3)
    targets = rng.random((blocks.shape[0], 8)).astype(np.float32)
    return blocks, targets


def test_forward_matches_oracle(L, batch):
    from oracle import mlp_oracle
    blocks, _ = batch
    net = L.EndpointNet(seed=5)
    y = net.forward(torch.from_numpy(blocks).cuda()).cpu().numpy().astype(np.float64)
    ref, _ = mlp_oracle.forward(net.state(), blocks)
    assert rel_err(y[:, :7], ref[:, :7]) < 1e-2
    assert np.abs(y[:, 7:]).max() < 1e-6  # padded outputs stay zero


def test_fused_forward_many_tiles(L):
    """The persistent inference kernel loops over tiles: more tiles than SMs and a ragged tail."""
    from oracle import mlp_oracle
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    n = sms * 128 * 2 + 37
    rng = np.random.default_rng(11)
    blocks = rng.integers(0, 256, size=(n, 64), dtype=np.uint8)
    net = L.EndpointNet(seed=9)
    y = net.forward(torch.from_numpy(blocks).cuda()).cpu().numpy().astype(np.float64)
    idx = np.concatenate([np.arange(0, 256), np.arange(n - 300, n)])   # first tiles and the tail
    ref, _ = mlp_oracle.forward(net.state(), blocks[idx])
    assert rel_err(y[idx, :7], ref[:, :7]) < 1e-2
    assert np.isfinite(y).all()
    assert np.abs(y[:, 7:]).max() < 1e-6


def test_gradients_match_oracle(L, batch):
    from oracle import mlp_oracle
    blocks, targets = batch
    net = L.EndpointNet(seed=6)
    loss = net.gradients(torch.from_numpy(blocks).cuda(), torch.from_numpy(targets).cuda())
    ref_loss, ref = mlp_oracle.gradients(net.state(), blocks, targets)
    assert abs(loss - ref_loss) / ref_loss < 1e-2
    for i, name in enumerate(L.PARAM_NAMES):
        g = net.get(i, grad=True).astype(np.float64)
        e = rel_err(g, ref[name])
        cos = float((g * ref[name]).sum() / (np.linalg.norm(g) * np.linalg.norm(ref[name]) + 1e-30))
        assert e < 3e-2 and cos > 0.999, (name, e, cos)


def test_quantile_bound_gradients_match_oracle(L, batch):
    from oracle import mlp_oracle
    blocks, targets = batch
    net = L.EndpointNet(seed=4)
    net.set_bound_loss(0.9, 0.25)
    loss = net.gradients(torch.from_numpy(blocks).cuda(), torch.from_numpy(targets).cuda())
    ref_loss, ref = mlp_oracle.gradients(net.state(), blocks, targets, tau=0.9, bw=0.25)
    assert abs(loss - ref_loss) / ref_loss < 1e-2
    for i, name in enumerate(L.PARAM_NAMES):
        g = net.get(i, grad=True).astype(np.float64)
        e = rel_err(g, ref[name])
        cos = float((g * ref[name]).sum() / (np.linalg.norm(g) * np.linalg.norm(ref[name]) + 1e-30))
        assert e < 3e-2 and cos > 0.999, (name, e, cos)


@pytest.fixture(scope="module")
def trained(L):
    blocks = L.training_blocks(4, 256, seed0=1000)          # 16,384 training blocks
    targets, _ = L.make_targets(blocks)
    net = L.EndpointNet(seed=7)
    losses = L.train(net, blocks, targets, steps=400, batch=1024, lr=1e-3)
    return net, losses


def test_training_reduces_loss(trained):
    _, losses = trained
    assert np.mean(losses[-20:]) < 0.5 * np.mean(losses[:5]), (losses[:5], losses[-20:])


def test_zero_threshold_falls_back_to_exact_optimizer(L, trained):
    import crunch2_gb300 as cg
    net, _ = trained
    blocks = torch.from_numpy(G.c0_blocks()).cuda()
    out, fb = net.encode(blocks, threshold=0.0, fallback_quality=4)
    assert fb == blocks.shape[0]
    assert torch.equal(out, cg.dxt1_optimize(blocks))


@pytest.mark.parametrize("quality", [0, 2, 3])
def test_fallback_quality_is_the_exact_optimizer_at_that_quality(L, trained, quality):
    import crunch2_gb300 as cg
    net, _ = trained
    blocks = torch.from_numpy(G.c0_blocks()).cuda()
    out, fb = net.encode(blocks, threshold=0.0, fallback_quality=quality)
    assert fb == blocks.shape[0]
    assert torch.equal(out, cg.dxt1_optimize(blocks, quality=quality))
    # crngpu_dxt1_learned is crngpu_dxt1_learned_ex with Uber fallback
    a = torch.empty_like(out)
    fa = L.ctypes.c_uint32(0)
    L._check(L._bind().crngpu_dxt1_learned(net.h, blocks.data_ptr(), blocks.shape[0], 1, 1.5, a.data_ptr(),
                                           L.ctypes.byref(fa), None), "crngpu_dxt1_learned")
    torch.cuda.synchronize()
    b, fb_b = net.encode(blocks, threshold=1.5, fallback_quality=4)
    assert torch.equal(a, b) and fa.value == fb_b
    with pytest.raises(cg.CrnGpuError):
        net.encode(blocks, threshold=1.5, fallback_quality=5)


def test_trained_network_beats_untrained(L, trained):
    from dxt_decode import rgb_rmse
    net, _ = trained
    held_out = L.training_blocks(1, 256, seed0=50000)
    host = held_out.cpu().numpy()
    untrained = L.EndpointNet(seed=8)
    res = {}
    for name, n_ in (("trained", net), ("untrained", untrained)):
        out, fb = n_.encode(held_out, threshold=1.5)
        nofb, _ = n_.encode(held_out, threshold=1e30)
        res[name] = (rgb_rmse(out.cpu().numpy(), host), fb, rgb_rmse(nofb.cpu().numpy(), host))
    import crunch2_gb300 as cg
    plain = rgb_rmse(cg.dxt1_optimize(held_out).cpu().numpy(), host)
    print("plain", plain, "trained (rmse, fallbacks, rmse without fallback)", res["trained"],
          "untrained", res["untrained"])
    assert res["trained"][2] < res["untrained"][2]      # better proposals before any fallback
    assert res["trained"][1] < res["untrained"][1]      # fewer blocks need the exact optimizer


def test_shipped_network_on_held_out_textures(L):
    """Config 4's evaluation at a reduced size: the shipped weights on two held-out 2048 x 2048
    textures from config 4's evaluation seed range, at config 4's fallback threshold (1.5): RGB
    RMSE within 0.1 of the plain optimizer's, and faster than the plain optimizer. (bench.py runs
    the full 32 x 4096^2 evaluation.)"""
    r = L.config4(weights=L.WEIGHTS, eval_textures=2, eval_size=2048, threshold=L.DEFAULT_THRESHOLD)
    got = r["learned"][0]
    print({k: r[k] for k in ("plain_mtexel_s", "rmse_plain")}, got)
    assert got["rmse_learned"] - r["rmse_plain"] <= 0.1
    assert got["speedup"] > 2.0
    assert 0.0 < got["fallback_frac"] < 0.25
