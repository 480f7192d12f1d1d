"""Bounded waits inside the kernels, with every first wait forced to give up at once.

Each wait on an mbarrier is bounded. When a staging wait runs out, the DXT1 encoders and the
TMA expansion variants read global memory instead, so their output must not change. When a wait
on a tcgen05 MMA runs out, the MLP call must fail with an error status and leave the context
usable. crngpu_force_wait_timeouts(1) sets the first-wait bound to zero polls (the copies and
MMAs still complete, and are drained with the normal long bound before a CTA exits), so these
tests run the fallback code without anything on the GPU hanging or faulting.
"""
import numpy as np
import pytest

import golden_util as G

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

TMA_VARIANTS = (18, 19, 20)  # the expansion variants that stage index records by bulk copies


@pytest.fixture(scope="module")
def cg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import crunch2_gb300
    crunch2_gb300.lib()
    return crunch2_gb300


@pytest.fixture()
def forced(cg):
    cg.wait_counters(reset=True)
    cg.force_wait_timeouts(True)
    try:
        yield cg
    finally:
        cg.force_wait_timeouts(False)


def test_normal_runs_count_no_timeouts(cg):
    cg.wait_counters(reset=True)
    blocks = torch.from_numpy(G.c0_blocks()).cuda()
    cg.dxt1_optimize(blocks)
    torch.cuda.synchronize()
    assert cg.wait_counters() == {k: 0 for k in cg.wait_counters()}


def test_encoder_staging_fallback_is_bit_identical(cg, forced):
    blocks = torch.from_numpy(np.concatenate([G.c0_blocks(), G.blocks()["edge_in"]])).cuda()
    cg.force_wait_timeouts(False)
    want = cg.dxt1_optimize(blocks).cpu().numpy()
    cg.wait_counters(reset=True)
    cg.force_wait_timeouts(True)
    got = cg.dxt1_optimize(blocks).cpu().numpy()
    c = cg.wait_counters()
    assert np.array_equal(got, want)
    assert c["encode_stage_timeouts"] > 0, c
    assert c["encode_drain_failures"] == 0, c


def test_batched_encoder_staging_fallback_is_bit_identical(cg, forced):
    from crunch2_gb300 import texgen
    levels = texgen.mip_chain(texgen.colour_texture(160, 96, 5))
    rgba = torch.from_numpy(np.concatenate([l.reshape(-1) for l in levels])).cuda()
    out = torch.zeros(cg.mip_chain_blocks(160, 96, len(levels)) * 8, dtype=torch.uint8, device="cuda")
    cg.force_wait_timeouts(False)
    with cg.EncodeBatch([(rgba, out, 160, 96, len(levels), cg.FMT_DXT1)]) as b:
        b.launch()
        torch.cuda.synchronize()
        want = out.cpu().numpy()
        out.zero_()
        cg.wait_counters(reset=True)
        cg.force_wait_timeouts(True)
        b.launch()
        torch.cuda.synchronize()
    c = cg.wait_counters()
    assert np.array_equal(out.cpu().numpy(), want)
    assert c["encode_stage_timeouts"] > 0, c
    assert c["encode_drain_failures"] == 0, c


def test_tma_expansion_fallback_writes_golden_levels(cg, forced):
    man = G.manifest()
    names = sorted(man)
    ctxs = [cg.unpack_begin(G.crn_bytes(n)) for n in names]
    outs = [torch.full((sum(l["bytes"] for l in man[n]["levels"]),), 0xCD, dtype=torch.uint8, device="cuda")
            for n in names]
    try:
        with cg.UnpackBatch([(c, 0, c.levels, o) for c, o in zip(ctxs, outs)]) as batch:
            for v in TMA_VARIANTS:
                batch.set_variant(v)
                cg.wait_counters(reset=True)
                for o in outs:
                    o.fill_(0xCD)
                batch.launch()
                batch.status()
                c = cg.wait_counters()
                assert c["expand_stage_timeouts"] > 0, (v, c)
                assert c["expand_drain_failures"] == 0, (v, c)
                for n, o in zip(names, outs):
                    host = o.cpu().numpy()
                    pos = 0
                    for lvl, info in enumerate(man[n]["levels"]):
                        assert G.sha(host[pos:pos + info["bytes"]]) == info["sha256"], (v, n, lvl)
                        pos += info["bytes"]
    finally:
        for c in ctxs:
            c.close()


def test_mma_wait_timeout_is_an_error_and_the_context_recovers(cg, forced):
    from crunch2_gb300 import learned
    learned._bind()
    net = learned.default_net()
    blocks = torch.from_numpy(G.c0_blocks()).cuda()
    cg.force_wait_timeouts(False)
    want, want_fb = net.encode(blocks)
    want = want.cpu().numpy()
    y_want = net.forward(blocks[:512]).cpu().numpy()
    cg.wait_counters(reset=True)
    cg.force_wait_timeouts(True)
    with pytest.raises(cg.CrnGpuError) as e:
        net.encode(blocks)
    assert e.value.code == cg.E_DEVICE
    with pytest.raises(cg.CrnGpuError):
        net.forward(blocks[:512])
    targets = torch.zeros((512, 8), dtype=torch.float32, device="cuda")
    with pytest.raises(cg.CrnGpuError):                 # the training GEMMs (k_gemm_tc)
        net.gradients(blocks[:512], targets)
    assert cg.wait_counters()["mma_wait_timeouts"] > 0
    cg.force_wait_timeouts(False)
    again, fb = net.encode(blocks)
    assert fb == want_fb and np.array_equal(again.cpu().numpy(), want)
    assert np.array_equal(net.forward(blocks[:512]).cpu().numpy(), y_want)
    assert np.isfinite(net.gradients(blocks[:512], targets))
