"""The neural IBL shader on the GPU, through the C ABI: the tensor-core kernels against the CPU
oracle (oracle/nn_oracle.py: forward, gradients, Adam, record sampling), the capture of training
records by the plain PBR shader, the fused raster variant (coverage and depth identical to the
plain shader), and the whole train / evaluate / fall-back pipeline, which must show what the
trained network gains over the method without it."""
import numpy as np
import pytest

from oracle import nn_oracle as O
from softglrender_gb300 import api as A
from softglrender_gb300 import scenes as S
from softglrender_gb300.neural import NeuralShader, pbr_programs, train_neural_ibl

pytestmark = pytest.mark.gpu


def _records(n, seed):
    """Synthetic records with the shader's input ranges: unit N and V, roughness, metallic,
    albedo in [0, 1], NdotV; targets a smooth function of them."""
    rng = np.random.default_rng(seed)
    N = rng.normal(size=(n, 3))
    N /= np.linalg.norm(N, axis=1, keepdims=True)
    V = rng.normal(size=(n, 3))
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    rough, metal = rng.uniform(0.05, 1, n), rng.uniform(0, 1, n)
    alb = rng.uniform(0, 1, (n, 3))
    ndv = np.maximum((N * V).sum(1), 0)
    rec = np.zeros((n, 16), np.float32)
    rec[:, 0:3], rec[:, 3:6], rec[:, 6], rec[:, 7], rec[:, 8:11], rec[:, 11] = N, V, rough, metal, alb, ndv
    sky = 0.5 + 0.4 * N[:, 1:2]
    rec[:, 12:15] = np.sqrt(alb * sky * (1 - 0.5 * metal[:, None]) + 0.2 * ndv[:, None] * (1 - rough[:, None]))
    return rec


@pytest.fixture()
def net(cuda_lib):
    r = A.Renderer(cuda_lib, 0)
    n = NeuralShader(r, seed=5)
    yield n
    n.destroy()
    r.destroy()


def test_infer_matches_oracle(net):
    rec = _records(1000, 1)   # 7 full tiles + a ragged one
    net.set_records(rec)
    y = net.infer()
    ref, _ = O.forward(O.unflatten(net.get_params()), rec[:, :12], use_bf16=True)
    scale = np.abs(ref).max()
    assert np.abs(y - ref).max() <= 2e-3 * scale + 1e-4, np.abs(y - ref).max()


def test_gradients_match_oracle(net):
    rec = _records(1000, 2)
    net.set_records(rec)
    g, loss = net.gradients(0, len(rec))
    p = O.unflatten(net.get_params())
    ref_loss, ref = O.loss_and_grad(p, rec[:, :12], rec[:, 12:15], use_bf16=True)
    assert loss == pytest.approx(ref_loss, rel=1e-3)
    gg = O.unflatten(g)
    for k in O.ORDER:
        err = np.linalg.norm(gg[k] - ref[k]) / max(np.linalg.norm(ref[k]), 1e-12)
        assert err < 2e-2, (k, err)


def test_gradients_are_deterministic(net):
    rec = _records(5000, 3)
    net.set_records(rec)
    g1, l1 = net.gradients(0, len(rec))
    g2, l2 = net.gradients(0, len(rec))
    assert np.array_equal(g1, g2) and l1 == l2


def test_adam_step_matches_oracle(net):
    rec = _records(3000, 4)
    net.set_records(rec)
    p0 = net.get_params()
    lr, batch, seed = 1e-3, 2048, 11
    net.train(1, batch, lr=lr, seed=seed)
    p1 = net.get_params()
    idx = O.sample_indices(seed, 0, batch, len(rec))
    _, g = O.loss_and_grad(O.unflatten(p0), rec[idx, :12], rec[idx, 12:15], use_bf16=True)
    p = O.unflatten(p0)
    m = {k: np.zeros_like(v) for k, v in p.items()}
    v = {k: np.zeros_like(q) for k, q in p.items()}
    O.adam_step(p, g, m, v, 1, lr)
    d_gpu, d_ref = p1 - p0, O.flatten(p) - p0
    # the first Adam step moves every parameter with a non-negligible gradient by about lr
    gf = np.abs(O.flatten(g))
    sig = gf > 1e-5
    agree = np.abs(d_gpu[sig] - d_ref[sig]) <= 0.05 * lr
    assert agree.mean() > 0.99, agree.mean()


def test_training_reduces_loss(net):
    rec = _records(1 << 16, 5)
    net.set_records(rec)
    _, l0 = net.gradients(0, 8192)
    net.train(300, 8192, lr=2e-3)
    _, l1 = net.gradients(0, 8192)
    assert l1 < 0.1 * l0, (l0, l1)


def _small_pbr(view=0):
    return S.config_pbr(width=320, height=180, lon=96, lat=48, tex=128, prefilter=64, irradiance=16, view=view)


def test_capture_records_plain_shader_fragments(cuda_lib):
    r = A.Renderer(cuda_lib, 0)
    net = NeuralShader(r, seed=1)
    inst = S.SceneInstance(r, _small_pbr())
    r.setStatsLevel(2)
    net.capture(1 << 20, 1)
    inst.render()
    r.waitIdle()
    net.stop_capture()
    frags = r.drawStats()["fragments_shaded"]
    n = net.record_count()
    assert n == frags > 1000
    rec = net.get_records()
    assert np.all(np.isfinite(rec))
    np.testing.assert_allclose(np.linalg.norm(rec[:, 0:3], axis=1), 1.0, atol=1e-4)   # N
    np.testing.assert_allclose(np.linalg.norm(rec[:, 3:6], axis=1), 1.0, atol=1e-4)   # V
    assert rec[:, 6:11].min() >= 0 and rec[:, 6:11].max() <= 1
    assert rec[:, 12:15].min() >= 0
    # a stride keeps every k-th fragment
    net.capture(1 << 20, 4)
    inst.render()
    net.stop_capture()
    assert net.record_count() == (frags + 3) // 4
    net.destroy()
    r.destroy()


def test_neural_raster_keeps_coverage_and_depth(cuda_lib):
    r = A.Renderer(cuda_lib, 0)
    net = NeuralShader(r, seed=2)
    inst = S.SceneInstance(r, _small_pbr(view=2))
    r.setStatsLevel(2)
    inst.render()
    plain = inst.outputs()
    fp = r.drawStats()["fragments_shaded"]
    for prog in pbr_programs(inst):
        net.bind(prog)
    inst.render()
    neural = inst.outputs()
    fn = r.drawStats()["fragments_shaded"]
    assert fp == fn
    assert np.array_equal(plain["depth"].view(np.uint32), neural["depth"].view(np.uint32))
    # background (clear colour) pixels are identical: coverage is unchanged
    bg = np.array([5, 5, 7, 255], np.uint8)   # ClearStates (0.02, 0.02, 0.03, 1.0) as RGBA8
    cov_p = np.any(plain["resolved"] != bg, axis=-1)
    cov_n = np.any(neural["resolved"] != bg, axis=-1)
    assert np.array_equal(cov_p, cov_n) or (cov_p != cov_n).mean() < 1e-4
    net.destroy()
    r.destroy()


def test_neural_pipeline_gains_over_the_method_without_it(cuda_lib):
    """Train on captures of 8 orbit views, evaluate on 4 held-out views: the trained network must
    be far closer to the plain shader than the shader without its IBL term and than the untrained
    network, and the fall-back decision must follow the threshold."""
    r = A.Renderer(cuda_lib, 0)
    kw = dict(width=320, height=180, lon=96, lat=48, tex=128, prefilter=64, irradiance=16)
    inst, net, rep = train_neural_ibl(r, kw, train_views=8, test_views=4, records=1 << 18, steps=3000,
                                      batch=1 << 14, lr=3e-3, seed=3)
    print("neural PSNR per held-out view:", [round(x, 2) for x in rep.psnr_views],
          "without IBL:", [round(x, 2) for x in rep.psnr_without],
          "untrained:", [round(x, 2) for x in rep.psnr_untrained], "loss", rep.final_loss)
    assert rep.records > 100000
    assert min(rep.psnr_views) > max(rep.psnr_without) + 6.0
    assert min(rep.psnr_views) > max(rep.psnr_untrained) + 6.0
    assert rep.bound == (rep.psnr_mean >= 40.0)
    net.destroy()
    r.destroy()


@pytest.mark.parametrize("deferred", [True, False])
def test_neural_wait_timeouts_reach_the_host(cuda_lib, deferred):
    """A tensor-core wait that times out is reported through the sticky flags (bit 6). The test hook
    reports a timeout after each wait has completed normally (nothing is abandoned in flight);
    without it a frame reports nothing."""
    r = A.Renderer(cuda_lib, 0)
    r.setDeferredShading(deferred)
    net = NeuralShader(r, seed=4)
    inst = S.SceneInstance(r, _small_pbr(view=1))
    for prog in pbr_programs(inst):
        net.bind(prog)
    inst.render()
    assert r.getOverflow() == 0
    NeuralShader.set_test_flags(r, 1)
    inst.render()
    assert r.getOverflow() & 64
    NeuralShader.set_test_flags(r, 0)
    inst.render()
    assert r.getOverflow() == 0
    with pytest.raises(A.SoftGLError):
        NeuralShader.set_test_flags(r, 2)
    net.destroy()
    r.destroy()


def test_per_material_fallback_in_one_submission(cuda_lib):
    """Two PBR materials (the same material maps under two environments, the second a differently
    tinted sky) in one uneven batch: the network is trained on material 0 only, each material keeps
    it only if its lowest held-out PSNR reaches the threshold, and in the same submission the
    material that fell back renders exactly as the plain shader while the other one uses the
    network."""
    from softglrender_gb300.neural import bind_per_material, evaluate_material
    from softglrender_gb300.uneven import UnevenBatch, UnevenConfig
    r = A.Renderer(cuda_lib, 0)
    kw = dict(width=320, height=180, lon=96, lat=48, tex=128, prefilter=64, irradiance=16)
    inst, net, rep = train_neural_ibl(r, kw, train_views=8, test_views=2, records=1 << 18, steps=3000,
                                      batch=1 << 14, lr=3e-3, seed=3, baselines=False)
    d0 = evaluate_material(r, net, "env0", dict(kw, ibl_variant=0), views=[20, 21])
    d1 = evaluate_material(r, net, "env1", dict(kw, ibl_variant=1), views=[20, 21])
    print("material PSNR min:", round(d0.psnr_min, 2), round(d1.psnr_min, 2))
    assert d0.psnr_min > d1.psnr_min + 3.0     # the network only knows environment 0
    threshold = 0.5 * (d0.psnr_min + d1.psnr_min)
    d0.threshold_db = d1.threshold_db = threshold
    cfg = UnevenConfig(scenes=6, tri_min=2000, tri_max=20000, resolutions=(64, 128), seed=5100, pbr_tex=128,
                       prefilter=64, irradiance=16, blinn_tex=64, pbr_materials=2)
    u = UnevenBatch(r, cfg)
    u.render()
    r.waitIdle()
    plain = {s: u.outputs(s) for s in u.items}
    bound = bind_per_material(net, {"env0": u.pbr_programs(0), "env1": u.pbr_programs(1)},
                              {"env0": d0, "env1": d1})
    assert bound == {"env0": True, "env1": False}
    u.render()
    r.waitIdle()
    for s, it in u.items.items():
        o = u.outputs(s)
        if not it["pbr"] or it["material"] == 1:   # plain shader: bit for bit
            for k in plain[s]:
                assert np.array_equal(o[k].view(np.uint8), plain[s][k].view(np.uint8)), (s, k)
        else:                                      # the network: same coverage and depth, colour changed
            assert np.array_equal(o["depth"].view(np.uint32), plain[s]["depth"].view(np.uint32))
            assert not np.array_equal(o["resolved"], plain[s]["resolved"])
    net.destroy()
    r.destroy()
