"""The learned QLT closure on the GPU.

* The training kernels' loss gradient against the CPU reference
  (oracle/surrogate_ref.py, itself pinned to finite differences).
* The FP32 forward against the CPU reference on the trained parameters, the
  BF16 and FP16 tensor-core forwards (the ones fused into the push) against
  the plain closure, for hidden widths 64 (the default) and 32, and the
  plain-closure fallback outside the box.
* The two engines that serve the network (block-collective tcgen05 with
  activations in tensor memory, the default; warp-collective mma.sync) on
  the same trained weights: the same inputs served, outputs equal to FP32
  rounding (the tensor cores associate the sums differently and the
  tcgen05 engine carries the biases as 16-bit head + remainder inputs of
  the GEMMs, so a 16-bit activation can round the other way: median
  relative difference <= 2e-5, every output within 3 %), and the same
  accuracy against the plain closure.
* The mixed focused push served by the network, on either engine, against
  the FP64 oracle with the plain closure: momentum spectrum L1 <= 1 %,
  chi-square p > 0.01, and the in-kernel judge's record of the network's
  per-step error.
"""
from __future__ import annotations

import numpy as np
import pytest

import surrogate_ref as sr
from test_gpu_statistics import _chi2_same, _spectrum

pytestmark = pytest.mark.gpu

TRAIN = dict(samples=524288, steps=8000, batch=4096, learning_rate=1e-2, seed=2024)


def _train(ctx, kpt, binding, element_type):
    params = binding.default_params(kperp_over_kpara=0.05, focused=1, closure=2)
    settings = kpt.settings_from_dict(params)
    return params, settings, ctx.train_surrogate(settings, element_type=element_type,
                                                 hidden_width=32, **TRAIN)


@pytest.fixture(scope="module")
def trained(ctx, kpt, binding):
    params, settings, surrogate = _train(ctx, kpt, binding, kpt.SURROGATE_BF16)
    yield params, settings, surrogate
    ctx.set_surrogate(None)
    surrogate.close()


@pytest.fixture(scope="module")
def trained64(ctx, kpt, binding):
    params = binding.default_params(kperp_over_kpara=0.05, focused=1, closure=2)
    settings = kpt.settings_from_dict(params)
    surrogate = ctx.train_surrogate(settings, element_type=kpt.SURROGATE_BF16, hidden_width=64,
                                    **TRAIN)
    yield params, settings, surrogate
    ctx.set_surrogate(None)
    surrogate.close()


@pytest.fixture(scope="module")
def trained64fp16(ctx, kpt, binding):
    params = binding.default_params(kperp_over_kpara=0.05, focused=1, closure=2)
    settings = kpt.settings_from_dict(params)
    surrogate = ctx.train_surrogate(settings, element_type=kpt.SURROGATE_FP16, hidden_width=64,
                                    **TRAIN)
    yield params, settings, surrogate
    ctx.set_surrogate(None)
    surrogate.close()


@pytest.fixture(scope="module")
def trained16(ctx, kpt, binding):
    params, settings, surrogate = _train(ctx, kpt, binding, kpt.SURROGATE_FP16)
    yield params, settings, surrogate
    ctx.set_surrogate(None)
    surrogate.close()


def _box_inputs(rng, n, norm, inside=True):
    lo, hi = norm["in_lo"], norm["in_hi"]
    feat = rng.uniform(lo, hi, (n, 5))
    sign = np.where(rng.uniform(size=n) < 0.5, -1.0, 1.0)
    mu = sign * np.exp(feat[:, 0])
    return np.stack([mu, feat[:, 1], feat[:, 2], np.exp(feat[:, 3]), feat[:, 4]], axis=1)


def _plain(params, inputs):
    mu, lp, lb, s2, gk = inputs.T
    p, b = np.exp(lp), np.exp(lb)
    d, dd, _, _ = sr.qlt_targets(mu, p, b, s2, gk, p0=params["p0"],
                                 particle_v0=params["particle_v0"],
                                 qlt_omega0=params["qlt_omega0"], qlt_lc=params["qlt_lc"],
                                 qlt_h0=params["qlt_h0"])
    k = sr.kappa_parallel(p, b, p0=params["p0"], kpara0=params["kpara0"],
                          gamma_turb=params["gamma_turb"])
    return d, dd, np.log(k)


@pytest.mark.parametrize("hidden", [32, 64])
def test_gradient_matches_cpu_reference(ctx, hidden):
    rng = np.random.default_rng(21)
    o = sr.layout(hidden)
    params = rng.normal(0.0, 0.3, o["N_PARAMS"]).astype(np.float32)
    x = rng.uniform(-1.0, 1.0, (1024, 5)).astype(np.float32)
    t = rng.normal(0.0, 1.0, (1024, 3)).astype(np.float32)
    loss, grad = ctx.surrogate_gradient(params, x, t, hidden)
    ref_loss, ref_grad = sr.loss_and_gradient(params.astype(np.float64), x.astype(np.float64),
                                              t.astype(np.float64))
    assert loss == pytest.approx(ref_loss, rel=1e-5)
    scale = np.abs(ref_grad).max()
    assert np.abs(grad - ref_grad).max() <= 1e-5 * scale
    # every block of the parameter vector, relative to its own scale
    for lo, hi in ((o["W1"], o["B1"]), (o["B1"], o["W2"]), (o["W2"], o["B2"]),
                   (o["B2"], o["W3"]), (o["W3"], o["B3"]), (o["B3"], o["N_PARAMS"])):
        block = np.abs(ref_grad[lo:hi]).max()
        assert np.abs(grad[lo:hi] - ref_grad[lo:hi]).max() <= 1e-4 * block, (lo, hi)


def _errors(params, inputs, out):
    d, dd, lk = _plain(params, inputs)
    return (np.abs(out[:, 0] - d) / d, np.abs(out[:, 2] - lk),
            np.abs(out[:, 1] - dd) / np.maximum(np.abs(dd), d))


@pytest.mark.parametrize("width", [32, 64])
def test_trained_network_forward_and_accuracy(trained, trained16, trained64, width):
    params, _, surrogate = trained if width == 32 else trained64
    assert surrogate.hidden_width == width
    assert surrogate.final_loss < 1e-3
    weights, norm = surrogate.parameters()
    rng = np.random.default_rng(5)
    inputs = _box_inputs(rng, 20000, norm)
    fp32, served32 = surrogate.evaluate(inputs, tensor_cores=False)
    bf16, served16 = surrogate.evaluate(inputs, tensor_cores=True)
    assert served32.all() and served16.all()
    # FP32 SIMT forward == CPU reference forward of the same parameters
    ref = sr.evaluate(weights, norm, inputs, p0=params["p0"], qlt_h0=params["qlt_h0"],
                      particle_v0=params["particle_v0"], qlt_omega0=params["qlt_omega0"],
                      qlt_lc=params["qlt_lc"], kpara0=params["kpara0"],
                      gamma_turb=params["gamma_turb"])
    assert np.allclose(fp32[:, 0], ref[:, 0], rtol=2e-4)
    assert np.allclose(fp32[:, 1], ref[:, 1], rtol=2e-3, atol=2e-4 * np.abs(ref[:, 1]).max())
    assert np.allclose(fp32[:, 2], ref[:, 2], rtol=0, atol=2e-4 * np.abs(ref[:, 2]).max())
    # accuracy against the plain closure: FP32 network, BF16 and FP16 tensor-core paths
    _, _, surrogate16 = trained16
    fp16, _ = surrogate16.evaluate(inputs, tensor_cores=True)
    fp16_simt, _ = surrogate16.evaluate(inputs, tensor_cores=False)
    p99 = {}
    for name, out in (("fp32", fp32), ("bf16", bf16), ("fp16", fp16), ("fp16-net fp32", fp16_simt)):
        err_d, err_k, err_dd = _errors(params, inputs, out)
        p99[name] = np.quantile(err_d, 0.99)
        print(f"{name}: D rel err median {np.median(err_d):.2e} p99 {p99[name]:.2e}"
              f" max {err_d.max():.2e}; ln kappa abs err p99 {np.quantile(err_k, 0.99):.2e};"
              f" dD/dmu p99 {np.quantile(err_dd, 0.99):.2e}")
        assert np.median(err_d) < 0.03, name
        assert p99[name] < 0.12, name
        assert np.quantile(err_k, 0.99) < 0.08, name
        assert np.quantile(err_dd, 0.99) < 0.15, name
    # FP16 serving adds little to the network's own error; BF16 adds more
    assert p99["fp16"] < p99["fp16-net fp32"] + 0.01


@pytest.mark.parametrize("net", ["trained", "trained16", "trained64", "trained64fp16"])
def test_engines_agree(kpt, net, request):
    params, _, surrogate = request.getfixturevalue(net)
    _, norm = surrogate.parameters()
    rng = np.random.default_rng(17)
    inputs = _box_inputs(rng, 20000, norm)  # 156 blocks of 128 and a ragged one
    inputs[:50, 0] *= 1e-3  # some below mu_cut: the plain closure
    outs = {}
    default_engine = surrogate.engine
    try:
        for engine in (kpt.ENGINE_TCGEN05, kpt.ENGINE_MMA_SYNC):
            surrogate.engine = engine
            outs[engine] = surrogate.evaluate(inputs)
    finally:
        surrogate.engine = default_engine
    with pytest.raises(kpt.KptError, match="unknown engine"):
        surrogate.engine = 7
    (tc, served_tc), (warp, served_warp) = outs[kpt.ENGINE_TCGEN05], outs[kpt.ENGINE_MMA_SYNC]
    assert np.array_equal(served_tc, served_warp)
    assert not served_tc[:50].any() and served_tc[50:].all()
    np.testing.assert_array_equal(tc[:50], warp[:50])
    for c in range(3):
        scale = np.abs(warp[:, c]) if c == 0 else np.abs(warp[:, c]).max()
        rel = np.abs(tc[:, c] - warp[:, c]) / scale
        assert np.median(rel) <= 2e-5, (c, np.median(rel))
        assert rel.max() <= 3e-2, (c, rel.max())
    p99 = [np.quantile(_errors(params, inputs[50:], out[50:])[0], 0.99) for out in (tc, warp)]
    assert p99[0] <= p99[1] + 0.005, p99


def test_fallback_outside_the_box_is_the_plain_closure(trained):
    params, _, surrogate = trained
    _, norm = surrogate.parameters()
    rng = np.random.default_rng(8)
    inside = _box_inputs(rng, 64, norm)
    small_mu = inside.copy()
    small_mu[:, 0] = rng.uniform(-0.5, 0.5, 64) * norm["mu_cut"]
    small_mu[small_mu[:, 0] == 0.0, 0] = 1e-3 * norm["mu_cut"]
    big_p = inside.copy()
    big_p[:, 1] = norm["in_hi"][1] + 1.0
    for case in (small_mu, big_p):
        out, served = surrogate.evaluate(case)
        assert not served.any()
        d, dd, lk = _plain(params, case)
        assert np.allclose(out[:, 0], d, rtol=1e-12)
        assert np.allclose(out[:, 1], dd, rtol=1e-9, atol=1e-12 * np.abs(d).max())
        assert np.allclose(out[:, 2], lk, rtol=0, atol=1e-12)


@pytest.mark.parametrize("engine", ["tcgen05", "mma_sync"])
@pytest.mark.parametrize("net", ["trained", "trained16", "trained64", "trained64fp16"])
def test_surrogate_push_matches_fp64_spectrum(ctx, kpt, oracle, binding, fields_mod, net, engine,
                                              request):
    params, settings, surrogate = request.getfixturevalue(net)
    default_engine = surrogate.engine
    surrogate.engine = kpt.ENGINE_TCGEN05 if engine == "tcgen05" else kpt.ENGINE_MMA_SYNC
    ye = fields_mod.stretched_edges(128, -2.0, 2.0)
    f0 = fields_mod.harris_field(64, 128, y_edges=ye, island_amplitude=0.1, noise=0.01, seed=5)
    f1 = fields_mod.harris_field(64, 128, y_edges=ye, island_amplitude=0.1, noise=0.01, seed=6)
    n, frame, seed = 6000, 7, 99
    plain = dict(params, closure=1)
    grid = oracle.grid(f0.x_edges, f0.y_edges)
    start = binding.empty_particles(n)
    count = oracle.inject(grid, plain, frame * 0.1, frame, seed, n, 0, n, start)
    ref = {k: v.copy() for k, v in start.items()}
    ref_steps = oracle.push(grid, oracle.table(f0, True), oracle.table(f1, True), plain,
                            frame * 0.1, frame, seed, count, ref)
    oracle.free_grid(grid)
    lower = ctx.field(f0, kpt.TABLE_FOCUSED21, kpt.PRECISION_MIXED)
    upper = ctx.field(f1, kpt.TABLE_FOCUSED21, kpt.PRECISION_MIXED)
    parts = ctx.particles(n)
    parts.upload(start, count)
    with pytest.raises(kpt.KptError, match="set_surrogate"):
        ctx.set_surrogate(None)
        ctx.push_interval(parts, lower, upper, settings, frame, seed)
    ctx.set_surrogate(surrogate)
    ctx.surrogate_judge()
    stats = ctx.push_interval(parts, lower, upper, settings, frame, seed)
    judge = ctx.surrogate_judge()
    got = parts.download()
    assert stats.failed == 0
    h_ref = _spectrum(ref["p"], ref["w"], ref["status"])
    h = _spectrum(got["p"], got["w"], got["status"])
    l1 = np.abs(h - h_ref).sum() / h_ref.sum()
    print(f"surrogate push: L1 {l1:.4f}, judge {judge}")
    assert l1 <= 0.01
    assert _chi2_same(h, h_ref) > 0.01
    mu_ref = np.histogram(ref["mu"][ref["status"] == 0], bins=16, range=(-1, 1))[0]
    mu_got = np.histogram(got["mu"][got["status"] == 0], bins=16, range=(-1, 1))[0]
    assert _chi2_same(mu_got.astype(float), mu_ref.astype(float)) > 0.01
    assert judge["evaluations"] + judge["fallbacks"] == stats.particle_steps
    # the network hands over to the plain closure continuously at mu_cut, so
    # particles do not pile up near mu = 0 (where the pitch-angle limiters
    # make the steps tiny): the substep count stays that of the plain closure
    assert abs(stats.particle_steps / ref_steps.sum() - 1.0) < 0.05
    assert stats.max_steps < settings.max_steps
    assert judge["evaluations"] > 0.9 * stats.particle_steps
    assert judge["judged"] > 0 and judge["max_rel_error"] < 0.2
    # the network is trained for one set of physics constants
    other = kpt.settings_from_dict(dict(params, kpara0=params["kpara0"] * 2))
    with pytest.raises(kpt.KptError, match="trained"):
        ctx.push_interval(parts, lower, upper, other, frame, seed)
    surrogate.engine = default_engine
    for f in (lower, upper):
        f.close()
    parts.close()


@pytest.mark.parametrize("net", ["trained64", "trained"])
def test_tcgen05_push_does_not_depend_on_the_schedule(ctx, kpt, fields_mod, net, request):
    """Each particle's row of the block-collective GEMMs is computed alone
    (no row sees another), and the noise is keyed by particle: the same
    population pushed unsorted, cell-sorted, and with 1 or 2 blocks per SM
    (other rows beside every particle, other lockstep partners) ends bit for
    bit the same."""
    _, settings, surrogate = request.getfixturevalue(net)
    default_engine = surrogate.engine
    assert default_engine == (kpt.ENGINE_TCGEN05 if net == "trained64" else kpt.ENGINE_MMA_SYNC)
    surrogate.engine = kpt.ENGINE_TCGEN05
    ye = fields_mod.stretched_edges(128, -2.0, 2.0)
    f0 = fields_mod.harris_field(64, 128, y_edges=ye, island_amplitude=0.1, noise=0.01, seed=5)
    f1 = fields_mod.harris_field(64, 128, y_edges=ye, island_amplitude=0.1, noise=0.01, seed=6)
    lower = ctx.field(f0, kpt.TABLE_FOCUSED21, kpt.PRECISION_MIXED)
    upper = ctx.field(f1, kpt.TABLE_FOCUSED21, kpt.PRECISION_MIXED)
    ctx.set_surrogate(surrogate)
    n = 5000
    parts = ctx.particles(n)
    ctx.inject(parts, lower, settings, n, 7, 99)
    start = parts.download(n)
    results = []
    try:
        for sort, blocks in ((False, 0), (True, 0), (True, 1), (False, 2)):
            ctx.set_push_schedule(kpt.SCHEDULE_REFILL, blocks)
            parts.upload(start, n)
            if sort:
                ctx.sort(parts, lower, 8, 8)
            stats = ctx.push_interval(parts, lower, upper, settings, 7, 99)
            results.append((parts.download(n), stats.particle_steps))
    finally:
        ctx.set_push_schedule(kpt.SCHEDULE_REFILL, 0)
        surrogate.engine = default_engine
    base, steps = results[0]
    assert steps > 0
    for other, other_steps in results[1:]:
        assert other_steps == steps
        for name in base:
            assert np.array_equal(base[name], other[name]), name
    for f in (lower, upper):
        f.close()
    parts.close()


def test_tcgen05_completion_wait_is_bounded(trained64, kpt):
    """A completion that never comes (no MMA issued): every block gives up
    after its bounded wait, reports it, frees its tensor memory and returns;
    the engine then serves the network as before."""
    params, _, surrogate = trained64
    timed_out, finished = surrogate.check_timeout(blocks=8, polls=64)
    assert (timed_out, finished) == (8, 8)
    _, norm = surrogate.parameters()
    inputs = _box_inputs(np.random.default_rng(2), 1000, norm)
    out, served = surrogate.evaluate(inputs)
    assert served.all() and np.isfinite(out).all()
    with pytest.raises(kpt.KptError, match="polls"):
        surrogate.check_timeout(blocks=1, polls=0)
