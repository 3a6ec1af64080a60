"""Radiance cache: the GPU forward/backward kernels against the CPU
restatement (oracle/cache_ref.py), the restatement against finite
differences, training, and the cache inside the renderer."""
import importlib
import math

import numpy as np
import pytest

from oracle import cache_ref as cr

LO, HI = (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)


def batch(n, seed):
    rng = np.random.default_rng(seed)
    rec = np.zeros((n, 16), np.float32)
    rec[:, 0:3] = rng.uniform(-1, 1, (n, 3))
    d = rng.normal(size=(n, 3))
    rec[:, 3:6] = d / np.linalg.norm(d, axis=1, keepdims=True)
    nn = rng.normal(size=(n, 3))
    rec[:, 6:9] = nn / np.linalg.norm(nn, axis=1, keepdims=True)
    rec[:, 9:12] = rng.uniform(0, 1, (n, 3))
    rec[:, 12:15] = rng.uniform(0, 1, (n, 3))
    p = rec[:, 0:3]
    tgt = np.stack([1.0 + np.sin(3 * p[:, 0]) * np.cos(2 * p[:, 1]),
                    0.5 + 0.5 * p[:, 2] ** 2,
                    np.exp(-np.sum(p * p, axis=1))], axis=1).astype(np.float32)
    tgt *= 0.5 + rec[:, 9:12]
    return rec, tgt


def random_params(seed, log2_table):
    rng = np.random.default_rng(seed)
    mlp = np.zeros(cr.n_params(), np.float32)
    for l in range(cr.LAYERS):
        k, n = cr.layer_shape(l)
        lim = math.sqrt(6.0 / (k + n))
        mlp[cr.layer_off(l):cr.layer_off(l) + k * n] = rng.uniform(-lim, lim, k * n)
    grid = rng.uniform(-0.5, 0.5, cr.LEVELS * (1 << log2_table) * 2).astype(np.float32)
    return mlp, grid


def test_restatement_backward_matches_finite_differences():
    log2 = 10
    res = cr.resolutions()
    rec, tgt = batch(64, 1)
    mlp, grid = random_params(2, log2)
    grid = grid.astype(np.float16).astype(np.float32)  # the table holds fp16 values
    loss, gm, gg, pred = cr.loss_and_grads(rec, tgt, mlp, grid, LO, HI, res, log2, exact=True)
    den = pred * pred + 0.01  # the loss treats its denominator as a constant

    def loss_at(m, g):
        x = cr.encode(rec, g, LO, HI, res, log2, exact=True)
        p, _ = cr.forward(x, m, exact=True)
        return float(((p[:, :3] - tgt) ** 2 / den).sum() / len(rec))

    rng = np.random.default_rng(3)
    eps = 1e-4
    for i in rng.choice(cr.n_params(), 24, replace=False):
        m1, m2 = mlp.astype(np.float64).copy(), mlp.astype(np.float64).copy()
        m1[i] += eps
        m2[i] -= eps
        fd = (loss_at(m1, grid) - loss_at(m2, grid)) / (2 * eps)
        assert abs(fd - gm[i]) <= 1e-4 + 2e-3 * abs(fd), (i, fd, gm[i])
    touched = np.flatnonzero(gg)
    for i in rng.choice(touched, 24, replace=False):
        g1, g2 = grid.astype(np.float64).copy(), grid.astype(np.float64).copy()
        g1[i] += eps
        g2[i] -= eps
        fd = (loss_at(mlp, g1) - loss_at(mlp, g2)) / (2 * eps)
        assert abs(fd - gg[i]) <= 1e-4 + 2e-3 * abs(fd), (i, fd, gg[i])


@pytest.fixture(scope="module")
def cache_mod(pt, gpu_lib):
    return importlib.import_module("hala-pathtracer_gb300.cache")


def gpu_cache(cache_mod, log2, seed):
    c = cache_mod.RadianceCache(log2_table_size=log2, seed=seed, batch_size=4096)
    c.set_bounds(LO, HI)
    mlp, grid = random_params(seed, log2)
    c.set_params(mlp, grid)
    return c, mlp, grid.astype(np.float16).astype(np.float32)


@pytest.mark.gpu
def test_gpu_forward_matches_cpu(cache_mod):
    log2 = 14
    c, mlp, grid = gpu_cache(cache_mod, log2, 5)
    rec, _ = batch(1000, 6)  # not a multiple of 16: ragged last tile
    got = c.infer(rec)
    x = cr.encode(rec, grid, LO, HI, cr.resolutions(), log2)
    want = cr.forward(x, mlp)[0][:, :3]
    scale = np.abs(want).max()
    assert np.abs(got - want).max() <= 2e-2 * scale, np.abs(got - want).max() / scale


@pytest.mark.gpu
@pytest.mark.parametrize("n", [16, 777, 5000])
def test_gpu_gradients_match_cpu(cache_mod, n):
    log2 = 14
    c, mlp, grid = gpu_cache(cache_mod, log2, 7)
    rec, tgt = batch(n, 8)
    gm, gg, loss = c.gradients(rec, tgt)
    loss_c, gm_c, gg_c, _ = cr.loss_and_grads(rec, tgt, mlp, grid, LO, HI, cr.resolutions(), log2)
    assert abs(loss - loss_c) <= 1e-2 * abs(loss_c) + 1e-6
    for l in range(cr.LAYERS):
        k, m = cr.layer_shape(l)
        a = gm[cr.layer_off(l):cr.layer_off(l) + k * m]
        b = gm_c[cr.layer_off(l):cr.layer_off(l) + k * m]
        err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        assert err < 2e-2, (l, err)
    err = np.linalg.norm(gg - gg_c) / max(np.linalg.norm(gg_c), 1e-30)
    assert err < 2e-2, err
    # no gradient lands where the CPU has none
    assert np.all(gg[gg_c == 0] == 0)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [64, 1000, 70000])
def test_tensor_core_weight_gradients_match_the_warp_kernel(cache_mod, n):
    """The weight gradients of the tcgen05 kernel (TMEM accumulators) equal
    those of the warp-level mma.sync kernel up to fp32 summation order, for
    ragged batches (n not a multiple of the 64-row chunk) and batches over
    several 1024-row blocks."""
    log2 = 14
    out = []
    for kernel in (0, 1):
        c = cache_mod.RadianceCache(log2_table_size=log2, seed=5, weight_grad_kernel=kernel)
        c.set_bounds(LO, HI)
        mlp, grid = random_params(9, log2)
        c.set_params(mlp, grid)
        rec, tgt = batch(n, 10)
        out.append(c.gradients(rec, tgt))
        c.close()
    (ga, gga, la), (gb, ggb, lb) = out
    # loss and table gradient: the same kernel, float atomics in any order
    assert abs(la - lb) <= 1e-5 * abs(lb)
    assert np.linalg.norm(gga - ggb) <= 1e-5 * np.linalg.norm(ggb)
    for l in range(cr.LAYERS):
        k, m = cr.layer_shape(l)
        a = ga[cr.layer_off(l):cr.layer_off(l) + k * m]
        b = gb[cr.layer_off(l):cr.layer_off(l) + k * m]
        err = np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)
        assert err < 1e-4, (l, err)
        assert np.count_nonzero(b) == 0 or np.count_nonzero(a) > 0


@pytest.mark.gpu
def test_gpu_training_fits_a_smooth_field(cache_mod):
    c = cache_mod.RadianceCache(log2_table_size=16, seed=11, batch_size=4096)
    c.set_bounds(LO, HI)
    rec, tgt = batch(16384, 12)
    test_rec, test_tgt = batch(2048, 13)

    def held_out_error():
        pred = c.infer(test_rec)
        return np.abs(pred - test_tgt).mean() / np.abs(test_tgt).mean()

    before = held_out_error()
    first = c.train(rec, tgt, steps=1)
    last = c.train(rec, tgt, steps=60)
    assert last < 0.2 * first, (first, last)
    # the fit generalises to positions it has not seen (the finest hash
    # levels memorise, the coarse ones and the MLP interpolate)
    after = held_out_error()
    assert after < 0.35 and after < 0.4 * before, (before, after)


@pytest.mark.gpu
def test_renderer_with_cache(pt, scenes):
    sc = scenes.cornell(64, 64, 8, max_depth=8, rr_depth=0, seed=1)
    r = pt.renderer_for(sc)
    r.set_radiance_cache(query_depth=1, train_shift=4, warmup_frames=2, batch_size=4096)
    r.render(8)
    st = r.stats()
    assert st.cache_queries > 0 and st.cache_train_samples > 0 and st.cache_train_steps > 0
    img = r.image(0)[..., :3]
    assert np.all(np.isfinite(img))
    plain = pt.renderer_for(sc)
    plain.render(8)
    ref = plain.image(0)[..., :3]
    assert abs(img.mean() - ref.mean()) < 0.25 * ref.mean()
    # detaching restores the unbiased tracer bit for bit
    r.set_radiance_cache(False)
    r.reset()
    r.render(8)
    assert np.array_equal(r.image(0), plain.image(0))


@pytest.mark.gpu
def test_cache_skips_glossy_and_glass_vertices(pt, scenes):
    """The cache vertex is used only where the surface is diffuse, or Disney
    without a glass lobe and at least min_roughness rough. On the Disney grid
    with min_roughness above every material's roughness no vertex qualifies:
    nothing is queried or trained, and the image is the plain tracer's bit
    for bit; with the default some vertices qualify."""
    sc = scenes.tiny_variants()["disney"]
    plain = pt.renderer_for(sc)
    plain.render(sc.spp)
    r = pt.renderer_for(sc)
    r.set_radiance_cache(min_roughness=2.0, warmup_frames=1)
    r.render(sc.spp)
    st = r.stats()
    assert st.cache_queries == 0 and st.cache_train_samples == 0
    for k in range(4):
        assert np.array_equal(r.image(k).view(np.uint8), plain.image(k).view(np.uint8)), f"image {k} differs"
    r2 = pt.renderer_for(sc)
    r2.set_radiance_cache(warmup_frames=0)
    r2.render(sc.spp)
    assert r2.stats().cache_queries > 0


@pytest.mark.gpu
def test_cache_rmse_against_the_fp64_oracle(pt, scenes):
    """What the trained cache changes against the plain tracer on the
    Cornell box, judged against the 4096-spp FP64 oracle image: paths end
    at the first bounce (far fewer rays per path) while the error at equal
    samples per pixel stays close to the unbiased tracer's."""
    import os
    import bench
    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", "cornell128_4096spp_fp64.npz"))
    ref = ref["radiance"].astype(np.float64)
    s = scenes.cornell(128, 128, 256, max_depth=8, rr_depth=0, seed=1)
    chunks = [1, 1, 2, 4, 8, 16, 32, 64, 127]
    plain = bench.cache_curves(pt, s, ref, chunks)
    cached = bench.cache_curves(pt, s, ref, chunks, {"steps_per_pass": 4})
    assert cached[-1][3] < 0.6 * plain[-1][3], (plain[-1], cached[-1])
    assert cached[-1][2] < 1.25 * plain[-1][2], (plain[-1], cached[-1])
    # the error keeps falling with more samples (no divergence)
    assert cached[-1][2] < 0.5 * cached[3][2]


@pytest.mark.gpu
def test_cache_benchmark_runs(cache_mod):
    c = cache_mod.RadianceCache(batch_size=4096)
    infer_ms, train_ms = c.benchmark(1 << 14, 2)
    assert infer_ms > 0 and train_ms > 0
