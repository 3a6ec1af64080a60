"""CPU tests of the oracle: portable math accuracy, RNG and tonemap known
answers restated independently in numpy, BSDF and environment-sampling
consistency, BVH vs brute force. No GPU."""
import ctypes as C
import math

import numpy as np
import pytest


def _ulp_err(got, ref):
    ref = np.asarray(ref, np.float64)
    ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    ulp = np.maximum(ulp, np.float64(np.spacing(np.float32(1.17549435e-38))))
    return np.abs(got.astype(np.float64) - ref) / ulp


@pytest.mark.parametrize("fn,lo,hi,bound", [
    (0, -7.0, 7.0, 2.0), (1, -7.0, 7.0, 2.0), (2, -1.5, 1.5, 3.0), (3, -87.0, 88.0, 1.5),
    (6, -1.0, 1.0, 1.5)])
def test_pmath_unary_accuracy(oracle_mod, fn, lo, hi, bound):
    x = np.random.default_rng(fn).uniform(lo, hi, 50000).astype(np.float32)
    ref = [np.sin, np.cos, np.tan, np.exp, None, None, np.arccos][fn](x.astype(np.float64))
    assert _ulp_err(oracle_mod.pmath(fn, x), ref).max() <= bound


def test_pmath_log_atan2_pow_accuracy(oracle_mod):
    rng = np.random.default_rng(7)
    x = np.exp(rng.uniform(-80, 80, 50000)).astype(np.float32)
    assert _ulp_err(oracle_mod.pmath(4, x), np.log(x.astype(np.float64))).max() <= 1.5
    y, z = rng.normal(size=50000).astype(np.float32), rng.normal(size=50000).astype(np.float32)
    assert _ulp_err(oracle_mod.pmath(7, y, z), np.arctan2(y.astype(np.float64), z.astype(np.float64))).max() <= 3.0
    b = rng.uniform(0, 4, 50000).astype(np.float32)
    e = rng.uniform(-5, 5, 50000).astype(np.float32)
    ref = np.power(b.astype(np.float64), e.astype(np.float64))
    got = oracle_mod.pmath(5, b, e).astype(np.float64)
    ok = np.isfinite(ref) & (ref > 1e-30)
    assert (np.abs(got[ok] - ref[ok]) / ref[ok]).max() < 5e-6


def test_pmath_special_values(oracle_mod):
    f = oracle_mod.pmath
    assert f(3, np.array([-200.0, 200.0], np.float32)).tolist() == [0.0, float("inf")]
    assert f(4, np.array([0.0], np.float32))[0] == -np.inf
    assert np.isnan(f(4, np.array([-1.0], np.float32))[0])
    p = f(5, np.array([0.0, 2.0, 7.0], np.float32), np.array([5.0, 0.0, 1.0], np.float32))
    assert p[0] == 0.0 and p[1] == 1.0 and abs(p[2] - 7.0) <= 7.0 * 2.0 ** -22
    assert np.isnan(f(6, np.array([1.5], np.float32))[0])
    assert f(7, np.array([0.0], np.float32), np.array([0.0], np.float32))[0] == 0.0


def _pcg4d(v):
    """Independent numpy restatement of wltcRS.glsl:22-28 (uint32 arithmetic)."""
    v = np.array(v, np.uint32)
    with np.errstate(over="ignore"):
        v = v * np.uint32(1664525) + np.uint32(1013904223)
        v[0] += v[1] * v[3]; v[1] += v[2] * v[0]; v[2] += v[0] * v[1]; v[3] += v[1] * v[2]
        v ^= v >> np.uint32(16)
        v[0] += v[1] * v[3]; v[1] += v[2] * v[0]; v[2] += v[0] * v[1]; v[3] += v[1] * v[2]
    return v


def test_pcg4d_and_rand_sequence(oracle_mod):
    lib = oracle_mod.lib()
    rng = np.random.default_rng(3)
    for _ in range(200):
        v = rng.integers(0, 2**32, 4, dtype=np.uint64).astype(np.uint32)
        a = (C.c_uint32 * 4)(*v.tolist())
        lib.or_pcg4d(a)
        assert list(a) == _pcg4d(v).tolist()
    # rand(): rng_initialize(pixel, frame) then s0.x / 2^32 (wltcRS.glsl:9-32)
    px, py, fr = 17, 5, 9
    out = (C.c_float * 6)()
    lib.or_rand_seq(px, py, fr, 6, out)
    s = np.array([px, py, fr, px + py], np.uint32)
    for k in range(6):
        s = _pcg4d(s)
        assert out[k] == np.float32(np.float32(s[0]) * np.float32(2.0 ** -32))
        assert 0.0 <= out[k] <= 1.0


def test_blue_noise_substitute_is_rgba8(oracle_mod):
    lib = oracle_mod.lib()
    out = (C.c_float * 4)()
    for x, y in [(0, 0), (1023, 1023), (17, 900)]:
        lib.or_blue_noise(x, y, out)
        v = _pcg4d([x, y, 0x2545F491, 0x9E3779B9])
        assert list(out) == [np.float32(float(c >> 24)) / np.float32(255.0) for c in v]


def _tonemap_np(c, ev, enable, aces, simple):
    """numpy restatement of pathtracer.rgen.glsl:280-301 and common/tonemap.glsl."""
    c = np.asarray(c, np.float64) * 2.0 ** ev
    lum = lambda v: 0.212671 * v[0] + 0.715160 * v[1] + 0.072169 * v[2]
    if enable:
        if aces and simple:
            c = np.clip((c * (2.51 * c + 0.03)) / (c * (2.43 * c + 0.59) + 0.14), 0, 1)
        elif aces:
            i = np.array([[0.59719, 0.35458, 0.04823], [0.07600, 0.90834, 0.01566], [0.02840, 0.13383, 0.83777]])
            o = np.array([[1.60475, -0.53108, -0.07367], [-0.10208, 1.10813, -0.00605], [-0.00327, -0.07276, 1.07602]])
            c = i @ c
            c = (c * (c + 0.0245786) - 0.000090537) / (c * (0.983729 * c + 0.4329510) + 0.238081)
            c = np.clip(o @ c, 0, 1)
        else:
            c = c / (1.0 + lum(c) / 1.5)
    return np.where(c <= 0.0031308, 12.92 * c, 1.055 * np.power(np.maximum(c, 0), 1 / 2.4) - 0.055)


@pytest.mark.parametrize("mode", [(1, 1, 0), (1, 1, 1), (1, 0, 0), (0, 0, 0)])
def test_tonemap_matches_restatement(oracle_mod, mode):
    lib = oracle_mod.lib()
    rng = np.random.default_rng(5)
    for _ in range(50):
        c = rng.uniform(0, 4, 3).astype(np.float32)
        ev = float(rng.uniform(-2, 2))
        out = (C.c_float * 3)()
        lib.or_tonemap((C.c_float * 3)(*c), ev, *mode, out)
        assert np.allclose(list(out), _tonemap_np(c, ev, *mode), rtol=2e-5, atol=2e-6)


def _tbn():
    return (C.c_float * 9)(1, 0, 0, 0, 1, 0, 0, 0, 1)


@pytest.mark.parametrize("kind,rough,metal,trans", [(0, 0.0, 0, 0), (0, 0.4, 0, 0), (1, 0.3, 0.0, 0.0),
                                                    (1, 0.6, 1.0, 0.0), (1, 0.2, 0.0, 1.0)])
def test_bsdf_sample_consistent_with_eval(oracle_mod, scenes, kind, rough, metal, trans):
    """disney_sample / diffuse sample return the eval of the sampled direction."""
    lib = oracle_mod.lib()
    m = scenes.material((0.7, 0.5, 0.3), mtype=kind, roughness=rough, metallic=metal,
                        specular_transmission=trans)
    rng = np.random.default_rng(11)
    N = (C.c_float * 3)(0, 0, 1)
    for _ in range(200):
        v = rng.normal(size=3)
        v[2] = abs(v[2]) + 0.05
        v /= np.linalg.norm(v)
        V = (C.c_float * 3)(*v)
        s0 = (C.c_uint32 * 4)(*rng.integers(0, 2**32, 4, dtype=np.uint64).astype(np.uint32).tolist())
        f, L, pdf, fl = (C.c_float * 3)(), (C.c_float * 3)(), C.c_float(), C.c_uint32()
        lib.or_bsdf_sample(kind, C.byref(m), _tbn(), 1.0 / 1.5, 0, 0, V, N, s0, f, L, C.byref(pdf), C.byref(fl))
        fe, pe = (C.c_float * 3)(), C.c_float()
        lib.or_bsdf_eval(kind, C.byref(m), _tbn(), 1.0 / 1.5, 0, 1, V, N, L, fe, C.byref(pe))
        assert list(fe) == list(f) and pe.value == pdf.value


def test_lambert_white_furnace(oracle_mod, scenes):
    """E[f cos / pdf] of Lambert sampling equals the albedo (inc/bxdf/lambert.glsl)."""
    lib = oracle_mod.lib()
    m = scenes.material((0.8, 0.6, 0.4))
    V, N = (C.c_float * 3)(0.3, 0.2, 0.93), (C.c_float * 3)(0, 0, 1)
    acc = np.zeros(3)
    n = 4000
    for k in range(n):
        s0 = (C.c_uint32 * 4)(k, 7, 11, k * 3)
        f, L, pdf, fl = (C.c_float * 3)(), (C.c_float * 3)(), C.c_float(), C.c_uint32()
        lib.or_bsdf_sample(0, C.byref(m), _tbn(), 1.0, 0, 0, V, N, s0, f, L, C.byref(pdf), C.byref(fl))
        acc += np.array(list(f)) / pdf.value
    assert np.allclose(acc / n, [0.8, 0.6, 0.4], rtol=1e-5)


def test_oracle_bvh_matches_brute_force(oracle_mod, scenes):
    sc = scenes.tiny_variants()["icosphere"]
    o = oracle_mod.Oracle(sc)
    rng = np.random.default_rng(2)
    pts = np.concatenate([m[0][:, :3] for m in sc.meshes])
    rays = np.zeros((3000, 8), np.float32)
    rays[:, :3] = rng.uniform(pts.min(0), pts.max(0), (3000, 3))
    d = rng.normal(size=(3000, 3))
    rays[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays[:, 7] = 1e4
    assert np.array_equal(o.trace_rays(rays), o.trace_rays(rays, brute_force=True))
    rays[:, 7] = rng.uniform(0.05, 2.0, 3000)
    assert np.array_equal(o.trace_rays(rays, any_hit=True)[:, 3], o.trace_rays(rays, any_hit=True, brute_force=True)[:, 3])


def test_env_sampling_matches_luminance_distribution(oracle_mod, scenes):
    """With the environment as the only light, the alias-table sampler's pdf
    integrates the per-texel luminance distribution (inc/env_map.glsl:6-37):
    a converged render of a white diffuse plane agrees between two seeds."""
    sc = scenes.Scene("env_plane")
    w = sc.add_material(scenes.material((0.9, 0.9, 0.9)))
    sc.add_mesh(*scenes.quad_mesh((-5, -5, 0), (10, 0, 0), (0, 10, 0)), w)
    sc.cameras.append(scenes.look_at((0, -3, 2), (0, 0, 0), 40.0))
    sc.env_rgb = scenes.synthetic_sky(64, 32, sun_peak=50.0, sun_sigma_deg=8.0)
    sc.width, sc.height, sc.max_depth, sc.rr_depth = 16, 16, 2, 0
    a = oracle_mod.Oracle(sc, seed=0)
    a.render(256)
    b = oracle_mod.Oracle(sc, seed=1000)
    b.render(256)
    ia, ib = a.image(0)[..., :3].mean(), b.image(0)[..., :3].mean()
    assert abs(ia - ib) / ia < 0.03
