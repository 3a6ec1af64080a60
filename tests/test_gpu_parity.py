"""CUDA path vs the CPU oracle (needs a GPU).

Parity bar: BVH closest-hit ids/t/u/v bit-exact against brute force (device
and oracle); per-path radiance within 1e-4 relative wherever the
hit-sequence hash agrees (same per-pixel RNG stream on both sides). Because
the shading code rounds like the oracle (no contraction, portable
transcendentals), the tests also require every hash to agree and every
per-path radiance and accumulated pixel to be bit-identical.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-4      # per-path radiance, relative
ABS_FLOOR = 1e-6    # absolute floor for near-black paths
MIN_AGREE = 0.97    # fraction of paths whose hit sequence must agree


def _random_rays(scene_bounds, n, seed):
    rng = np.random.default_rng(seed)
    lo, hi = scene_bounds
    o = rng.uniform(lo, hi, size=(n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = o
    rays[:, 3] = 0.0
    rays[:, 4:7] = d
    rays[:, 7] = 1e4
    return rays


def _bounds(scene):
    pts = np.concatenate([m[0][:, :3] for m in scene.meshes])
    return pts.min(0), pts.max(0)


@pytest.mark.parametrize("name", ["cornell", "disney", "icosphere", "media"])
def test_bvh_closest_bitexact(pt, scenes, oracle_mod, name):
    sc = scenes.tiny_variants()[name]
    r = pt.renderer_for(sc)
    o = oracle_mod.Oracle(sc)
    rays = _random_rays(_bounds(sc), 4000, 11)
    hb = r.trace_rays(rays)
    hf = r.trace_rays(rays, brute_force=True)
    ho = o.trace_rays(rays, brute_force=True)
    tri = (hf[:, 3] & 0x80000000) == 0
    # triangles (and misses): bit-exact on t, u, v and id
    assert np.array_equal(hb[tri], hf[tri])
    assert np.array_equal(hf[tri], ho[tri])
    # analytic lights: same id; t within float rounding of the light test
    lt = ~tri & (hf[:, 3] != 0xFFFFFFFF)
    assert np.array_equal(hb[lt, 3], hf[lt, 3])
    assert np.array_equal(hf[lt, 3], ho[lt, 3])
    tf, to = hf[lt, 0].view(np.float32), ho[lt, 0].view(np.float32)
    assert np.allclose(tf, to, rtol=1e-5)


@pytest.mark.parametrize("name", ["cornell", "disney"])
def test_bvh_axis_aligned_rays(pt, scenes, oracle_mod, name):
    """Directions with exactly-zero components (orthographic cameras, walls)."""
    sc = scenes.tiny_variants()[name]
    r = pt.renderer_for(sc)
    o = oracle_mod.Oracle(sc)
    rng = np.random.default_rng(9)
    lo, hi = _bounds(sc)
    dirs = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                     [0, 0.6, -0.8], [0.6, 0, 0.8], [-0.8, 0.6, 0], [0, -0.6, 0.8]], np.float32)
    n = 3000
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform(lo, hi, size=(n, 3))
    rays[:, 4:7] = dirs[rng.integers(0, len(dirs), n)]
    rays[:, 7] = 1e4
    hb = r.trace_rays(rays)
    ho = o.trace_rays(rays, brute_force=True)
    tri = (ho[:, 3] & 0x80000000) == 0
    assert np.array_equal(hb[tri], ho[tri])
    assert np.array_equal(hb[:, 3], ho[:, 3])
    rays[:, 7] = rng.uniform(0.05, 2.0, n)
    assert np.array_equal(r.trace_rays(rays, any_hit=True)[:, 3], o.trace_rays(rays, any_hit=True)[:, 3])


@pytest.mark.parametrize("freq", [16, 72])
def test_bvh_large_scene_bitexact(pt, scenes, freq):
    """Scenes that take every build path: 5,122 triangles (one-block levels
    and whole subtrees) and 103,682 (also the multi-block top levels).
    Closest hits and any-hit answers equal brute force over all triangles."""
    sc = scenes.displaced_icosphere(64, 36, 1, freq=freq)
    sc.lights = []
    r = pt.renderer_for(sc)
    assert r.stats().triangles == 20 * freq * freq + 2
    rays = _random_rays(_bounds(sc), 4000, 13)
    assert np.array_equal(r.trace_rays(rays), r.trace_rays(rays, brute_force=True))
    rays[:, 7] = np.random.default_rng(4).uniform(0.01, 1.0, len(rays))
    a = r.trace_rays(rays, any_hit=True)
    b = r.trace_rays(rays, any_hit=True, brute_force=True)
    assert np.array_equal(a[:, 3], b[:, 3])


@pytest.mark.parametrize("build", [0, 1])
def test_bvh_degenerate_geometry(pt, scenes, build):
    """Inputs where no SAH plane separates the centroids, so every build tier
    falls back to median splits: 20,000 copies of one triangle (multi-block,
    one-block and whole-subtree tasks), 3,000 triangles in one plane, 600
    triangles sharing a centroid. Closest hits (equal distances resolved by
    the lower id) and any-hit answers equal brute force, with the default
    build and with the fast one (equal Morton codes ordered by index)."""
    sc = scenes.tiny_variants()["cornell"]
    sc.meshes = []
    sc.lights = []
    mat = sc.add_material(scenes.material())
    rng = np.random.default_rng(17)
    tri = np.array([[0.2, 0.2, 0.3], [0.8, 0.3, 0.4], [0.4, 0.9, 0.6]])
    z = np.zeros((3, 3))
    sc.add_mesh(scenes.pack_vertices(tri, z, z, np.zeros((3, 2))), np.tile(np.arange(3, dtype=np.uint32), 20000), mat)
    flat = rng.uniform(0, 1, size=(9000, 3))
    flat[:, 2] = 0.5
    n = np.zeros((9000, 3))
    sc.add_mesh(scenes.pack_vertices(flat, n, n, np.zeros((9000, 2))), np.arange(9000, dtype=np.uint32), mat)
    c = np.array([0.5, 0.5, 0.5])
    nested = np.concatenate([c + s * (tri - tri.mean(0)) for s in np.linspace(0.05, 1.5, 600)])
    n = np.zeros((1800, 3))
    sc.add_mesh(scenes.pack_vertices(nested, n, n, np.zeros((1800, 2))), np.arange(1800, dtype=np.uint32), mat)
    r = pt.renderer_for(sc, bvh_build=build)
    assert r.stats().triangles == 23600
    rays = _random_rays((np.zeros(3), np.ones(3)), 4000, 23)
    assert np.array_equal(r.trace_rays(rays), r.trace_rays(rays, brute_force=True))
    rays[:, 7] = rng.uniform(0.01, 1.0, len(rays))
    assert np.array_equal(r.trace_rays(rays, any_hit=True)[:, 3],
                          r.trace_rays(rays, any_hit=True, brute_force=True)[:, 3])


@pytest.mark.parametrize("name", ["cornell", "icosphere"])
def test_bvh_any_hit(pt, scenes, oracle_mod, name):
    sc = scenes.tiny_variants()[name]
    r = pt.renderer_for(sc)
    o = oracle_mod.Oracle(sc)
    rays = _random_rays(_bounds(sc), 4000, 5)
    rays[:, 7] = np.random.default_rng(3).uniform(0.01, 3.0, len(rays))
    a = r.trace_rays(rays, any_hit=True)
    b = r.trace_rays(rays, any_hit=True, brute_force=True)
    c = o.trace_rays(rays, any_hit=True, brute_force=True)
    assert np.array_equal(a[:, 3], b[:, 3])
    assert np.array_equal(b[:, 3], c[:, 3])


@pytest.mark.parametrize("name", ["cornell", "disney", "icosphere", "media"])
def test_per_path_radiance(pt, scenes, oracle_mod, name):
    sc = scenes.tiny_variants()[name]
    r = pt.renderer_for(sc, keep_samples=True)
    r.render(sc.spp)
    rad_g, hash_g = r.samples()
    o = oracle_mod.Oracle(sc)
    WH = sc.width * sc.height
    rad_o, hash_o = o.trace_paths(np.arange(WH), 0, sc.spp)
    rad_o = rad_o.reshape(-1, 3)
    hash_o = hash_o.reshape(-1)
    agree = hash_g == hash_o
    assert agree.mean() >= MIN_AGREE, f"hit sequences agree on {agree.mean():.4f} of paths"
    assert agree.all(), f"{(~agree).sum()} of {len(agree)} hit sequences differ"
    assert np.array_equal(rad_g.view(np.uint32), rad_o.view(np.uint32)), "per-path radiance not bit-identical"
    a, b = rad_g[agree].astype(np.float64), rad_o[agree].astype(np.float64)
    assert np.isfinite(a).all()
    err = np.abs(a - b)
    tol = REL_TOL * np.maximum(np.abs(a), np.abs(b)) + ABS_FLOOR
    bad = (err > tol).any(axis=1)
    idx = np.nonzero(agree)[0][bad][:5]
    detail = "; ".join(f"path {k}: gpu {rad_g[k]} oracle {rad_o[k]}" for k in idx)
    assert not bad.any(), f"{bad.sum()} agreeing paths differ; worst {err.max():.3g}; {detail}"


def test_accumulated_images(pt, scenes, oracle_mod):
    sc = scenes.tiny_variants()["cornell"]
    r = pt.renderer_for(sc, keep_samples=True)
    r.render(sc.spp)
    o = oracle_mod.Oracle(sc)
    o.render(sc.spp)
    _, hash_g = r.samples()
    WH = sc.width * sc.height
    _, hash_o = o.trace_paths(np.arange(WH), 0, sc.spp)
    same = (hash_g.reshape(sc.spp, WH) == hash_o.reshape(sc.spp, WH)).all(0).reshape(sc.height, sc.width)
    assert same.all()
    for which in (0, 1, 2, 3):
        assert np.array_equal(r.image(which), o.image(which)), f"image {which} differs"
    assert r.stats().frame_index == sc.spp


def _golden_scene_names():
    import os
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(here, "golden"))
    import pin_scenes
    return sorted(pin_scenes.PIN_SCENES)


@pytest.mark.parametrize("name", _golden_scene_names())
def test_gpu_matches_reference_golden(pt, name):
    """GPU images bit-identical to the reference's own shaders (golden fixtures)."""
    import os
    import pin_scenes
    here = os.path.dirname(os.path.abspath(__file__))
    g = np.load(os.path.join(here, "golden", f"ref_{name}.npz"))
    sc = pin_scenes.PIN_SCENES[name]()
    r = pt.renderer_for(sc)
    r.render(int(g["frames"]))
    for k, which in (("accum", 0), ("albedo", 1), ("normal", 2), ("final", 3)):
        got = r.image(which)
        if which == 3:
            assert np.array_equal(got, g[k]), f"{name}: final image differs"
        else:
            assert np.array_equal(got.view(np.uint32), g[k].view(np.uint32)), f"{name}: {k} differs"


def test_converges_to_the_fp64_oracle(pt, scenes):
    """The 128x128 Cornell box rendered on the GPU with an independent seed
    against the oracle's 4096-spp FP64 image: the error falls as 1/sqrt(spp)
    and the mean difference stays within its noise (no bias)."""
    import os
    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", "cornell128_4096spp_fp64.npz"))
    ref = ref["radiance"].astype(np.float64)
    s = scenes.cornell(128, 128, 1024, max_depth=8, rr_depth=0, seed=1)
    r = pt.renderer_for(s, seed=7)
    err = {}
    for total, step in ((64, 64), (256, 192), (1024, 768)):
        r.render(step)
        d = r.image(0)[..., :3].astype(np.float64) - ref
        err[total] = float(np.sqrt((d ** 2).mean()))
    assert 0.4 < err[256] / err[64] < 0.62, err
    assert 0.4 < err[1024] / err[256] < 0.62, err
    npix = d.shape[0] * d.shape[1]
    for c in range(3):
        dc = d[..., c].ravel()
        assert abs(dc.mean()) < 5.0 * dc.std() / np.sqrt(npix), (c, dc.mean(), dc.std())


def test_every_disney_kernel_matches_the_oracle(pt, scenes, oracle_mod):
    """Disney materials of both Disney kernels: no transmission (the kernel
    without the glass lobe), partial and full transmission, and out-of-range
    parameters whose glass weight is negative (kept on the kernel with every
    lobe). Per-path radiance and hit sequences equal the oracle's bit for
    bit."""
    sc = scenes.tiny_variants()["disney"]
    variants = [dict(specular_transmission=0.0), dict(specular_transmission=0.5),
                dict(specular_transmission=1.0), dict(metallic=1.25, specular_transmission=0.3)]
    for k, m in enumerate(sc.materials[1:]):
        for field, value in variants[k % 4].items():
            setattr(m, field, value)
    r = pt.renderer_for(sc, keep_samples=True)
    r.render(sc.spp)
    rad_g, hash_g = r.samples()
    o = oracle_mod.Oracle(sc)
    WH = sc.width * sc.height
    rad_o, hash_o = o.trace_paths(np.arange(WH), 0, sc.spp)
    assert np.array_equal(hash_g, hash_o.reshape(-1))
    assert np.array_equal(rad_g.view(np.uint32), rad_o.reshape(-1, 3).view(np.uint32))


@pytest.mark.parametrize("size", [(16384, 4), (2048, 1024)])
def test_env_alias_tables_both_builders(pt, scenes, oracle_mod, size):
    """The environment's alias tables come from the one-warp-per-row builder
    when a row fits in shared memory (2048 wide) and from the one-thread-per-
    row builder otherwise (16384 texels x 16 B per row): per-path radiance
    and hit sequences equal the oracle's bit for bit either way."""
    sc = scenes.tiny_variants()["disney"]
    sc.env_rgb = scenes.synthetic_sky(*size)
    r = pt.renderer_for(sc, keep_samples=True)
    r.render(sc.spp)
    rad_g, hash_g = r.samples()
    o = oracle_mod.Oracle(sc)
    WH = sc.width * sc.height
    rad_o, hash_o = o.trace_paths(np.arange(WH), 0, sc.spp)
    assert np.array_equal(hash_g, hash_o.reshape(-1))
    assert np.array_equal(rad_g.view(np.uint32), rad_o.reshape(-1, 3).view(np.uint32))


@pytest.mark.parametrize("freq", [6, 72, 361])
def test_fast_bvh_build_bitexact(pt, abi, scenes, freq):
    """The fast builder (linear BVH over Morton codes, PT_BVH_BUILD_FAST) on
    displaced icospheres of 722, 103,682 and 2,606,422 triangles plus the
    ground quad (the oversized triangles take their own subtree): closest
    hits and any-hit answers equal brute force, and a render equals the
    default build's image bit for bit."""
    sc = scenes.displaced_icosphere(48, 32, 2, freq=freq)
    sc.lights = []
    r = pt.renderer_for(sc, bvh_build=abi.BVH_BUILD_FAST)
    st = r.stats()
    assert st.triangles == sc.num_triangles and st.bvh_nodes > 0
    rays = _random_rays(_bounds(sc), 4000, 31)
    cam = np.array(sc.cameras[0].position, np.float32)
    tgt = np.array([0.0, 0.0, 1.15]) + np.random.default_rng(32).uniform(-1.0, 1.0, size=(2000, 3))
    rays[:2000, 0:3] = cam
    dc = tgt - cam
    rays[:2000, 4:7] = dc / np.linalg.norm(dc, axis=1, keepdims=True)
    assert np.array_equal(r.trace_rays(rays), r.trace_rays(rays, brute_force=True))
    rays[:, 7] = np.random.default_rng(33).uniform(0.01, 2.0, len(rays))
    assert np.array_equal(r.trace_rays(rays, any_hit=True)[:, 3],
                          r.trace_rays(rays, any_hit=True, brute_force=True)[:, 3])
    r.render(sc.spp)
    d = pt.renderer_for(sc)
    d.render(sc.spp)
    for k in (0, 1, 2, 3):
        assert np.array_equal(r.image(k).view(np.uint8), d.image(k).view(np.uint8)), k
