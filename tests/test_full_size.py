"""Parity at the benchmarked sizes (needs a GPU).

The renders the benchmark times, at their full size and through the default
path (default wavefront size, the bounce graph), checked against the oracle
on seeded pixel samples: every path of those pixels (all frames) must have
the oracle's hit-sequence hash and radiance bit for bit, and the accumulated
pixel must equal the oracle's running mean in frame order
(pathtracer.rgen.glsl:259-278). The BVH of the 2.6M-triangle icosphere (built
by the multi-block tier) is checked against brute force over all triangles.

Workloads: the 9x9 Disney grid under the HDR sky (1920x1080, 64 spp, depth
12), the displaced icosphere (2.6M triangles, 1920x1080, 32 spp, depth 8),
the media box (1024x1024, 128 spp, depth 32).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PIXELS = 4096


def bit_equal(a, b):
    """Element-wise: the same float32 bits, or both NaN (a path whose
    throughput turns non-finite gives NaN on both sides, as the reference
    does, but the NaN's payload differs between the CPU and the GPU)."""
    return (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))


def check_workload(pt, oracle_mod, sc, seed):
    WH = sc.width * sc.height
    r = pt.renderer_for(sc, keep_samples=1)
    r.render(sc.spp)
    st = r.stats()
    assert st.paths == WH * sc.spp
    pix = np.sort(np.random.default_rng(seed).choice(WH, PIXELS, replace=False)).astype(np.uint64)
    paths = (np.arange(sc.spp, dtype=np.uint64)[:, None] * np.uint64(WH) + pix[None, :]).reshape(-1)
    rad_g, hash_g = r.read_samples(paths)
    acc = r.image(0).reshape(-1, 4)[pix.astype(np.int64), :3]
    r.close()
    o = oracle_mod.Oracle(sc)
    rad_o, hash_o = o.trace_paths(pix.astype(np.uint32), 0, sc.spp)
    rad_o = rad_o.reshape(-1, 3)
    hash_o = hash_o.reshape(-1)
    bad = np.nonzero(hash_g != hash_o)[0]
    assert len(bad) == 0, f"{len(bad)} of {len(paths)} hit sequences differ, first path {paths[bad[0]]}"
    same = bit_equal(rad_g, rad_o).all(1)
    assert same.all(), f"{(~same).sum()} of {len(paths)} per-path radiances differ"
    ref = oracle_mod.running_mean(rad_o.reshape(sc.spp, PIXELS, 3))
    assert bit_equal(np.ascontiguousarray(acc), ref).all(), "accumulated pixels differ"
    return st


def test_disney_grid_full_size(pt, scenes, oracle_mod):
    """1920x1080 x 64 spp in one wavefront of the default size (2^27 paths
    when the device has room), bounce graph, as the benchmark renders it."""
    sc = scenes.disney_grid()
    st = check_workload(pt, oracle_mod, sc, 101)
    assert st.max_bounces_seen >= 2


def test_displaced_icosphere_full_size(pt, scenes, oracle_mod):
    """2.6M triangles: closest hits and any-hit answers of the device BVH
    equal brute force over every triangle, then per-path parity of the
    1920x1080 x 32 spp render."""
    sc = scenes.displaced_icosphere()
    assert sc.num_triangles == 2606422
    r = pt.renderer_for(sc)
    assert r.stats().triangles == sc.num_triangles
    pts = np.concatenate([m[0][:, :3] for m in sc.meshes])
    lo, hi = pts.min(0), pts.max(0)
    rng = np.random.default_rng(29)
    n = 4096
    rays = np.zeros((n, 8), np.float32)
    # half from random points in the box, half from the camera towards the sphere
    rays[:, 0:3] = rng.uniform(lo, hi, size=(n, 3))
    d = rng.normal(size=(n, 3))
    rays[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays[:, 7] = 1e4
    cam = np.array(sc.cameras[0].position, np.float32)
    tgt = np.array([0.0, 0.0, 1.15]) + rng.uniform(-1.0, 1.0, size=(n // 2, 3))  # the sphere
    dc = tgt - cam
    rays[: n // 2, 0:3] = cam
    rays[: n // 2, 4:7] = dc / np.linalg.norm(dc, axis=1, keepdims=True)
    hb = r.trace_rays(rays)
    hf = r.trace_rays(rays, brute_force=True)
    assert np.array_equal(hb, hf)
    assert (hf[:, 3] != 0xFFFFFFFF).mean() > 0.3
    rays[:, 7] = rng.uniform(0.01, 2.0, n)
    a = r.trace_rays(rays, any_hit=True)
    b = r.trace_rays(rays, any_hit=True, brute_force=True)
    assert np.array_equal(a[:, 3], b[:, 3])
    r.close()
    check_workload(pt, oracle_mod, sc, 103)


def test_media_box_full_size(pt, scenes, oracle_mod):
    """1024x1024 x 128 spp at depth 32 (delta tracking, transmittance loop)."""
    sc = scenes.media_box()
    st = check_workload(pt, oracle_mod, sc, 107)
    assert st.max_bounces_seen > 12
