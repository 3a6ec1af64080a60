"""The allocation-free BVH rebuild, pt_bvh_build_noalloc.

Some hosts may not call cudaMalloc or cudaFree while they run: they reserve
their device pools at start-up and rebuild the BVH of animated geometry every
frame inside that budget. pt_bvh_build_noalloc serves them by building into
caller-owned buffers, with its scratch in a fixed library-owned device array.

The tests build the BVH of a scene through that entry point twice in a row
and check each result against the library's ordinary build (the one
pt_renderer_commit runs): the same binary node count, the triangles in leaf
order a permutation of the input, and the closest hit of every test ray
found by walking the returned nodes bit-identical (t, u, v, triangle id) to
pt_renderer_trace_rays on the committed renderer. Scenes: a small icosphere
(under the ordinary build's multi-block threshold) and a soup of exactly
PT_NOALLOC_MAX_TRIANGLES = 65,536 triangles (the largest input, where the
ordinary build splits the top levels with all blocks and the allocation-free
one with one block per task). The device's free memory is the same before
and after the second call. An input above the limit is refused with a reason.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

f32 = np.float32
MISS = 0xFFFFFFFF


def _world_triangles(scene):
    """Triangle v0/e1/e2 in world space with the float32 operation order of
    the library's upload (rows of the 3x4 transform, then e = v - v0)."""
    v0s, e1s, e2s = [], [], []
    for verts, idx, tr_cm, _ in scene.meshes:
        T = tr_cm.reshape(4, 4).T.astype(np.float32)  # row-major object-to-world
        p = verts[:, 0:3].astype(np.float32)
        w = np.empty_like(p)
        for r in range(3):
            w[:, r] = ((T[r, 0] * p[:, 0] + T[r, 1] * p[:, 1]) + T[r, 2] * p[:, 2]) + T[r, 3]
        t = idx.reshape(-1, 3)
        a, b, c = w[t[:, 0]], w[t[:, 1]], w[t[:, 2]]
        v0s.append(a)
        e1s.append(b - a)
        e2s.append(c - a)
    out = []
    for arr in (np.concatenate(v0s), np.concatenate(e1s), np.concatenate(e2s)):
        q = np.zeros((len(arr), 4), np.float32)
        q[:, :3] = arr
        out.append(q)
    return out


def _intersect(o, d, v0, e1, e2, tmin, tmax):
    """Moller-Trumbore with the library's operation order (float32, no FMA)."""
    def cross(a, b):
        return (f32(a[1] * b[2]) - f32(a[2] * b[1]), f32(a[2] * b[0]) - f32(a[0] * b[2]),
                f32(a[0] * b[1]) - f32(a[1] * b[0]))

    def dot(a, b):
        return f32(f32(a[0] * b[0]) + f32(a[1] * b[1])) + f32(a[2] * b[2])

    pvec = cross(d, e2)
    det = dot(e1, pvec)
    if det == 0:
        return None
    inv = f32(1.0) / det
    tvec = (o[0] - v0[0], o[1] - v0[1], o[2] - v0[2])
    u = f32(dot(tvec, pvec) * inv)
    if u < 0 or u > 1:
        return None
    qvec = cross(tvec, e1)
    v = f32(dot(d, qvec) * inv)
    if v < 0 or f32(u + v) > 1:
        return None
    t = f32(dot(e2, qvec) * inv)
    if t < tmin or t > tmax:
        return None
    return t, u, v


def _box_hit(lo, hi, o, d, tmax):
    """Conservative slab test in float64 (boxes are already widened)."""
    tn, tf = 0.0, float(tmax)
    for k in range(3):
        if d[k] == 0.0:
            if o[k] < lo[k] - 1e-6 or o[k] > hi[k] + 1e-6:
                return False
            continue
        t0, t1 = (lo[k] - o[k]) / d[k], (hi[k] - o[k]) / d[k]
        if t0 > t1:
            t0, t1 = t1, t0
        tn, tf = max(tn, t0), min(tf, t1)
    return tn <= tf * (1.0 + 1e-6) + 1e-6


def _closest(nodes, tris, o, d, tmin, tmax):
    """Walks the returned nodes: lexicographic minimum of (t, triangle id)."""
    nf = nodes.reshape(-1, 16)
    ni = nf.view(np.int32)
    tu = tris.view(np.uint32)
    best_t, best_id, bu, bv = f32(tmax), MISS, f32(0), f32(0)
    o64, d64 = o.astype(np.float64), d.astype(np.float64)
    stack = [0]
    while stack:
        link = stack.pop()
        if link >= 0:
            row, links = nf[link].astype(np.float64), ni[link, 12:14]
            for c in range(2):
                base = 4 * c
                lo = (row[base], row[base + 2], row[8 + 2 * c])
                hi = (row[base + 1], row[base + 3], row[9 + 2 * c])
                if _box_hit(lo, hi, o64, d64, best_t):
                    stack.append(int(links[c]))
        else:
            ul = link & 0xFFFFFFFF
            start, count = ul & 0x03FFFFFF, (ul >> 26) & 0x1F
            for s in range(start, start + count):
                tid = int(tu[3 * s, 3])
                r = _intersect(o, d, tris[3 * s, :3], tris[3 * s + 1, :3], tris[3 * s + 2, :3], tmin, best_t)
                if r is not None and (r[0] < best_t or tid < best_id):
                    best_t, best_id, bu, bv = r[0], tid, r[1], r[2]
    if best_id == MISS:
        return np.array([np.float32(1e6).view(np.uint32), 0, 0, MISS], np.uint32)
    return np.array([f32(best_t).view(np.uint32), f32(bu).view(np.uint32), f32(bv).view(np.uint32), best_id],
                    np.uint32)


def _soup(scenes, n, seed):
    """n small random triangles in the unit cube, one material, a camera."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.0, 1.0, size=(n, 1, 3))
    pos = (c + rng.uniform(-0.02, 0.02, size=(n, 3, 3))).reshape(-1, 3)
    z = np.zeros((3 * n, 3))
    s = scenes.Scene("soup")
    m = s.add_material(scenes.material())
    s.add_mesh(scenes.pack_vertices(pos, z + [0, 0, 1], z + [1, 0, 0], np.zeros((3 * n, 2))),
               np.arange(3 * n, dtype=np.uint32), m)
    s.cameras.append(scenes.look_at((0.5, -2.0, 0.5), (0.5, 0.5, 0.5), 40.0))
    s.width, s.height, s.spp = 16, 16, 1
    return s


def _check_noalloc_build(pt, sc, nrays, seed):
    torch = pytest.importorskip("torch")
    pt.build()
    lib = pt.load_library()
    sc.lights = []  # triangles only: the walk below does not include analytic lights
    r = pt.renderer_for(sc)
    n = sc.num_triangles
    binary_nodes = r.stats().bvh_binary_nodes
    rng = np.random.default_rng(seed)
    pts = np.concatenate([m[0][:, :3] for m in sc.meshes])
    rays = np.zeros((nrays, 8), np.float32)
    rays[:, 0:3] = rng.uniform(pts.min(0), pts.max(0), size=(nrays, 3))
    dirs = rng.normal(size=(nrays, 3))
    rays[:, 4:7] = dirs / np.linalg.norm(dirs, axis=1, keepdims=True)
    rays[:, 7] = 1e4
    expected = r.trace_rays(rays)
    r.close()

    v0, e1, e2 = (torch.from_numpy(a).cuda() for a in _world_triangles(sc))
    nodes = torch.empty((4 * 2 * n, 4), device="cuda")
    tri_sorted = torch.empty((3 * n, 4), device="cuda")
    for call in range(2):
        nodes.fill_(float("nan"))
        tri_sorted.fill_(float("nan"))
        nn = C.c_uint32(0)
        err = C.create_string_buffer(256)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        st = lib.pt_bvh_build_noalloc(v0.data_ptr(), e1.data_ptr(), e2.data_ptr(), n, nodes.data_ptr(), 2 * n,
                                      tri_sorted.data_ptr(), C.byref(nn), None, err, 256)
        torch.cuda.synchronize()
        assert st == 0, err.value.decode()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before, "device memory changed during the call"
        assert nn.value == binary_nodes, (nn.value, binary_nodes)
        hn = nodes[:4 * nn.value].cpu().numpy()
        ht = tri_sorted.cpu().numpy()
        ids = ht[0::3, 3].view(np.uint32)
        assert np.array_equal(np.sort(ids), np.arange(n, dtype=np.uint32))
        got = np.stack([_closest(hn, ht, rays[k, 0:3], rays[k, 4:7], f32(rays[k, 3]), f32(rays[k, 7]))
                        for k in range(len(rays))])
        assert np.array_equal(got, expected), f"call {call}: {(got != expected).any(1).sum()} rays differ"
        assert (expected[:, 3] != MISS).any()


def test_noalloc_bvh_matches_renderer_build(pt, scenes):
    _check_noalloc_build(pt, scenes.tiny_variants()["icosphere"], 256, 21)


def test_noalloc_bvh_at_the_size_limit(pt, scenes):
    sc = _soup(scenes, pt.abi.NOALLOC_MAX_TRIANGLES, 5)
    assert sc.num_triangles == 65536
    _check_noalloc_build(pt, sc, 96, 22)


def test_noalloc_bvh_rejects_oversized_input(pt):
    pt.build()
    lib = pt.load_library()
    nn = C.c_uint32(7)
    err = C.create_string_buffer(256)
    too_many = pt.abi.NOALLOC_MAX_TRIANGLES + 1
    st = lib.pt_bvh_build_noalloc(None, None, None, too_many, None, 0, None, C.byref(nn), None, err, 256)
    assert st == pt.abi.PT_ERR_INVALID_ARG
    assert b"65536" in err.value and nn.value == 0
