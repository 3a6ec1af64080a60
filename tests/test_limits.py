"""Limits that must be reported, not hidden (needs a GPU).

A traversal that runs out of stack skips a subtree and one that reaches its
visit cap stops early; either makes the call that saw it fail with
PT_ERR_TRAVERSAL instead of returning a silently wrong image. Scenes the leaf
links cannot address (2^26 triangles or more) are refused at set_scene. The
default wavefront is sized from the free device memory.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_traversal_stack_overflow_is_reported(pt, abi, scenes):
    sc = scenes.tiny_variants()["icosphere"]
    r = pt.renderer_for(sc)
    r.render(1)
    good = r.image(0).copy()
    r.reset()
    r.set_traversal_limits(stack_entries=1)
    with pytest.raises(pt.PTError) as e:
        r.render(1)
    assert e.value.status == abi.PT_ERR_TRAVERSAL
    assert "stack" in str(e.value)
    pts = np.concatenate([m[0][:, :3] for m in sc.meshes])
    centre = 0.5 * (pts.min(0) + pts.max(0))
    rays = np.zeros((256, 8), np.float32)
    rays[:, 0:3] = np.array(sc.cameras[0].position)
    d = centre + np.random.default_rng(3).normal(size=(256, 3)) * 0.3 - rays[:, 0:3]
    rays[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays[:, 7] = 1e4
    with pytest.raises(pt.PTError) as e:
        r.trace_rays(rays)
    assert e.value.status == abi.PT_ERR_TRAVERSAL
    # back to the defaults: the same render as before, no error
    r.set_traversal_limits(0, 0)
    r.reset()
    r.render(1)
    assert np.array_equal(r.image(0).view(np.uint32), good.view(np.uint32))


def test_traversal_visit_cap_is_reported(pt, abi, scenes):
    sc = scenes.tiny_variants()["cornell"]
    r = pt.renderer_for(sc)
    r.set_traversal_limits(max_visits=1)
    with pytest.raises(pt.PTError) as e:
        r.render(1)
    assert e.value.status == abi.PT_ERR_TRAVERSAL
    assert "visits" in str(e.value)
    with pytest.raises(pt.PTError):
        r.set_traversal_limits(stack_entries=97)


def test_scene_beyond_leaf_addressing_is_refused(pt, abi, scenes):
    """2^26 triangles cannot be addressed by a 26-bit leaf start: refused
    before any index is read or anything is uploaded."""
    sc = scenes.tiny_variants()["cornell"]
    d = sc.desc()
    verts = np.zeros((3, 11), np.float32)
    idx = np.zeros(3, np.uint32)
    d.primitives[0].vertices = verts.ctypes.data_as(C.POINTER(C.c_float))
    d.primitives[0].num_vertices = 3
    d.primitives[0].indices = idx.ctypes.data_as(C.POINTER(C.c_uint32))
    d.primitives[0].num_indices = 3 * (1 << 26)  # never read: the size check comes first
    r = pt.Renderer(sc.config())
    with pytest.raises(pt.PTError) as e:
        r.set_scene(d)
    assert e.value.status == abi.PT_ERR_UNSUPPORTED
    assert "2^26" in str(e.value)


def test_default_wavefront_is_sized_from_free_memory(pt, scenes):
    import torch
    sc = scenes.cornell(64, 64, 4)
    r = pt.renderer_for(sc, wave_paths=0)
    free, _ = torch.cuda.mem_get_info()
    r.render(4)
    w = r.stats().wave_paths
    assert w == 64 * 64 * 4  # the render is smaller than any default wavefront
    r.render(60)  # a larger call is not held to the first call's size
    assert r.stats().wave_paths == 64 * 64 * 60
    big = scenes.cornell(1024, 1024, 64)
    r2 = pt.renderer_for(big, wave_paths=0)
    r2.render(64)
    w2 = r2.stats().wave_paths
    per_path = 268
    assert w2 & (w2 - 1) == 0 and (1 << 16) <= w2 <= (1 << 27)
    assert w2 * per_path <= free // 2 or w2 == (1 << 16)
