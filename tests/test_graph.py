"""The bounce loop as one CUDA graph launch per wave (default) against the
host-driven loop (one read-back per bounce, PT_PROFILE_HOST_LOOP): the
kernels are the same, so images, ray counts and bounce counts must be
identical. Small wavefronts exercise several grid buckets, many waves and
the graph's reuse across waves and renders (needs a GPU)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _render(pt, abi, sc, flags, spp, tail=None, **cfg):
    r = pt.renderer_for(sc, **cfg)
    r.set_profiling(flags)
    if tail is not None:
        r.set_tail_paths(tail)
    r.render(spp)
    st = r.stats()
    imgs = [r.image(w) for w in (0, 1, 2, 3)]
    r.close()
    return imgs, (st.closest_rays, st.shadow_rays, st.max_bounces_seen, st.paths)


@pytest.mark.parametrize("name", ["cornell", "disney", "icosphere", "media"])
@pytest.mark.parametrize("wave", [0, 5000, 70000])
def test_graph_matches_host_loop(pt, abi, scenes, name, wave):
    sc = scenes.tiny_variants()[name]
    a, sa = _render(pt, abi, sc, 0, sc.spp, wave_paths=wave)
    b, sb = _render(pt, abi, sc, abi.PROFILE_HOST_LOOP, sc.spp, wave_paths=wave)
    assert sa == sb, f"stats differ: graph {sa} host loop {sb}"
    for k in range(4):
        assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), f"image {k} differs"


def _pin_scene(name):
    import os
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(here, "golden"))
    import pin_scenes
    return pin_scenes.PIN_SCENES[name]()


@pytest.mark.parametrize("name", ["cornell", "disney", "icosphere", "media", "pin:transparent", "pin:textured",
                                  "pin:media_transparent"])
def test_wave_tail_matches_wavefront(pt, abi, scenes, name):
    """The wave tail (one kernel carrying each remaining path to its end)
    against the per-bounce wavefront: off, the automatic threshold, 4096,
    and every bounce of every wave in the tail, with the bounce graph and the host
    loop, over small and large wavefronts. Images, ray counts and bounce
    counts must be identical."""
    sc = _pin_scene(name[4:]) if name.startswith("pin:") else scenes.tiny_variants()[name]
    ref, sref = _render(pt, abi, sc, abi.PROFILE_HOST_LOOP, sc.spp, tail=0, wave_paths=70000)
    for flags in (0, abi.PROFILE_HOST_LOOP):
        for tail in (abi.TAIL_PATHS_AUTO, 4096, 1 << 31):
            for wave in (0, 5000):
                b, sb = _render(pt, abi, sc, flags, sc.spp, tail=tail, wave_paths=wave)
                where = f"flags {flags} tail {tail} wave {wave}"
                assert sb == sref, f"stats differ ({where}): {sb} against {sref}"
                for k in range(4):
                    assert np.array_equal(b[k].view(np.uint8), ref[k].view(np.uint8)), f"image {k} differs ({where})"


def test_wave_tail_progressive_frames(pt, abi, scenes):
    """One sample per render call on a frame large enough that the first
    bounces run as wavefront launches and the rest in the tail."""
    sc = scenes.disney_grid(160, 90, 6, segments=16, rings=8, env_size=(256, 128))
    out = []
    for tail in (0, 4096):
        r = pt.renderer_for(sc)
        r.set_tail_paths(tail)
        for _ in range(sc.spp):
            r.render(1)
        out.append(([r.image(w) for w in (0, 1, 2, 3)], r.stats().frame_index))
        r.close()
    assert out[0][1] == out[1][1] == sc.spp
    for k in range(4):
        assert np.array_equal(out[0][0][k].view(np.uint8), out[1][0][k].view(np.uint8)), f"image {k} differs"


def test_graph_progressive_frames(pt, abi, scenes):
    """One frame per render call, as an interactive host drives it: the graph
    is captured once and relaunched; the result equals one call of all frames."""
    sc = scenes.tiny_variants()["disney"]
    r = pt.renderer_for(sc)
    for _ in range(sc.spp):
        r.render(1)
    per_frame = [r.image(w) for w in (0, 3)]
    r.close()
    whole, _ = _render(pt, abi, sc, abi.PROFILE_HOST_LOOP, sc.spp)
    assert np.array_equal(per_frame[0].view(np.uint32), whole[0].view(np.uint32))
    assert np.array_equal(per_frame[1], whole[3])


@pytest.mark.parametrize("name", ["cornell", "disney"])
def test_resume_from_saved_accumulation(pt, abi, scenes, name):
    """Checkpoint after some frames, resume in a new renderer, finish: the
    images equal an uninterrupted render bit for bit."""
    sc = scenes.tiny_variants()[name]
    first = 3
    a = pt.renderer_for(sc)
    a.render(first)
    saved = [a.image(w) for w in (abi.IMAGE_ACCUM, abi.IMAGE_ALBEDO, abi.IMAGE_NORMAL)]
    frames = a.stats().frame_index
    a.close()
    assert frames == first
    b = pt.renderer_for(sc)
    b.load_accumulation(*saved, frames)
    assert np.array_equal(b.image(abi.IMAGE_ACCUM).view(np.uint32), saved[0].view(np.uint32))
    b.render(4)
    whole = pt.renderer_for(sc)
    whole.render(first + 4)
    assert b.stats().frame_index == whole.stats().frame_index == first + 4
    for w in (abi.IMAGE_ACCUM, abi.IMAGE_ALBEDO, abi.IMAGE_NORMAL, abi.IMAGE_FINAL):
        assert np.array_equal(b.image(w).view(np.uint8), whole.image(w).view(np.uint8)), f"image {w} differs"
