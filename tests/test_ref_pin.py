"""The reference's own shaders, compiled as host code (oracle/_ref), against
the CPU oracle, rendered live. Runs only where the reference checkout
exists; the committed golden fixtures carry the same check elsewhere."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import pin_scenes  # noqa: E402

ref = pytest.importorskip("oracle.ref.ref")
if not ref.available():
    pytest.skip("reference checkout not present", allow_module_level=True)


@pytest.mark.parametrize("name", ["cornell", "media_transparent", "lights_icosphere", "textured"])
def test_reference_shaders_match_oracle_over_more_frames(oracle_mod, name):
    sc = pin_scenes.PIN_SCENES[name]()
    frames = sc.spp + 3
    r = ref.RefRenderer(sc)
    r.render(frames)
    o = oracle_mod.Oracle(sc)
    o.render(frames)
    for which in (0, 1, 2, 3):
        a, b = r.image(which), o.image(which)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), f"{name}: image {which} differs"


def test_golden_fixtures_are_current():
    """The committed fixtures equal a fresh render of the reference's shaders."""
    for name, fn in pin_scenes.PIN_SCENES.items():
        sc = fn()
        r = ref.RefRenderer(sc)
        r.render(sc.spp)
        g = np.load(os.path.join(HERE, "golden", f"ref_{name}.npz"))
        assert np.array_equal(r.image(0).view(np.uint32), g["accum"].view(np.uint32)), name
        assert np.array_equal(r.image(3), g["final"]), name


@pytest.mark.parametrize("name", ["cornell", "thin_lens_reinhard", "ortho_sky"])
def test_loaded_blue_noise_texture_matches_the_reference_shaders(oracle_mod, name):
    """With a loaded blue-noise texture (load_blue_noise_texture) the
    reference's rand4blue and camera shaders and the oracle give the same
    images, bit for bit."""
    sc = pin_scenes.PIN_SCENES[name]()
    sc.blue_noise = np.random.default_rng(13).integers(0, 256, (1024, 1024, 4)).astype(np.uint8)
    r = ref.RefRenderer(sc)
    r.render(sc.spp)
    o = oracle_mod.Oracle(sc)
    o.render(sc.spp)
    for which in (0, 1, 2, 3):
        assert np.array_equal(r.image(which).view(np.uint32), o.image(which).view(np.uint32)), which
    plain = oracle_mod.Oracle(pin_scenes.PIN_SCENES[name]())
    plain.render(sc.spp)
    assert not np.array_equal(plain.image(0), o.image(0))
