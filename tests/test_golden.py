"""The CPU oracle against golden images produced by the reference's own
shaders (tests/golden/ref_*.npz, made by tests/golden/make_golden.py from the
GLSL compiled as host code). Bit-identical accumulation, albedo, normal and
final images for every pin scene."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import pin_scenes  # noqa: E402


def load_golden(name):
    return np.load(os.path.join(HERE, "golden", f"ref_{name}.npz"))


@pytest.mark.parametrize("name", sorted(pin_scenes.PIN_SCENES))
def test_oracle_matches_reference_golden(oracle_mod, name):
    g = load_golden(name)
    sc = pin_scenes.PIN_SCENES[name]()
    o = oracle_mod.Oracle(sc)
    o.render(int(g["frames"]))
    for k, which in (("accum", 0), ("albedo", 1), ("normal", 2), ("final", 3)):
        got = o.image(which)
        want = g[k]
        if which == 3:
            assert np.array_equal(got, want), f"{name}: final image differs"
        else:
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), f"{name}: {k} differs"


def test_golden_covers_every_permutation():
    perms = {str(load_golden(n)["permutation"]) for n in pin_scenes.PIN_SCENES}
    assert perms == {"base", "transparent", "medium", "medium_transparent"}
