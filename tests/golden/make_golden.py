#!/usr/bin/env python3
"""Regenerates tests/golden/ref_<scene>.npz from the reference's own shaders.

Needs the reference checkout: the shaders are compiled as host code by
oracle/ref/build_ref.py (GLSL read where it lies) and run by the pipeline
stand-in oracle/ref/ref_harness.inl. Each fixture holds the four images the
reference's raygen shader writes (accumulation, albedo, normal, RGBA8 final)
after `frames` progressive frames of one pin scene (tests/golden/pin_scenes.py).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import pin_scenes  # noqa: E402
from oracle.ref.ref import RefRenderer, available  # noqa: E402


def main():
    if not available():
        raise SystemExit("the reference checkout is not available")
    for name, fn in pin_scenes.PIN_SCENES.items():
        sc = fn()
        r = RefRenderer(sc)
        r.render(sc.spp)
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), accum=r.image(0), albedo=r.image(1),
                            normal=r.image(2), final=r.image(3), frames=np.int32(sc.spp),
                            permutation=np.array(r.perm))
        print(name, r.perm, sc.width, sc.height, sc.spp)


if __name__ == "__main__":
    main()
