"""Generates tests/golden/cornell128_4096spp_fp64.npz: the 128 x 128 Cornell
box (max depth 8, no Russian roulette) rendered by the CPU oracle with 4096
samples per pixel and FP64 accumulation. It is the ground truth of the
radiance-cache RMSE-versus-time comparison; its RNG seed (7777) differs from
the seeds of the renders it judges, so its residual noise is independent of
theirs.

Run from the repository root: python tests/golden/make_cache_reference.py
"""
import importlib
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

SPP = 4096
SEED = 7777


def scene():
    sc = importlib.import_module("hala-pathtracer_gb300.scenes")
    return sc.cornell(128, 128, SPP, max_depth=8, rr_depth=0, seed=SEED)


def main():
    from oracle import oracle
    oracle.build()
    s = scene()
    o = oracle.Oracle(s)
    t = time.time()
    o.render(SPP, fp64=True)
    img = o.image(0)[..., :3].astype(np.float32)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cornell128_4096spp_fp64.npz")
    np.savez_compressed(out, radiance=img, spp=SPP, seed=SEED, width=128, height=128, max_depth=8, rr_depth=0)
    print(f"wrote {out} in {time.time() - t:.1f} s")


if __name__ == "__main__":
    main()
