"""Serving workload: a seeded mix of render jobs with Poisson arrivals, and
the loop that plays it against a `serve.Server`.

The mix draws each job's scene uniformly from the four procedural workloads
(Cornell box, Disney sphere grid under an HDR sky, displaced icosphere with
analytic lights, media box), perturbs its materials and lights with the job's
own seed, and draws its resolution log-uniformly in pixel count between
128 x 128 and 1920 x 1080 (keeping the workload's aspect ratio) and its
samples per pixel log-uniformly in 1..256. Jobs share their base scene's
geometry arrays; only materials and lights are copied.
"""
import copy
import math
import threading
import time

import numpy as np

from . import abi
from . import scenes as sc

BASE_BUILDERS = {
    "cornell": lambda: sc.cornell(),
    "disney_grid": lambda: sc.disney_grid(),
    "displaced_icosphere": lambda: sc.displaced_icosphere(),
    "media_box": lambda: sc.media_box(),
}


def tiny_bases():
    """Small base scenes for tests (the same four kinds, little geometry)."""
    t = sc.tiny_variants()
    return {"cornell": t["cornell"], "disney_grid": t["disney"], "displaced_icosphere": t["icosphere"],
            "media_box": t["media"]}


def perturb(base, rng):
    """Shallow copy of `base` with jittered materials and lights."""
    s = copy.copy(base)
    s._keep = []
    mats = []
    for m in base.materials:
        m2 = abi.Material.from_buffer_copy(m)
        f = rng.uniform(0.8, 1.2, 3)
        for k in range(3):
            m2.base_color[k] = float(min(1.0, max(0.0, m.base_color[k] * f[k])))
        m2.roughness = float(min(1.0, max(0.0, m.roughness + rng.uniform(-0.1, 0.1))))
        sc.preprocess_material(m2)
        mats.append(m2)
    s.materials = mats
    lights = []
    for li in base.lights:
        l2 = abi.Light.from_buffer_copy(li)
        g = float(rng.uniform(0.7, 1.3))
        for k in range(3):
            l2.intensity[k] = li.intensity[k] * g
        lights.append(l2)
    s.lights = lights
    s.env_intensity = float(base.env_intensity * rng.uniform(0.7, 1.3))
    return s


class MixJob:
    def __init__(self, index, arrival_s, kind, scene, frames):
        self.index = index
        self.arrival_s = arrival_s
        self.kind = kind
        self.scene = scene
        self.frames = frames
        self.job_id = None
        self.info = None

    @property
    def paths(self):
        return self.scene.width * self.scene.height * self.frames


def job_mix(n_jobs=256, rate=20.0, seed=0, bases=None, min_pixels=128 * 128, max_pixels=1920 * 1080,
            max_spp=256):
    """The job list: arrival time (s), scene kind, perturbed scene, spp."""
    rng = np.random.default_rng(seed)
    bases = bases if bases is not None else {k: b() for k, b in BASE_BUILDERS.items()}
    kinds = sorted(bases)
    gaps = rng.exponential(1.0 / rate, n_jobs)
    arrivals = np.cumsum(gaps) - gaps[0]
    jobs = []
    for i in range(n_jobs):
        kind = kinds[int(rng.integers(len(kinds)))]
        base = bases[kind]
        pixels = math.exp(rng.uniform(math.log(min_pixels), math.log(max_pixels)))
        aspect = base.width / base.height
        w = max(1, int(round(math.sqrt(pixels * aspect))))
        h = max(1, int(round(pixels / w)))
        spp = int(min(max_spp, max(1, round(math.exp(rng.uniform(0.0, math.log(max_spp)))))))
        s = perturb(base, rng)
        s.width, s.height, s.spp = w, h, spp
        jobs.append(MixJob(i, float(arrivals[i]), kind, s, spp))
    return jobs


def play(server, jobs, time_scale=1.0, release=True, cache=None):
    """Submits each job at its arrival time, waits for all of them and
    returns a summary: job latencies (submit to done, server clock), their
    p50/p99, and paths/s over the span from the first submit to the last
    completion. With `cache` (pt_cache_config fields as a dict), every job
    whose scene has no participating medium renders with an online radiance
    cache (the cache does not handle media)."""
    def wants_cache(j):
        return cache is not None and all(m.medium.type == abi.MEDIUM_NONE for m in j.scene.materials)
    descs = [server.job_desc(j.scene, j.frames, cache if wants_cache(j) else None) for j in jobs]
    t0 = time.perf_counter()
    done = threading.Event()
    waiter_err = []

    def waiter():
        try:
            for j in jobs:
                while j.job_id is None:
                    time.sleep(0.0005)
                server.wait(j.job_id)
                j.info = server.poll(j.job_id)
                if release:
                    server.release(j.job_id)
        except Exception as e:  # surfaced to the caller below
            waiter_err.append(e)
        finally:
            done.set()

    th = threading.Thread(target=waiter, daemon=True)
    th.start()
    for j, (jd, keep) in zip(jobs, descs):
        delay = j.arrival_s * time_scale - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        j.job_id = server.submit_desc(jd)
    done.wait()
    th.join()
    if waiter_err:
        raise waiter_err[0]
    return summarize(jobs)


def summarize(jobs):
    ok = [j for j in jobs if j.info is not None and j.info.state == abi.JOB_DONE]
    lat = np.array([j.info.done_ms - j.info.submit_ms for j in ok], np.float64)
    queue = np.array([j.info.admit_ms - j.info.submit_ms for j in ok], np.float64)
    span_ms = (max(j.info.done_ms for j in ok) - min(j.info.submit_ms for j in ok)) if ok else 0.0
    paths = sum(j.paths for j in ok)
    return {
        "jobs": len(jobs),
        "done": len(ok),
        "failed": sum(1 for j in jobs if j.info is not None and j.info.state == abi.JOB_FAILED),
        "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
        "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
        "mean_ms": float(lat.mean()) if len(lat) else None,
        "p50_queue_ms": float(np.percentile(queue, 50)) if len(queue) else None,
        "span_s": span_ms / 1e3,
        "paths": int(paths),
        "paths_per_s": paths / (span_ms / 1e3) if span_ms > 0 else None,
    }
