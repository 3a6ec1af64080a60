#!/usr/bin/env python3
"""Benchmark of the GB300 wavefront path tracer (paths/s).

One step = one complete render of the workload: W x H pixels x spp
progressive frames through the full integrator (camera, closest hit,
shading, next-event estimation, accumulation, tonemap). The default workload
is the 9x9 Disney sphere grid under a 2048x1024 HDR sky, 1920x1080, 64 spp,
depth 12, Russian roulette from depth 4, all synthetic.

`value` is paths/s with the scene already resident in HBM (device time of the
K timed renders, CUDA events on the renderer's stream; each wave's bounces
run as one CUDA graph launch unless --bounce-loop host). `e2e` is the same
metric through the public API from host buffers: scene upload, BVH build,
environment tables, the render and the image read-back are all inside its
timed region. The roofline's closest-hit launch times come from K further
renders of the same workload with CUDA events around every launch (the
host-driven bounce loop; events cannot sit inside the graph).

--impl reference times the CPU restatement of the reference integrator on
the host cores over a bounded sample of the same workload.

Multi-GPU: every rank renders the full workload's pixels for its own range of
frames (rank r: frames r * spp .. (r + 1) * spp - 1 of one render), so N
ranks render one image of N * spp samples; the accumulators are merged once
after the timed steps (partition.merge_accumulation, one all-reduce).
Per-rank work is fixed as N grows: scaling "weak".
"""
import argparse
import importlib
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

WORKLOADS = {
    "disney_grid_1080p_64spp": ("disney_grid", {}),
    "cornell_256_16spp": ("cornell", {}),
    "displaced_icosphere_1080p_32spp": ("displaced_icosphere", {}),
    "media_box_1024_128spp": ("media_box", {}),
}
DEFAULT_WORKLOAD = "disney_grid_1080p_64spp"
L2_FLUSH_BYTES = 256 << 20  # > 129 MB L2
# DRAM bytes (read + write) per closest-hit ray of k_trace: ncu's DRAM bytes
# of every k_trace launch of one 480x270x64 render of the Disney grid (its
# bounces 0-10, MB each, from profiles/k_trace_disney_grid_480x270_bvh4.md)
# over that render's 19,520,376 closest-hit rays.
TRACE_DRAM_MB_PER_BOUNCE = (744.49, 851.96, 559.77, 616.26, 419.36, 123.11, 61.27, 42.23, 29.07, 21.45, 15.81)
TRACE_DRAM_BYTES_PER_RAY = sum(TRACE_DRAM_MB_PER_BOUNCE) * 1e6 / 19520376


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def rank_seed(seed, rank, frames):
    """RNG seed of a rank: the seed is added to the frame index, so rank r
    renders frames [r * frames, (r + 1) * frames) of one render of
    world * frames frames (partition.frame_range with equal blocks)."""
    return seed + rank * frames


def max_over_ranks(x, device="cuda"):
    """The slowest rank's time (the job's time) when running under
    torch.distributed; x itself on a single process."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms into a CSV
    (in $PT_BENCH_CLOCKS_DIR, else the temporary directory); the JSON line
    carries the median SM clock under load and the throttle reasons seen."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        out_dir = os.environ.get("PT_BENCH_CLOCKS_DIR", tempfile.gettempdir())
        self.path = os.path.join(out_dir, f"hala_pt_clocks_gpu{gpu_index}_pid{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[3][k].lower().startswith("active")})
        loaded = [r for r in rows if r[2] > 200.0] or rows
        return {"sm_mhz": statistics.median(r[0] for r in loaded), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def _cpu_pixels(scene, npix, seed=1234):
    """A seeded set of distinct pixels, sorted (rows top to bottom)."""
    import numpy as np
    WH = scene.width * scene.height
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(WH, size=min(WH, npix), replace=False)).astype(np.uint32)


def _cpu_rate_probe(o, scene, threads):
    """Paths/s of the oracle on 512 pixels x all frames (thread start-up and
    caches warmed first)."""
    pix = _cpu_pixels(scene, 512, 99)
    o.trace_paths(pix[:64], 0, 1, threads)
    t0 = time.perf_counter()
    o.trace_paths(pix, 0, scene.spp, threads)
    return len(pix) * scene.spp / max(time.perf_counter() - t0, 1e-9)


def cpu_baseline(scene, seconds=12.0, threads=0, gpu_accum=None):
    """The oracle (CPU restatement of the reference integrator) on the host
    cores over a bounded, seeded sample of the workload: a fixed set of
    pixels, each rendered for all of the workload's frames (the same RNG
    stream as the GPU), sized to about `seconds` of CPU work.

    With `gpu_accum` (the accumulated image of the GPU's timed render), the
    sample doubles as the parity check of that render: the oracle's running
    mean of each sampled pixel must equal the GPU's pixel bit for bit."""
    import numpy as np
    from oracle import oracle
    oracle.build()
    o = oracle.Oracle(scene)
    WH = scene.width * scene.height
    rate = _cpu_rate_probe(o, scene, threads)
    npix = int(max(256, min(WH, seconds * rate / scene.spp)))
    pix = _cpu_pixels(scene, npix)
    t0 = time.perf_counter()
    rad, _ = o.trace_paths(pix, 0, scene.spp, threads)
    dt = time.perf_counter() - t0
    cores = threads if threads > 0 else (os.cpu_count() or 1)
    # one core, for the per-core rate (a short sample spread over the image)
    one = pix[::max(1, npix // 1024)]
    t1 = time.perf_counter()
    o.trace_paths(one, 0, scene.spp, 1)
    single = len(one) * scene.spp / (time.perf_counter() - t1)
    out = {"value": npix * scene.spp / dt, "unit": "paths/s", "cores": cores, "kind": "port",
           "single_thread_paths_per_s": single, "cpu_bvh_build_s": o.commit_s,
           "sample": f"{npix} seeded random pixels x all {scene.spp} frames of the full workload ({dt:.1f} s)"}
    if gpu_accum is not None:
        ref = oracle.running_mean(rad)
        got = np.ascontiguousarray(gpu_accum.reshape(-1, 4)[pix.astype(np.int64), :3])
        # bit for bit; a NaN equals a NaN (the payload of a NaN differs between CPU and GPU)
        same = ((got.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(got) & np.isnan(ref))).all(1)
        bad = np.nonzero(~same)[0]
        out["parity"] = {"pixels_checked": int(npix), "paths_covered": int(npix * scene.spp),
                         "mismatched_pixels": int(len(bad)), "nan_pixels": int(np.isnan(ref).any(1).sum()),
                         "first_mismatches": [{"pixel": int(pix[k]), "gpu": got[k].tolist(), "oracle": ref[k].tolist()}
                                              for k in bad[:4]],
                         "check": "accumulated pixels of the last timed GPU render against the oracle's running "
                                  "mean of the same pixels' paths, bit for bit (NaN equals NaN)"}
    return out


def run_reference(args, scene, workload):
    """The CPU arm: the oracle port of the reference integrator on all host
    threads. One step = one fully timed render of a seeded sample of the
    workload's pixels, each for all of its frames; the sample is sized so that
    the whole run ends within a few minutes."""
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    from oracle import oracle
    oracle.build()
    o = oracle.Oracle(scene)
    rate = _cpu_rate_probe(o, scene, 0)
    per_step_s = min(4.0, 120.0 / (args.warmup + args.steps))
    WH = scene.width * scene.height
    npix = int(max(256, min(WH, per_step_s * rate / scene.spp)))
    pix = _cpu_pixels(scene, npix)
    dts = []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        o.trace_paths(pix, 0, scene.spp, 0)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            dts.append(dt)
    paths_step = npix * scene.spp
    v = paths_step * len(dts) / sum(dts)
    cores = os.cpu_count() or 1
    sample = f"{npix} seeded random pixels x all {scene.spp} frames per step ({paths_step} paths)"
    line = {
        "impl": "reference", "metric": "paths/s", "value": v, "unit": "paths/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(dts) / len(dts),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload,
        "step": {"paths": paths_step, "pixels": npix, "frames": scene.spp,
                 "note": "each step renders a seeded sample of the workload (paths/s is a rate: the cost of a "
                         "path does not depend on how many are rendered)"},
        "cpu_baseline": {"value": v, "unit": "paths/s", "cores": cores, "kind": "port", "sample": sample,
                         "cpu_bvh_build_s": o.commit_s},
        "e2e": {"value": v, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def progressive_frames(r, abi, frames):
    """One sample per render call, as an interactive host drives the renderer:
    device ms per frame with the bounce graph and with the host-driven loop."""
    out = {}
    for label, flags in (("graph_ms_per_frame", 0), ("host_loop_ms_per_frame", abi.PROFILE_HOST_LOOP)):
        r.set_profiling(flags)
        r.reset()
        r.render(1)
        ms = []
        for _ in range(frames):
            r.render(1)
            ms.append(r.stats().render_ms)
        out[label] = statistics.median(ms)
    r.set_profiling(0)
    return out


def l2_copy_bandwidth(torch, mib=32, reps=64):
    """GB/s (read + write) of a device copy between two buffers that stay in
    the 129 MB L2: the ceiling for L2-served traffic the roofline's L2
    fraction is quoted against. The copies are replayed from a CUDA graph so
    that launch gaps do not count; best of five replays."""
    n = (mib << 20) // 4
    a = torch.ones(n, dtype=torch.float32, device="cuda")
    b = torch.empty_like(a)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for _ in range(3):
            b.copy_(a)
    torch.cuda.current_stream().wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        for _ in range(reps):
            b.copy_(a)
    g.replay()
    best = None
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        g.replay()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    return 2.0 * (mib << 20) * reps / (best / 1e3) / 1e9


def workloads_leg(pt):
    """The other configurations of the benchmark, each at its full size: the
    Cornell box, the 2.6M-triangle displaced icosphere (with its BVH rebuilt
    before every frame) and the media box; each also on the host cores over
    a seeded pixel sample (the oracle; for the icosphere its BVH build is
    timed separately), which also checks the GPU's accumulated pixels."""
    scenes = importlib.import_module("hala-pathtracer_gb300.scenes")
    abi = importlib.import_module("hala-pathtracer_gb300.abi")
    out = {}
    for name, fn in (("cornell_256_16spp", scenes.cornell), ("displaced_icosphere_1080p_32spp",
                                                               scenes.displaced_icosphere),
                     ("media_box_1024_128spp", scenes.media_box)):
        s = fn()
        r = pt.renderer_for(s)
        r.render(s.spp)  # warm-up at the full size: wavefront buffers and the bounce graph
        r.reset()
        r.render(s.spp)
        st = r.stats()
        row = {"paths": st.paths, "render_ms": st.render_ms, "paths_per_s": st.paths / (st.render_ms / 1e3),
               "rays_per_s": (st.closest_rays + st.shadow_rays) / (st.render_ms / 1e3), "triangles": s.num_triangles,
               "bvh_build_ms": st.bvh_build_ms}
        r.set_profiling(abi.PROFILE_HOST_LOOP)
        r.reset()
        r.render(s.spp)
        row["host_loop_render_ms"] = r.stats().render_ms
        r.set_profiling(0)
        if name.startswith("displaced"):
            # BVH rebuilt and timed per frame, with the default (SAH) and the
            # fast (Morton-ordered linear BVH) builder
            for key, mode in (("per_frame_rebuild", abi.BVH_BUILD_SAH), ("per_frame_rebuild_fast", abi.BVH_BUILD_FAST)):
                r.set_bvh_build(mode)
                r.commit()
                r.reset()
                r.render(1)  # warm-up of this tree
                r.reset()
                total, build = 0.0, 0.0
                for _ in range(s.spp):
                    r.commit()
                    build += r.stats().bvh_build_ms
                    r.render(1)
                    total += r.stats().render_ms
                total += build
                row[key] = {"paths_per_s": st.paths / (total / 1e3), "ms_total": total,
                            "build_ms_per_frame": build / s.spp, "render_ms_per_frame": (total - build) / s.spp}
            r.set_bvh_build(abi.BVH_BUILD_SAH)
            r.commit()
        r.reset()
        r.render(s.spp)  # the render whose pixels the CPU sample checks (the rebuild loop above changed accum)
        acc = r.image(abi.IMAGE_ACCUM)
        r.close()
        cb = cpu_baseline(s, seconds=8.0, gpu_accum=acc)
        row["parity"] = cb.pop("parity")
        row["cpu_oracle"] = cb
        row["speedup_vs_cpu"] = row["paths_per_s"] / cb["value"]
        out[name] = row
    return out


def cache_mlp_roofline():
    """Device-timed radiance-cache kernels on 2^22 seeded records against the
    measured bf16 tensor peak: 43,008 MLP FLOPs per query (2 x 21,504
    weights), three times that per training sample (forward, input and
    weight gradients)."""
    cache = importlib.import_module("hala-pathtracer_gb300.cache")
    c = cache.RadianceCache()
    n = 1 << 22
    infer_ms, train_ms = c.benchmark(n, 5)
    c.close()
    flops = 2.0 * 21504
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak, kind = float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        peak, kind = 1900.0, "fallback"
    inf_tf = flops * n / (infer_ms / 1e3) / 1e12
    trn_tf = 3.0 * flops * n / (train_ms / 1e3) / 1e12
    return {"kernel": "k_cache_infer (hash grid + 6-layer BF16 MLP, mma.sync)", "bound": "tensor",
            "queries": n, "infer_ms": infer_ms, "queries_per_s": n / (infer_ms / 1e3), "achieved": inf_tf,
            "peak": peak, "peak_kind": kind, "unit": "TFLOP/s", "frac": inf_tf / peak,
            "train_ms_per_pass": train_ms, "train_tflops": trn_tf, "train_frac": trn_tf / peak}


def cache_curves(pt, scene, ref, chunks, cache_options=None):
    """Progressive render; after each chunk: (spp, device ms so far, RMSE
    against `ref`, rays per path so far)."""
    import numpy as np
    r = pt.renderer_for(scene)
    if cache_options is not None:
        r.set_radiance_cache(**cache_options)
    out, t, done, rays = [], 0.0, 0, 0
    for c in chunks:
        r.render(c)
        st = r.stats()
        t += st.render_ms
        done += c
        rays += st.closest_rays + st.shadow_rays
        err = float(np.sqrt(((r.image(0)[..., :3].astype(np.float64) - ref) ** 2).mean()))
        out.append((done, t, err, rays / (done * scene.width * scene.height)))
    r.close()
    return out


def time_to_error(curve, target):
    """Device time at which a curve first reaches `target` RMSE (log-log
    interpolation between checkpoints), or None."""
    prev = None
    for spp, t, e, _ in curve:
        if e <= target:
            if prev is None:
                return t
            (t0, e0), (t1, e1) = prev, (t, e)
            if e0 <= e1:
                return t1
            f = (math.log(e0) - math.log(target)) / (math.log(e0) - math.log(e1))
            return math.exp(math.log(t0) + f * (math.log(t1) - math.log(t0)))
        prev = (t, e)
    return None


def radiance_cache_leg(pt, target_spp=256):
    """RMSE against the 4096-spp FP64 oracle image of the 128 x 128 Cornell
    box (tests/golden/cornell128_4096spp_fp64.npz) versus device time, for
    the plain tracer and with the online radiance cache."""
    import numpy as np
    scenes = importlib.import_module("hala-pathtracer_gb300.scenes")
    ref = np.load(os.path.join(ROOT, "tests", "golden", "cornell128_4096spp_fp64.npz"))["radiance"].astype(np.float64)
    s = scenes.cornell(128, 128, 1024, max_depth=8, rr_depth=0, seed=1)
    chunks = [1, 1, 2, 4, 8, 16, 32, 64, 128, 256, 512]
    warm = pt.renderer_for(s)
    warm.render(2)
    warm.set_radiance_cache()
    warm.render(4)
    warm.close()
    plain = cache_curves(pt, s, ref, chunks)
    cached = cache_curves(pt, s, ref, chunks, {})
    target = next(e for spp, t, e, _ in plain if spp == target_spp)
    t_plain = next(t for spp, t, e, _ in plain if spp == target_spp)
    t_cache = time_to_error(cached, target)
    return {
        "scene": "cornell 128x128, depth 8, no RR", "reference": "oracle 4096 spp FP64",
        "target_rmse": target, "plain_ms_to_target": t_plain, "cache_ms_to_target": t_cache,
        "time_ratio": (t_cache / t_plain) if t_cache else None,
        "plain_rmse_1024spp": plain[-1][2], "cache_rmse_1024spp": cached[-1][2],
        "plain_rays_per_path": plain[-1][3], "cache_rays_per_path": cached[-1][3],
        "plain_ms_1024spp": plain[-1][1], "cache_ms_1024spp": cached[-1][1],
    }


def serving_leg(n_jobs=256, rate=20.0, seed=0, cache=None):
    """The serving mix: `n_jobs` render jobs with Poisson arrivals at `rate`
    jobs/s, scenes drawn from the four workloads with seed-perturbed
    materials and lights, resolution log-uniform 128^2..1920x1080, spp
    log-uniform 1..256, all through one pt_server. With `cache` (a dict of
    radiance-cache options), every job without participating media renders
    with an online radiance cache."""
    jm = importlib.import_module("hala-pathtracer_gb300.jobmix")
    serve = importlib.import_module("hala-pathtracer_gb300.serve")
    jobs = jm.job_mix(n_jobs=n_jobs, rate=rate, seed=seed)
    with serve.Server() as srv:
        # first launches of every kernel variant outside the measured mix
        warm = jm.job_mix(n_jobs=8, rate=1000.0, seed=seed + 1, bases=jm.tiny_bases(), min_pixels=16 * 16,
                          max_pixels=64 * 64, max_spp=2)
        for j in warm:
            srv.wait(srv.submit(j.scene, j.frames))
        base = srv.stats()
        res = jm.play(srv, jobs, cache=cache)
        st = srv.stats()
    res.update({
        "arrival_rate_jobs_per_s": rate,
        "wavefronts": st.wavefronts - base.wavefronts,
        "device_busy_s": (st.busy_ms - base.busy_ms) / 1e3,
        "rays_per_s": ((st.closest_rays - base.closest_rays) + (st.shadow_rays - base.shadow_rays)) /
        max(res["span_s"], 1e-9),
        "peak_resident_gb": st.peak_resident_bytes / 1e9,
        "kernel_launches": st.kernel_launches - base.kernel_launches,
    })
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="resolution scale of the workload (profiling captures of a smaller case)")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving mix")
    ap.add_argument("--no-cache", action="store_true", help="skip the radiance-cache comparison")
    ap.add_argument("--no-workloads", action="store_true", help="skip the other workloads' table")
    ap.add_argument("--serving-jobs", type=int, default=256)
    ap.add_argument("--bounce-loop", default="graph", choices=["graph", "host"],
                    help="bounce loop of the timed steps: one CUDA graph per wave, or one host read-back per bounce")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    scenes = importlib.import_module("hala-pathtracer_gb300.scenes")
    fn, kw = WORKLOADS[args.workload]
    scene = getattr(scenes, fn)(**kw)
    if args.scale != 1.0:
        scene.width = max(1, int(round(scene.width * args.scale)))
        scene.height = max(1, int(round(scene.height * args.scale)))
    workload = {"workload": args.workload, "width": scene.width, "height": scene.height, "spp": scene.spp,
                "max_depth": scene.max_depth, "rr_depth": scene.rr_depth, "triangles": scene.num_triangles,
                "paths_per_step": scene.width * scene.height * scene.spp,
                "l2": "flushed between steps (256 MiB write)"}
    if args.impl == "reference":
        return run_reference(args, scene, workload)

    import numpy as np
    import torch
    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    pt = importlib.import_module("hala-pathtracer_gb300")
    abi = pt.abi
    pt.build()

    scene.seed = rank_seed(scene.seed, rank, scene.spp)  # this rank's frames of the job
    r = pt.renderer_for(scene)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    loop_flags = abi.PROFILE_HOST_LOOP if args.bounce_loop == "host" else 0
    r.set_profiling(loop_flags)
    # warm-up
    for _ in range(args.warmup):
        r.reset()
        r.render(scene.spp)
    # traversal work per closest-hit ray (counting kernels, outside the timed region)
    r.set_profiling(abi.PROFILE_COUNT)
    r.reset()
    r.render(max(1, scene.spp // 8))
    cs = r.stats()
    nodes_per_ray = cs.trav_nodes / max(cs.closest_rays, 1)
    tris_per_ray = cs.trav_tris / max(cs.closest_rays, 1)
    r.set_profiling(loop_flags)
    r.reset()
    r.render(scene.spp)  # the bounce graph is captured here, outside the timed steps

    clocks = ClockSampler(local)
    barrier()
    clocks.start()
    step_ms, closest, shadow, launches = [], 0, 0, 0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        r.reset()
        r.render(scene.spp)
        st = r.stats()
        step_ms.append(st.render_ms)
        closest += st.closest_rays
        shadow += st.shadow_rays
        launches += st.kernel_launches
    barrier()
    clk = clocks.stop()
    timed_accum = r.image(abi.IMAGE_ACCUM)  # the last timed render, for the parity check
    wave_paths = r.stats().wave_paths
    total_ms = max_over_ranks(sum(step_ms))
    paths_step = scene.width * scene.height * scene.spp
    value = ws * paths_step * args.steps / (total_ms / 1e3)
    rays_per_s = ws * (closest + shadow) / (total_ms / 1e3)

    merge = None
    if ws > 1:
        # the job's one collective: the frame-weighted mean of the ranks'
        # accumulators (an all-reduce of W x H x 4 floats per image)
        part = importlib.import_module("hala-pathtracer_gb300.partition")
        imgs = [torch.empty((scene.height, scene.width, 4), dtype=torch.float32, device="cuda") for _ in range(3)]
        for which, t in zip((abi.IMAGE_ACCUM, abi.IMAGE_ALBEDO, abi.IMAGE_NORMAL), imgs):
            r.image_into(which, t.data_ptr(), t.numel() * 4)
        barrier()
        t0 = time.perf_counter()
        merged, total_frames = part.merge_accumulation(imgs, scene.spp)
        torch.cuda.synchronize()
        merge = {"frames_total": total_frames, "ms": 1e3 * (time.perf_counter() - t0),
                 "bytes_per_rank": 3 * imgs[0].numel() * 4}
        del merged

    # the same steps again with CUDA events around every closest-hit launch
    # (host-driven bounce loop: events cannot sit inside the bounce graph)
    r.set_profiling(abi.PROFILE_TRACE_TIMING)
    host_ms, trace_ms, trace_launches, t_closest = [], 0.0, 0, 0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        r.reset()
        r.render(scene.spp)
        st = r.stats()
        host_ms.append(st.render_ms)
        trace_ms += st.trace_ms
        trace_launches += st.trace_launches
        t_closest += st.closest_rays
    r.set_profiling(0)
    progressive = progressive_frames(r, abi, 16)

    # end to end through the public API, host buffers in and images out
    e2e_ms = []
    h2d = sum(v.nbytes + i.nbytes for v, i, _, _ in scene.meshes) + 144 * len(scene.materials) + \
        64 * len(scene.lights) + 64 * len(scene.cameras)
    if scene.env_rgb is not None:
        h2d += scene.env_rgb.shape[0] * scene.env_rgb.shape[1] * 16
    d2h = scene.width * scene.height * (4 + 16)
    for k in range(args.warmup + args.steps):
        flush.zero_()
        barrier()
        t0 = time.perf_counter()
        rr = pt.renderer_for(scene)
        rr.render(scene.spp)
        _img = rr.image(abi.IMAGE_FINAL)
        _acc = rr.image(abi.IMAGE_ACCUM)
        rr.close()
        barrier()
        if k >= args.warmup:
            e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_total = max_over_ranks(sum(e2e_ms))
    e2e_value = ws * paths_step * args.steps / (e2e_total / 1e3)

    # roofline of the closest-hit kernel (algorithmic bytes per traced ray)
    bytes_per_ray = 32 + 16 + 128 * nodes_per_ray + 48 * tris_per_ray  # 128-B 4-wide nodes, 48-B triangles
    avg_launch_ms = trace_ms / max(trace_launches, 1)
    achieved = bytes_per_ray * t_closest / (trace_ms / 1e3) / 1e9 if trace_ms > 0 else 0.0
    peak, peak_kind = _peaks()
    traffic = TRACE_DRAM_BYTES_PER_RAY * t_closest / max(trace_launches, 1)
    dram_gbs = traffic / (avg_launch_ms / 1e3) / 1e9 if avg_launch_ms > 0 else 0.0
    l2_gbs = l2_copy_bandwidth(torch)
    line = {
        "metric": "paths/s", "value": value, "unit": "paths/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload,
        "rays": {"rays_per_s": rays_per_s, "closest_rays_per_step": closest / args.steps,
                 "shadow_rays_per_step": shadow / args.steps},
        "wave_paths": wave_paths,
        "e2e": {"value": e2e_value, "unit": "paths/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_total / args.steps},
        "roofline": {"kernel": "k_trace (closest hit)", "bound": "hbm", "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic,
                     "traffic_note": "ncu DRAM bytes per closest-hit ray over every k_trace launch of a 480x270x64 "
                                     "render x rays per launch",
                     "dram_achieved_gbs": dram_gbs, "dram_frac": dram_gbs / peak,
                     "l2": {"achieved": achieved, "peak": l2_gbs, "frac": achieved / l2_gbs if l2_gbs else None,
                            "peak_kind": "measured here: copies between two 32 MiB buffers resident in L2, replayed "
                                         "from a CUDA graph"},
                     "limiter": "issue and dependent-load latency: the BVH and triangles stay in L2 (68-81% L2 "
                                "hit rate), DRAM carries ~180 B per ray (90 B on bounce 0), mostly path state; ncu "
                                "shows 62-66% issue active and 8-11 of 32 lanes active per instruction (divergent "
                                "traversal lengths)",
                     "bytes_per_ray": bytes_per_ray, "nodes_per_ray": nodes_per_ray, "tris_per_ray": tris_per_ray,
                     "avg_launch_ms": avg_launch_ms, "launches": trace_launches,
                     "trace_share_of_step": trace_ms / max(sum(host_ms), 1e-9),
                     "timing": "events around each launch in K further steps of the same render"},
        "bounce_loop": {"timed_steps": args.bounce_loop, "ms_per_step": total_ms / args.steps,
                        "host_loop_ms_per_step": sum(host_ms) / args.steps,
                        "progressive_1spp": progressive},
        "gpu_launches": launches,
        "clocks": clk,
    }
    if merge is not None:
        line["merge"] = merge
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cb = cpu_baseline(scene, gpu_accum=timed_accum)
            line["parity"] = cb.pop("parity")
            line["cpu_baseline"] = cb
        except Exception as e:  # the checker is optional for the GPU number
            line["cpu_baseline"] = {"error": str(e)}
    r.close()
    if rank == 0 and ws == 1 and not args.no_workloads:
        try:
            line["workloads"] = workloads_leg(pt)
        except Exception as e:
            line["workloads"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0 and ws == 1 and not args.no_cache:
        try:
            line["cache_mlp_roofline"] = cache_mlp_roofline()
        except Exception as e:
            line["cache_mlp_roofline"] = {"error": f"{type(e).__name__}: {e}"}
        try:
            line["radiance_cache"] = radiance_cache_leg(pt)
        except Exception as e:
            line["radiance_cache"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0 and ws == 1 and not args.no_serving:
        try:
            line["serving"] = serving_leg(n_jobs=args.serving_jobs)
        except Exception as e:
            line["serving"] = {"error": f"{type(e).__name__}: {e}"}
        if not args.no_cache:
            try:
                sv = serving_leg(n_jobs=args.serving_jobs, cache={})
                sv["cache"] = "jobs without media rendered with the online radiance cache (default options)"
                line["serving_with_cache"] = sv
            except Exception as e:
                line["serving_with_cache"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
