"""One image from several GPUs: the frames of a progressive render split
across ranks, the ranks' accumulators merged once at the end.

A pixel's random sequence depends only on the pixel and the frame index
(common/wltcRS.glsl:9-19 seeds the RNG from (x, y, frame)), and the
tracer configuration's `seed` is added to the frame index. So rank r renders
the contiguous frames [lo_r, hi_r) of the whole render by rendering
hi_r - lo_r frames with seed + lo_r: its paths are exactly the paths of those
frames of a single-GPU render. Its accumulators hold the running mean of
its frames (pathtracer.rgen.glsl:259-278); the merged image is the mean over
all frames, the frame-count-weighted mean of the ranks' accumulators
(sum_r F_r * A_r / sum_r F_r). That sum is the one collective of the job (an
all-reduce of W x H x 4 floats per image); scene, BVH and environment are
replicated and nothing else is exchanged. The result equals a single render
of all frames up to float32 rounding of the running means.

Works with any torch.distributed backend: NCCL with CUDA tensors on GPUs,
gloo with CPU tensors.
"""
import importlib

import numpy as np


def frame_range(total_frames, rank, world):
    """Contiguous frames [lo, hi) of `rank`: blocks of total // world frames,
    the first total % world ranks one more."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(int(total_frames), int(world))
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def merge_accumulation(images, frames, group=None):
    """Frame-weighted mean of every rank's accumulation images.

    images: sequence of float32 tensors (H, W, 4) of this rank (accum, albedo,
    normal, ...); frames: the number of frames they hold (0 is allowed).
    Returns (merged tensors, total frames); every rank gets the same result.
    """
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size(group) == 1:
        return [img.to(torch.float32).clone() for img in images], int(frames)
    dev = images[0].device
    n = torch.tensor([float(frames)], dtype=torch.float64, device=dev)
    weighted = [img.to(torch.float32) * float(frames) for img in images]
    dist.all_reduce(n, op=dist.ReduceOp.SUM, group=group)
    for w in weighted:
        dist.all_reduce(w, op=dist.ReduceOp.SUM, group=group)
    total = float(n.item())
    if total <= 0:
        raise ValueError("no frames were rendered on any rank")
    merged = []
    for w in weighted:
        m = w / total
        m[..., 3] = 1.0  # the accumulators' alpha (pathtracer.rgen.glsl:271-277)
        merged.append(m)
    return merged, int(round(total))


def render_partitioned(scene, frames, group=None, **cfg_over):
    """Renders `frames` progressive frames of `scene` split across the ranks
    of `group` (one GPU per rank, torch.cuda's current device) and merges them.
    Returns (renderer, frames_here); on every rank the renderer then holds the
    merged accumulation (the images of the whole render)."""
    import torch
    import torch.distributed as dist
    pt = importlib.import_module("hala-pathtracer_gb300")
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    lo, hi = frame_range(frames, rank, world)
    cfg_over = dict(cfg_over)
    cfg_over["seed"] = int(cfg_over.get("seed", scene.seed)) + lo
    r = pt.renderer_for(scene, **cfg_over)
    if hi > lo:
        r.render(hi - lo)
    H, W = r.height, r.width
    imgs = [torch.empty((H, W, 4), dtype=torch.float32, device="cuda") for _ in range(3)]
    for which, t in zip((pt.abi.IMAGE_ACCUM, pt.abi.IMAGE_ALBEDO, pt.abi.IMAGE_NORMAL), imgs):
        r.image_into(which, t.data_ptr(), t.numel() * 4)
    torch.cuda.synchronize()
    merged, total = merge_accumulation(imgs, hi - lo, group)
    torch.cuda.synchronize()
    r.load_accumulation_ptr(merged[0].data_ptr(), merged[1].data_ptr(), merged[2].data_ptr(), total)
    return r, hi - lo


def merge_host_images(per_rank, frames):
    """Reference merge of host images (tests): frame-weighted mean in
    float32 of [(H, W, 4) arrays] with their frame counts."""
    acc = np.zeros_like(per_rank[0], np.float32)
    for img, f in zip(per_rank, frames):
        acc += np.asarray(img, np.float32) * np.float32(f)
    out = acc / np.float32(sum(frames))
    out[..., 3] = 1.0
    return out
