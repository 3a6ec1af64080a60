"""Frames of one render split across ranks and merged (the multi-GPU form
of a render): the frame ranges tile the render, and the merge of two gloo
ranks' oracle renders equals the oracle's single render of all frames within
float32 rounding of the running means. CPU only; the GPU form
(partition.render_partitioned over NCCL) runs the same merge on device
tensors."""
import importlib
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


@pytest.fixture(scope="module")
def part(pt):
    return importlib.import_module("hala-pathtracer_gb300.partition")


def test_frame_ranges_tile_the_render(part):
    for total in (1, 7, 64, 129):
        for world in (1, 2, 3, 8):
            rs = [part.frame_range(total, r, world) for r in range(world)]
            assert rs[0][0] == 0 and rs[-1][1] == total
            assert all(rs[k][1] == rs[k + 1][0] for k in range(world - 1))
            sizes = [b - a for a, b in rs]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        part.frame_range(8, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, frames, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    part = importlib.import_module("hala-pathtracer_gb300.partition")
    scenes = importlib.import_module("hala-pathtracer_gb300.scenes")
    from oracle import oracle
    sc = scenes.cornell(20, 16, frames, max_depth=6, rr_depth=2, seed=3)
    lo, hi = part.frame_range(frames, rank, world)
    o = oracle.Oracle(sc, seed=sc.seed + lo)
    o.render(hi - lo, threads=1)
    imgs = [torch.from_numpy(o.image(k)) for k in (0, 1, 2)]
    merged, total = part.merge_accumulation(imgs, hi - lo)
    out[rank] = ([m.numpy() for m in merged], total, [i.numpy() for i in imgs], (lo, hi))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world,frames", [(2, 8), (3, 7)])
def test_merged_ranks_equal_one_render(oracle_mod, scenes, part, world, frames):
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, _free_port(), frames, out), nprocs=world, start_method="spawn")
    sc = scenes.cornell(20, 16, frames, max_depth=6, rr_depth=2, seed=3)
    o = oracle_mod.Oracle(sc)
    o.render(frames)
    for r in range(world):
        merged, total, _, _ = out[r]
        assert total == frames
        for k in (0, 1, 2):
            want = o.image(k)
            np.testing.assert_allclose(merged[k], want, rtol=2e-6 * frames, atol=1e-7)
    # every rank got the same merge, and it is the host reference merge
    per_rank = [out[r][2][0] for r in range(world)]
    counts = [out[r][3][1] - out[r][3][0] for r in range(world)]
    ref = part.merge_host_images(per_rank, counts)
    for r in range(world):
        np.testing.assert_allclose(out[r][0][0], ref, rtol=1e-6, atol=1e-7)
    # a rank's frames are those frames of the single render: rank 0's image
    # is the single render stopped after its frames
    lo, hi = out[0][3]
    o0 = oracle_mod.Oracle(sc)
    o0.render(hi - lo)
    assert np.array_equal(o0.image(0), out[0][2][0])


@pytest.mark.gpu
def test_gpu_frame_ranges_merge_to_one_render(pt, scenes, part):
    """On one GPU: the frames of a render split over three renderers (seed
    offset by each range's first frame), merged by the frame-weighted mean,
    equal the single render within float32 rounding; a one-rank
    render_partitioned (device images, no collective) is the single render
    bit for bit."""
    import torch
    sc = scenes.cornell(64, 48, 10, max_depth=6, rr_depth=2, seed=3)
    full = pt.renderer_for(sc)
    full.render(sc.spp)
    want = [full.image(k) for k in (0, 1, 2)]
    per, counts = [], []
    for rank in range(3):
        lo, hi = part.frame_range(sc.spp, rank, 3)
        r = pt.renderer_for(sc, seed=sc.seed + lo)
        r.render(hi - lo)
        per.append([r.image(k) for k in (0, 1, 2)])
        counts.append(hi - lo)
        r.close()
    for k in (0, 1, 2):
        merged = part.merge_host_images([p[k] for p in per], counts)
        np.testing.assert_allclose(merged, want[k], rtol=2e-5, atol=1e-7)
    r1, n1 = part.render_partitioned(sc, sc.spp)
    assert n1 == sc.spp
    torch.cuda.synchronize()
    for k in (0, 1, 2, 3):
        assert np.array_equal(r1.image(k).view(np.uint8), full.image(k).view(np.uint8)), k
    assert r1.stats().frame_index == sc.spp
