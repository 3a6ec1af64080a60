"""Job server (pt_server_*): continuous batching into shared wavefronts.

The serving claim is that a job's images do not depend on what shared its
wavefronts: every job here is rendered once through the server, mixed with
jobs of other scenes, resolutions, sample counts and feature permutations,
and once alone through pt_renderer; the accumulated, albedo, normal and
final images must be bit-identical. Fault tests make their faults on the
host (invalid job, over-budget job, injected admission failure, cancelled
jobs) -- nothing faults the GPU.
"""
import importlib
import math

import numpy as np
import pytest

from tests.golden import pin_scenes

IMAGES = (0, 1, 2, 3)  # accum, albedo, normal, final


@pytest.fixture(scope="module")
def serve(pt, gpu_lib):
    return importlib.import_module("hala-pathtracer_gb300.serve")


@pytest.fixture(scope="module")
def jobmix(pt):
    return importlib.import_module("hala-pathtracer_gb300.jobmix")


def alone(pt, scene, frames):
    r = pt.renderer_for(scene)
    r.render(frames)
    out = [r.image(k) for k in IMAGES]
    r.close()
    return out


def mixed_jobs(jobmix):
    jobs = [(name, getattr(pin_scenes, name)()) for name in
            ("cornell", "disney_ibl", "lights_icosphere", "media", "transparent", "media_transparent",
             "ortho_sky", "thin_lens_reinhard", "no_tonemap", "textured")]
    mix = jobmix.job_mix(n_jobs=6, rate=100.0, seed=5, bases=jobmix.tiny_bases(), min_pixels=8 * 8,
                         max_pixels=48 * 40, max_spp=4)
    jobs += [(f"mix{j.index}_{j.kind}", j.scene) for j in mix]
    return jobs


@pytest.mark.gpu
@pytest.mark.parametrize("wave,quantum", [(2048, 256), (1 << 16, 1 << 12)])
def test_jobs_bit_identical_alone_and_in_the_mix(pt, serve, jobmix, wave, quantum):
    jobs = mixed_jobs(jobmix)
    with serve.Server(wave_paths=wave, quantum_paths=quantum) as srv:
        srv.pause(True)  # queue everything first so the jobs share wavefronts
        ids = [srv.submit(s) for _, s in jobs]
        srv.pause(False)
        for jid in ids:
            assert srv.wait(jid, 120000)
        st = srv.stats()
        assert st.jobs_done == len(jobs)
        assert st.paths == sum(s.width * s.height * s.spp for _, s in jobs)
        # jobs really shared wavefronts: fewer wavefronts than jobs x passes
        assert st.wavefronts < sum(math.ceil(s.width * s.height * s.spp / quantum) for _, s in jobs)
        for (name, s), jid in zip(jobs, ids):
            got = [srv.image(jid, k) for k in IMAGES]
            ref = alone(pt, s, s.spp)
            for k in IMAGES:
                assert np.array_equal(got[k].view(np.uint8), ref[k].view(np.uint8)), f"{name}: image {k} differs"
            srv.release(jid)
        assert srv.stats().resident_bytes == 0


@pytest.mark.gpu
def test_job_larger_than_a_wavefront(pt, serve, scenes):
    s = scenes.cornell(40, 32, 5, max_depth=6, rr_depth=2, seed=3)
    with serve.Server(wave_paths=1000, quantum_paths=300) as srv:
        jid = srv.submit(s)
        assert srv.wait(jid, 60000)
        info = srv.poll(jid)
        assert info.state == 2 and info.paths_done == 40 * 32 * 5
        got = srv.image(jid, 0)
    assert np.array_equal(got, alone(pt, s, 5)[0])


@pytest.mark.gpu
def test_rejects_invalid_and_over_budget_jobs(pt, serve, scenes):
    s = scenes.cornell(16, 16, 1)
    with serve.Server(hbm_budget_bytes=16 << 10) as srv:  # 16 KiB: no job fits
        with pytest.raises(pt.PTError) as e:
            srv.submit(s)
        assert e.value.status == 2  # PT_ERR_OOM
    with serve.Server() as srv:
        with pytest.raises(pt.PTError) as e:
            srv.submit(s, width=0)
        assert e.value.status == 1
        with pytest.raises(pt.PTError) as e:
            srv.submit(s, frames=0)
        assert e.value.status == 1
        bad = scenes.cornell(16, 16, 1)
        v, i, tr, m = bad.meshes[0]
        i = i.copy()
        i[0] = 10 ** 6  # index out of range
        bad.meshes[0] = (v, i, tr, m)
        with pytest.raises(pt.PTError) as e:
            srv.submit(bad)
        assert e.value.status == 1
        assert srv.stats().jobs_rejected == 3


@pytest.mark.gpu
def test_injected_admission_failure_leaves_other_jobs_intact(pt, serve, scenes):
    jobs = [scenes.cornell(20, 20, 2, seed=k) for k in range(3)]
    with serve.Server(fail_admission_of_job=2) as srv:
        ids = [srv.submit(s) for s in jobs]
        for jid in ids:
            assert srv.wait(jid, 60000)
        infos = [srv.poll(j) for j in ids]
        assert [i.state for i in infos] == [2, 3, 2]
        assert infos[1].status == 2 and b"injected" in infos[1].error
        with pytest.raises(pt.PTError):
            srv.image(ids[1], 0)
        for k in (0, 2):
            assert np.array_equal(srv.image(ids[k], 0), alone(pt, jobs[k], 2)[0])
        st = srv.stats()
        assert st.jobs_failed == 1 and st.jobs_done == 2


@pytest.mark.gpu
def test_cancel_queued_and_running_jobs(pt, serve, scenes):
    s = scenes.cornell(24, 24, 2)
    with serve.Server(max_jobs=1) as srv:
        srv.pause(True)
        a = srv.submit(s)
        b = srv.submit(s)
        # a is admitted (the only slot), b waits for the slot
        for _ in range(2000):
            if srv.poll(a).state == 1:
                break
            srv.wait(a, 5)
        assert srv.poll(a).state == 1 and srv.poll(b).state == 0
        assert not srv.wait(b, 50)  # still queued: the wait times out
        srv.cancel(b)
        assert srv.poll(b).state == 4
        srv.cancel(a)  # running: retired at the next wavefront boundary
        assert srv.wait(a, 10000) and srv.poll(a).state == 4
        c = srv.submit(s)
        srv.pause(False)
        assert srv.wait(c, 60000) and srv.poll(c).state == 2
        assert np.array_equal(srv.image(c, 3), alone(pt, s, 2)[3])
        st = srv.stats()
        assert st.jobs_cancelled == 2 and st.jobs_done == 1 and st.paths == 24 * 24 * 2


@pytest.mark.gpu
def test_budget_admits_one_job_at_a_time(pt, serve, scenes):
    jobs = [scenes.cornell(32, 32, 2, seed=k) for k in range(4)]
    with serve.Server() as probe:
        one = probe.poll(probe.submit(jobs[0])).device_bytes
    with serve.Server(hbm_budget_bytes=int(one * 1.5)) as srv:
        ids = [srv.submit(s) for s in jobs]
        for jid in ids:
            assert srv.wait(jid, 60000)
            assert srv.poll(jid).state == 2
            srv.release(jid)  # frees the images so the next job fits
        st = srv.stats()
        assert st.jobs_done == 4
        assert st.peak_resident_bytes <= int(one * 1.5)


def test_job_mix_is_seeded_and_within_bounds(jobmix):
    bases = jobmix.tiny_bases()
    a = jobmix.job_mix(n_jobs=200, rate=20.0, seed=1, bases=bases)
    b = jobmix.job_mix(n_jobs=200, rate=20.0, seed=1, bases=bases)
    assert [(j.kind, j.scene.width, j.scene.height, j.frames) for j in a] == \
           [(j.kind, j.scene.width, j.scene.height, j.frames) for j in b]
    arr = np.array([j.arrival_s for j in a])
    assert arr[0] == 0.0 and np.all(np.diff(arr) >= 0)
    assert 0.03 < np.diff(arr).mean() < 0.07  # Poisson at 20 jobs/s
    px = np.array([j.scene.width * j.scene.height for j in a])
    assert px.min() >= 0.9 * 128 * 128 and px.max() <= 1.1 * 1920 * 1080
    spp = np.array([j.frames for j in a])
    assert spp.min() >= 1 and spp.max() <= 256
    assert {j.kind for j in a} == set(bases)
    # perturbation touches materials and lights, never the shared geometry
    for j in a[:20]:
        base = bases[j.kind]
        assert j.scene.meshes is base.meshes
        assert len(j.scene.materials) == len(base.materials)


@pytest.mark.gpu
def test_radiance_cache_jobs_alone_and_in_the_mix(pt, serve, scenes):
    """Jobs with an online radiance cache run their passes on their own,
    between the shared wavefronts of plain jobs. The cache's hash-table
    gradients are summed with float atomics, whose order varies from run to
    run, so a cached render is reproducible to within that training noise,
    not bit for bit: a cached job's accumulated image alone on a server, in a
    mix with plain and other cached jobs, and through pt_renderer with the
    same frames per render call agree within 2% relative RMS (the stated
    tolerance). Plain jobs in the mix stay bit-identical. A cached job on a
    scene with media is refused at submit."""
    cache = dict(paths_per_pass=1 << 14, batch_size=4096, log2_table_size=14, steps_per_pass=2)
    a = scenes.cornell(48, 32, 12, max_depth=6, rr_depth=2, seed=3)
    b = scenes.cornell(40, 40, 9, max_depth=5, rr_depth=2, seed=4)
    plain = pin_scenes.disney_ibl()
    with serve.Server(wave_paths=1 << 14, quantum_paths=1 << 12) as srv:
        ja = srv.submit(a, cache=cache)
        assert srv.wait(ja, 120000)
        alone_a = [srv.image(ja, k) for k in IMAGES]
    with serve.Server(wave_paths=1 << 14, quantum_paths=1 << 12) as srv:
        srv.pause(True)
        ids = [srv.submit(plain), srv.submit(a, cache=cache), srv.submit(b, cache=cache), srv.submit(plain)]
        srv.pause(False)
        for jid in ids:
            assert srv.wait(jid, 120000)
            assert srv.poll(jid).state == pt.abi.JOB_DONE, srv.poll(jid).error
        mixed_a = [srv.image(ids[1], k) for k in IMAGES]
        plain_imgs = [srv.image(ids[0], k) for k in IMAGES]
        st = srv.stats()
        assert st.paths == 2 * plain.width * plain.height * plain.spp + a.width * a.height * 12 + \
            b.width * b.height * 9
        with pytest.raises(pt.PTError) as e:
            srv.submit(scenes.media_box(16, 16, 1), cache=cache)
        assert e.value.status == pt.abi.PT_ERR_UNSUPPORTED
    def rel_rms(x, y):
        x, y = x[..., :3].astype(np.float64), y[..., :3].astype(np.float64)
        return float(np.sqrt(((x - y) ** 2).mean() / max((y ** 2).mean(), 1e-30)))
    assert rel_rms(mixed_a[0], alone_a[0]) < 2e-2
    assert rel_rms(mixed_a[1], alone_a[1]) < 1e-6 and rel_rms(mixed_a[2], alone_a[2]) < 1e-6  # first-hit AOVs
    ref = alone(pt, plain, plain.spp)
    for k in IMAGES:
        assert np.array_equal(plain_imgs[k].view(np.uint8), ref[k].view(np.uint8)), k
    # the server's turns are render calls of whole passes: 16384 paths = 10.67
    # frames of 48 x 32, so turns of 11 frames, then the last frame
    r = pt.renderer_for(a, wave_paths=1 << 14)
    r.set_radiance_cache(**cache)
    r.render(11)
    r.render(1)
    assert rel_rms(r.image(0), alone_a[0]) < 2e-2
    assert r.stats().frame_index == 12
    # and the cache did take part: the cached render is not the plain one
    plain_a = alone(pt, a, 12)
    assert rel_rms(alone_a[0], plain_a[0]) > 1e-4
