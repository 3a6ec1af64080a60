"""Job server: many render jobs sharing the GPU's wavefronts (pt_server_*).

A job is what a reference host does for one image -- HalaRenderer::new,
set_scene, set_envmap or sky colours, set_env_intensity, set_exposure_value,
commit and `frames` render() calls (src/bin/hala-pathtracer.rs:128-285) --
submitted as one call. The server admits queued jobs while their device
memory fits its HBM budget, keeps each admitted job's scene, BVH and images
on the device, and packs the paths of all admitted jobs into shared
wavefronts. A job's images are bit-identical to those of `renderer_for` on the
same scene.
"""
import ctypes as C

import numpy as np

from . import abi
from . import PTError, _cache_config, _f4, load_library


class Server:
    def __init__(self, hbm_budget_bytes=0, max_jobs=0, wave_paths=0, quantum_paths=0, use_graphs=False,
                 fail_admission_of_job=0):
        self._lib = load_library()
        cfg = abi.ServerConfig()
        cfg.hbm_budget_bytes = int(hbm_budget_bytes)
        cfg.max_jobs = int(max_jobs)
        cfg.wave_paths = int(wave_paths)
        cfg.quantum_paths = int(quantum_paths)
        cfg.use_graphs = 1 if use_graphs else 0
        cfg.fail_admission_of_job = int(fail_admission_of_job)
        h = C.c_void_p()
        st = self._lib.pt_server_create(C.byref(cfg), C.byref(h))
        if st != abi.PT_OK:
            raise PTError(st, "pt_server_create failed (no CUDA device)")
        self._h = h
        self._shapes = {}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pt_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != abi.PT_OK:
            msg = self._lib.pt_server_last_error(self._h)
            raise PTError(st, msg.decode() if msg else "")

    def job_desc(self, scene, frames=None, cache=None, **cfg_over):
        """pt_job_desc for a scenes.Scene, set up the way `renderer_for` sets
        up a renderer; `cache` (a dict of pt_cache_config fields, {} for the
        defaults) renders the job with an online radiance cache. Returns
        (desc, keepalive)."""
        desc = scene.desc()
        jd = abi.JobDesc()
        jd.scene = C.pointer(desc)
        jd.config = scene.config(**cfg_over)
        jd.frames = int(scene.spp if frames is None else frames)
        jd.camera_index = 0
        keep = [scene, desc]
        if cache is not None:
            cc = _cache_config(**cache)
            keep.append(cc)
            jd.cache = C.addressof(cc)
        if scene.env_rgb is not None:
            env = np.ascontiguousarray(scene.env_rgb, np.float32)
            keep.append(env)
            jd.env_rgb = env.ctypes.data_as(C.POINTER(C.c_float))
            jd.env_width, jd.env_height = env.shape[1], env.shape[0]
            jd.env_rotation_deg = float(scene.env_rotation_deg)
            jd.ground_color = _f4((0.0, 0.0, 0.0, 1.0))
            jd.sky_color = _f4((0.0, 0.0, 0.0, 1.0))
        else:
            jd.ground_color = _f4(scene.ground_color)
            jd.sky_color = _f4(scene.sky_color)
        jd.env_intensity = float(scene.env_intensity)
        jd.exposure_value = float(scene.exposure_value)
        return jd, keep

    def submit(self, scene, frames=None, cache=None, **cfg_over):
        """Queues one job; returns its id. The scene's arrays are copied."""
        jd, keep = self.job_desc(scene, frames, cache, **cfg_over)
        return self.submit_desc(jd)

    def submit_desc(self, job_desc):
        jid = C.c_uint64()
        self._check(self._lib.pt_server_submit(self._h, C.byref(job_desc), C.byref(jid)))
        self._shapes[jid.value] = (job_desc.config.height, job_desc.config.width)
        return jid.value

    def poll(self, job_id):
        info = abi.JobInfo()
        self._check(self._lib.pt_server_poll(self._h, int(job_id), C.byref(info)))
        return info

    def wait(self, job_id, timeout_ms=0):
        """True when the job reached a final state, False on timeout."""
        st = self._lib.pt_server_wait(self._h, int(job_id), int(timeout_ms))
        if st == abi.PT_ERR_TIMEOUT:
            return False
        self._check(st)
        return True

    def image(self, job_id, which=abi.IMAGE_ACCUM):
        """One image of a finished job: (H, W, 4) float32, or uint8 for IMAGE_FINAL."""
        info = self.poll(job_id)
        if info.state != abi.JOB_DONE:
            raise PTError(info.status or abi.PT_ERR_NOT_READY,
                          f"job {info.id} is {abi.JOB_STATE_NAMES.get(info.state)}: {info.error.decode()}")
        h, w = self._shapes[job_id]
        out = np.empty((h, w, 4), np.uint8 if which == abi.IMAGE_FINAL else np.float32)
        self._check(self._lib.pt_server_read_image(self._h, int(job_id), int(which), out.ctypes.data, out.nbytes))
        return out

    def cancel(self, job_id):
        self._check(self._lib.pt_server_cancel(self._h, int(job_id)))

    def release(self, job_id):
        self._check(self._lib.pt_server_release(self._h, int(job_id)))
        self._shapes.pop(job_id, None)

    def pause(self, paused=True):
        self._check(self._lib.pt_server_pause(self._h, 1 if paused else 0))

    def stats(self):
        s = abi.ServerStats()
        self._check(self._lib.pt_server_get_stats(self._h, C.byref(s)))
        return s

