"""GB300 wavefront path tracer: Python host over the libhalapt C ABI.

`Renderer` mirrors the operator surface of the reference's `HalaRenderer`
(crate hala-renderer as called from src/bin/hala-pathtracer.rs:128-285):
new -> set_scene -> set_envmap | set_ground_color/set_sky_color ->
set_env_intensity -> set_exposure_value -> commit -> render ... ->
save_images, with the same argument meaning. Errors raise `PTError`
carrying the C status and the library's last-error text, the way the
reference propagates `anyhow::Result`.

All compute runs in libhalapt.so (hand-written CUDA for sm_103a). There is
no CPU fallback: if the library is missing or no GPU is present, the
constructor raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from . import scenes  # noqa: F401  (procedural workloads)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libhalapt.so")
_lib = None


class PTError(RuntimeError):
    def __init__(self, status, message):
        self.status = status
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {message}")


def load_library(path=None):
    """Loads libhalapt.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise PTError(abi.PT_ERR_NOT_READY, f"{p} is missing; run build() first")
        _lib = abi.bind(C.CDLL(p), abi.RENDERER_SIGNATURES)
    return _lib


def build(force=False):
    from . import buildlib as _b
    return _b.build(force=force)


def _f4(v):
    v = list(v) + [1.0] * (4 - len(v))
    return (C.c_float * 4)(*v[:4])


class Renderer:
    """One progressive renderer (HalaRenderer::new, src/bin/hala-pathtracer.rs:128-138)."""

    def __init__(self, config):
        self._lib = load_library()
        self.config = config
        h = C.c_void_p()
        st = self._lib.pt_renderer_create(C.byref(config), C.byref(h))
        if st != abi.PT_OK:
            raise PTError(st, "pt_renderer_create failed (invalid config or no CUDA device)")
        self._h = h
        self.width, self.height = config.width, config.height
        self._keep = []

    # -- lifecycle ---------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._lib.pt_renderer_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != abi.PT_OK:
            msg = self._lib.pt_renderer_last_error(self._h)
            raise PTError(st, msg.decode() if msg else "")

    # -- operator surface ----------------------------------------------------
    def set_scene(self, scene):
        """HalaRenderer::set_scene. `scene` is a scenes.Scene or an abi.SceneDesc."""
        desc = scene.desc() if hasattr(scene, "desc") else scene
        self._keep = [scene, desc]
        self._check(self._lib.pt_renderer_set_scene(self._h, C.byref(desc)))

    def set_envmap(self, rgb, rotation_degrees=0.0):
        """HalaRenderer::set_envmap with decoded pixels: (H, W, 3) float32, row 0 = zenith."""
        if rgb is None:
            self._check(self._lib.pt_renderer_set_envmap(self._h, None, 0, 0, 0.0))
            return
        a = np.ascontiguousarray(rgb, np.float32)
        self._check(self._lib.pt_renderer_set_envmap(self._h, a.ctypes.data_as(C.POINTER(C.c_float)),
                                                     a.shape[1], a.shape[0], float(rotation_degrees)))

    def set_envmap_file(self, path, rotation_degrees=0.0):
        """HalaRenderer::set_envmap(&hdri_file, rotation): the OpenEXR file read
        by the library itself (pt_renderer_set_envmap_file)."""
        self._check(self._lib.pt_renderer_set_envmap_file(self._h, None if path is None else str(path).encode(),
                                                          float(rotation_degrees)))

    def set_scene_file(self, path):
        """HalaScene::new(scene_file) + set_scene: the glTF 2.0 file read by the
        library itself (pt_renderer_set_scene_file)."""
        self._check(self._lib.pt_renderer_set_scene_file(self._h, str(path).encode()))

    def load_blue_noise_texture(self, path):
        """HalaRenderer::load_blue_noise_texture: the camera jitter's RGBA8
        texture from an 8-bit PNG (None: the substitute table)."""
        self._check(self._lib.pt_renderer_load_blue_noise_texture(self._h, None if path is None else
                                                                   str(path).encode()))

    def set_blue_noise(self, rgba8):
        """The same texture from (1024, 1024, 4) uint8 texels (None: the substitute)."""
        if rgba8 is None:
            self._check(self._lib.pt_renderer_set_blue_noise(self._h, None))
            return
        a = np.ascontiguousarray(rgba8, np.uint8)
        if a.shape != (abi.PT_BLUE_NOISE_SIZE, abi.PT_BLUE_NOISE_SIZE, 4):
            raise ValueError(f"blue-noise texels must be ({abi.PT_BLUE_NOISE_SIZE}, {abi.PT_BLUE_NOISE_SIZE}, 4)")
        self._check(self._lib.pt_renderer_set_blue_noise(self._h, a.ctypes.data))

    def set_ground_color(self, rgba):
        self._check(self._lib.pt_renderer_set_ground_color(self._h, _f4(rgba)))

    def set_sky_color(self, rgba):
        self._check(self._lib.pt_renderer_set_sky_color(self._h, _f4(rgba)))

    def set_env_intensity(self, v):
        self._check(self._lib.pt_renderer_set_env_intensity(self._h, float(v)))

    def set_exposure_value(self, v):
        self._check(self._lib.pt_renderer_set_exposure_value(self._h, float(v)))

    def set_camera_index(self, i):
        self._check(self._lib.pt_renderer_set_camera_index(self._h, int(i)))

    def commit(self):
        self._check(self._lib.pt_renderer_commit(self._h))

    def render(self, frames=1):
        """update + render: `frames` progressive frames of 1 sample per pixel."""
        self._check(self._lib.pt_renderer_render(self._h, int(frames)))

    def reset(self):
        self._check(self._lib.pt_renderer_reset(self._h))

    def load_accumulation(self, accum, albedo, normal, frame_index):
        """Resumes from saved (H, W, 4) float32 accum / albedo / normal images
        holding `frame_index` frames (image() and stats().frame_index of the
        saved renderer); later frames continue bit-identically."""
        imgs = [np.ascontiguousarray(a, np.float32) for a in (accum, albedo, normal)]
        for a in imgs:
            if a.shape != (self.height, self.width, 4):
                raise ValueError(f"image shape {a.shape} != {(self.height, self.width, 4)}")
        self._check(self._lib.pt_renderer_load_accumulation(self._h, *(a.ctypes.data for a in imgs),
                                                            int(frame_index)))

    def wait_idle(self):
        self._check(self._lib.pt_renderer_wait_idle(self._h))

    def save_images(self, prefix):
        """Writes <prefix>_color/_albedo/_normal.pfm and <prefix>_final.ppm."""
        self._check(self._lib.pt_renderer_save_images(self._h, str(prefix).encode()))

    # -- read-back -----------------------------------------------------------
    def image(self, which=abi.IMAGE_ACCUM):
        if which == abi.IMAGE_FINAL:
            out = np.empty((self.height, self.width, 4), np.uint8)
        else:
            out = np.empty((self.height, self.width, 4), np.float32)
        self._check(self._lib.pt_renderer_read_image(self._h, which, out.ctypes.data, out.nbytes))
        return out

    def image_into(self, which, ptr, nbytes):
        """Copies one image into memory at address `ptr` (host, or device
        memory of the renderer's device, e.g. a torch tensor's data_ptr())."""
        self._check(self._lib.pt_renderer_read_image(self._h, which, C.c_void_p(ptr), int(nbytes)))

    def load_accumulation_ptr(self, accum_ptr, albedo_ptr, normal_ptr, frame_index):
        """load_accumulation from raw addresses (host or device memory), each
        W * H float4."""
        self._check(self._lib.pt_renderer_load_accumulation(self._h, C.c_void_p(accum_ptr), C.c_void_p(albedo_ptr),
                                                            C.c_void_p(normal_ptr), int(frame_index)))

    def samples(self):
        """Per-path radiance (n, 3) and hit-sequence hash (n,) of the last render
        (needs keep_samples); path k is frame k // (W*H), pixel k % (W*H)."""
        n = self.stats().paths
        rad = np.empty((n, 3), np.float32)
        hsh = np.empty((n,), np.uint32)
        self._check(self._lib.pt_renderer_read_image(self._h, abi.IMAGE_SAMPLE_RADIANCE, rad.ctypes.data, rad.nbytes))
        self._check(self._lib.pt_renderer_read_image(self._h, abi.IMAGE_SAMPLE_HASH, hsh.ctypes.data, hsh.nbytes))
        return rad, hsh

    def read_samples(self, paths):
        """Per-path radiance (n, 3) and hash (n,) of the last render call for the
        path indices `paths` (k = frame_local * W * H + pixel), gathered on the
        device (needs keep_samples)."""
        idx = np.ascontiguousarray(paths, np.uint64)
        rad = np.empty((len(idx), 3), np.float32)
        hsh = np.empty((len(idx),), np.uint32)
        self._check(self._lib.pt_renderer_read_samples(self._h, idx.ctypes.data, len(idx), rad.ctypes.data,
                                                       hsh.ctypes.data))
        return rad, hsh

    def set_bvh_build(self, mode):
        """abi.BVH_BUILD_SAH (default) or abi.BVH_BUILD_FAST for the next commit()."""
        self._check(self._lib.pt_renderer_set_bvh_build(self._h, int(mode)))

    def set_tail_paths(self, paths):
        """Live paths at or below which a wave's remaining bounces run as one
        kernel (0: never; abi.TAIL_PATHS_AUTO: chosen from the scene, the
        default); the images do not depend on it."""
        self._check(self._lib.pt_renderer_set_tail_paths(self._h, int(paths)))

    def set_traversal_limits(self, stack_entries=0, max_visits=0):
        """Traversal stack entries (1..96) and node visits per ray; 0 = default."""
        self._check(self._lib.pt_renderer_set_traversal_limits(self._h, int(stack_entries), int(max_visits)))

    def stats(self):
        s = abi.Stats()
        self._check(self._lib.pt_renderer_get_stats(self._h, C.byref(s)))
        return s

    def set_radiance_cache(self, enable=True, **options):
        """Attaches a new online radiance cache (options: pt_cache_config
        fields) or, with enable=False, detaches it (plain unbiased tracer)."""
        cfg = _cache_config(**options) if enable else None
        self._check(self._lib.pt_renderer_set_radiance_cache(self._h, C.byref(cfg) if cfg is not None else None))

    def set_profiling(self, flags):
        """abi.PROFILE_TRACE_TIMING | abi.PROFILE_COUNT | abi.PROFILE_HOST_LOOP, or 0
        (0: each wave's bounces run as one CUDA graph launch)."""
        self._check(self._lib.pt_renderer_set_profiling(self._h, int(flags)))

    def stream(self):
        p = C.c_void_p()
        self._check(self._lib.pt_renderer_get_stream(self._h, C.byref(p)))
        return p.value or 0

    def trace_rays(self, rays, any_hit=False, brute_force=False):
        """rays (n, 8) float32: origin, tmin, direction, tmax -> hits (n, 4) uint32."""
        rays = np.ascontiguousarray(rays, np.float32)
        hits = np.empty((len(rays), 4), np.uint32)
        self._check(self._lib.pt_renderer_trace_rays(self._h, rays.ctypes.data_as(C.POINTER(C.c_float)),
                                                     len(rays), int(any_hit), int(brute_force),
                                                     hits.ctypes.data_as(C.POINTER(C.c_uint32))))
        return hits


def renderer_for(scene, bvh_build=None, **cfg_over):
    """Creates, fills and commits a renderer for a procedural scene, in the
    order of src/bin/hala-pathtracer.rs:128-213 (`bvh_build`: the BVH
    builder, abi.BVH_BUILD_SAH by default)."""
    r = Renderer(scene.config(**cfg_over))
    if bvh_build is not None:
        r.set_bvh_build(bvh_build)
    r.set_scene(scene)
    if getattr(scene, "blue_noise", None) is not None:
        r.set_blue_noise(scene.blue_noise)
    if scene.env_rgb is not None:
        r.set_envmap(scene.env_rgb, scene.env_rotation_deg)
    else:
        r.set_ground_color(scene.ground_color)
        r.set_sky_color(scene.sky_color)
    r.set_env_intensity(scene.env_intensity)
    r.set_exposure_value(scene.exposure_value)
    r.commit()
    return r


def read_gltf(path):
    """A glTF 2.0 scene through the library's own reader (pt_gltf_load), copied
    out as a scenes.Scene: meshes (vertices, indices, column-major transform,
    material), materials, lights, cameras and textures, plus `skipped_images`
    (the number of images that were not PNG)."""
    lib = load_library()
    h = C.c_void_p()
    err = C.create_string_buffer(512)
    st = lib.pt_gltf_load(str(path).encode(), C.byref(h), err, 512)
    if st != abi.PT_OK:
        raise PTError(st, err.value.decode())
    try:
        d = lib.pt_gltf_scene_desc(h).contents
        s = scenes.Scene(os.path.splitext(os.path.basename(str(path)))[0])
        for k in range(d.num_primitives):
            p = d.primitives[k]
            v = np.ctypeslib.as_array(p.vertices, (p.num_vertices * 11,)).reshape(-1, 11).copy() \
                if p.num_vertices else np.zeros((0, 11), np.float32)
            i = np.ctypeslib.as_array(p.indices, (p.num_indices,)).copy() if p.num_indices else np.zeros(0, np.uint32)
            s.meshes.append((v, i, np.array(list(p.transform), np.float32), int(p.material_index)))
        s.materials = [abi.Material.from_buffer_copy(d.materials[k]) for k in range(d.num_materials)]
        s.lights = [abi.Light.from_buffer_copy(d.lights[k]) for k in range(d.num_lights)]
        s.cameras = [abi.Camera.from_buffer_copy(d.cameras[k]) for k in range(d.num_cameras)]
        for k in range(d.num_textures):
            t = d.textures[k]
            s.textures.append(np.ctypeslib.as_array(t.rgba, (t.height * t.width * 4,)).reshape(t.height, t.width, 4)
                              .copy())
        s.skipped_images = int(lib.pt_gltf_skipped_images(h))
        return s
    finally:
        lib.pt_gltf_free(h)


def read_png_rgba8(path):
    """(H, W, 4) uint8 texels of an 8-bit PNG through the library's own
    reader (pt_png_read_rgba8)."""
    lib = load_library()
    w, h = C.c_uint32(), C.c_uint32()
    err = C.create_string_buffer(256)
    st = lib.pt_png_read_rgba8(str(path).encode(), None, 0, C.byref(w), C.byref(h), err, 256)
    if st != abi.PT_OK:
        raise PTError(st, err.value.decode())
    out = np.empty((h.value, w.value, 4), np.uint8)
    st = lib.pt_png_read_rgba8(str(path).encode(), out.ctypes.data, out.size, C.byref(w), C.byref(h), err, 256)
    if st != abi.PT_OK:
        raise PTError(st, err.value.decode())
    return out


def read_exr(path):
    """(H, W, 3) float32 pixels of an OpenEXR file through the library's own
    reader (pt_exr_read_rgb)."""
    lib = load_library()
    w, h = C.c_uint32(), C.c_uint32()
    err = C.create_string_buffer(256)
    st = lib.pt_exr_read_rgb(str(path).encode(), None, 0, C.byref(w), C.byref(h), err, 256)
    if st != abi.PT_OK:
        raise PTError(st, err.value.decode())
    out = np.empty((h.value, w.value, 3), np.float32)
    st = lib.pt_exr_read_rgb(str(path).encode(), out.ctypes.data, out.size, C.byref(w), C.byref(h), err, 256)
    if st != abi.PT_OK:
        raise PTError(st, err.value.decode())
    return out


def _cache_config(**kw):
    cfg = abi.CacheConfig()
    load_library().pt_cache_config_default(C.byref(cfg))
    for k, v in kw.items():
        if not hasattr(cfg, k):
            raise TypeError(f"unknown radiance-cache option {k}")
        setattr(cfg, k, v)
    return cfg
