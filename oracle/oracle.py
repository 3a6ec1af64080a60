"""ctypes wrapper of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the
benchmark's CPU-baseline leg as the checker. The product package never
imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
SOURCES = [os.path.join(HERE, "pt_oracle.cpp")]
HEADERS = [os.path.join(HERE, "pt_oracle.h"), os.path.join(HERE, "vec.h"), os.path.join(HERE, "pmath.h"),
           os.path.join(HERE, "..", "include", "hala_pt.h")]


def build(force=False):
    """Compiles liboracle.so with g++ (no fast-math, no FMA contraction)."""
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    if not force and os.path.exists(LIB_PATH):
        mt = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(s) <= mt for s in SOURCES + HEADERS):
            return LIB_PATH
    tmp = LIB_PATH + ".tmp"
    import platform
    # hardware fused multiply-add where the ISA needs a flag for it (x86-64);
    # explicit std::fma only, no contraction of other expressions
    isa = ["-mfma"] if platform.machine() in ("x86_64", "AMD64") else []
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-pthread"] + isa + ["-o", tmp] + SOURCES
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        import importlib
        abi = importlib.import_module("hala-pathtracer_gb300.abi")
        path = build()
        L = C.CDLL(path)
        P = C.c_void_p
        sig = {
            "or_create": (P, [C.POINTER(abi.TracerConfig)]),
            "or_destroy": (None, [P]),
            "or_set_scene": (C.c_int, [P, C.POINTER(abi.SceneDesc)]),
            "or_set_envmap": (C.c_int, [P, C.POINTER(C.c_float), C.c_uint32, C.c_uint32, C.c_float]),
            "or_set_ground_color": (None, [P, C.POINTER(C.c_float)]),
            "or_set_sky_color": (None, [P, C.POINTER(C.c_float)]),
            "or_set_env_intensity": (None, [P, C.c_float]),
            "or_set_exposure_value": (None, [P, C.c_float]),
            "or_set_camera_index": (None, [P, C.c_uint32]),
            "or_set_blue_noise": (None, [P, C.c_void_p]),
            "or_commit": (C.c_int, [P]),
            "or_features": (C.c_uint32, [P]),
            "or_render": (C.c_int, [P, C.c_uint32, C.c_int]),
            "or_render_fp64": (C.c_int, [P, C.c_uint32, C.c_int]),
            "or_reset": (None, [P]),
            "or_read_image": (C.c_int, [P, C.c_int, C.c_void_p, C.c_size_t]),
            "or_trace_paths": (C.c_int, [P, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint32), C.c_uint32,
                                         C.POINTER(C.c_float), C.POINTER(C.c_uint32), C.c_int]),
            "or_set_brute": (None, [P, C.c_int]),
            "or_trace_path_rays": (C.c_int, [P, C.c_uint32, C.c_uint32, C.POINTER(C.c_float), C.c_uint32,
                                             C.POINTER(C.c_uint32)]),
            "or_trace_rays": (C.c_int, [P, C.POINTER(C.c_float), C.c_uint32, C.c_int, C.c_int,
                                        C.POINTER(C.c_uint32), C.c_int]),
            "or_counters": (None, [P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                   C.POINTER(C.c_uint64)]),
            "or_pcg4d": (None, [C.POINTER(C.c_uint32)]),
            "or_rand_seq": (None, [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.c_float)]),
            "or_blue_noise": (None, [C.c_uint32, C.c_uint32, C.POINTER(C.c_float)]),
            "or_bsdf_eval": (None, [C.c_int, C.POINTER(abi.Material), C.POINTER(C.c_float), C.c_float,
                                    C.c_uint32, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                    C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float)]),
            "or_bsdf_sample": (None, [C.c_int, C.POINTER(abi.Material), C.POINTER(C.c_float), C.c_float,
                                      C.c_uint32, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                      C.POINTER(C.c_uint32), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                      C.POINTER(C.c_float), C.POINTER(C.c_uint32)]),
            "or_pmath": (None, [C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                C.c_uint32]),
            "or_tonemap": (None, [C.POINTER(C.c_float), C.c_float, C.c_int, C.c_int, C.c_int,
                                  C.POINTER(C.c_float)]),
        }
        for k, (r, a) in sig.items():
            f = getattr(L, k)
            f.restype = r
            f.argtypes = a
        _lib = L
    return _lib


def pmath(fn, x, y=None):
    """Evaluates the oracle's portable float32 function `fn` (see or_pmath)."""
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(np.zeros_like(x) if y is None else y, np.float32)
    out = np.empty_like(x)
    lib().or_pmath(fn, _fp(x), _fp(y), _fp(out), len(x))
    return out


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _up(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


class Oracle:
    """CPU oracle renderer for one scene (same operator surface as the GPU)."""

    def __init__(self, scene, **cfg_over):
        L = lib()
        self.scene = scene
        self.cfg = scene.config(**cfg_over)
        self.h = L.or_create(C.byref(self.cfg))
        if not self.h:
            raise ValueError("or_create failed")
        self._desc = scene.desc()
        rc = L.or_set_scene(self.h, C.byref(self._desc))
        if rc != 0:
            raise ValueError(f"or_set_scene failed: {rc}")
        ptr, w, h = scene.env_pointer()
        if ptr is not None:
            L.or_set_envmap(self.h, ptr, w, h, scene.env_rotation_deg)
        g = (C.c_float * 4)(*scene.ground_color)
        s = (C.c_float * 4)(*scene.sky_color)
        L.or_set_ground_color(self.h, g)
        L.or_set_sky_color(self.h, s)
        L.or_set_env_intensity(self.h, scene.env_intensity)
        L.or_set_exposure_value(self.h, scene.exposure_value)
        bn = getattr(scene, "blue_noise", None)
        if bn is not None:
            self._blue_noise = np.ascontiguousarray(bn, np.uint8)
            assert self._blue_noise.shape == (1024, 1024, 4)
            L.or_set_blue_noise(self.h, self._blue_noise.ctypes.data)
        import time
        t0 = time.perf_counter()
        rc = L.or_commit(self.h)
        self.commit_s = time.perf_counter() - t0  # CPU BVH build (+ environment tables)
        if rc != 0:
            raise ValueError(f"or_commit failed: {rc}")
        self.width, self.height = self.cfg.width, self.cfg.height

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_destroy(self.h)
            self.h = None

    @property
    def features(self):
        return lib().or_features(self.h)

    def render(self, frames, threads=0, fp64=False):
        fn = lib().or_render_fp64 if fp64 else lib().or_render
        rc = fn(self.h, frames, threads)
        if rc != 0:
            raise RuntimeError(f"oracle render failed: {rc}")

    def reset(self):
        lib().or_reset(self.h)

    def image(self, which=0):
        n = self.width * self.height
        if which == 3:
            out = np.zeros((self.height, self.width, 4), np.uint8)
        else:
            out = np.zeros((self.height, self.width, 4), np.float32)
        rc = lib().or_read_image(self.h, which, out.ctypes.data, out.nbytes)
        if rc != 0:
            raise RuntimeError(f"read_image failed {rc}")
        return out

    def trace_paths(self, pixels, first_frame, nframes, threads=0):
        pixels = np.ascontiguousarray(pixels, np.uint32)
        rad = np.zeros((nframes, len(pixels), 3), np.float32)
        hsh = np.zeros((nframes, len(pixels)), np.uint32)
        rc = lib().or_trace_paths(self.h, first_frame, nframes, _up(pixels), len(pixels), _fp(rad),
                                  _up(hsh), threads)
        if rc != 0:
            raise RuntimeError(f"trace_paths failed {rc}")
        return rad, hsh

    def path_rays(self, pixel, frame):
        """The rays one path traces, in order: (n, 11) float32 rows of origin,
        tmin, direction, tmax, kind (0 closest hit, 1 any hit), result bits
        (hit id or occluded), t."""
        cap = 4096
        out = np.zeros((cap, 11), np.float32)
        n = C.c_uint32()
        rc = lib().or_trace_path_rays(self.h, int(pixel), int(frame), _fp(out), cap, C.byref(n))
        if rc != 0:
            raise RuntimeError(f"trace_path_rays failed {rc}")
        return out[:min(n.value, cap)]

    def set_brute_force(self, on=True):
        """Trace paths against every triangle instead of the BVH."""
        lib().or_set_brute(self.h, 1 if on else 0)

    def trace_rays(self, rays, any_hit=False, brute_force=False, threads=0):
        rays = np.ascontiguousarray(rays, np.float32)
        hits = np.zeros((len(rays), 4), np.uint32)
        rc = lib().or_trace_rays(self.h, _fp(rays), len(rays), int(any_hit), int(brute_force),
                                 _up(hits), threads)
        if rc != 0:
            raise RuntimeError(f"trace_rays failed {rc}")
        return hits

    def counters(self):
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        lib().or_counters(self.h, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, c.value


def running_mean(rad):
    """Accumulated pixels of (frames, pixels, 3) float32 per-path radiance in
    frame order, the way pathtracer.rgen.glsl:259-278 accumulates: frame 0
    stored, then mix(a, x, 1 / (f + 1)) in float32, each operation rounded."""
    a = np.array(rad[0], np.float32, copy=True)
    one = np.float32(1.0)
    for f in range(1, rad.shape[0]):
        t = one / (np.float32(f) + one)
        a = a * (one - t) + rad[f] * t
    return a
