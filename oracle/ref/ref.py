"""ctypes wrapper of the reference's own shaders compiled as host code.

TEST INFRASTRUCTURE ONLY: used to pin the CPU oracle against the reference
(tests/test_ref_pin.py) and to regenerate tests/golden fixtures. Available
only where the reference checkout exists (oracle/ref/build_ref.py).
"""
import ctypes as C
import importlib

import numpy as np

from . import build_ref


def available():
    return bool(build_ref.build())


def permutation(scene):
    medium = any(m.medium.type != 0 for m in scene.materials)
    transparent = any(m.opacity < 1.0 for m in scene.materials)
    if medium:
        return "medium_transparent" if transparent else "medium"
    return "transparent" if transparent else "base"


_libs = {}


def _lib(perm):
    if perm not in _libs:
        abi = importlib.import_module("hala-pathtracer_gb300.abi")
        path = build_ref.build(perms=[perm])[perm]
        L = C.CDLL(path)
        P = C.c_void_p
        for name, res, args in [
            ("ref_create", P, [C.POINTER(abi.TracerConfig)]),
            ("ref_destroy", None, [P]),
            ("ref_set_scene", C.c_int, [P, C.POINTER(abi.SceneDesc)]),
            ("ref_set_envmap", C.c_int, [P, C.POINTER(C.c_float), C.c_uint32, C.c_uint32, C.c_float]),
            ("ref_set_colors", None, [P, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
            ("ref_set_env_intensity", None, [P, C.c_float]),
            ("ref_set_blue_noise", None, [P, C.c_void_p]),
            ("ref_set_exposure_value", None, [P, C.c_float]),
            ("ref_commit", C.c_int, [P]),
            ("ref_render", C.c_int, [P, C.c_uint32, C.c_int]),
            ("ref_read_image", C.c_int, [P, C.c_int, C.c_void_p, C.c_size_t]),
        ]:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _libs[perm] = L
    return _libs[perm]


class RefRenderer:
    """The reference's raygen/hit/miss/callable shaders run by the host harness."""

    def __init__(self, scene, **cfg_over):
        if scene.seed != 0 or cfg_over.get("seed", 0) != 0:
            raise ValueError("the reference seeds its RNG with the frame index only: use seed 0")
        self.perm = permutation(scene)
        self.L = _lib(self.perm)
        self.scene = scene
        self.cfg = scene.config(**cfg_over)
        self.h = self.L.ref_create(C.byref(self.cfg))
        self._desc = scene.desc()
        self.L.ref_set_scene(self.h, C.byref(self._desc))
        ptr, w, h = scene.env_pointer()
        if ptr is not None:
            self.L.ref_set_envmap(self.h, ptr, w, h, scene.env_rotation_deg)
        self.L.ref_set_colors(self.h, (C.c_float * 4)(*scene.ground_color), (C.c_float * 4)(*scene.sky_color))
        self.L.ref_set_env_intensity(self.h, scene.env_intensity)
        self.L.ref_set_exposure_value(self.h, scene.exposure_value)
        bn = getattr(scene, "blue_noise", None)
        if bn is not None:
            self._blue_noise = np.ascontiguousarray(bn, np.uint8)
            self.L.ref_set_blue_noise(self.h, self._blue_noise.ctypes.data)
        self.L.ref_commit(self.h)
        self.width, self.height = self.cfg.width, self.cfg.height

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_destroy(self.h)
            self.h = None

    def render(self, frames, threads=0):
        self.L.ref_render(self.h, frames, threads)

    def image(self, which=0):
        dt = np.uint8 if which == 3 else np.float32
        out = np.zeros((self.height, self.width, 4), dt)
        rc = self.L.ref_read_image(self.h, which, out.ctypes.data, out.nbytes)
        if rc != 0:
            raise RuntimeError(f"ref_read_image failed {rc}")
        return out
