"""ctypes mirror of include/hala_pt.h (the C ABI of the GB300 path tracer).

The struct layouts follow shaders/src/hala-pathtracer/inc/types.glsl of the
reference (Camera :2-11, Light :14-39, Medium :42-49, Material :52-83,
Vertex/Primitive :86-110) field by field.
"""
import ctypes as C

PT_OK = 0
PT_ERR_INVALID_ARG = 1
PT_ERR_OOM = 2
PT_ERR_CUDA = 3
PT_ERR_TIMEOUT = 4
PT_ERR_NOT_READY = 5
PT_ERR_UNSUPPORTED = 6
PT_ERR_STATE = 7
PT_ERR_CANCELLED = 8
PT_ERR_TRAVERSAL = 9

STATUS_NAMES = {
    0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "CUDA_ERROR", 4: "TIMEOUT",
    5: "NOT_READY", 6: "UNSUPPORTED", 7: "BAD_STATE", 8: "CANCELLED", 9: "TRAVERSAL_LIMIT",
}

PT_MAX_CAMERAS = 8
PT_MAX_LIGHTS = 16
PT_INVALID_INDEX = 0xFFFFFFFF
PT_BLUE_NOISE_SIZE = 1024

LIGHT_POINT, LIGHT_DIRECTIONAL, LIGHT_SPOT, LIGHT_QUAD, LIGHT_SPHERE = 0, 1, 2, 3, 4
MEDIUM_NONE, MEDIUM_ABSORB, MEDIUM_SCATTER, MEDIUM_EMISSIVE = 0, 1, 2, 3
MATERIAL_DIFFUSE, MATERIAL_DISNEY = 0, 1
CAMERA_PERSPECTIVE, CAMERA_ORTHOGRAPHIC = 0, 1

IMAGE_ACCUM, IMAGE_ALBEDO, IMAGE_NORMAL, IMAGE_FINAL = 0, 1, 2, 3
IMAGE_SAMPLE_RADIANCE, IMAGE_SAMPLE_HASH = 4, 5

FEATURE_MEDIUM, FEATURE_VOL_MIS, FEATURE_TRANSPARENT = 1, 2, 4

HIT_MISS = 0xFFFFFFFF
HIT_LIGHT_BIT = 0x80000000

F3 = C.c_float * 3


class Camera(C.Structure):
    _fields_ = [("position", F3), ("right", F3), ("up", F3), ("forward", F3),
                ("yfov", C.c_float), ("focal_distance_or_xmag", C.c_float),
                ("aperture_or_ymag", C.c_float), ("type", C.c_uint32)]


class Light(C.Structure):
    _fields_ = [("intensity", F3), ("position", F3), ("u", F3), ("v", F3),
                ("radius", C.c_float), ("area", C.c_float), ("type", C.c_int32)]


class Medium(C.Structure):
    _fields_ = [("color", F3), ("density", C.c_float), ("anisotropy", C.c_float),
                ("type", C.c_uint32)]


class Material(C.Structure):
    _fields_ = [("medium", Medium), ("base_color", F3), ("opacity", C.c_float),
                ("emission", F3), ("anisotropic", C.c_float), ("metallic", C.c_float),
                ("roughness", C.c_float), ("subsurface", C.c_float),
                ("specular_tint", C.c_float), ("sheen", C.c_float), ("sheen_tint", C.c_float),
                ("clearcoat", C.c_float), ("clearcoat_roughness", C.c_float),
                ("clearcoat_tint", F3), ("specular_transmission", C.c_float),
                ("ior", C.c_float), ("ax", C.c_float), ("ay", C.c_float),
                ("base_color_map_index", C.c_uint32), ("normal_map_index", C.c_uint32),
                ("metallic_roughness_map_index", C.c_uint32),
                ("emission_map_index", C.c_uint32), ("type", C.c_uint32)]


class Primitive(C.Structure):
    _fields_ = [("vertices", C.POINTER(C.c_float)), ("num_vertices", C.c_uint32),
                ("indices", C.POINTER(C.c_uint32)), ("num_indices", C.c_uint32),
                ("transform", C.c_float * 16), ("material_index", C.c_uint32)]


class Texture(C.Structure):
    _fields_ = [("rgba", C.POINTER(C.c_float)), ("width", C.c_uint32), ("height", C.c_uint32)]


class SceneDesc(C.Structure):
    _fields_ = [("primitives", C.POINTER(Primitive)), ("num_primitives", C.c_uint32),
                ("materials", C.POINTER(Material)), ("num_materials", C.c_uint32),
                ("lights", C.POINTER(Light)), ("num_lights", C.c_uint32),
                ("cameras", C.POINTER(Camera)), ("num_cameras", C.c_uint32),
                ("textures", C.POINTER(Texture)), ("num_textures", C.c_uint32)]


class TracerConfig(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("max_depth", C.c_uint32),
                ("rr_depth", C.c_uint32), ("enable_tonemap", C.c_int32),
                ("enable_aces", C.c_int32), ("use_simple_aces", C.c_int32),
                ("seed", C.c_uint32), ("max_samples", C.c_uint64),
                ("wave_paths", C.c_uint32), ("keep_samples", C.c_uint32)]


class Stats(C.Structure):
    _fields_ = [("frame_index", C.c_uint64), ("paths", C.c_uint64),
                ("closest_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("render_ms", C.c_double), ("trace_ms", C.c_double),
                ("bvh_build_ms", C.c_double), ("bvh_nodes", C.c_uint64),
                ("triangles", C.c_uint64), ("features", C.c_uint32),
                ("max_bounces_seen", C.c_uint32), ("trace_launches", C.c_uint64),
                ("trav_nodes", C.c_uint64), ("trav_tris", C.c_uint64),
                ("kernel_launches", C.c_uint64), ("cache_queries", C.c_uint64),
                ("cache_train_samples", C.c_uint64), ("cache_train_steps", C.c_uint64),
                ("cache_loss", C.c_double), ("wave_paths", C.c_uint64),
                ("bvh_binary_nodes", C.c_uint64)]


class CacheConfig(C.Structure):
    _fields_ = [("query_depth", C.c_uint32), ("train_shift", C.c_uint32), ("batch_size", C.c_uint32),
                ("log2_table_size", C.c_uint32), ("learning_rate", C.c_float),
                ("min_resolution", C.c_uint32), ("max_resolution", C.c_uint32), ("seed", C.c_uint32),
                ("warmup_frames", C.c_uint32), ("paths_per_pass", C.c_uint32), ("steps_per_pass", C.c_uint32),
                ("weight_grad_kernel", C.c_uint32), ("min_roughness", C.c_float)]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_jobs", C.c_uint32),
                ("wave_paths", C.c_uint32), ("quantum_paths", C.c_uint32),
                ("use_graphs", C.c_uint32), ("fail_admission_of_job", C.c_uint64)]


class JobDesc(C.Structure):
    _fields_ = [("scene", C.POINTER(SceneDesc)), ("config", TracerConfig),
                ("frames", C.c_uint32), ("camera_index", C.c_uint32),
                ("env_rgb", C.POINTER(C.c_float)), ("env_width", C.c_uint32),
                ("env_height", C.c_uint32), ("env_rotation_deg", C.c_float),
                ("ground_color", C.c_float * 4), ("sky_color", C.c_float * 4),
                ("env_intensity", C.c_float), ("exposure_value", C.c_float),
                ("cache", C.c_void_p)]


class JobInfo(C.Structure):
    _fields_ = [("id", C.c_uint64), ("state", C.c_int32), ("status", C.c_int32),
                ("paths_total", C.c_uint64), ("paths_done", C.c_uint64),
                ("device_bytes", C.c_uint64), ("submit_ms", C.c_double),
                ("admit_ms", C.c_double), ("done_ms", C.c_double), ("error", C.c_char * 128)]


class ServerStats(C.Structure):
    _fields_ = [("jobs_submitted", C.c_uint64), ("jobs_done", C.c_uint64),
                ("jobs_failed", C.c_uint64), ("jobs_cancelled", C.c_uint64),
                ("jobs_rejected", C.c_uint64), ("jobs_queued", C.c_uint32),
                ("jobs_running", C.c_uint32), ("resident_bytes", C.c_uint64),
                ("peak_resident_bytes", C.c_uint64), ("wavefronts", C.c_uint64),
                ("paths", C.c_uint64), ("closest_rays", C.c_uint64),
                ("shadow_rays", C.c_uint64), ("kernel_launches", C.c_uint64),
                ("graph_launches", C.c_uint64), ("busy_ms", C.c_double),
                ("uptime_ms", C.c_double)]


JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_FAILED, JOB_CANCELLED = range(5)
JOB_STATE_NAMES = {0: "queued", 1: "running", 2: "done", 3: "failed", 4: "cancelled"}

PROFILE_TRACE_TIMING = 1
PROFILE_COUNT = 2
PROFILE_HOST_LOOP = 4
NOALLOC_MAX_TRIANGLES = 65536
BVH_BUILD_SAH, BVH_BUILD_FAST = 0, 1
TAIL_PATHS_AUTO = 0xFFFFFFFF


def make_config(width, height, max_depth=8, rr_depth=0, enable_tonemap=True, enable_aces=True,
                use_simple_aces=False, seed=0, max_samples=0, wave_paths=0, keep_samples=False):
    cfg = TracerConfig()
    cfg.width, cfg.height = int(width), int(height)
    cfg.max_depth, cfg.rr_depth = int(max_depth), int(rr_depth)
    cfg.enable_tonemap = 1 if enable_tonemap else 0
    cfg.enable_aces = 1 if enable_aces else 0
    cfg.use_simple_aces = 1 if use_simple_aces else 0
    cfg.seed = int(seed)
    cfg.max_samples = int(max_samples)
    cfg.wave_paths = int(wave_paths)
    cfg.keep_samples = 1 if keep_samples else 0
    return cfg


# The exported symbols of libhalapt.so with their ctypes signatures.
RENDERER_SIGNATURES = {
    "pt_renderer_create": (C.c_int, [C.POINTER(TracerConfig), C.POINTER(C.c_void_p)]),
    "pt_renderer_destroy": (None, [C.c_void_p]),
    "pt_renderer_last_error": (C.c_char_p, [C.c_void_p]),
    "pt_renderer_set_scene": (C.c_int, [C.c_void_p, C.POINTER(SceneDesc)]),
    "pt_renderer_set_envmap": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_uint32,
                                         C.c_uint32, C.c_float]),
    "pt_renderer_set_envmap_file": (C.c_int, [C.c_void_p, C.c_char_p, C.c_float]),
    "pt_renderer_set_scene_file": (C.c_int, [C.c_void_p, C.c_char_p]),
    "pt_renderer_load_blue_noise_texture": (C.c_int, [C.c_void_p, C.c_char_p]),
    "pt_renderer_set_blue_noise": (C.c_int, [C.c_void_p, C.c_void_p]),
    "pt_png_read_rgba8": (C.c_int, [C.c_char_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_uint32),
                                    C.POINTER(C.c_uint32), C.c_char_p, C.c_size_t]),
    "pt_gltf_load": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p), C.c_char_p, C.c_size_t]),
    "pt_gltf_scene_desc": (C.POINTER(SceneDesc), [C.c_void_p]),
    "pt_gltf_skipped_images": (C.c_uint32, [C.c_void_p]),
    "pt_gltf_free": (None, [C.c_void_p]),
    "pt_exr_read_rgb": (C.c_int, [C.c_char_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_uint32),
                                  C.POINTER(C.c_uint32), C.c_char_p, C.c_size_t]),
    "pt_renderer_set_ground_color": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "pt_renderer_set_sky_color": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "pt_renderer_set_env_intensity": (C.c_int, [C.c_void_p, C.c_float]),
    "pt_renderer_set_exposure_value": (C.c_int, [C.c_void_p, C.c_float]),
    "pt_renderer_set_camera_index": (C.c_int, [C.c_void_p, C.c_uint32]),
    "pt_renderer_commit": (C.c_int, [C.c_void_p]),
    "pt_renderer_render": (C.c_int, [C.c_void_p, C.c_uint32]),
    "pt_renderer_reset": (C.c_int, [C.c_void_p]),
    "pt_renderer_load_accumulation": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64]),
    "pt_renderer_read_image": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]),
    "pt_renderer_save_images": (C.c_int, [C.c_void_p, C.c_char_p]),
    "pt_renderer_wait_idle": (C.c_int, [C.c_void_p]),
    "pt_renderer_get_stats": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    "pt_renderer_get_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "pt_renderer_set_profiling": (C.c_int, [C.c_void_p, C.c_uint32]),
    "pt_renderer_trace_rays": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_uint32,
                                         C.c_int32, C.c_int32, C.POINTER(C.c_uint32)]),
    "pt_renderer_set_bvh_build": (C.c_int, [C.c_void_p, C.c_uint32]),
    "pt_renderer_set_traversal_limits": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32]),
    "pt_renderer_set_tail_paths": (C.c_int, [C.c_void_p, C.c_uint32]),
    "pt_renderer_read_samples": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    "pt_bvh_build_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                       C.c_uint32, C.c_void_p, C.POINTER(C.c_uint32), C.c_void_p,
                                       C.c_char_p, C.c_size_t]),
    "pt_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]),
    "pt_server_destroy": (None, [C.c_void_p]),
    "pt_server_last_error": (C.c_char_p, [C.c_void_p]),
    "pt_server_submit": (C.c_int, [C.c_void_p, C.POINTER(JobDesc), C.POINTER(C.c_uint64)]),
    "pt_server_poll": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(JobInfo)]),
    "pt_server_wait": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint32]),
    "pt_server_read_image": (C.c_int, [C.c_void_p, C.c_uint64, C.c_int, C.c_void_p, C.c_size_t]),
    "pt_server_cancel": (C.c_int, [C.c_void_p, C.c_uint64]),
    "pt_server_release": (C.c_int, [C.c_void_p, C.c_uint64]),
    "pt_server_pause": (C.c_int, [C.c_void_p, C.c_int32]),
    "pt_server_get_stats": (C.c_int, [C.c_void_p, C.POINTER(ServerStats)]),
    "pt_cache_config_default": (None, [C.POINTER(CacheConfig)]),
    "pt_cache_create": (C.c_int, [C.POINTER(CacheConfig), C.POINTER(C.c_void_p)]),
    "pt_cache_destroy": (None, [C.c_void_p]),
    "pt_cache_last_error": (C.c_char_p, [C.c_void_p]),
    "pt_cache_set_bounds": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "pt_cache_num_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "pt_cache_get_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "pt_cache_set_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "pt_cache_infer": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "pt_cache_gradients": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                     C.c_void_p, C.POINTER(C.c_float)]),
    "pt_cache_train": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                 C.POINTER(C.c_float)]),
    "pt_cache_benchmark": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double)]),
    "pt_renderer_set_radiance_cache": (C.c_int, [C.c_void_p, C.POINTER(CacheConfig)]),
    "pt_material_preprocess": (None, [C.POINTER(Material)]),
    "pt_material_default": (None, [C.POINTER(Material)]),
    "pt_abi_version": (C.c_uint32, []),
}


def bind(lib, signatures):
    for name, (res, args) in signatures.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib
