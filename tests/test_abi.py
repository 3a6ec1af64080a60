"""The C ABI library: it builds for sm_103a, loads, and exports every entry
point include/hala_pt.h declares (no GPU needed)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "hala_pt.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pt_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "pt_renderer_create" in syms and "pt_renderer_render" in syms
    assert len(syms) >= 20


def test_library_exports_every_declared_symbol(gpu_lib):
    for s in declared_symbols():
        assert hasattr(gpu_lib, s), f"{s} is declared but not exported"


def test_python_binding_covers_header(pt):
    from importlib import import_module
    abi = import_module("hala-pathtracer_gb300.abi")
    assert set(declared_symbols()) <= set(abi.RENDERER_SIGNATURES)


def test_material_preprocess_matches_python(gpu_lib, scenes):
    abi = scenes.abi
    for mtype in (abi.MATERIAL_DIFFUSE, abi.MATERIAL_DISNEY):
        for rough in (0.0, 0.05, 0.3, 0.77, 1.0):
            for aniso in (0.0, 0.5, 1.0):
                m = scenes.material(mtype=mtype, roughness=rough, anisotropic=aniso)
                ax, ay = m.ax, m.ay
                gpu_lib.pt_material_preprocess(C.byref(m))
                assert (m.ax, m.ay) == (ax, ay)


def test_config_validation_without_gpu(gpu_lib, scenes):
    """Invalid configs are rejected before any device work (tracer.rs:43-49)."""
    abi = scenes.abi
    h = C.c_void_p()
    bad = abi.make_config(0, 16)
    assert gpu_lib.pt_renderer_create(C.byref(bad), C.byref(h)) == abi.PT_ERR_INVALID_ARG
    bad = abi.make_config(16, 16, max_depth=2, rr_depth=3)
    assert gpu_lib.pt_renderer_create(C.byref(bad), C.byref(h)) == abi.PT_ERR_INVALID_ARG
    assert gpu_lib.pt_renderer_create(None, C.byref(h)) == abi.PT_ERR_INVALID_ARG
    assert gpu_lib.pt_abi_version() == 1


def _header_structs():
    """Field names, in order, of every struct the header defines."""
    text = open(os.path.join(ROOT, "include", "hala_pt.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for m in re.finditer(r"(?:typedef\s+)?struct\s+(pt_[a-z_]+)\s*\{(.*?)\}", text, flags=re.S):
        fields = []
        for decl in m.group(2).split(";"):
            decl = decl.strip()
            if not decl:
                continue
            # "type a, b" or "type name[3]" or "const T* name"
            names = decl.split()[-1] if "," not in decl else decl.split(None, 1)[1]
            for n in names.split(","):
                n = n.strip().lstrip("*")
                n = re.sub(r"\[.*\]", "", n)
                fields.append(n)
        out[m.group(1)] = fields
    return out


def test_python_structs_follow_the_header():
    """Every ctypes mirror of a header struct has the header's fields in the
    header's order (an appended or reordered field breaks the ABI)."""
    from importlib import import_module
    abi = import_module("hala-pathtracer_gb300.abi")
    pairs = {"pt_camera": abi.Camera, "pt_light": abi.Light, "pt_medium": abi.Medium, "pt_material": abi.Material,
             "pt_primitive": abi.Primitive, "pt_texture": abi.Texture, "pt_scene_desc": abi.SceneDesc,
             "pt_tracer_config": abi.TracerConfig, "pt_stats": abi.Stats, "pt_cache_config": abi.CacheConfig,
             "pt_server_config": abi.ServerConfig, "pt_job_desc": abi.JobDesc, "pt_job_info": abi.JobInfo,
             "pt_server_stats": abi.ServerStats}
    structs = _header_structs()
    for cname, py in pairs.items():
        assert cname in structs, cname
        py_fields = [f[0] for f in py._fields_]
        assert py_fields == structs[cname], (cname, py_fields, structs[cname])


def test_python_constants_follow_the_header():
    from importlib import import_module
    abi = import_module("hala-pathtracer_gb300.abi")
    text = open(os.path.join(ROOT, "include", "hala_pt.h")).read()
    defines = {k: int(v.rstrip("uU"), 0) for k, v in re.findall(r"#define\s+(PT_[A-Z0-9_]+)\s+(0x[0-9A-Fa-f]+u?|\d+u?)\b",
                                                                  text)}
    names = {"PT_PROFILE_TRACE_TIMING": "PROFILE_TRACE_TIMING", "PT_PROFILE_COUNT": "PROFILE_COUNT",
             "PT_PROFILE_HOST_LOOP": "PROFILE_HOST_LOOP", "PT_BVH_BUILD_SAH": "BVH_BUILD_SAH",
             "PT_BVH_BUILD_FAST": "BVH_BUILD_FAST", "PT_TAIL_PATHS_AUTO": "TAIL_PATHS_AUTO",
             "PT_NOALLOC_MAX_TRIANGLES": "NOALLOC_MAX_TRIANGLES", "PT_MAX_CAMERAS": "PT_MAX_CAMERAS",
             "PT_MAX_LIGHTS": "PT_MAX_LIGHTS", "PT_INVALID_INDEX": "PT_INVALID_INDEX"}
    for c, p in names.items():
        assert c in defines, c
        assert getattr(abi, p) == defines[c], (c, defines[c], getattr(abi, p))
    for name, value in re.findall(r"\b(PT_ERR_[A-Z_]+|PT_OK)\s*=\s*(\d+)", text):
        assert getattr(abi, name) == int(value), name
