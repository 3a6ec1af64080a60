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
