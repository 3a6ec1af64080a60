"""Scene and image I/O through the GPU renderer (needs a GPU).

Scenes loaded by gltf.py and environments loaded by exr.py are rendered by
the CUDA path and compared with the oracle (per path, bit for bit) or with
the reference-generated golden images; the CLI's output files are read back
and compared with the images of the renderer calls they stand for.
"""
import base64
import importlib
import json
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REF_ASSETS = os.path.join(os.environ.get("HALA_REFERENCE", "/root/reference"), "assets")
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def io(pt):
    return {k: importlib.import_module(f"hala-pathtracer_gb300.{k}") for k in ("gltf", "exr", "png", "pfm", "config",
                                                                                "cli")}


def same_as_oracle(pt, oracle_mod, s):
    """Per-path radiance and hit sequences, then all four images, bit for bit."""
    WH = s.width * s.height
    r = pt.renderer_for(s, keep_samples=1)
    r.render(s.spp)
    rad_g, hash_g = r.samples()
    o = oracle_mod.Oracle(s)
    rad_o, hash_o = o.trace_paths(np.arange(WH), 0, s.spp)
    assert np.array_equal(hash_g, hash_o.reshape(-1)), "hit sequences differ"
    assert np.array_equal(rad_g.view(np.uint32), rad_o.reshape(-1, 3).view(np.uint32)), "radiance differs"
    o.render(s.spp)
    for which in (0, 1, 2, 3):
        a, b = r.image(which), o.image(which)
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), f"image {which} differs"
    r.close()


def loaded_copy(io, s, tmp_path):
    """s written as glTF and read back, with the tracer settings carried over."""
    p = io["gltf"].save_scene(s, str(tmp_path / s.name))
    t = io["gltf"].load_scene(p, s.width, s.height)
    t.spp, t.max_depth, t.rr_depth, t.seed = s.spp, s.max_depth, s.rr_depth, s.seed
    t.env_rgb, t.env_rotation_deg, t.env_intensity = s.env_rgb, s.env_rotation_deg, s.env_intensity
    t.ground_color, t.sky_color, t.exposure_value, t.tonemap = s.ground_color, s.sky_color, s.exposure_value, s.tonemap
    return t


@pytest.mark.parametrize("name", ["lights_icosphere", "media", "thin_lens_reinhard", "ortho_sky", "transparent"])
def test_gltf_scene_renders_on_the_gpu_like_the_oracle(pt, io, oracle_mod, tmp_path, name):
    from tests.golden import pin_scenes
    t = loaded_copy(io, pin_scenes.PIN_SCENES[name](), tmp_path)
    same_as_oracle(pt, oracle_mod, t)


def test_gltf_textures_render_on_the_gpu_like_the_oracle(pt, io, oracle_mod, tmp_path):
    """A hand-written glTF: a room of two quads, a PNG base-colour texture
    (sRGB, data URI), a metallic-roughness texture on a Disney material, a
    rectangle light from the extras, a thin-lens camera."""
    rng = np.random.default_rng(8)
    tex = rng.integers(0, 256, size=(8, 8, 4), dtype=np.uint8)
    tex[..., 3] = 255
    pth = str(tmp_path / "t.png")
    io["png"].write(pth, tex)
    uri = "data:image/png;base64," + base64.b64encode(open(pth, "rb").read()).decode()
    pos = np.array([[-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0],
                    [-1, 1, 0], [1, 1, 0], [1, 1, 2], [-1, 1, 2]], np.float32)
    uv = np.array([[0, 0], [2, 0], [2, 2], [0, 2], [0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    idx = np.array([0, 1, 2, 0, 2, 3, 4, 5, 6, 4, 6, 7], np.uint16)
    blob = pos.tobytes() + uv.tobytes() + idx.tobytes()
    doc = {
        "asset": {"version": "2.0"}, "scene": 0, "scenes": [{"nodes": [0, 1, 2, 3]}],
        "nodes": [{"mesh": 0}, {"mesh": 1},
                  {"camera": 0, "translation": [0, -3.5, 1.0], "rotation": [math.sin(math.pi / 4), 0, 0,
                                                                           math.cos(math.pi / 4)]},
                  {"extensions": {"KHR_lights_punctual": {"light": 0}}, "translation": [0, 0, 1.9],
                   "rotation": [1, 0, 0, 0]}],
        "meshes": [{"primitives": [{"attributes": {"POSITION": 0, "TEXCOORD_0": 1}, "indices": 2, "material": 0}]},
                   {"primitives": [{"attributes": {"POSITION": 0, "TEXCOORD_0": 1}, "indices": 3, "material": 1}]}],
        "materials": [{"pbrMetallicRoughness": {"baseColorFactor": [0.9, 0.8, 0.7, 1.0],
                                                "baseColorTexture": {"index": 0}}},
                      {"pbrMetallicRoughness": {"baseColorFactor": [0.6, 0.6, 0.7, 1.0], "metallicFactor": 0.8,
                                                "roughnessFactor": 0.6, "metallicRoughnessTexture": {"index": 0}},
                       "extras": {"type": "disney", "clearcoat": 0.4}}],
        "textures": [{"source": 0}], "images": [{"uri": uri}],
        "accessors": [{"bufferView": 0, "componentType": 5126, "count": 8, "type": "VEC3"},
                      {"bufferView": 1, "componentType": 5126, "count": 8, "type": "VEC2"},
                      {"bufferView": 2, "componentType": 5123, "count": 6, "type": "SCALAR"},
                      {"bufferView": 3, "componentType": 5123, "count": 6, "type": "SCALAR"}],
        "bufferViews": [{"buffer": 0, "byteOffset": 0, "byteLength": 96},
                        {"buffer": 0, "byteOffset": 96, "byteLength": 64},
                        {"buffer": 0, "byteOffset": 160, "byteLength": 12},
                        {"buffer": 0, "byteOffset": 172, "byteLength": 12}],
        "buffers": [{"byteLength": len(blob),
                     "uri": "data:application/octet-stream;base64," + base64.b64encode(blob).decode()}],
        "cameras": [{"type": "perspective", "perspective": {"yfov": 0.7},
                     "extras": {"aperture": 0.01, "focal_distance": 3.5}}],
        "extensions": {"KHR_lights_punctual": {"lights": [{"type": "point", "color": [1, 0.9, 0.8], "intensity": 6.0,
                                                           "extras": {"type": 1, "param0": 0.6, "param1": 0.4}}]}},
    }
    p = str(tmp_path / "hand.gltf")
    json.dump(doc, open(p, "w"))
    s = io["gltf"].load_scene(p, 24, 20)
    assert len(s.textures) >= 1 and s.materials[0].base_color_map_index < len(s.textures)
    s.spp, s.max_depth, s.rr_depth = 3, 6, 2
    same_as_oracle(pt, oracle_mod, s)


def test_exr_environment_renders_like_the_reference(pt, io, tmp_path):
    """The Disney pin scene's HDR sky written as a float ZIP OpenEXR and read
    back by exr.py: the GPU images equal the reference-generated golden images
    of the scene with the in-memory sky."""
    from tests.golden import pin_scenes
    s = pin_scenes.disney_ibl()
    p = str(tmp_path / "sky.exr")
    io["exr"].write(p, s.env_rgb, half=False, compression="ZIP")
    s.env_rgb = io["exr"].read_rgb(p)
    g = np.load(os.path.join(HERE, "golden", "ref_disney_ibl.npz"))
    r = pt.renderer_for(s)
    r.render(int(g["frames"]))
    for k, which in (("accum", 0), ("albedo", 1), ("normal", 2), ("final", 3)):
        assert np.array_equal(r.image(which).view(np.uint8), g[k].view(np.uint8)), k


def test_half_float_exr_environment_on_the_gpu(pt, io, oracle_mod, tmp_path):
    """A half-float RLE-free OpenEXR sky: what exr.py decodes is what both the
    GPU and the oracle render, path for path."""
    from tests.golden import pin_scenes
    s = pin_scenes.disney_ibl()
    p = str(tmp_path / "sky16.exr")
    io["exr"].write(p, s.env_rgb, half=True, compression="ZIP")
    s.env_rgb = io["exr"].read_rgb(p)
    assert np.array_equal(s.env_rgb, pin_scenes.disney_ibl().env_rgb.astype(np.float16).astype(np.float32))
    same_as_oracle(pt, oracle_mod, s)


def _read_ppm(path):
    raw = open(path, "rb").read()
    parts = raw.split(maxsplit=4)
    assert parts[0] == b"P6"
    w, h = int(parts[1]), int(parts[2])
    return np.frombuffer(parts[4], np.uint8, w * h * 3).reshape(h, w, 3)


def test_cli_output_equals_the_renderer_images(pt, io, tmp_path):
    """The reference's YAML schema end to end: a glTF scene and an EXR HDRI
    through the CLI. Each file it writes, read back, equals the image of the
    renderer calls src/bin/hala-pathtracer.rs makes for that config
    (HalaRenderer::new from the tracer section, set_scene, set_envmap with the
    rotation, set_env_intensity, set_exposure_value, commit, max_samples
    frames), bit for bit."""
    from tests.golden import pin_scenes
    s = pin_scenes.disney_ibl()
    io["gltf"].save_scene(s, str(tmp_path / "scene"))
    io["exr"].write(str(tmp_path / "sky.exr"), s.env_rgb)
    (tmp_path / "c.yaml").write_text(
        "window:\n  width: 32\n  height: 18\ntracer:\n  max_depth: 12\n  rr_depth: 4\n  exposure_value: -1.0\n"
        "  tonemap:\n    enable: true\n    enable_aces: true\n    use_simple_aces: false\n  max_samples: 2\n"
        "scene_file: ./scene.gltf\nhdri_file: ./sky.exr\nhdri_rotation: 77.8\nenv_intensity: 0.7\n"
        "ground_color: [0.0, 0.0, 0.0]\nsky_color: [0.0, 0.0, 0.0]\n")
    out = str(tmp_path / "img")
    assert io["cli"].main(["-c", str(tmp_path / "c.yaml"), "--out", out]) == 0

    cfg = io["config"].load_app_config(str(tmp_path / "c.yaml"))
    scene = io["gltf"].load_scene(str(tmp_path / "scene.gltf"), 32, 18)
    r = pt.Renderer(io["config"].tracer_config(cfg))
    r.set_scene(scene)
    r.set_envmap(io["exr"].read_rgb(str(tmp_path / "sky.exr")), 77.8)
    r.set_env_intensity(0.7)
    r.set_exposure_value(-1.0)
    r.commit()
    r.render(2)
    for suffix, which in (("_color.pfm", 0), ("_albedo.pfm", 1), ("_normal.pfm", 2)):
        got = io["pfm"].read(out + suffix)
        want = r.image(which)[..., :3]
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), suffix
    final = r.image(3)[..., :3]
    assert final.max() > 0
    png8 = np.round(io["png"].read(out + "_final.png")[..., :3] * 255.0).astype(np.uint8)  # read() gives [0, 1]
    assert np.array_equal(png8, final)
    assert np.array_equal(_read_ppm(out + "_final.ppm"), final)
    # and the scene is the one written: the same images as the in-memory scene
    s2 = pin_scenes.disney_ibl()
    s2.seed = 0
    ref = pt.renderer_for(s2)
    ref.render(2)
    a, b = ref.image(0), r.image(0)
    assert np.abs(a - b).max() <= 1e-3 * max(1.0, float(np.abs(a).max()))


@pytest.mark.skipif(not os.path.isdir(REF_ASSETS), reason="reference assets not present")
def test_reference_cornell_gltf_on_the_gpu(pt, io, oracle_mod):
    """The reference's own assets/cornell-box.gltf loaded by gltf.py, rendered
    by the GPU and by the oracle: the same paths bit for bit."""
    s = io["gltf"].load_scene(os.path.join(REF_ASSETS, "cornell-box.gltf"), 40, 30)
    s.spp, s.max_depth, s.rr_depth = 3, 8, 4
    same_as_oracle(pt, oracle_mod, s)


def test_envmap_file_entry_point(pt, io, tmp_path):
    """pt_renderer_set_envmap_file (the library's own EXR reader, for hosts
    without a Python loader) gives the images of set_envmap with exr.py's
    pixels, bit for bit; a file it cannot read is refused with the reason."""
    from tests.golden import pin_scenes
    s = pin_scenes.disney_ibl()
    p = str(tmp_path / "sky.exr")
    io["exr"].write(p, s.env_rgb, half=True, compression="ZIP")
    a = pt.renderer_for(s)
    a.set_envmap_file(p, s.env_rotation_deg)
    a.commit()
    a.render(2)
    s.env_rgb = io["exr"].read_rgb(p)
    b = pt.renderer_for(s)
    b.render(2)
    for k in (0, 1, 2, 3):
        assert np.array_equal(a.image(k).view(np.uint8), b.image(k).view(np.uint8)), k
    bad = tmp_path / "bad.exr"
    bad.write_bytes(b"not an exr")
    with pytest.raises(pt.PTError, match="not an OpenEXR"):
        a.set_envmap_file(str(bad), 0.0)


@pytest.mark.parametrize("name", ["lights_icosphere", "media", "hand"])
def test_scene_file_entry_point(pt, io, tmp_path, name):
    """pt_renderer_set_scene_file (the library's own glTF reader, for hosts
    without a Python loader) renders like set_scene with gltf.py's scene of
    the same file, bit for bit; a file it cannot read is refused with the
    reason."""
    from tests.golden import pin_scenes
    if name == "hand":
        from tests.test_gltf_c import _document
        doc, blob = _document(tmp_path)
        doc = dict(doc, buffers=[{"byteLength": len(blob), "uri": "data:application/octet-stream;base64," +
                                  base64.b64encode(blob).decode()}])
        p = str(tmp_path / "hand.gltf")
        with open(p, "w") as f:
            json.dump(doc, f)
        s = io["gltf"].load_scene(p, 48, 32)
        s.spp, s.max_depth, s.rr_depth = 2, 6, 3
    else:
        src = pin_scenes.PIN_SCENES[name]()
        p = io["gltf"].save_scene(src, str(tmp_path / name))
        s = loaded_copy(io, src, tmp_path)
    a = pt.renderer_for(s)
    a.set_scene_file(p)
    a.commit()
    a.render(s.spp)
    b = pt.renderer_for(s)
    b.render(s.spp)
    # textures decode through powf on both sides; where the two loaders'
    # texels agree exactly (every scene here on one machine) so do the images
    c = pt.read_gltf(p)
    exact = all(np.array_equal(x, y) for x, y in zip(c.textures, s.textures))
    for k in (0, 1, 2, 3):
        if exact:
            assert np.array_equal(a.image(k).view(np.uint8), b.image(k).view(np.uint8)), k
        else:
            assert np.allclose(a.image(k), b.image(k), rtol=1e-4, atol=1e-5), k
    bad = tmp_path / "bad.gltf"
    bad.write_text("{\"asset\": ")
    with pytest.raises(pt.PTError, match="bad.gltf"):
        a.set_scene_file(str(bad))
    a.close()
    b.close()
