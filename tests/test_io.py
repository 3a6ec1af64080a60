"""Scene and image I/O: OpenEXR HDRIs, PNG textures and output, the glTF
loader with the renderer's extras, and config-file path resolution. CPU only
(the renders here use the CPU oracle as the checker)."""
import importlib
import json
import math
import os
import struct
import zlib

import numpy as np
import pytest

REF_ASSETS = os.path.join(os.environ.get("HALA_REFERENCE", "/root/reference"), "assets")


@pytest.fixture(scope="module")
def exr(pt):
    return importlib.import_module("hala-pathtracer_gb300.exr")


@pytest.fixture(scope="module")
def png(pt):
    return importlib.import_module("hala-pathtracer_gb300.png")


@pytest.fixture(scope="module")
def gltf(pt):
    return importlib.import_module("hala-pathtracer_gb300.gltf")


# ----------------------------------------------------------------- OpenEXR

@pytest.mark.parametrize("half,comp", [(False, "ZIP"), (True, "ZIP"), (False, "NONE"), (True, "NONE")])
def test_exr_round_trip(exr, tmp_path, half, comp):
    rng = np.random.default_rng(1)
    img = np.exp(rng.normal(0, 2, (37, 53, 3))).astype(np.float32)  # HDR range, ragged last ZIP block
    p = str(tmp_path / "a.exr")
    exr.write(p, img, half=half, compression=comp)
    back = exr.read_rgb(p)
    want = img.astype(np.float16).astype(np.float32) if half else img
    assert back.shape == img.shape and np.array_equal(back, want)


def _rle(raw):
    out = bytearray()
    i = 0
    while i < len(raw):
        j = i
        while j < len(raw) and j - i < 127 and raw[j] == raw[i]:
            j += 1
        if j - i >= 3:
            out += struct.pack("b", j - i - 1) + raw[i:i + 1]
            i = j
        else:
            k = min(len(raw), i + 126)
            out += struct.pack("b", -(k - i)) + raw[i:k]
            i = k
    return bytes(out)


def test_exr_rle_and_raw_blocks(exr):
    """An RLE file assembled here from the format description: one FLOAT
    channel Y, predictor + byte reordering before run-length coding; the
    second line is stored raw (compressed size = raw size)."""
    W, H = 6, 2
    rows = [np.array([1, 1, 1, 2, 2, 3], np.float32), np.array([0.5] * 6, np.float32)]

    def attr(n, t, v):
        return n.encode() + b"\0" + t.encode() + b"\0" + struct.pack("<i", len(v)) + v

    hdr = struct.pack("<iI", 20000630, 2)
    hdr += attr("channels", "chlist", b"Y\0" + struct.pack("<iB3xii", 2, 0, 1, 1) + b"\0")
    hdr += attr("compression", "compression", b"\x01")
    hdr += attr("dataWindow", "box2i", struct.pack("<iiii", 0, 0, W - 1, H - 1))
    hdr += attr("displayWindow", "box2i", struct.pack("<iiii", 0, 0, W - 1, H - 1))
    hdr += attr("lineOrder", "lineOrder", b"\0") + b"\0"
    raw0 = rows[0].tobytes()
    c0 = _rle(exr._apply_predictor_reorder(raw0))
    chunk0 = struct.pack("<ii", 0, len(c0)) + c0
    chunk1 = struct.pack("<ii", 1, len(rows[1].tobytes())) + rows[1].tobytes()
    base = len(hdr) + 16
    data = hdr + struct.pack("<QQ", base, base + len(chunk0)) + chunk0 + chunk1
    ch, _ = exr.read(data)
    assert np.array_equal(ch["Y"], np.stack(rows))
    rgb = exr.read_rgb(data)
    assert rgb.shape == (H, W, 3) and np.array_equal(rgb[..., 1], np.stack(rows))


def test_exr_refuses_unsupported(exr, tmp_path):
    p = str(tmp_path / "b.exr")
    exr.write(p, np.ones((4, 4, 3), np.float32), compression="NONE")
    data = bytearray(open(p, "rb").read())
    i = data.index(b"compression\0compression\0") + len(b"compression\0compression\0") + 4
    data[i] = 4  # PIZ
    with pytest.raises(exr.ExrError, match="PIZ"):
        exr.read(bytes(data))
    with pytest.raises(exr.ExrError):
        exr.read(b"not an exr")


# ----------------------------------------------------------------- PNG

def _png_bytes(rows_filtered, W, H, depth, ctype, plte=None):
    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)
    out = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", W, H, depth, ctype, 0, 0, 0))
    if plte is not None:
        out += chunk(b"PLTE", plte)
    return out + chunk(b"IDAT", zlib.compress(rows_filtered)) + chunk(b"IEND", b"")


def _filter_rows(img_bytes, stride, bpp, ftypes):
    """Encoder side of the five PNG filters (the spec's definitions)."""
    out = bytearray()
    prev = bytes(stride)
    for y, row in enumerate(img_bytes):
        f = ftypes[y % len(ftypes)]
        enc = bytearray(stride)
        for i in range(stride):
            a = row[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            if f == 0:
                pred = 0
            elif f == 1:
                pred = a
            elif f == 2:
                pred = b
            elif f == 3:
                pred = (a + b) >> 1
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
            enc[i] = (row[i] - pred) & 0xFF
        out += bytes([f]) + enc
        prev = row
    return bytes(out)


def test_png_all_filters_rgba8_and_rgb16(png):
    rng = np.random.default_rng(2)
    img = rng.integers(0, 256, (9, 7, 4), dtype=np.uint8)
    rows = [img[y].tobytes() for y in range(9)]
    data = _png_bytes(_filter_rows(rows, 28, 4, [0, 1, 2, 3, 4]), 7, 9, 8, 6)
    got = png.read(data)
    assert np.array_equal(np.round(got * 255).astype(np.uint8), img)
    img16 = rng.integers(0, 65536, (5, 4, 3), dtype=np.uint16)
    rows = [img16[y].astype(">u2").tobytes() for y in range(5)]
    data = _png_bytes(_filter_rows(rows, 24, 6, [4, 3, 1]), 4, 5, 16, 2)
    got = png.read(data)
    assert np.array_equal(np.round(got[..., :3] * 65535).astype(np.uint16), img16)
    assert np.all(got[..., 3] == 1.0)


def test_png_palette_grey_and_writer(png, tmp_path):
    pal = bytes([255, 0, 0, 0, 255, 0, 0, 0, 255, 10, 20, 30])
    idx = np.array([[0, 1, 2, 3], [3, 2, 1, 0]], np.uint8)
    packed = [bytes([(r[0] << 6) | (r[1] << 4) | (r[2] << 2) | r[3]]) for r in idx]
    got = png.read(_png_bytes(_filter_rows(packed, 1, 1, [0]), 4, 2, 2, 3, pal))
    assert np.array_equal(np.round(got[..., :3] * 255).astype(np.uint8), np.frombuffer(pal, np.uint8).reshape(4, 3)[idx])
    img = np.random.default_rng(3).integers(0, 256, (6, 5, 3), dtype=np.uint8)
    p = str(tmp_path / "o.png")
    png.write(p, img)
    assert np.array_equal(np.round(png.read(p)[..., :3] * 255).astype(np.uint8), img)


# ----------------------------------------------------------------- glTF

def _same_scene(a, b, scenes):
    assert len(a.meshes) == len(b.meshes)
    for (va, ia, ta, ma), (vb, ib, tb, mb) in zip(a.meshes, b.meshes):
        assert np.array_equal(va, vb) and np.array_equal(ia, ib) and ma == mb
        assert np.allclose(ta, tb, atol=1e-6)
    for ma, mb in zip(a.materials, b.materials):
        assert bytes(ma) == bytes(mb)
    for la, lb in zip(a.lights, b.lights):
        assert la.type == lb.type
        for f in ("intensity", "position", "u", "v"):
            assert np.allclose(list(getattr(la, f)), list(getattr(lb, f)), rtol=1e-5, atol=1e-6), f
    for ca, cb in zip(a.cameras, b.cameras):
        for f in ("position", "right", "up", "forward"):
            assert np.allclose(list(getattr(ca, f)), list(getattr(cb, f)), atol=1e-6)
        assert (ca.type, ca.yfov, ca.focal_distance_or_xmag, ca.aperture_or_ymag) == \
               (cb.type, cb.yfov, cb.focal_distance_or_xmag, cb.aperture_or_ymag)


@pytest.mark.parametrize("name", ["lights_icosphere", "media", "thin_lens_reinhard", "ortho_sky"])
def test_gltf_round_trip(gltf, scenes, tmp_path, name, oracle_mod):
    from tests.golden import pin_scenes
    s = pin_scenes.PIN_SCENES[name]()
    p = gltf.save_scene(s, str(tmp_path / name))
    t = gltf.load_scene(p, s.width, s.height)
    _same_scene(s, t, scenes)
    # rendered by the oracle: same image up to the light round trip's rounding
    t.spp, t.max_depth, t.rr_depth, t.seed = s.spp, s.max_depth, s.rr_depth, s.seed
    t.env_rgb, t.env_rotation_deg, t.env_intensity = s.env_rgb, s.env_rotation_deg, s.env_intensity
    t.ground_color, t.sky_color, t.exposure_value, t.tonemap = s.ground_color, s.sky_color, s.exposure_value, s.tonemap
    a = oracle_mod.Oracle(s)
    a.render(s.spp)
    b = oracle_mod.Oracle(t)
    b.render(s.spp)
    ia, ib = a.image(0)[..., :3], b.image(0)[..., :3]
    assert np.abs(ia - ib).max() <= 1e-3 * max(1.0, float(np.abs(ia).max()))


def test_gltf_textures_and_extras(gltf, png, tmp_path):
    """Hand-written glTF: TRS node, data-URI PNG colour texture (sRGB),
    metallic-roughness texture, material and light extras."""
    tex = np.zeros((2, 2, 4), np.uint8)
    tex[..., :3] = [[[255, 128, 0], [0, 0, 0]], [[64, 64, 64], [255, 255, 255]]]
    tex[..., 3] = 255
    pth = str(tmp_path / "t.png")
    png.write(pth, tex)
    uri = "data:image/png;base64," + __import__("base64").b64encode(open(pth, "rb").read()).decode()
    pos = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32)
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    idx = np.array([0, 1, 2, 0, 2, 3], np.uint16)
    blob = pos.tobytes() + uv.tobytes() + idx.tobytes()
    doc = {
        "asset": {"version": "2.0"}, "scene": 0, "scenes": [{"nodes": [0, 1, 2]}],
        "nodes": [{"mesh": 0, "translation": [0, 0, 1], "rotation": [0, 0, math.sin(math.pi / 4), math.cos(math.pi / 4)],
                   "scale": [2, 2, 2]},
                  {"camera": 0, "translation": [0, 0, 5]},
                  {"extensions": {"KHR_lights_punctual": {"light": 0}}, "translation": [0, 0, 3]}],
        "meshes": [{"primitives": [{"attributes": {"POSITION": 0, "TEXCOORD_0": 1}, "indices": 2, "material": 0}]}],
        "materials": [{"pbrMetallicRoughness": {"baseColorFactor": [0.5, 1.0, 1.0, 1.0], "baseColorTexture": {"index": 0},
                                                "metallicFactor": 0.25, "roughnessFactor": 0.5,
                                                "metallicRoughnessTexture": {"index": 0}},
                       "extras": {"type": "disney", "clearcoat": 0.7, "sheen": 0.3,
                                  "medium": {"type": "scatter", "color": [0.9, 0.8, 0.7], "density": 2.0,
                                             "anisotropy": 0.4}}}],
        "textures": [{"source": 0}], "images": [{"uri": uri}],
        "accessors": [{"bufferView": 0, "componentType": 5126, "count": 4, "type": "VEC3"},
                      {"bufferView": 1, "componentType": 5126, "count": 4, "type": "VEC2"},
                      {"bufferView": 2, "componentType": 5123, "count": 6, "type": "SCALAR"}],
        "bufferViews": [{"buffer": 0, "byteOffset": 0, "byteLength": 48}, {"buffer": 0, "byteOffset": 48, "byteLength": 32},
                        {"buffer": 0, "byteOffset": 80, "byteLength": 12}],
        "buffers": [{"byteLength": len(blob), "uri": "data:application/octet-stream;base64," +
                     __import__("base64").b64encode(blob).decode()}],
        "cameras": [{"type": "perspective", "perspective": {"yfov": 0.5}, "extras": {"aperture": 0.1,
                                                                                      "focal_distance": 4.0}}],
        "extensions": {"KHR_lights_punctual": {"lights": [{"type": "point", "color": [1, 0.5, 0.25], "intensity": 2.0,
                                                           "extras": {"type": 1, "param0": 0.5, "param1": 0.25}}]}},
    }
    p = str(tmp_path / "hand.gltf")
    json.dump(doc, open(p, "w"))
    s = gltf.load_scene(p, 32, 24)
    assert (s.width, s.height) == (32, 24)
    v, i, tr, mi = s.meshes[0]
    M = np.asarray(tr).reshape(4, 4).T
    assert np.allclose(M[:3, 3], [0, 0, 1]) and np.allclose(M[:3, :3] @ [1, 0, 0], [0, 2, 0], atol=1e-6)
    assert np.allclose(v[:, 3:6], [0, 0, 1])  # smooth normals computed
    m = s.materials[0]
    assert m.type == 1 and abs(m.clearcoat - 0.7) < 1e-7 and abs(m.sheen - 0.3) < 1e-7
    assert m.medium.type == 2 and abs(m.medium.density - 2.0) < 1e-7
    col = s.textures[m.base_color_map_index]
    lin = gltf.srgb_to_linear(tex[..., :3] / 255.0)
    assert np.allclose(col[..., :3], lin * [0.5, 1.0, 1.0], atol=1e-6)
    mr = s.textures[m.metallic_roughness_map_index]
    assert np.allclose(mr[..., 2], tex[..., 2] / 255.0 * 0.25) and np.allclose(mr[..., 1], tex[..., 1] / 255.0 * 0.5)
    L = s.lights[0]
    assert L.type == 3 and abs(L.area - 0.125) < 1e-7
    assert np.allclose(list(L.intensity), np.array([1, 0.5, 0.25]) * 2.0 * 4.0 / 0.125)
    c = s.cameras[0]
    assert np.allclose(list(c.forward), [0, 0, -1]) and abs(c.aperture_or_ymag - 0.1) < 1e-7


@pytest.mark.skipif(not os.path.isdir(REF_ASSETS), reason="reference assets not present")
def test_reference_assets_load_and_render(gltf, oracle_mod):
    s = gltf.load_scene(os.path.join(REF_ASSETS, "cornell-box.gltf"), 32, 24)
    assert len(s.meshes) == 7 and len(s.lights) == 1 and len(s.cameras) == 1
    L = s.lights[0]
    assert L.type == 3 and abs(L.area - 0.47 * 0.38) < 1e-6
    assert abs(s.cameras[0].yfov - 0.2563342779540469) < 1e-7
    assert all(m.type == 0 for m in s.materials)  # Lambert: no metal, no transmission
    s.spp, s.max_depth, s.rr_depth = 2, 8, 4
    o = oracle_mod.Oracle(s)
    o.render(2)
    img = o.image(0)[..., :3]
    assert np.all(np.isfinite(img)) and img.mean() > 0
    t = gltf.load_scene(os.path.join(REF_ASSETS, "orthographic_camera.gltf"), 32, 24)
    c = t.cameras[0]
    assert c.type == 1 and abs(c.focal_distance_or_xmag - 5.107142925262451) < 1e-6
    assert t.lights[0].type == 1


def test_config_paths_resolve_like_the_reference(pt, tmp_path, monkeypatch):
    cli = importlib.import_module("hala-pathtracer_gb300.cli")
    conf = tmp_path / "conf"
    conf.mkdir()
    (tmp_path / "assets").mkdir()
    (tmp_path / "assets" / "x.gltf").write_text("{}")
    monkeypatch.chdir(tmp_path)
    assert cli.resolve("./assets/x.gltf", str(conf)) == "./assets/x.gltf"
    monkeypatch.chdir(conf)
    assert cli.resolve("./assets/x.gltf", str(conf)) == os.path.join(str(tmp_path), "./assets/x.gltf")


# ----------------------------------------------------------------- PFM

def test_pfm_round_trip_and_layout(pt, tmp_path):
    """Rows are stored bottom to top, little-endian with a negative scale."""
    pfm = importlib.import_module("hala-pathtracer_gb300.pfm")
    rng = np.random.default_rng(4)
    img = rng.normal(size=(7, 11, 3)).astype(np.float32)
    img[0, 0] = [np.inf, -0.0, np.nan]
    p = str(tmp_path / "a.pfm")
    pfm.write(p, img)
    raw = open(p, "rb").read()
    assert raw.startswith(b"PF\n11 7\n-1.0\n")
    body = np.frombuffer(raw[len(b"PF\n11 7\n-1.0\n"):], "<f4").reshape(7, 11, 3)
    assert np.array_equal(body[-1].view(np.uint32), img[0].view(np.uint32))  # top row stored last
    back = pfm.read(p)
    assert np.array_equal(back.view(np.uint32), img.view(np.uint32))
    # big-endian files (positive scale) read too
    big = b"PF\n11 7\n1.0\n" + np.ascontiguousarray(img[::-1]).astype(">f4").tobytes()
    assert np.array_equal(pfm.read(big).view(np.uint32), img.view(np.uint32))
    with pytest.raises(pfm.PfmError):
        pfm.read(b"P6\n1 1\n255\n\0\0\0")
    with pytest.raises(pfm.PfmError):
        pfm.read(raw[:-4])
