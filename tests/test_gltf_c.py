"""The library's own glTF 2.0 reader (pt_gltf_load, behind
pt_renderer_set_scene_file) against the Python loader gltf.py: the same
vertices, indices, transforms, materials, lights and cameras, bit for bit,
and the same textures, for the pin scenes written as glTF, a hand-written
document that exercises the rest of the mapping (node hierarchy, GLB and
external buffers, strided and normalized accessors, missing normals and
tangents, every light kind, orthographic camera, alpha modes, extensions,
PNG colour types and bit depths, a skipped JPEG), the reference's own
assets where the checkout is present, and malformed files. Loads
libhalapt.so on the CPU; no GPU call."""
import base64
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
def gltf(pt):
    return importlib.import_module("hala-pathtracer_gb300.gltf")


@pytest.fixture(scope="module")
def lib(pt):
    pt.build()
    return pt.load_library()


def _same(py, c):
    """Python-loaded scene `py` against the library's `c`: exact except the
    textures, where sRGB decoding calls powf (numpy's float32 power may take
    another implementation): within 2 ulp there."""
    assert len(py.meshes) == len(c.meshes)
    for (va, ia, ta, ma), (vb, ib, tb, mb) in zip(py.meshes, c.meshes):
        assert va.dtype == vb.dtype == np.float32 and np.array_equal(va, vb)
        assert np.array_equal(ia.astype(np.uint32), ib) and ma == mb
        assert np.array_equal(np.asarray(ta, np.float32), tb)
    assert [bytes(m) for m in py.materials] == [bytes(m) for m in c.materials]
    assert [bytes(x) for x in py.lights] == [bytes(x) for x in c.lights]
    assert [bytes(x) for x in py.cameras] == [bytes(x) for x in c.cameras]
    assert len(py.textures) == len(c.textures)
    for ta, tb in zip(py.textures, c.textures):
        assert ta.shape == tb.shape
        np.testing.assert_allclose(tb, ta, rtol=2.4e-7, atol=0)
    assert len(getattr(py, "skipped_images", [])) == c.skipped_images


@pytest.mark.parametrize("name", ["cornell", "disney_ibl", "lights_icosphere", "media", "transparent",
                                  "media_transparent", "ortho_sky", "thin_lens_reinhard", "no_tonemap", "textured"])
def test_pin_scenes_read_like_the_python_loader(pt, lib, gltf, tmp_path, name):
    from tests.golden import pin_scenes
    s = pin_scenes.PIN_SCENES[name]()
    p = gltf.save_scene(s, str(tmp_path / name))
    _same(gltf.load_scene(p), pt.read_gltf(p))


# ----------------------------------------------------------------- a hand-written document

def _png(pixels, depth, ctype, plte=None, trns=None):
    """PNG bytes of an (H, W, channels) integer array, filter 0 rows."""
    a = np.asarray(pixels)
    H, W = a.shape[:2]
    if depth == 16:
        rows = [a[y].astype(">u2").tobytes() for y in range(H)]
    elif depth == 8:
        rows = [a[y].astype(np.uint8).tobytes() for y in range(H)]
    else:
        rows = []
        for y in range(H):
            bits = "".join(format(int(v), f"0{depth}b") for v in a[y].reshape(-1))
            bits += "0" * (-len(bits) % 8)
            rows.append(bytes(int(bits[k:k + 8], 2) for k in range(0, len(bits), 8)))
    raw = b"".join(b"\0" + r for r in rows)

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)
    out = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", W, H, depth, ctype, 0, 0, 0))
    if plte is not None:
        out += chunk(b"PLTE", bytes(plte))
    if trns is not None:
        out += chunk(b"tRNS", bytes(trns))
    return out + chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b"")


def _uri(b, mime="application/octet-stream"):
    return f"data:{mime};base64," + base64.b64encode(b).decode()


def _document(tmp_path):
    """(doc, external buffer bytes): two meshes under a node hierarchy, four
    materials, six images, five lights, two cameras."""
    rng = np.random.default_rng(11)
    blob = bytearray()
    views, accessors = [], []

    def add(arr, ctype, typ, normalized=False, stride=0, buffer=0):
        a = np.ascontiguousarray(arr)
        while len(blob) % 4:
            blob.append(0)
        off = len(blob)
        if stride:
            item = a.itemsize * a.shape[1]
            rows = bytearray(stride * len(a))
            for k in range(len(a)):
                rows[k * stride:k * stride + item] = a[k].tobytes()
            blob.extend(rows)
        else:
            blob.extend(a.tobytes())
        v = {"buffer": buffer, "byteOffset": off, "byteLength": len(blob) - off}
        if stride:
            v["byteStride"] = stride
        views.append(v)
        acc = {"bufferView": len(views) - 1, "componentType": ctype, "count": len(a), "type": typ}
        if normalized:
            acc["normalized"] = True
        accessors.append(acc)
        return len(accessors) - 1

    # mesh 0: a displaced grid without normals or tangents, u8 normalized
    # texcoords, u16 indices
    n = 5
    xs, ys = np.meshgrid(np.linspace(-1, 1, n), np.linspace(-1, 1, n))
    pos0 = np.stack([xs, ys, 0.2 * rng.standard_normal(xs.shape)], -1).reshape(-1, 3).astype(np.float32)
    uv0 = rng.integers(0, 256, (n * n, 2)).astype(np.uint8)
    quads = [(y * n + x, y * n + x + 1, (y + 1) * n + x + 1, (y + 1) * n + x) for y in range(n - 1)
             for x in range(n - 1)]
    idx0 = np.array([[a, b, c, a, c, d] for a, b, c, d in quads], np.uint16).reshape(-1)
    # mesh 1: interleaved (strided) positions, normals and tangents, i16
    # normalized texcoords, no indices
    pos1 = rng.standard_normal((9, 3)).astype(np.float32)
    nrm1 = rng.standard_normal((9, 3)).astype(np.float32)
    nrm1 /= np.linalg.norm(nrm1, axis=1, keepdims=True)
    tan1 = np.concatenate([rng.standard_normal((9, 3)), np.ones((9, 1))], 1).astype(np.float32)
    uv1 = rng.integers(-32768, 32768, (9, 2)).astype(np.int16)
    a_pos0, a_uv0, a_idx0 = add(pos0, 5126, "VEC3"), add(uv0, 5121, "VEC2", normalized=True), add(idx0, 5123, "SCALAR")
    a_pos1 = add(pos1, 5126, "VEC3", stride=16)
    a_nrm1, a_tan1 = add(nrm1, 5126, "VEC3", stride=20), add(tan1, 5126, "VEC4")
    a_uv1 = add(uv1, 5122, "VEC2", normalized=True)

    # images: 8-bit RGBA, 16-bit RGB, palette with tRNS, 4-bit grey, grey +
    # alpha, and a JPEG the readers skip
    img8 = rng.integers(0, 256, (3, 4, 4))
    img16 = rng.integers(0, 65536, (2, 3, 3))
    pal_idx = rng.integers(0, 4, (4, 5, 1))
    plte = rng.integers(0, 256, 12).tolist()
    grey4 = rng.integers(0, 16, (3, 3, 1))
    ga = rng.integers(0, 256, (2, 2, 2))
    images = [{"uri": _uri(_png(img8, 8, 6), "image/png")},
              {"uri": _uri(_png(img16, 16, 2), "image/png")},
              {"uri": "pal tex.png"},
              {"uri": _uri(_png(grey4, 4, 0), "image/png")},
              {"uri": _uri(_png(ga, 8, 4), "image/png")},
              {"uri": _uri(b"\xff\xd8\xff\xe0 not decoded", "image/jpeg")}]
    (tmp_path / "pal tex.png").write_bytes(_png(pal_idx, 2, 3, plte, trns=[255, 0, 128]))
    textures = [{"source": k} for k in range(6)] + [{}]  # the last one has no source

    materials = [
        {"pbrMetallicRoughness": {"baseColorFactor": [0.9, 0.5, 0.25, 0.6], "baseColorTexture": {"index": 0},
                                  "metallicFactor": 0.0, "roughnessFactor": 0.7,
                                  "metallicRoughnessTexture": {"index": 1}},
         "normalTexture": {"index": 3}, "emissiveTexture": {"index": 4}, "emissiveFactor": [1.0, 0.5, 0.0],
         "extensions": {"KHR_materials_emissive_strength": {"emissiveStrength": 3.0}},
         "alphaMode": "BLEND"},
        {"pbrMetallicRoughness": {"baseColorFactor": [0.2, 0.3, 0.4, 0.3], "metallicFactor": 0.8,
                                  "roughnessFactor": 0.15, "baseColorTexture": {"index": 2}},
         "alphaMode": "MASK", "alphaCutoff": 0.25,
         "extensions": {"KHR_materials_ior": {"ior": 1.33}, "KHR_materials_transmission": {"transmissionFactor": 0.5},
                        "KHR_materials_clearcoat": {"clearcoatFactor": 0.6, "clearcoatRoughnessFactor": 0.2}},
         "extras": {"anisotropic": 0.5, "sheen_tint": 0.25, "clearcoat_tint": [0.9, 0.8, 0.7],
                    "medium": {"type": "emissive", "color": [2.0, 1.0, 0.5], "density": 0.5}}},
        {"pbrMetallicRoughness": {"baseColorTexture": {"index": 5}, "metallicFactor": 0.0},
         "emissiveTexture": {"index": 6}, "extras": {"type": "1", "roughness": 0.45, "subsurface": 0.3,
                                                       "medium": {"type": 1, "density": 4}}},
        {"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}, "baseColorFactor": [0.9, 0.5, 0.25, 1],
                                  "metallicFactor": 0},
         "extras": {"type": "lambert", "roughness": 0.3}},
    ]
    s2 = math.sqrt(0.5)
    nodes = [
        {"children": [1, 2], "translation": [0.5, -1.0, 2.0], "rotation": [0.0, 0.0, math.sin(0.3), math.cos(0.3)],
         "scale": [1.5, 1.5, 1.5]},
        {"mesh": 0, "rotation": [s2 * math.sin(0.2), 0.0, 0.0, math.cos(0.2)]},
        {"mesh": 1, "matrix": [0.5, 0, 0, 0, 0, 0.5, 0, 0, 0, 0, 0.5, 0, 1.0, 2.0, 3.0, 1]},
        {"camera": 0, "translation": [0, -6, 1], "rotation": [s2, 0, 0, s2]},
        {"camera": 1, "translation": [0, 0, 8]},
        {"extensions": {"KHR_lights_punctual": {"light": 0}}, "translation": [0, 0, 4],
         "rotation": [1.0, 0.0, 0.0, 0.0]},
        {"extensions": {"KHR_lights_punctual": {"light": 1}}, "translation": [1, 1, 3]},
        {"extensions": {"KHR_lights_punctual": {"light": 2}}, "rotation": [0.3, 0.2, 0.1, 0.927]},
        {"extensions": {"KHR_lights_punctual": {"light": 3}}, "translation": [-2, 0, 3],
         "rotation": [0.0, 0.3826834, 0.0, 0.9238795]},
        {"extensions": {"KHR_lights_punctual": {"light": 4}}, "translation": [2, 0, 3]},
    ]
    lights = [{"type": "point", "color": [1, 0.9, 0.8], "intensity": 30.0,
               "extras": {"type": 1, "param0": 0.6, "param1": 0.4}},
              {"type": "point", "intensity": 5.0, "extras": {"type": 2, "param0": 0.25}},
              {"type": "directional", "color": [1.0, 0.95, 0.9], "intensity": 2.0, "extras": {"cone_deg": 1.5}},
              {"type": "spot", "intensity": 40.0, "spot": {"innerConeAngle": 0.2, "outerConeAngle": 0.5}},
              {"type": "point", "extras": {"rgb": [3.0, 2.0, 1.0]}}]
    cameras = [{"type": "perspective", "perspective": {"yfov": 0.7, "znear": 0.01},
                "extras": {"aperture": 0.05, "focal_distance": 6.0}},
               {"type": "orthographic", "orthographic": {"xmag": 3.0, "ymag": 2.0, "znear": 0.1, "zfar": 50}}]
    doc = {"asset": {"version": "2.0"}, "scene": 0, "scenes": [{"nodes": [0, 3, 4, 5, 6, 7, 8, 9]}],
           "nodes": nodes,
           "meshes": [{"primitives": [{"attributes": {"POSITION": a_pos0, "TEXCOORD_0": a_uv0}, "indices": a_idx0,
                                       "material": 0},
                                      {"attributes": {"POSITION": a_pos0}, "indices": a_idx0, "mode": 1}]},
                      {"primitives": [{"attributes": {"POSITION": a_pos1, "NORMAL": a_nrm1, "TANGENT": a_tan1,
                                                      "TEXCOORD_0": a_uv1}, "material": 1},
                                      {"attributes": {"POSITION": a_pos1}},
                                      {"attributes": {"POSITION": a_pos0}, "indices": a_idx0, "material": 2},
                                      {"attributes": {"POSITION": a_pos1}, "material": 3}]}],
           "materials": materials, "textures": textures, "images": images,
           "accessors": accessors, "bufferViews": views, "cameras": cameras,
           "extensionsUsed": ["KHR_lights_punctual"],
           "extensions": {"KHR_lights_punctual": {"lights": lights}}}
    return doc, bytes(blob)


def test_hand_written_document_reads_like_the_python_loader(pt, lib, gltf, tmp_path):
    doc, blob = _document(tmp_path)
    # .gltf with an external buffer whose name has a space
    (tmp_path / "geo data.bin").write_bytes(blob)
    d = dict(doc, buffers=[{"byteLength": len(blob), "uri": "geo%20data.bin"}])
    p = tmp_path / "hand.gltf"
    p.write_text(json.dumps(d, indent=1))
    py, c = gltf.load_scene(str(p)), pt.read_gltf(str(p))
    _same(py, c)
    assert len(c.meshes) == 5 and len(c.materials) == 5 and len(c.lights) == 5 and len(c.cameras) == 2
    # six images: the JPEG is skipped, and the fourth material's colour map
    # is the first one's (same image and factor), baked once
    assert len(c.textures) == 5 and c.skipped_images == 1
    assert c.materials[3].base_color_map_index == c.materials[0].base_color_map_index
    assert sorted(L.type for L in c.lights) == [0, 1, 2, 3, 4]
    # the same document as .glb (JSON chunk + BIN chunk)
    d = dict(doc, buffers=[{"byteLength": len(blob)}])
    js = json.dumps(d).encode()
    js += b" " * (-len(js) % 4)
    b = blob + b"\0" * (-len(blob) % 4)
    glb = struct.pack("<4sII", b"glTF", 2, 12 + 8 + len(js) + 8 + len(b)) + struct.pack("<I4s", len(js), b"JSON") + \
        js + struct.pack("<I4s", len(b), b"BIN\0") + b
    g = tmp_path / "hand.glb"
    g.write_bytes(glb)
    _same(gltf.load_scene(str(g)), pt.read_gltf(str(g)))
    # and with the buffer as a data URI
    d = dict(doc, buffers=[{"byteLength": len(blob), "uri": _uri(blob)}])
    q = tmp_path / "inline.gltf"
    q.write_text(json.dumps(d))
    _same(gltf.load_scene(str(q)), pt.read_gltf(str(q)))


@pytest.mark.skipif(not os.path.isdir(REF_ASSETS), reason="reference assets not present")
@pytest.mark.parametrize("name", ["cornell-box.gltf", "orthographic_camera.gltf"])
def test_reference_assets_read_like_the_python_loader(pt, lib, gltf, name):
    p = os.path.join(REF_ASSETS, name)
    _same(gltf.load_scene(p), pt.read_gltf(p))


def test_malformed_files_are_refused_with_a_reason(pt, lib, tmp_path):
    import ctypes as C
    abi = importlib.import_module("hala-pathtracer_gb300.abi")

    def load(path):
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        st = lib.pt_gltf_load(str(path).encode(), C.byref(h), err, 512)
        assert not h.value
        return st, err.value.decode()

    cases = {
        "missing.gltf": None,
        "bad.gltf": "{\"asset\": {\"version\": \"2.0\"}, \"nodes\": [",
        "nocam.gltf": json.dumps({"asset": {"version": "2.0"}, "nodes": []}),
        "sparse.gltf": json.dumps({"asset": {"version": "2.0"}, "scenes": [{"nodes": [0, 1]}],
                                   "nodes": [{"mesh": 0}, {"camera": 0}], "cameras": [{"type": "perspective"}],
                                   "meshes": [{"primitives": [{"attributes": {"POSITION": 0}}]}],
                                   "accessors": [{"componentType": 5126, "count": 3, "type": "VEC3",
                                                  "sparse": {"count": 1}}]}),
        "huge.gltf": json.dumps({"asset": {"version": "2.0"}, "scenes": [{"nodes": [0, 1]}],
                                 "nodes": [{"mesh": 0}, {"camera": 0}], "cameras": [{"type": "perspective"}],
                                 "meshes": [{"primitives": [{"attributes": {"POSITION": 0}}]}],
                                 "accessors": [{"componentType": 5126, "count": 2147483647, "type": "MAT4"}]}),
        "overrun.gltf": json.dumps({"asset": {"version": "2.0"}, "scenes": [{"nodes": [0, 1]}],
                                    "nodes": [{"mesh": 0}, {"camera": 0}], "cameras": [{"type": "perspective"}],
                                    "meshes": [{"primitives": [{"attributes": {"POSITION": 0}}]}],
                                    "accessors": [{"bufferView": 0, "componentType": 5126, "count": 2147483647,
                                                   "type": "VEC3", "byteOffset": 4}],
                                    "bufferViews": [{"buffer": 0, "byteLength": 12, "byteStride": 4096}],
                                    "buffers": [{"byteLength": 12, "uri": _uri(bytes(12))}]}),
        "cycle.gltf": json.dumps({"asset": {"version": "2.0"}, "scenes": [{"nodes": [0]}],
                                  "nodes": [{"children": [1], "camera": 0}, {"children": [0]}],
                                  "cameras": [{"type": "perspective"}]}),
        "short.gltf": json.dumps({"asset": {"version": "2.0"}, "scenes": [{"nodes": [0, 1]}],
                                  "nodes": [{"mesh": 0}, {"camera": 0}], "cameras": [{"type": "perspective"}],
                                  "meshes": [{"primitives": [{"attributes": {"POSITION": 0}}]}],
                                  "accessors": [{"bufferView": 0, "componentType": 5126, "count": 3,
                                                 "type": "VEC3"}],
                                  "bufferViews": [{"buffer": 0, "byteLength": 12}],
                                  "buffers": [{"byteLength": 12, "uri": _uri(bytes(12))}]}),
    }
    for name, text in cases.items():
        p = tmp_path / name
        if text is not None:
            p.write_text(text)
        st, why = load(p)
        assert st == abi.PT_ERR_INVALID_ARG and name.split(".")[0] in why and len(why) > len(str(p)) + 2, (name, why)


def test_mutated_documents_are_read_or_refused(pt, lib, tmp_path):
    """Seeded byte mutations of the hand-written document (JSON syntax,
    numbers, indices, base64 of the buffers and PNGs): every one is either
    read or refused with PT_ERR_INVALID_ARG and a reason, never a crash."""
    import ctypes as C
    import random
    abi = importlib.import_module("hala-pathtracer_gb300.abi")
    doc, blob = _document(tmp_path)
    text = json.dumps(dict(doc, buffers=[{"byteLength": len(blob), "uri": _uri(blob)}])).encode()
    rng = random.Random(7)
    seen = {abi.PT_OK: 0, abi.PT_ERR_INVALID_ARG: 0}
    p = tmp_path / "m.gltf"
    for _ in range(400):
        b = bytearray(text)
        for _ in range(rng.randint(1, 6)):
            k = rng.randrange(len(b))
            op = rng.random()
            if op < 0.4:
                b[k] = rng.randrange(256)
            elif op < 0.6:
                del b[k:k + rng.randint(1, 16)]
            elif op < 0.8:
                b[k:k] = bytes(rng.choice(b'0123456789-.eE[]{}",:') for _ in range(rng.randint(1, 4)))
            else:
                b[k:k] = rng.choice([b"-1", b"99999999999", b"1e308", b"4294967295", b"2147483648"])
        p.write_bytes(bytes(b))
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        st = lib.pt_gltf_load(str(p).encode(), C.byref(h), err, 512)
        assert st in seen, st
        seen[st] += 1
        if st == abi.PT_OK:
            lib.pt_gltf_free(h)
        else:
            assert not h.value and err.value
    assert seen[abi.PT_OK] > 0 and seen[abi.PT_ERR_INVALID_ARG] > 0
