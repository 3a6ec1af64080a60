"""glTF 2.0 scene loader (and writer) with the renderer's custom extras:
the drop-in for `HalaScene::new(scene_file)` (src/bin/hala-pathtracer.rs:98),
whose glTF code (crate gltf 1.4.1, inside the renderer crate) is not part of
the reference checkout. The mapping below is therefore specified here:

Geometry   every TRIANGLES primitive of every mesh node of the default
           scene, in node order; POSITION, NORMAL (smooth normals when
           absent), TANGENT xyz (an orthogonal tangent when absent),
           TEXCOORD_0 (zeros when absent); the node's world matrix becomes
           the primitive transform.
Materials  pbrMetallicRoughness factors, emissiveFactor (times
           KHR_materials_emissive_strength), KHR_materials_ior,
           KHR_materials_transmission, KHR_materials_clearcoat, and alpha
           (BLEND: opacity = base alpha; MASK: 0/1 against alphaCutoff).
           Material `extras` override any pt_material field by name and
           select the model: "type" = "diffuse" | "disney" (or 0 | 1);
           without it a material is diffuse (Lambert / Oren-Nayar) unless it
           is metallic, transmissive or clear-coated. A "medium" extra
           {"type": "absorb" | "scatter" | "emissive", "color", "density",
           "anisotropy"} attaches a participating medium.
Textures   PNG images (file, data URI or buffer view). The shaders replace
           the material value with the texel (pathtracer.rgen.glsl:121-133),
           so the loader bakes glTF's factor x texture product into the map;
           colour and emission maps are converted from sRGB to linear.
Lights     KHR_lights_punctual point / spot / directional, intensity =
           colour x intensity. The extras {"type": 1, "param0": w,
           "param1": h} turn a light into a w x h rectangle emitting along
           the node's -Z axis, and {"type": 2, "param0": r} into a sphere of
           radius r; their radiance is that of a Lambertian emitter of the
           same power as the punctual light (4 pi intensity).
Cameras    perspective (yfov; extras "aperture", "focal_distance") and
           orthographic (xmag, ymag), looking along the node's -Z with +Y up.
"""
import base64
import json
import math
import os
import struct

import numpy as np

from . import abi
from . import png as pngmod
from . import scenes as sc

COMPONENT = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
NCOMP = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT4": 16}
NORM_SCALE = {5120: 127.0, 5121: 255.0, 5122: 32767.0, 5123: 65535.0}
MEDIUM_NAMES = {"absorb": abi.MEDIUM_ABSORB, "scatter": abi.MEDIUM_SCATTER, "emissive": abi.MEDIUM_EMISSIVE}


class GltfError(ValueError):
    pass


def srgb_to_linear(c):
    c = np.asarray(c, np.float32)
    return np.where(c <= 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4).astype(np.float32)


def _read_document(path):
    with open(path, "rb") as f:
        data = f.read()
    if data[:4] == b"glTF":
        _magic, _ver, _length = struct.unpack_from("<4sII", data, 0)
        pos, doc, bin_chunk = 12, None, None
        while pos < len(data):
            n, typ = struct.unpack_from("<I4s", data, pos)
            chunk = data[pos + 8:pos + 8 + n]
            pos += 8 + n
            if typ == b"JSON":
                doc = json.loads(chunk.decode("utf-8"))
            elif typ == b"BIN\0":
                bin_chunk = chunk
        if doc is None:
            raise GltfError("GLB without a JSON chunk")
        return doc, bin_chunk
    return json.loads(data.decode("utf-8")), None


def _uri_bytes(uri, base):
    if uri.startswith("data:"):
        return base64.b64decode(uri.split(",", 1)[1])
    with open(os.path.join(base, uri.replace("%20", " ")), "rb") as f:
        return f.read()


class _Doc:
    def __init__(self, path):
        self.path = path
        self.base = os.path.dirname(os.path.abspath(path))
        self.j, glb_bin = _read_document(path)
        self.buffers = []
        for i, b in enumerate(self.j.get("buffers", [])):
            if "uri" in b:
                self.buffers.append(_uri_bytes(b["uri"], self.base))
            elif i == 0 and glb_bin is not None:
                self.buffers.append(glb_bin)
            else:
                raise GltfError(f"buffer {i} has no data")

    def view_bytes(self, vi):
        v = self.j["bufferViews"][vi]
        b = self.buffers[v["buffer"]]
        off = v.get("byteOffset", 0)
        return b[off:off + v["byteLength"]], v.get("byteStride", 0)

    def accessor(self, ai):
        a = self.j["accessors"][ai]
        if "sparse" in a:
            raise GltfError("sparse accessors are not supported")
        dt = COMPONENT[a["componentType"]]
        nc = NCOMP[a["type"]]
        count = a["count"]
        item = np.dtype(dt).itemsize * nc
        if "bufferView" not in a:
            out = np.zeros((count, nc), dt)
        else:
            raw, stride = self.view_bytes(a["bufferView"])
            off = a.get("byteOffset", 0)
            if stride and stride != item:
                rows = np.frombuffer(raw, np.uint8, count=(count - 1) * stride + item, offset=off)
                rows = np.lib.stride_tricks.as_strided(rows, (count, item), (stride, 1))
                out = np.frombuffer(rows.copy().tobytes(), dt).reshape(count, nc)
            else:
                out = np.frombuffer(raw, dt, count * nc, off).reshape(count, nc)
        if a.get("normalized") and dt != np.float32:
            out = np.maximum(out.astype(np.float32) / NORM_SCALE[a["componentType"]], -1.0)
        return out


def _node_matrix(n):
    if "matrix" in n:
        return np.asarray(n["matrix"], np.float64).reshape(4, 4).T  # column-major in the file
    t = np.asarray(n.get("translation", [0, 0, 0]), np.float64)
    x, y, z, w = n.get("rotation", [0, 0, 0, 1])
    s = np.asarray(n.get("scale", [1, 1, 1]), np.float64)
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    M = np.eye(4)
    M[:3, :3] = R * s[None, :]
    M[:3, 3] = t
    return M


def _walk(doc):
    """(node index, world matrix) for every node of the default scene."""
    j = doc.j
    scenes = j.get("scenes", [])
    roots = scenes[j.get("scene", 0)]["nodes"] if scenes else list(range(len(j.get("nodes", []))))
    out = []

    def visit(i, parent):
        n = j["nodes"][i]
        M = parent @ _node_matrix(n)
        out.append((i, M))
        for c in n.get("children", []):
            visit(c, M)

    for r in roots:
        visit(r, np.eye(4))
    return out


class _Textures:
    """Loads each image once and bakes factor x texture maps on demand."""

    def __init__(self, doc, scene):
        self.doc, self.scene = doc, scene
        self.images, self.baked = {}, {}
        self.skipped = []

    def image(self, ii):
        if ii not in self.images:
            im = self.doc.j["images"][ii]
            if "uri" in im:
                data = _uri_bytes(im["uri"], self.doc.base)
            else:
                data, _ = self.doc.view_bytes(im["bufferView"])
            if not data.startswith(pngmod.SIGNATURE):
                self.images[ii] = None
                self.skipped.append(im.get("uri", f"image {ii}"))
            else:
                self.images[ii] = pngmod.read(data)
        return self.images[ii]

    def bake(self, tex_info, factor, kind):
        """kind: 'srgb' (colour/emission), 'mr' (B metallic, G roughness) or 'linear'."""
        if tex_info is None:
            return abi.PT_INVALID_INDEX
        ti = tex_info["index"]
        src = self.doc.j["textures"][ti].get("source")
        if src is None:
            return abi.PT_INVALID_INDEX
        key = (src, kind, tuple(np.round(np.asarray(factor, np.float64), 7)))
        if key not in self.baked:
            img = self.image(src)
            if img is None:
                return abi.PT_INVALID_INDEX
            t = img.copy()
            if kind == "srgb":
                t[..., :3] = srgb_to_linear(t[..., :3]) * np.asarray(factor, np.float32)[:3]
            elif kind == "mr":
                t[..., 2] *= factor[0]  # metallic in blue
                t[..., 1] *= factor[1]  # roughness in green
            self.baked[key] = self.scene.add_texture(t.astype(np.float32))
        return self.baked[key]


def _material(doc, m, tex):
    pbr = m.get("pbrMetallicRoughness", {})
    ext = m.get("extensions", {})
    extras = m.get("extras", {}) or {}
    bc = pbr.get("baseColorFactor", [1, 1, 1, 1])
    metallic = float(pbr.get("metallicFactor", 1.0))
    rough = float(pbr.get("roughnessFactor", 1.0))
    emis = np.asarray(m.get("emissiveFactor", [0, 0, 0]), np.float64)
    emis = emis * float(ext.get("KHR_materials_emissive_strength", {}).get("emissiveStrength", 1.0))
    ior = float(ext.get("KHR_materials_ior", {}).get("ior", 1.5))
    trans = float(ext.get("KHR_materials_transmission", {}).get("transmissionFactor", 0.0))
    cc = ext.get("KHR_materials_clearcoat", {})
    clearcoat = float(cc.get("clearcoatFactor", 0.0))
    cc_rough = float(cc.get("clearcoatRoughnessFactor", 0.0))
    opacity = 1.0
    mode = m.get("alphaMode", "OPAQUE")
    if mode == "BLEND":
        opacity = float(bc[3])
    elif mode == "MASK":
        opacity = 1.0 if float(bc[3]) >= float(m.get("alphaCutoff", 0.5)) else 0.0
    mtype = abi.MATERIAL_DISNEY if (metallic > 0 or trans > 0 or clearcoat > 0) else abi.MATERIAL_DIFFUSE
    t = extras.get("type")
    if t is not None:
        mtype = {"diffuse": abi.MATERIAL_DIFFUSE, "lambert": abi.MATERIAL_DIFFUSE, "disney": abi.MATERIAL_DISNEY}.get(
            str(t).lower(), int(t) if str(t).isdigit() else abi.MATERIAL_DIFFUSE)
    mat = sc.material(tuple(bc[:3]), mtype, roughness=rough, metallic=metallic, specular_transmission=trans,
                      ior=ior, opacity=opacity, emission=tuple(emis), clearcoat=clearcoat,
                      clearcoat_roughness=cc_rough)
    for name, value in extras.items():
        if name in ("type", "medium"):
            continue
        if hasattr(mat, name):
            field = getattr(mat, name)
            if hasattr(field, "__len__"):
                field[:] = list(value)[:len(field)]
            else:
                setattr(mat, name, float(value))
    med = extras.get("medium")
    if med:
        mt = med.get("type", "absorb")
        mat.medium.type = MEDIUM_NAMES.get(str(mt).lower(), int(mt) if str(mt).isdigit() else abi.MEDIUM_NONE)
        mat.medium.color[:] = med.get("color", [1, 1, 1])
        mat.medium.density = float(med.get("density", 0.0))
        mat.medium.anisotropy = float(med.get("anisotropy", 0.0))
    mat.base_color_map_index = tex.bake(pbr.get("baseColorTexture"), list(mat.base_color), "srgb")
    mat.metallic_roughness_map_index = tex.bake(pbr.get("metallicRoughnessTexture"), (mat.metallic, mat.roughness),
                                                "mr")
    mat.emission_map_index = tex.bake(m.get("emissiveTexture"), list(mat.emission), "srgb")
    mat.normal_map_index = tex.bake(m.get("normalTexture"), (1, 1, 1), "linear")
    return sc.preprocess_material(mat)


def _light(L, M):
    color = np.asarray(L.get("color", [1, 1, 1]), np.float64)
    inten = float(L.get("intensity", 1.0))
    extras = L.get("extras", {}) or {}
    # an "rgb" extra gives the intensity per channel directly
    I = np.asarray(extras["rgb"], np.float64) if "rgb" in extras else color * inten
    pos = M[:3, 3]
    X, Y, Z = (M[:3, k] for k in range(3))
    fwd = -Z / max(np.linalg.norm(Z), 1e-30)
    etype = int(extras.get("type", 0))
    if etype == 1:  # rectangle
        w, h = float(extras.get("param0", 1.0)), float(extras.get("param1", 1.0))
        u = X / np.linalg.norm(X) * w
        v = Y / np.linalg.norm(Y) * h
        area = w * h
        radiance = I * 4.0 / max(area, 1e-30)
        return sc.quad_light(pos - 0.5 * u - 0.5 * v, u, v, radiance)
    if etype == 2:  # sphere
        r = float(extras.get("param0", 0.1))
        return sc.sphere_light(pos, r, I / (math.pi * r * r))
    kind = L.get("type", "point")
    if kind == "directional":
        return sc.directional_light(fwd, I, float(extras.get("cone_deg", 0.0)))
    if kind == "spot":
        spot = L.get("spot", {})
        inner = math.degrees(float(spot.get("innerConeAngle", 0.0)))
        outer = math.degrees(float(spot.get("outerConeAngle", math.pi / 4)))
        return sc.spot_light(pos, fwd, I, inner, outer)
    return sc.point_light(pos, I)


def _camera(c, M):
    cam = abi.Camera()
    X, Y, Z = (M[:3, k] / np.linalg.norm(M[:3, k]) for k in range(3))
    cam.position[:] = M[:3, 3]
    cam.right[:] = X
    cam.up[:] = Y
    cam.forward[:] = -Z
    extras = c.get("extras", {}) or {}
    if c.get("type") == "orthographic":
        o = c["orthographic"]
        cam.type = abi.CAMERA_ORTHOGRAPHIC
        cam.yfov = float(extras.get("yfov", 0.0))  # unused by the orthographic ray
        cam.focal_distance_or_xmag = float(o["xmag"])
        cam.aperture_or_ymag = float(o["ymag"])
    else:
        p = c.get("perspective", {})
        cam.type = abi.CAMERA_PERSPECTIVE
        cam.yfov = float(p.get("yfov", math.radians(40.0)))
        cam.focal_distance_or_xmag = float(extras.get("focal_distance", 1.0))
        cam.aperture_or_ymag = float(extras.get("aperture", 0.0))
    return cam


def load_scene(path, width=None, height=None):
    """Reads a .gltf / .glb file into a scenes.Scene."""
    doc = _Doc(path)
    j = doc.j
    s = sc.Scene(os.path.splitext(os.path.basename(path))[0])
    tex = _Textures(doc, s)
    for m in j.get("materials", []):
        s.add_material(_material(doc, m, tex))
    default_mat = None
    lights_ext = j.get("extensions", {}).get("KHR_lights_punctual", {}).get("lights", [])
    for ni, M in _walk(doc):
        n = j["nodes"][ni]
        if "mesh" in n:
            for prim in j["meshes"][n["mesh"]]["primitives"]:
                if prim.get("mode", 4) != 4:
                    continue
                at = prim["attributes"]
                pos = doc.accessor(at["POSITION"]).astype(np.float64)
                idx = (doc.accessor(prim["indices"]).reshape(-1).astype(np.uint32) if "indices" in prim
                       else np.arange(len(pos), dtype=np.uint32))
                nrm = doc.accessor(at["NORMAL"]).astype(np.float64) if "NORMAL" in at else \
                    sc.smooth_normals(pos, idx.reshape(-1, 3))
                tan = doc.accessor(at["TANGENT"])[:, :3].astype(np.float64) if "TANGENT" in at else \
                    sc._orthogonal_tangent(nrm)
                uv = doc.accessor(at["TEXCOORD_0"]).astype(np.float64) if "TEXCOORD_0" in at else \
                    np.zeros((len(pos), 2))
                mi = prim.get("material")
                if mi is None:
                    if default_mat is None:
                        default_mat = s.add_material(sc.material((0.8, 0.8, 0.8)))
                    mi = default_mat
                s.add_mesh(sc.pack_vertices(pos, nrm, tan, uv), idx, mi, transform=M.astype(np.float32))
        if "camera" in n and len(s.cameras) < abi.PT_MAX_CAMERAS:
            s.cameras.append(_camera(j["cameras"][n["camera"]], M))
        li = n.get("extensions", {}).get("KHR_lights_punctual", {}).get("light")
        if li is not None and len(s.lights) < abi.PT_MAX_LIGHTS:
            s.lights.append(_light(lights_ext[li], M))
    if not s.cameras:
        raise GltfError("the scene has no camera")
    if width:
        s.width = int(width)
    if height:
        s.height = int(height)
    s.skipped_images = tex.skipped
    return s


# --------------------------------------------------------------------------- writer

def save_scene(scene, path):
    """Writes a scenes.Scene as .gltf + .bin with the extras above (every
    material field, area lights as extras), for round trips and tools.
    Texture maps are not written."""
    base = os.path.splitext(path)[0]
    binname = os.path.basename(base) + ".bin"
    blob = bytearray()
    accessors, views, meshes, nodes = [], [], [], []

    def add(arr, ctype, typ, target):
        a = np.ascontiguousarray(arr)
        while len(blob) % 4:
            blob.append(0)
        views.append({"buffer": 0, "byteOffset": len(blob), "byteLength": a.nbytes, "target": target})
        blob.extend(a.tobytes())
        acc = {"bufferView": len(views) - 1, "componentType": ctype, "count": len(a), "type": typ}
        if typ == "VEC3" and ctype == 5126:
            acc["min"] = a.min(0).tolist()
            acc["max"] = a.max(0).tolist()
        accessors.append(acc)
        return len(accessors) - 1

    for k, (v, i, tr, mat) in enumerate(scene.meshes):
        attrs = {"POSITION": add(v[:, 0:3].astype(np.float32), 5126, "VEC3", 34962),
                 "NORMAL": add(v[:, 3:6].astype(np.float32), 5126, "VEC3", 34962),
                 "TANGENT": add(np.concatenate([v[:, 6:9], np.ones((len(v), 1), np.float32)], 1), 5126, "VEC4",
                                34962),
                 "TEXCOORD_0": add(v[:, 9:11].astype(np.float32), 5126, "VEC2", 34962)}
        ind = add(np.asarray(i, np.uint32), 5125, "SCALAR", 34963)
        meshes.append({"primitives": [{"attributes": attrs, "indices": ind, "material": int(mat)}]})
        M = np.asarray(tr, np.float64).reshape(4, 4)  # stored column-major
        nodes.append({"mesh": k, "matrix": M.reshape(-1).tolist()})
    materials = []
    for m in scene.materials:
        extras = {"type": "disney" if m.type == abi.MATERIAL_DISNEY else "diffuse"}
        for f in ("opacity", "anisotropic", "metallic", "roughness", "subsurface", "specular_tint", "sheen",
                  "sheen_tint", "clearcoat", "clearcoat_roughness", "specular_transmission", "ior"):
            extras[f] = float(getattr(m, f))
        extras["clearcoat_tint"] = list(m.clearcoat_tint)
        extras["emission"] = list(m.emission)
        if m.medium.type != abi.MEDIUM_NONE:
            inv = {v: k for k, v in MEDIUM_NAMES.items()}
            extras["medium"] = {"type": inv[m.medium.type], "color": list(m.medium.color),
                                "density": float(m.medium.density), "anisotropy": float(m.medium.anisotropy)}
        materials.append({"pbrMetallicRoughness": {"baseColorFactor": list(m.base_color) + [1.0],
                                                   "metallicFactor": float(m.metallic),
                                                   "roughnessFactor": float(m.roughness)},
                          "extras": extras})
    lights = []
    for L in scene.lights:
        node = {"extensions": {"KHR_lights_punctual": {"light": len(lights)}}}
        if L.type == abi.LIGHT_QUAD:
            u, v = np.asarray(L.u, np.float64), np.asarray(L.v, np.float64)
            w, h = np.linalg.norm(u), np.linalg.norm(v)
            X, Y = u / w, v / h
            Z = np.cross(X, Y)
            M = np.eye(4)
            M[:3, 0], M[:3, 1], M[:3, 2] = X, Y, Z
            M[:3, 3] = np.asarray(L.position, np.float64) + 0.5 * u + 0.5 * v
            I = np.asarray(L.intensity, np.float64) * w * h / 4.0
            lights.append({"type": "point", "color": [1, 1, 1], "intensity": 1.0,
                           "extras": {"type": 1, "param0": w, "param1": h, "rgb": I.tolist()}})
            node["matrix"] = M.T.reshape(-1).tolist()
        elif L.type == abi.LIGHT_SPHERE:
            I = np.asarray(L.intensity, np.float64) * math.pi * L.radius ** 2
            lights.append({"type": "point", "color": [1, 1, 1], "intensity": 1.0,
                           "extras": {"type": 2, "param0": float(L.radius), "rgb": I.tolist()}})
            node["translation"] = list(L.position)
        else:
            kind = {abi.LIGHT_POINT: "point", abi.LIGHT_DIRECTIONAL: "directional", abi.LIGHT_SPOT: "spot"}[L.type]
            ent = {"type": kind, "color": [1, 1, 1], "intensity": 1.0, "extras": {"rgb": list(L.intensity)}}
            if kind == "directional" and L.v[0] > 0:
                ent["extras"]["cone_deg"] = math.degrees(math.acos(min(1.0, L.v[0])))
            node["translation"] = list(L.position)
            if kind in ("directional", "spot"):
                d = np.asarray(L.u, np.float64)
                z = -d / np.linalg.norm(d)
                x = np.cross([0.0, 0.0, 1.0] if abs(z[2]) < 0.9 else [1.0, 0.0, 0.0], z)
                x /= np.linalg.norm(x)
                y = np.cross(z, x)
                M = np.eye(4)
                M[:3, 0], M[:3, 1], M[:3, 2], M[:3, 3] = x, y, z, np.asarray(L.position, np.float64)
                node.pop("translation")
                node["matrix"] = M.T.reshape(-1).tolist()
            if kind == "spot":
                ent["spot"] = {"innerConeAngle": math.acos(max(-1.0, min(1.0, L.v[0]))),
                               "outerConeAngle": math.acos(max(-1.0, min(1.0, L.v[1])))}
            lights.append(ent)
        nodes.append(node)
    cameras = []
    for c in scene.cameras:
        X, Y, F = (np.asarray(a, np.float64) for a in (c.right, c.up, c.forward))
        M = np.eye(4)
        M[:3, 0], M[:3, 1], M[:3, 2], M[:3, 3] = X, Y, -F, np.asarray(c.position, np.float64)
        if c.type == abi.CAMERA_ORTHOGRAPHIC:
            cam = {"type": "orthographic", "orthographic": {"xmag": c.focal_distance_or_xmag,
                                                            "ymag": c.aperture_or_ymag, "znear": 0.01, "zfar": 1e4},
                   "extras": {"yfov": c.yfov}}
        else:
            cam = {"type": "perspective", "perspective": {"yfov": c.yfov, "znear": 0.01},
                   "extras": {"aperture": c.aperture_or_ymag, "focal_distance": c.focal_distance_or_xmag}}
        cameras.append(cam)
        nodes.append({"camera": len(cameras) - 1, "matrix": M.T.reshape(-1).tolist()})
    doc = {"asset": {"version": "2.0", "generator": "hala-pathtracer_gb300"},
           "extensionsUsed": ["KHR_lights_punctual"], "scene": 0,
           "scenes": [{"nodes": list(range(len(nodes)))}], "nodes": nodes, "meshes": meshes,
           "materials": materials, "accessors": accessors, "bufferViews": views, "cameras": cameras,
           "buffers": [{"byteLength": len(blob), "uri": binname}],
           "extensions": {"KHR_lights_punctual": {"lights": lights}}}
    with open(base + ".bin", "wb") as f:
        f.write(bytes(blob))
    with open(base + ".gltf", "w") as f:
        json.dump(doc, f, indent=1)
    return base + ".gltf"
