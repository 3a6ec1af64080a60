"""Procedural scenes for the benchmark workloads and the parity tests.

Every scene is synthetic and seeded; nothing is read from disk. The four
workloads are:

  cornell()      -- Cornell box, 34 triangles, one quad light, Lambert only,
                    perspective 40 deg, 256x256, 16 spp, depth 8, seed 1
  disney_grid()  -- 9x9 UV spheres (64x32 segments) + ground quad, Disney
                    materials (metallic by row, roughness by column, every
                    third sphere glass), 2048x1024 synthetic HDR sky with a
                    sun lobe of peak 5e4, 1920x1080, 64 spp, depth 12
  displaced_icosphere() -- geodesic sphere of ~2.6M triangles displaced by
                    6-octave value noise (seed 7), point + spot + sphere +
                    directional lights, Oren-Nayar and Disney materials,
                    1920x1080, 32 spp, depth 8
  media_box()    -- Cornell room with a scattering sphere, an emissive-medium
                    box and an absorbing fog slab (delta tracking), 1024x1024,
                    128 spp, depth 32

Materials carry the preprocessed ax/ay the shaders read (see
`preprocess_material`), and the Light/Camera/Material fields follow
inc/types.glsl of the reference.
"""
import ctypes as C
import math

import numpy as np

from . import abi

FRAC_PI_2 = np.float32(math.pi * 0.5)


# --------------------------------------------------------------------------- materials

def preprocess_material(m):
    """Fills ax/ay the way the shaders read them (float32 arithmetic).

    Disney (inc/bxdf/disney.glsl:420): GGX alphas from roughness^2 and the
    anisotropic aspect sqrt(1 - 0.9 anisotropic), clamped to >= 0.001.
    Diffuse (inc/bxdf/oren_nayar.glsl:35-46): Oren-Nayar A and B from
    sigma = roughness * pi/2.
    """
    f = np.float32
    r = f(m.roughness)
    if m.type == abi.MATERIAL_DISNEY:
        aspect = np.sqrt(f(1.0) - f(0.9) * f(m.anisotropic))
        m.ax = float(max(f(0.001), (r * r) / aspect))
        m.ay = float(max(f(0.001), (r * r) * aspect))
    else:
        sigma = r * FRAC_PI_2
        s2 = sigma * sigma
        m.ax = float(f(1.0) - s2 / (f(2.0) * (s2 + f(0.33))))
        m.ay = float(f(0.45) * s2 / (s2 + f(0.09)))
    return m


def material(base_color=(0.8, 0.8, 0.8), mtype=abi.MATERIAL_DIFFUSE, roughness=0.0, metallic=0.0,
             specular_transmission=0.0, ior=1.5, opacity=1.0, emission=(0, 0, 0), anisotropic=0.0,
             subsurface=0.0, specular_tint=0.0, sheen=0.0, sheen_tint=0.0, clearcoat=0.0,
             clearcoat_roughness=0.0, clearcoat_tint=(1, 1, 1), medium=None):
    m = abi.Material()
    m.base_color[:] = base_color
    m.opacity = opacity
    m.emission[:] = emission
    m.anisotropic = anisotropic
    m.metallic = metallic
    m.roughness = roughness
    m.subsurface = subsurface
    m.specular_tint = specular_tint
    m.sheen = sheen
    m.sheen_tint = sheen_tint
    m.clearcoat = clearcoat
    m.clearcoat_roughness = clearcoat_roughness
    m.clearcoat_tint[:] = clearcoat_tint
    m.specular_transmission = specular_transmission
    m.ior = ior
    m.base_color_map_index = abi.PT_INVALID_INDEX
    m.normal_map_index = abi.PT_INVALID_INDEX
    m.metallic_roughness_map_index = abi.PT_INVALID_INDEX
    m.emission_map_index = abi.PT_INVALID_INDEX
    m.type = mtype
    m.medium.color[:] = (0, 0, 0)
    m.medium.density = 0.0
    m.medium.anisotropy = 0.0
    m.medium.type = abi.MEDIUM_NONE
    if medium is not None:
        mtype_, color, density, aniso = medium
        m.medium.type = mtype_
        m.medium.color[:] = color
        m.medium.density = density
        m.medium.anisotropy = aniso
    return preprocess_material(m)


# --------------------------------------------------------------------------- lights / cameras

def quad_light(corner, u, v, radiance):
    L = abi.Light()
    L.type = abi.LIGHT_QUAD
    L.intensity[:] = radiance
    L.position[:] = corner
    L.u[:] = u
    L.v[:] = v
    L.radius = 0.0
    L.area = float(np.linalg.norm(np.cross(np.asarray(u, np.float64), np.asarray(v, np.float64))))
    return L


def point_light(position, intensity):
    L = abi.Light()
    L.type = abi.LIGHT_POINT
    L.intensity[:] = intensity
    L.position[:] = position
    return L


def spot_light(position, direction, intensity, inner_deg, outer_deg):
    L = abi.Light()
    L.type = abi.LIGHT_SPOT
    L.intensity[:] = intensity
    L.position[:] = position
    d = np.asarray(direction, np.float64)
    L.u[:] = d / np.linalg.norm(d)
    L.v[:] = (math.cos(math.radians(inner_deg)), math.cos(math.radians(outer_deg)), 0.0)
    return L


def directional_light(direction, intensity, cone_deg=0.0):
    """`direction` is the direction the light travels (Light.u)."""
    L = abi.Light()
    L.type = abi.LIGHT_DIRECTIONAL
    L.intensity[:] = intensity
    d = np.asarray(direction, np.float64)
    L.u[:] = d / np.linalg.norm(d)
    L.v[:] = (math.cos(math.radians(cone_deg)) if cone_deg > 0 else 0.0, 0.0, 0.0)
    return L


def sphere_light(center, radius, radiance):
    L = abi.Light()
    L.type = abi.LIGHT_SPHERE
    L.intensity[:] = radiance
    L.position[:] = center
    L.radius = radius
    L.area = float(4.0 * math.pi * radius * radius)
    return L


def look_at(eye, target, yfov_deg, up=(0.0, 0.0, 1.0), aperture=0.0, focal_distance=1.0,
            ortho=None):
    eye = np.asarray(eye, np.float64)
    fwd = np.asarray(target, np.float64) - eye
    fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, np.asarray(up, np.float64))
    right /= np.linalg.norm(right)
    upv = np.cross(right, fwd)
    cam = abi.Camera()
    cam.position[:] = eye
    cam.right[:] = right
    cam.up[:] = upv
    cam.forward[:] = fwd
    cam.yfov = math.radians(yfov_deg)
    if ortho is not None:
        cam.type = abi.CAMERA_ORTHOGRAPHIC
        cam.focal_distance_or_xmag, cam.aperture_or_ymag = ortho
    else:
        cam.type = abi.CAMERA_PERSPECTIVE
        cam.focal_distance_or_xmag = focal_distance
        cam.aperture_or_ymag = aperture
    return cam


# --------------------------------------------------------------------------- meshes

IDENTITY = np.eye(4, dtype=np.float32)


def _orthogonal_tangent(n):
    n = np.asarray(n, np.float64)
    up = np.where(np.abs(n[..., 2:3]) < 0.999, np.array([0.0, 0.0, 1.0]), np.array([1.0, 0.0, 0.0]))
    t = np.cross(up, n)
    return t / np.linalg.norm(t, axis=-1, keepdims=True)


def pack_vertices(pos, nrm, tan, uv):
    v = np.zeros((len(pos), 11), np.float32)
    v[:, 0:3] = pos
    v[:, 3:6] = nrm
    v[:, 6:9] = tan
    v[:, 9:11] = uv
    return v


def quad_mesh(corner, u, v):
    """Two triangles spanning corner + [0,1]u + [0,1]v, normal = u x v."""
    corner, u, v = (np.asarray(a, np.float64) for a in (corner, u, v))
    pos = np.array([corner, corner + u, corner + u + v, corner + v])
    n = np.cross(u, v)
    n /= np.linalg.norm(n)
    t = u / np.linalg.norm(u)
    verts = pack_vertices(pos, np.tile(n, (4, 1)), np.tile(t, (4, 1)),
                          np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float64))
    idx = np.array([0, 1, 2, 0, 2, 3], np.uint32)
    return verts, idx


def box_mesh(center, size, rot_z_deg=0.0):
    """Axis-aligned box rotated about z; 6 faces, 12 triangles, outward normals."""
    cx, cy, cz = center
    sx, sy, sz = (s * 0.5 for s in size)
    a = math.radians(rot_z_deg)
    R = np.array([[math.cos(a), -math.sin(a), 0.0], [math.sin(a), math.cos(a), 0.0], [0.0, 0.0, 1.0]])
    faces = []
    # (normal axis, sign)
    for axis in range(3):
        for sgn in (-1.0, 1.0):
            n = np.zeros(3)
            n[axis] = sgn
            u = np.zeros(3)
            v = np.zeros(3)
            ua, va = [(1, 2), (2, 0), (0, 1)][axis]
            u[ua] = 1.0
            v[va] = 1.0
            if sgn < 0:
                u, v = v, u
            half = np.array([sx, sy, sz])
            corner = n * half - u * half - v * half
            faces.append((corner, u * 2 * half, v * 2 * half))
    verts, idxs = [], []
    base = 0
    for corner, u, v in faces:
        vv, ii = quad_mesh(R @ corner, R @ u, R @ v)
        vv[:, 0:3] += (cx, cy, cz)
        verts.append(vv)
        idxs.append(ii + base)
        base += 4
    return np.concatenate(verts), np.concatenate(idxs).astype(np.uint32)


def uv_sphere(center, radius, segments=64, rings=32):
    """UV sphere; cap rings are single triangles (no degenerate triangles)."""
    th = np.linspace(0.0, math.pi, rings + 1)
    ph = np.linspace(0.0, 2.0 * math.pi, segments + 1)
    T, P = np.meshgrid(th, ph, indexing="ij")
    n = np.stack([np.sin(T) * np.cos(P), np.sin(T) * np.sin(P), np.cos(T)], -1).reshape(-1, 3)
    tan = np.stack([-np.sin(P), np.cos(P), np.zeros_like(P)], -1).reshape(-1, 3)
    uv = np.stack([P / (2 * math.pi), T / math.pi], -1).reshape(-1, 2)
    pos = n * radius + np.asarray(center, np.float64)
    idx = []
    W = segments + 1
    for r in range(rings):
        for s in range(segments):
            a = r * W + s
            b = a + W
            if r != 0:
                idx.append((a, b, a + 1))
            if r != rings - 1:
                idx.append((a + 1, b, b + 1))
    return pack_vertices(pos, n, tan, uv), np.asarray(idx, np.uint32).reshape(-1)


def _hash3(ix, iy, iz, seed):
    h = (ix.astype(np.uint64) * np.uint64(73856093)) ^ (iy.astype(np.uint64) * np.uint64(19349663)) ^ \
        (iz.astype(np.uint64) * np.uint64(83492791)) ^ np.uint64(seed * 2654435761 & 0xFFFFFFFF)
    h = h & np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(13)
    h = (h * np.uint64(0x5BD1E995)) & np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(15)
    return (h.astype(np.float64) / 4294967295.0) * 2.0 - 1.0


def value_noise3(p, seed):
    """Smooth (quintic) value noise in [-1, 1] on an integer lattice."""
    i = np.floor(p)
    f = p - i
    w = f * f * f * (f * (f * 6.0 - 15.0) + 10.0)
    i = i.astype(np.int64)
    out = 0.0
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                c = _hash3(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz, seed)
                wx = w[:, 0] if dx else 1.0 - w[:, 0]
                wy = w[:, 1] if dy else 1.0 - w[:, 1]
                wz = w[:, 2] if dz else 1.0 - w[:, 2]
                out = out + c * wx * wy * wz
    return out


def fractal_noise(p, octaves=6, seed=7, base_freq=2.0):
    amp, freq, total, norm = 1.0, base_freq, 0.0, 0.0
    for o in range(octaves):
        total = total + amp * value_noise3(p * freq, seed + 101 * o)
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


def _icosahedron():
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    return v, f


def geodesic_sphere(freq):
    """Icosphere with every face split into freq^2 triangles (20 freq^2 total),
    shared vertices merged so the mesh is watertight."""
    V, F = _icosahedron()
    # barycentric lattice of one face
    ij = [(i, j) for i in range(freq + 1) for j in range(freq + 1 - i)]
    lut = {p: k for k, p in enumerate(ij)}
    ij = np.asarray(ij, np.float64)
    tris = []
    for i in range(freq):
        for j in range(freq - i):
            tris.append((lut[(i, j)], lut[(i + 1, j)], lut[(i, j + 1)]))
            if j + 1 <= freq - i - 1:
                tris.append((lut[(i + 1, j)], lut[(i + 1, j + 1)], lut[(i, j + 1)]))
    tris = np.asarray(tris, np.int64)
    nloc = len(ij)
    a = ij[:, 0:1] / freq
    b = ij[:, 1:2] / freq
    pts = []
    for f in F:
        p = V[f[0]] * (1.0 - a - b) + V[f[1]] * a + V[f[2]] * b
        pts.append(p / np.linalg.norm(p, axis=1, keepdims=True))
    pts = np.concatenate(pts)
    allt = np.concatenate([tris + k * nloc for k in range(len(F))])
    key = np.round(pts * 1e9).astype(np.int64)
    _, first, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    uniq = pts[first]
    allt = inv.reshape(-1)[allt]
    return uniq, allt.astype(np.uint32).reshape(-1)


def smooth_normals(pos, idx):
    tri = idx.reshape(-1, 3).astype(np.int64)
    fn = np.cross(pos[tri[:, 1]] - pos[tri[:, 0]], pos[tri[:, 2]] - pos[tri[:, 0]])
    n = np.zeros_like(pos)
    for k in range(3):
        np.add.at(n, tri[:, k], fn)
    return n / np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)


# --------------------------------------------------------------------------- scene container

class Scene:
    """Host-side scene plus the tracer settings of its workload."""

    def __init__(self, name):
        self.name = name
        self.meshes = []   # (vertices [n,11] f32, indices u32, transform 4x4 f32 col-major, material)
        self.materials = []
        self.lights = []
        self.cameras = []
        self.env_rgb = None      # (H, W, 3) float32
        self.env_rotation_deg = 0.0
        self.ground_color = (0.0, 0.0, 0.0, 1.0)
        self.sky_color = (0.0, 0.0, 0.0, 1.0)
        self.env_intensity = 1.0
        self.exposure_value = 0.0
        self.width, self.height = 256, 256
        self.spp, self.max_depth, self.rr_depth, self.seed = 16, 8, 0, 0
        self.tonemap = (True, True, False)
        self.textures = []       # (H, W, 4) float32 RGBA, linear values
        self.blue_noise = None   # (1024, 1024, 4) uint8 camera-jitter texture, or None: the substitute
        self._keep = []

    def add_material(self, m):
        self.materials.append(m)
        return len(self.materials) - 1

    def add_texture(self, rgba):
        self.textures.append(np.ascontiguousarray(rgba, np.float32))
        return len(self.textures) - 1

    def add_mesh(self, verts, idx, mat, transform=None):
        tr = IDENTITY if transform is None else np.asarray(transform, np.float32)
        self.meshes.append((np.ascontiguousarray(verts, np.float32),
                            np.ascontiguousarray(idx, np.uint32).reshape(-1),
                            np.ascontiguousarray(tr.T.reshape(-1), np.float32), mat))

    @property
    def num_triangles(self):
        return sum(len(m[1]) // 3 for m in self.meshes)

    def config(self, **over):
        kw = dict(width=self.width, height=self.height, max_depth=self.max_depth,
                  rr_depth=self.rr_depth, enable_tonemap=self.tonemap[0],
                  enable_aces=self.tonemap[1], use_simple_aces=self.tonemap[2], seed=self.seed)
        kw.update(over)
        return abi.make_config(**kw)

    def desc(self):
        """ctypes pt_scene_desc; the arrays stay alive with this Scene."""
        prims = (abi.Primitive * max(1, len(self.meshes)))()
        keep = []
        for k, (v, i, tr, mat) in enumerate(self.meshes):
            prims[k].vertices = v.ctypes.data_as(C.POINTER(C.c_float))
            prims[k].num_vertices = len(v)
            prims[k].indices = i.ctypes.data_as(C.POINTER(C.c_uint32))
            prims[k].num_indices = len(i)
            prims[k].transform[:] = tr.tolist()
            prims[k].material_index = mat
            keep += [v, i]
        mats = (abi.Material * max(1, len(self.materials)))(*self.materials)
        lights = (abi.Light * max(1, len(self.lights)))(*self.lights)
        cams = (abi.Camera * max(1, len(self.cameras)))(*self.cameras)
        d = abi.SceneDesc()
        d.primitives, d.num_primitives = prims, len(self.meshes)
        d.materials, d.num_materials = mats, len(self.materials)
        d.lights, d.num_lights = lights, len(self.lights)
        d.cameras, d.num_cameras = cams, len(self.cameras)
        texs = (abi.Texture * max(1, len(self.textures)))()
        for k, t in enumerate(self.textures):
            texs[k].rgba = t.ctypes.data_as(C.POINTER(C.c_float))
            texs[k].height, texs[k].width = t.shape[0], t.shape[1]
            keep.append(t)
        d.textures, d.num_textures = texs, len(self.textures)
        self._keep = [prims, mats, lights, cams, texs, keep]
        return d

    def env_pointer(self):
        if self.env_rgb is None:
            return None, 0, 0
        e = np.ascontiguousarray(self.env_rgb, np.float32)
        self._keep_env = e
        return e.ctypes.data_as(C.POINTER(C.c_float)), e.shape[1], e.shape[0]


# --------------------------------------------------------------------------- workloads

def cornell(width=256, height=256, spp=16, max_depth=8, rr_depth=0, seed=1, boxes=True):
    """Cornell box: unit room (x right, y depth, z up) open towards -y."""
    s = Scene("cornell")
    white = s.add_material(material((0.73, 0.73, 0.73)))
    red = s.add_material(material((0.65, 0.05, 0.05)))
    green = s.add_material(material((0.12, 0.45, 0.15)))
    # room: floor, ceiling, back wall, left (red), right (green); normals face inwards
    s.add_mesh(*quad_mesh((0, 0, 0), (1, 0, 0), (0, 1, 0)), white)          # floor, +z
    s.add_mesh(*quad_mesh((0, 0, 1), (0, 1, 0), (1, 0, 0)), white)          # ceiling, -z
    s.add_mesh(*quad_mesh((0, 1, 0), (1, 0, 0), (0, 0, 1)), white)          # back, -y
    s.add_mesh(*quad_mesh((0, 0, 0), (0, 0, 1), (0, 1, 0)), red)            # left, +x
    s.add_mesh(*quad_mesh((1, 0, 0), (0, 1, 0), (0, 0, 1)), green)         # right, -x
    if boxes:
        s.add_mesh(*box_mesh((0.33, 0.62, 0.3), (0.28, 0.28, 0.6), 17.0), white)   # tall box
        s.add_mesh(*box_mesh((0.67, 0.35, 0.15), (0.28, 0.28, 0.3), -18.0), white)  # short box
    # 0.25 x 0.25 quad light just below the ceiling, emitting downwards
    s.lights.append(quad_light((0.375, 0.375, 0.999), (0.25, 0, 0), (0, 0.25, 0), (17.0, 17.0, 17.0)))
    s.cameras.append(look_at((0.5, -1.35, 0.5), (0.5, 0.5, 0.5), 40.0))
    s.width, s.height, s.spp, s.max_depth, s.rr_depth, s.seed = width, height, spp, max_depth, rr_depth, seed
    return s


def synthetic_sky(width=2048, height=1024, sun_peak=5e4, sun_elev_deg=35.0, sun_azim_deg=60.0,
                  sun_sigma_deg=1.0, noise_sigma=0.25, seed=3):
    """Equirect HDR sky: vertical gradient, Gaussian sun lobe, log-normal noise.

    Texel (x, y) is looked up for direction (-sin t cos p, sin t sin p, cos t)
    with t = pi (y + 0.5) / H and p = 2 pi (x + 0.5) / W (inc/env_map.glsl:15-26).
    """
    rng = np.random.default_rng(seed)
    y = (np.arange(height) + 0.5) / height
    x = (np.arange(width) + 0.5) / width
    th = (y * math.pi)[:, None]
    ph = (x * 2 * math.pi)[None, :]
    dx = -np.sin(th) * np.cos(ph)
    dy = np.sin(th) * np.sin(ph)
    dz = np.cos(th) * np.ones_like(ph)
    up = np.clip(dz, 0.0, 1.0)
    zenith = np.array([0.25, 0.45, 0.95])
    horizon = np.array([1.0, 0.95, 0.9])
    ground = np.array([0.18, 0.15, 0.12])
    sky = horizon * (1 - up[..., None]) + zenith * up[..., None]
    rgb = np.where((dz >= 0)[..., None], sky * 1.5, ground * 0.5)
    se, sa = math.radians(sun_elev_deg), math.radians(sun_azim_deg)
    sd = np.array([-math.cos(se) * math.cos(sa), math.cos(se) * math.sin(sa), math.sin(se)])
    cosang = np.clip(dx * sd[0] + dy * sd[1] + dz * sd[2], -1, 1)
    ang = np.arccos(cosang)
    lobe = sun_peak * np.exp(-0.5 * (ang / math.radians(sun_sigma_deg)) ** 2)
    rgb = rgb + lobe[..., None] * np.array([1.0, 0.92, 0.8])
    rgb = rgb * np.exp(rng.normal(0.0, noise_sigma, size=(height, width, 1)))
    return rgb.astype(np.float32)


def disney_grid(width=1920, height=1080, spp=64, max_depth=12, rr_depth=4, seed=0, segments=64,
                rings=32, env_size=(2048, 1024)):
    s = Scene("disney_grid")
    ground = s.add_material(material((0.5, 0.5, 0.5), abi.MATERIAL_DISNEY, roughness=0.5))
    s.add_mesh(*quad_mesh((-6, -6, 0), (12, 0, 0), (0, 12, 0)), ground)
    for row in range(9):
        for col in range(9):
            k = row * 9 + col
            glass = (k % 3) == 0
            m = material((0.9, 0.55, 0.3), abi.MATERIAL_DISNEY, roughness=0.05 + 0.95 * col / 8.0,
                         metallic=row / 8.0, specular_transmission=1.0 if glass else 0.0,
                         ior=1.5)
            mi = s.add_material(m)
            c = ((col - 4) * 1.0, (row - 4) * 1.0, 0.42)
            s.add_mesh(*uv_sphere(c, 0.4, segments, rings), mi)
    s.cameras.append(look_at((0.0, -9.5, 6.5), (0.0, -0.3, 0.0), 40.0))
    s.env_rgb = synthetic_sky(*env_size)
    s.env_intensity = 1.0
    s.width, s.height, s.spp, s.max_depth, s.rr_depth, s.seed = width, height, spp, max_depth, rr_depth, seed
    return s


def displaced_icosphere(width=1920, height=1080, spp=32, max_depth=8, rr_depth=4, seed=0, freq=361):
    s = Scene("displaced_icosphere")
    on = s.add_material(material((0.7, 0.6, 0.5), abi.MATERIAL_DIFFUSE,
                                 roughness=float(0.3 / (math.pi / 2))))  # Oren-Nayar sigma = 0.3
    dis = s.add_material(material((0.4, 0.5, 0.7), abi.MATERIAL_DISNEY, roughness=0.4))
    pos, idx = geodesic_sphere(freq)
    disp = 1.0 + 0.1 * fractal_noise(pos * 1.0, octaves=6, seed=7)
    pos = pos * disp[:, None]
    nrm = smooth_normals(pos, idx)
    tan = _orthogonal_tangent(nrm)
    uv = np.zeros((len(pos), 2))
    verts = pack_vertices(pos + np.array([0, 0, 1.15]), nrm, tan, uv)
    s.add_mesh(verts, idx, dis)
    s.add_mesh(*quad_mesh((-10, -10, 0), (20, 0, 0), (0, 20, 0)), on)
    s.lights.append(point_light((2.5, -2.0, 3.5), (12.0, 12.0, 12.0)))
    s.lights.append(spot_light((-2.5, -2.5, 4.0), (2.5, 2.5, -3.0), (40.0, 38.0, 35.0), 20.0, 30.0))
    s.lights.append(sphere_light((-1.8, 1.5, 2.8), 0.2, (30.0, 28.0, 25.0)))
    s.lights.append(directional_light((0.3, 0.5, -0.8), (1.2, 1.15, 1.1)))
    s.cameras.append(look_at((0.0, -4.8, 2.4), (0.0, 0.0, 1.0), 40.0))
    s.width, s.height, s.spp, s.max_depth, s.rr_depth, s.seed = width, height, spp, max_depth, rr_depth, seed
    return s


def media_box(width=1024, height=1024, spp=128, max_depth=32, rr_depth=4, seed=0):
    """Cornell room with participating media behind glass boundaries.

    A medium is entered when a path crosses a surface whose material carries
    it (pathtracer.rgen.glsl:235-242), so each medium sits behind a thin
    dielectric boundary: a scattering sphere (sigma_s 4, sigma_a 0.2, HG
    g 0.7), an emissive-medium box (emission coefficient 2) and an absorbing
    fog slab (sigma_a 0.02) filling the room.
    """
    s = cornell(width, height, spp, max_depth, rr_depth, seed, boxes=False)
    s.name = "media_box"
    sig_s, sig_a = 4.0, 0.2
    sig_t = sig_s + sig_a
    scat = s.add_material(material((1, 1, 1), abi.MATERIAL_DISNEY, roughness=0.02,
                                   specular_transmission=1.0, ior=1.33,
                                   medium=(abi.MEDIUM_SCATTER, (sig_s / sig_t,) * 3, sig_t, 0.7)))
    s.add_mesh(*uv_sphere((0.6, 0.55, 0.45), 0.3, 48, 24), scat)
    emis = s.add_material(material((1, 1, 1), abi.MATERIAL_DISNEY, roughness=0.02,
                                   specular_transmission=1.0, ior=1.05,
                                   medium=(abi.MEDIUM_EMISSIVE, (1.0, 0.5, 0.2), 2.0, 0.0)))
    s.add_mesh(*box_mesh((0.22, 0.3, 0.1), (0.16, 0.16, 0.2), 25.0), emis)
    fog = s.add_material(material((1, 1, 1), abi.MATERIAL_DISNEY, roughness=0.02,
                                  specular_transmission=1.0, ior=1.05,
                                  medium=(abi.MEDIUM_ABSORB, (0.0, 0.0, 0.0), 0.02, 0.0)))
    s.add_mesh(*box_mesh((0.5, 0.5, 0.5), (0.99, 0.99, 0.98), 0.0), fog)
    return s


# --------------------------------------------------------------------------- textures

def checker_texture(size=32, cells=8, c0=(0.9, 0.85, 0.75), c1=(0.15, 0.2, 0.35)):
    """RGBA checkerboard with a gentle gradient (so bilinear filtering shows)."""
    y, x = np.mgrid[0:size, 0:size]
    on = ((x * cells // size) + (y * cells // size)) % 2 == 0
    rgb = np.where(on[..., None], np.asarray(c0), np.asarray(c1))
    rgb = rgb * (0.75 + 0.25 * (x / max(1, size - 1)))[..., None]
    return np.concatenate([rgb, np.ones((size, size, 1))], -1).astype(np.float32)


def bump_normal_map(size=32, seed=5, strength=0.6):
    """Tangent-space normal map (RGB in [0,1]) of a smooth random height field."""
    rng = np.random.default_rng(seed)
    h = rng.normal(size=(size // 4, size // 4))
    h = np.kron(h, np.ones((4, 4)))
    for _ in range(2):
        h = 0.25 * (np.roll(h, 1, 0) + np.roll(h, -1, 0) + np.roll(h, 1, 1) + np.roll(h, -1, 1))
    gx = (np.roll(h, -1, 1) - np.roll(h, 1, 1)) * strength
    gy = (np.roll(h, -1, 0) - np.roll(h, 1, 0)) * strength
    n = np.stack([-gx, -gy, np.ones_like(gx)], -1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    return np.concatenate([n * 0.5 + 0.5, np.ones((size, size, 1))], -1).astype(np.float32)


def metallic_roughness_texture(size=16):
    """glTF layout: G = roughness (left to right), B = metallic (bottom to top)."""
    y, x = np.mgrid[0:size, 0:size]
    r = 0.05 + 0.9 * x / (size - 1)
    m = y / (size - 1)
    return np.stack([np.zeros_like(r), r, m, np.ones_like(r)], -1).astype(np.float32)


def tiny_variants():
    """Small versions of every workload for parity tests (seconds on one core)."""
    return {
        "cornell": cornell(48, 48, 4),
        "disney": disney_grid(64, 36, 2, segments=16, rings=8, env_size=(256, 128)),
        "icosphere": displaced_icosphere(64, 36, 2, freq=12),
        "media": media_box(40, 40, 2, max_depth=12),
    }


WORKLOADS = {
    "cornell_256_16spp": cornell,
    "disney_grid_1080p_64spp": disney_grid,
    "displaced_icosphere_1080p_32spp": displaced_icosphere,
    "media_box_1024_128spp": media_box,
}
