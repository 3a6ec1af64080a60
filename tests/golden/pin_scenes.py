"""Small scenes that pin the oracle and the GPU path to the reference's own
shaders: every feature permutation (base, TRANSPARENT, MEDIUM+VOL_MIS,
MEDIUM+VOL_MIS+TRANSPARENT), all five light types, sky and HDR environment,
Lambert / Oren-Nayar / Disney (glass, metal, clearcoat, sheen), perspective,
thin-lens and orthographic cameras, and every tonemap mode. Seed 0 (the
reference seeds its RNG with the frame index only)."""
import importlib

S = importlib.import_module("hala-pathtracer_gb300.scenes")
abi = S.abi


def _cornell_base(w, h, spp):
    s = S.cornell(w, h, spp, max_depth=6, rr_depth=2, seed=0)
    return s


def cornell():
    return _cornell_base(24, 24, 3)


def disney_ibl():
    s = S.disney_grid(32, 18, 2, segments=12, rings=6, env_size=(64, 32))
    s.env_rotation_deg = 77.8
    s.env_intensity = 0.7
    s.exposure_value = -1.0
    return s


def lights_icosphere():
    s = S.displaced_icosphere(32, 18, 2, freq=6)
    s.lights.append(S.directional_light((-0.2, 0.4, -0.9), (0.5, 0.5, 0.5), cone_deg=8.0))
    s.lights.append(S.quad_light((-1.0, -1.5, 3.0), (0.6, 0, 0), (0, 0.6, 0), (6.0, 6.0, 6.0)))
    s.materials[1].clearcoat = 0.8
    s.materials[1].clearcoat_roughness = 0.2
    s.materials[1].sheen = 0.5
    s.materials[1].sheen_tint = 0.3
    s.materials[1].specular_tint = 0.4
    s.materials[1].subsurface = 0.3
    s.materials[1].anisotropic = 0.5
    S.preprocess_material(s.materials[1])
    return s


def media():
    return S.media_box(24, 24, 2, max_depth=10, rr_depth=3, seed=0)


def transparent():
    s = _cornell_base(24, 24, 3)
    panel = s.add_material(S.material((0.9, 0.8, 0.2), opacity=0.5))
    s.add_mesh(*S.quad_mesh((0.2, 0.3, 0.1), (0.6, 0, 0), (0, 0, 0.6)), panel)
    clear = s.add_material(S.material((0.5, 0.9, 0.6), opacity=0.0))
    s.add_mesh(*S.quad_mesh((0.1, 0.8, 0.6), (0.3, 0, 0), (0, 0, 0.3)), clear)
    return s


def media_transparent():
    s = S.media_box(24, 24, 2, max_depth=10, rr_depth=3, seed=0)
    panel = s.add_material(S.material((0.8, 0.8, 0.8), opacity=0.6))
    s.add_mesh(*S.quad_mesh((0.15, 0.4, 0.2), (0.7, 0, 0), (0, 0, 0.5)), panel)
    return s


def ortho_sky():
    s = S.disney_grid(24, 16, 2, segments=10, rings=5, env_size=(8, 4))
    s.env_rgb = None
    s.ground_color = (0.2, 0.15, 0.1, 1.0)
    s.sky_color = (0.4 * 4, 0.6 * 4, 0.9 * 4, 1.0)
    s.cameras = [S.look_at((0.0, -9.0, 6.0), (0.0, 0.0, 0.0), 40.0, ortho=(5.0, 3.3))]
    s.tonemap = (True, True, True)
    return s


def thin_lens_reinhard():
    s = _cornell_base(24, 24, 3)
    s.cameras = [S.look_at((0.5, -1.35, 0.5), (0.5, 0.5, 0.5), 40.0, aperture=0.02, focal_distance=1.8)]
    s.tonemap = (True, False, False)
    s.exposure_value = 0.5
    return s


def no_tonemap():
    s = _cornell_base(16, 16, 2)
    s.tonemap = (False, False, False)
    return s


def textured():
    """Every material map: a checker base colour on the floor (uv repeated
    2.5 times, so the sampler wraps), a normal map on the back wall, a
    metallic/roughness map on a Disney box, an emission map on a panel."""
    s = S.cornell(24, 24, 3, max_depth=6, rr_depth=2, seed=0, boxes=False)
    checker = s.add_texture(S.checker_texture())
    bumps = s.add_texture(S.bump_normal_map())
    mr = s.add_texture(S.metallic_roughness_texture())
    glow = s.add_texture(S.checker_texture(8, 2, (3.0, 2.0, 0.5), (0.0, 0.0, 0.0)))
    floor = s.materials[0]
    m_floor = S.material((1, 1, 1))
    m_floor.base_color_map_index = checker
    m_wall = S.material((0.7, 0.7, 0.7))
    m_wall.normal_map_index = bumps
    m_box = S.material((0.8, 0.5, 0.3), abi.MATERIAL_DISNEY, roughness=0.5)
    m_box.metallic_roughness_map_index = mr
    m_glow = S.material((0.2, 0.2, 0.2))
    m_glow.emission_map_index = glow
    del floor
    fi, wi, bi, gi = (s.add_material(m) for m in (m_floor, m_wall, m_box, m_glow))
    v, i, tr, _ = s.meshes[0]
    v = v.copy()
    v[:, 9:11] *= 2.5
    s.meshes[0] = (v, i, tr, fi)
    v, i, tr, _ = s.meshes[2]
    s.meshes[2] = (v, i, tr, wi)
    s.add_mesh(*S.box_mesh((0.35, 0.55, 0.25), (0.3, 0.3, 0.5), 20.0), bi)
    s.add_mesh(*S.quad_mesh((0.6, 0.7, 0.05), (0.25, 0, 0), (0, 0, 0.25)), gi)
    return s


PIN_SCENES = {
    "cornell": cornell, "disney_ibl": disney_ibl, "lights_icosphere": lights_icosphere, "media": media,
    "transparent": transparent, "media_transparent": media_transparent, "ortho_sky": ortho_sky,
    "thin_lens_reinhard": thin_lens_reinhard, "no_tonemap": no_tonemap, "textured": textured,
}
