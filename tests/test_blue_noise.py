"""The camera jitter's blue-noise texture (load_blue_noise_texture,
src/bin/hala-pathtracer.rs:195; rand4blue, wltcRS.glsl:43-53).

CPU: the library's RGBA8 PNG reader (pt_png_read_rgba8) against png.py for
every 8-bit layout and the refusals; the oracle's texture path, fed the
substitute table itself, gives the substitute's images bit for bit, and
another table changes them. GPU: with a loaded texture the device paths
equal the oracle's with the same texture, bit for bit, and loading the PNG
file equals setting its texels."""
import importlib
import struct
import zlib

import numpy as np
import pytest


def _png(pixels, depth, ctype, plte=None, trns=None):
    from tests.test_gltf_c import _png as make
    return make(pixels, depth, ctype, plte, trns)


def substitute_table():
    """The substitute texels: top bytes of pcg4d(x, y, 0x2545F491, 0x9E3779B9)."""
    y, x = np.mgrid[0:1024, 0:1024].astype(np.uint32)
    v = [x.copy(), y.copy(), np.full_like(x, 0x2545F491), np.full_like(x, 0x9E3779B9)]
    with np.errstate(over="ignore"):
        v = [a * np.uint32(1664525) + np.uint32(1013904223) for a in v]
        for shift in (False, True):
            if shift:
                v = [a ^ (a >> np.uint32(16)) for a in v]
            v[0] += v[1] * v[3]
            v[1] += v[2] * v[0]
            v[2] += v[0] * v[1]
            v[3] += v[1] * v[2]
    return np.stack([(a >> np.uint32(24)).astype(np.uint8) for a in v], -1)


def test_png_rgba8_reader_matches_png_py(pt, tmp_path):
    png = importlib.import_module("hala-pathtracer_gb300.png")
    pt.build()
    rng = np.random.default_rng(2)
    cases = {
        "rgba": (rng.integers(0, 256, (5, 7, 4)), 8, 6, None, None),
        "rgb": (rng.integers(0, 256, (4, 3, 3)), 8, 2, None, None),
        "grey": (rng.integers(0, 256, (3, 6, 1)), 8, 0, None, None),
        "grey_alpha": (rng.integers(0, 256, (2, 5, 2)), 8, 4, None, None),
        "palette": (rng.integers(0, 5, (6, 4, 1)), 8, 3, rng.integers(0, 256, 15).tolist(), [10, 200]),
        "palette_2bit": (rng.integers(0, 4, (3, 9, 1)), 2, 3, rng.integers(0, 256, 12).tolist(), None),
    }
    for name, (px, depth, ctype, plte, trns) in cases.items():
        p = tmp_path / f"{name}.png"
        p.write_bytes(_png(px, depth, ctype, plte, trns))
        got = pt.read_png_rgba8(p)
        want = np.round(png.read(str(p)) * 255.0).astype(np.uint8)
        assert np.array_equal(got, want), name
    for name, (px, depth, ctype) in {"sixteen": (rng.integers(0, 65536, (2, 2, 3)), 16, 2),
                                     "grey4": (rng.integers(0, 16, (2, 2, 1)), 4, 0)}.items():
        p = tmp_path / f"{name}.png"
        p.write_bytes(_png(px, depth, ctype))
        with pytest.raises(pt.PTError, match="8-bit"):
            pt.read_png_rgba8(p)
    bad = tmp_path / "bad.png"
    bad.write_bytes(b"\x89PNG\r\n\x1a\n" + b"\0" * 10)
    with pytest.raises(pt.PTError, match="bad.png"):
        pt.read_png_rgba8(bad)


def test_oracle_texture_path(oracle_mod):
    from tests.golden import pin_scenes
    s = pin_scenes.PIN_SCENES["cornell"]()
    base = oracle_mod.Oracle(s)
    base.render(2)
    s.blue_noise = substitute_table()
    same = oracle_mod.Oracle(s)
    same.render(2)
    assert np.array_equal(base.image(0).view(np.uint32), same.image(0).view(np.uint32))
    s.blue_noise = np.random.default_rng(4).integers(0, 256, (1024, 1024, 4)).astype(np.uint8)
    other = oracle_mod.Oracle(s)
    other.render(2)
    assert not np.array_equal(base.image(0), other.image(0))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cornell", "thin_lens_reinhard", "ortho_sky"])
def test_loaded_texture_paths_match_the_oracle(pt, oracle_mod, tmp_path, name):
    from tests.golden import pin_scenes
    s = pin_scenes.PIN_SCENES[name]()
    tex = np.random.default_rng(9).integers(0, 256, (1024, 1024, 4)).astype(np.uint8)
    s.blue_noise = tex
    WH = s.width * s.height
    r = pt.renderer_for(s, keep_samples=1)
    r.render(s.spp)
    rad_g, hash_g = r.samples()
    o = oracle_mod.Oracle(s)
    rad_o, hash_o = o.trace_paths(np.arange(WH), 0, s.spp)
    assert np.array_equal(hash_g, hash_o.reshape(-1))
    assert np.array_equal(rad_g.view(np.uint32), rad_o.reshape(-1, 3).view(np.uint32))
    # the same texels from an 8-bit RGBA PNG, larger than 1024 x 1024 (the
    # top-left 1024 x 1024 are fetched)
    big = np.zeros((1030, 1100, 4), np.uint8)
    big[:1024, :1024] = tex
    p = tmp_path / "blue_noise.png"
    p.write_bytes(_png(big, 8, 6))
    s2 = pin_scenes.PIN_SCENES[name]()
    a = pt.renderer_for(s2)
    a.load_blue_noise_texture(p)
    a.render(s2.spp)
    b = pt.renderer_for(s)
    b.render(s.spp)
    for k in (0, 1, 2, 3):
        assert np.array_equal(a.image(k).view(np.uint8), b.image(k).view(np.uint8)), k
    # back to the substitute
    a.load_blue_noise_texture(None)
    a.reset()
    a.render(s2.spp)
    c = pt.renderer_for(s2)
    c.render(s2.spp)
    assert np.array_equal(a.image(0).view(np.uint8), c.image(0).view(np.uint8))
    small = tmp_path / "small.png"
    small.write_bytes(_png(tex[:512, :512], 8, 6))
    with pytest.raises(pt.PTError, match="smaller than 1024"):
        a.load_blue_noise_texture(small)
    for x in (r, a, b, c):
        x.close()


def test_mutated_pngs_are_read_or_refused(pt, tmp_path):
    """Seeded byte mutations of PNGs of four layouts (chunk lengths, header
    fields, compressed data): each is read or refused with a reason, never a
    crash."""
    import ctypes as C
    import random
    abi = importlib.import_module("hala-pathtracer_gb300.abi")
    pt.build()
    lib = pt.load_library()
    rng = np.random.default_rng(1)
    seeds = [_png(rng.integers(0, 256, (9, 7, 4)), 8, 6),
             _png(rng.integers(0, 4, (5, 6, 1)), 2, 3, rng.integers(0, 256, 12).tolist(), [1, 2]),
             _png(rng.integers(0, 65536, (3, 3, 3)), 16, 2), _png(rng.integers(0, 256, (4, 4, 2)), 8, 4)]
    r = random.Random(3)
    p = tmp_path / "m.png"
    seen = {abi.PT_OK: 0, abi.PT_ERR_INVALID_ARG: 0}
    for _ in range(600):
        b = bytearray(r.choice(seeds))
        for _ in range(r.randint(1, 4)):
            k = r.randrange(len(b))
            op = r.random()
            if op < 0.5:
                b[k] = r.randrange(256)
            elif op < 0.7:
                del b[k:k + r.randint(1, 8)]
            elif op < 0.85:
                b[k:k] = bytes(r.randrange(256) for _ in range(r.randint(1, 8)))
            else:
                b[k:k + 4] = r.choice([b"\xff\xff\xff\xff", b"\x7f\xff\xff\xff", b"\x00\x01\x00\x00", b"\0\0\0\0"])
        p.write_bytes(bytes(b))
        w, h = C.c_uint32(), C.c_uint32()
        err = C.create_string_buffer(256)
        st = lib.pt_png_read_rgba8(str(p).encode(), None, 0, C.byref(w), C.byref(h), err, 256)
        assert st in seen, st
        seen[st] += 1
        if st != abi.PT_OK:
            assert err.value
    assert seen[abi.PT_OK] > 0 and seen[abi.PT_ERR_INVALID_ARG] > 0
