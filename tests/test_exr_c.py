"""The library's own OpenEXR reader (pt_exr_read_rgb, behind
pt_renderer_set_envmap_file) against the Python loader exr.py: the same
floats, bit for bit, for every compression and pixel type they support and
for DEFLATE streams of all three block kinds (stored, fixed and dynamic
Huffman codes). Loads libhalapt.so on the CPU; no GPU call."""
import importlib
import struct
import zlib

import numpy as np
import pytest


@pytest.fixture(scope="module")
def exr(pt):
    return importlib.import_module("hala-pathtracer_gb300.exr")


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


def write_exr(path, channels, comp, exr, zlevel=6, strategy=zlib.Z_DEFAULT_STRATEGY, ymin=0):
    """channels: {name: (H, W) array of uint32 / float16 / float32}, written in
    sorted name order. comp 0 NONE, 1 RLE, 2 ZIPS, 3 ZIP."""
    names = sorted(channels)
    H, W = channels[names[0]].shape
    ptype = {np.dtype(np.uint32): 0, np.dtype(np.float16): 1, np.dtype(np.float32): 2}

    def attr(n, t, v):
        return n.encode() + b"\0" + t.encode() + b"\0" + struct.pack("<i", len(v)) + v
    chl = b"".join(n.encode() + b"\0" + struct.pack("<iB3xii", ptype[channels[n].dtype], 0, 1, 1) for n in names)
    hdr = struct.pack("<iI", 20000630, 2)
    hdr += attr("channels", "chlist", chl + b"\0")
    hdr += attr("compression", "compression", bytes([comp]))
    hdr += attr("dataWindow", "box2i", struct.pack("<iiii", 0, ymin, W - 1, ymin + H - 1))
    hdr += attr("lineOrder", "lineOrder", b"\0") + b"\0"
    lpb = 16 if comp == 3 else 1
    chunks = []
    for y0 in range(0, H, lpb):
        raw = b"".join(channels[n][y].tobytes() for y in range(y0, min(H, y0 + lpb)) for n in names)
        data = raw
        if comp == 1:
            data = _rle(exr._apply_predictor_reorder(raw))
        elif comp in (2, 3):
            c = zlib.compressobj(zlevel, zlib.DEFLATED, 15, 9, strategy)
            data = c.compress(exr._apply_predictor_reorder(raw)) + c.flush()
        if len(data) >= len(raw):
            data = raw
        chunks.append(struct.pack("<ii", ymin + y0, len(data)) + data)
    pos = len(hdr) + 8 * len(chunks)
    offs = []
    for c in chunks:
        offs.append(pos)
        pos += len(c)
    with open(path, "wb") as f:
        f.write(hdr + struct.pack(f"<{len(chunks)}Q", *offs) + b"".join(chunks))


def _hdr_image(H, W, seed):
    rng = np.random.default_rng(seed)
    img = np.exp(rng.normal(0, 2, (H, W, 3))).astype(np.float32)
    img[H // 2:, : W // 3] = 0.25  # runs for RLE and long DEFLATE matches
    return img


@pytest.mark.parametrize("comp", [0, 1, 2, 3])
@pytest.mark.parametrize("dtype", [np.float32, np.float16])
def test_rgb_files_read_like_exr_py(pt, gpu_lib, exr, tmp_path, comp, dtype):
    img = _hdr_image(37, 53, 3).astype(dtype)
    p = str(tmp_path / f"c{comp}.exr")
    write_exr(p, {"R": img[..., 0], "G": img[..., 1], "B": img[..., 2]}, comp, exr, ymin=-5)
    got = pt.read_exr(p)
    want = exr.read_rgb(p)
    assert got.shape == (37, 53, 3)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("level,strategy", [(0, zlib.Z_DEFAULT_STRATEGY), (1, zlib.Z_FIXED),
                                            (9, zlib.Z_DEFAULT_STRATEGY), (6, zlib.Z_HUFFMAN_ONLY),
                                            (6, zlib.Z_RLE)])
def test_deflate_block_kinds(pt, gpu_lib, exr, tmp_path, level, strategy):
    img = _hdr_image(64, 200, 5)
    p = str(tmp_path / "z.exr")
    write_exr(p, {"R": img[..., 0], "G": img[..., 1], "B": img[..., 2]}, 3, exr, zlevel=level, strategy=strategy)
    assert np.array_equal(pt.read_exr(p).view(np.uint32), exr.read_rgb(p).view(np.uint32))


def test_uint_and_luminance_channels(pt, gpu_lib, exr, tmp_path):
    rng = np.random.default_rng(2)
    y = rng.integers(0, 1 << 20, size=(9, 11), dtype=np.uint32)
    p = str(tmp_path / "y.exr")
    write_exr(p, {"Y": y}, 3, exr)
    got = pt.read_exr(p)
    assert np.array_equal(got, exr.read_rgb(p))
    assert np.array_equal(got[..., 1], y.astype(np.float32))
    # layer-qualified names with extra channels (A) around R, G, B
    img = _hdr_image(8, 12, 7)
    a = np.ones((8, 12), np.float16)
    q = str(tmp_path / "layer.exr")
    write_exr(q, {"diffuse.R": img[..., 0], "diffuse.G": img[..., 1], "diffuse.B": img[..., 2], "diffuse.A": a}, 2,
              exr)
    assert np.array_equal(pt.read_exr(q).view(np.uint32), exr.read_rgb(q).view(np.uint32))


def test_files_the_reader_refuses(pt, gpu_lib, exr, tmp_path):
    img = np.full((16, 40, 3), 0.75, np.float32)  # compressible: the chunk is a DEFLATE stream
    p = str(tmp_path / "ok.exr")
    write_exr(p, {"R": img[..., 0], "G": img[..., 1], "B": img[..., 2]}, 3, exr)
    data = bytearray(open(p, "rb").read())
    assert len(data) < 16 * 40 * 12

    def refused(raw, match):
        q = str(tmp_path / "bad.exr")
        open(q, "wb").write(bytes(raw))
        with pytest.raises(pt.PTError, match=match):
            pt.read_exr(q)

    i = data.index(b"compression\0compression\0") + len(b"compression\0compression\0") + 4
    piz = bytearray(data)
    piz[i] = 4
    refused(piz, "not supported")
    tiled = bytearray(data)
    tiled[4:8] = struct.pack("<I", 2 | 0x200)
    refused(tiled, "tiled")
    refused(data[: len(data) - 7], "corrupt|truncated")
    refused(b"not an exr file at all", "not an OpenEXR")
    broken = bytearray(data)
    broken[-3] ^= 0x5A  # inside the last chunk's DEFLATE stream (Adler-32 or codes)
    refused(broken, "corrupt")
    with pytest.raises(pt.PTError, match="cannot open"):
        pt.read_exr(str(tmp_path / "missing.exr"))


def test_mutated_files_are_read_or_refused(pt, exr, tmp_path):
    """Seeded byte mutations of EXR files (header attributes, offset table,
    chunk sizes, ZIP streams): each is read or refused with a reason, never a
    crash."""
    import ctypes as C
    import random
    abi = importlib.import_module("hala-pathtracer_gb300.abi")
    pt.build()
    lib = pt.load_library()
    rng = np.random.default_rng(1)
    seeds = []
    for k, (half, comp) in enumerate([(False, "ZIP"), (True, "ZIP"), (False, "NONE"), (True, "NONE")]):
        p = tmp_path / f"s{k}.exr"
        exr.write(str(p), (rng.random((19, 23, 3)) * 5).astype(np.float32), half=half, compression=comp)
        seeds.append(p.read_bytes())
    r = random.Random(5)
    p = tmp_path / "m.exr"
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
                b[k:k + 4] = r.choice([b"\xff\xff\xff\xff", b"\xff\xff\xff\x7f", b"\0\0\x01\0", b"\0\0\0\0"])
        p.write_bytes(bytes(b))
        w, h = C.c_uint32(), C.c_uint32()
        err = C.create_string_buffer(256)
        st = lib.pt_exr_read_rgb(str(p).encode(), None, 0, C.byref(w), C.byref(h), err, 256)
        if st == abi.PT_OK:
            out = np.empty((h.value, w.value, 3), np.float32)
            st = lib.pt_exr_read_rgb(str(p).encode(), out.ctypes.data, out.size, C.byref(w), C.byref(h), err, 256)
        assert st in seen, st
        seen[st] += 1
        if st != abi.PT_OK:
            assert err.value
    assert seen[abi.PT_OK] > 0 and seen[abi.PT_ERR_INVALID_ARG] > 0
