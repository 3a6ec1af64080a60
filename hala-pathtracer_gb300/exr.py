"""OpenEXR scanline images: the HDRI loader behind set_envmap and the writer
used for image output.

The reference loads its HDRIs with the `exr` crate (1.72.0) inside its
renderer crate (src/bin/hala-pathtracer.rs:203, `set_envmap(path,
rotation)`). This module reads the parts of the OpenEXR 2 file format that
HDRI files use: single-part scanline images, HALF / FLOAT / UINT channels,
compression NONE, RLE, ZIPS and ZIP. Tiled, deep and multi-part files and
the PIZ / PXR24 / B44 / DWA codecs are refused with a clear error.

Channel data of a block is stored line by line, channels in the (sorted)
order of the channel list. RLE and ZIP store it reordered (even bytes, then
odd bytes) and delta-coded before compression; a chunk whose compressed size
equals its raw size is stored raw.
"""
import struct
import zlib

import numpy as np

MAGIC = 20000630
COMPRESSION = {0: "NONE", 1: "RLE", 2: "ZIPS", 3: "ZIP", 4: "PIZ", 5: "PXR24", 6: "B44", 7: "B44A", 8: "DWAA",
               9: "DWAB"}
LINES_PER_BLOCK = {0: 1, 1: 1, 2: 1, 3: 16}
PIXEL_TYPES = {0: (np.uint32, 4), 1: (np.float16, 2), 2: (np.float32, 4)}


class ExrError(ValueError):
    pass


def _cstr(buf, pos):
    end = buf.index(b"\0", pos)
    return buf[pos:end].decode("latin-1"), end + 1


def _read_header(buf):
    if len(buf) < 8 or struct.unpack_from("<i", buf, 0)[0] != MAGIC:
        raise ExrError("not an OpenEXR file")
    version = struct.unpack_from("<I", buf, 4)[0]
    if version & 0x200:
        raise ExrError("tiled OpenEXR files are not supported")
    if version & 0x1800:
        raise ExrError("deep or multi-part OpenEXR files are not supported")
    pos = 8
    attrs = {}
    while True:
        if buf[pos] == 0:
            pos += 1
            break
        name, pos = _cstr(buf, pos)
        typ, pos = _cstr(buf, pos)
        size = struct.unpack_from("<i", buf, pos)[0]
        pos += 4
        attrs[name] = (typ, buf[pos:pos + size])
        pos += size
    return attrs, pos


def _channels(raw):
    chans, pos = [], 0
    while raw[pos] != 0:
        name, pos = _cstr(raw, pos)
        ptype, _plinear, xs, ys = struct.unpack_from("<iB3xii", raw, pos)
        pos += 16
        if xs != 1 or ys != 1:
            raise ExrError(f"channel {name} is subsampled")
        chans.append((name, ptype))
    return chans


def _undo_predictor_reorder(t):
    t = np.frombuffer(t, np.uint8).copy()
    # delta decoding: t[i] = t[i-1] + t[i] - 128 (mod 256)
    t[1:] -= 128
    t = np.cumsum(t, dtype=np.uint8)
    n = len(t)
    half = (n + 1) // 2
    out = np.empty(n, np.uint8)
    out[0::2] = t[:half]
    out[1::2] = t[half:]
    return out.tobytes()


def _apply_predictor_reorder(raw):
    r = np.frombuffer(raw, np.uint8)
    t = np.concatenate([r[0::2], r[1::2]])
    d = t.astype(np.int16)
    d[1:] = (t[1:].astype(np.int16) - t[:-1].astype(np.int16) + 128 + 256) & 0xFF
    return d.astype(np.uint8).tobytes()


def _rle_decode(data, expected):
    out = bytearray()
    i = 0
    while i < len(data):
        c = struct.unpack_from("b", data, i)[0]
        i += 1
        if c < 0:
            out += data[i:i - c]
            i -= c
        else:
            out += bytes([data[i]]) * (c + 1)
            i += 1
    if len(out) != expected:
        raise ExrError("corrupt RLE block")
    return bytes(out)


def read(path_or_bytes):
    """Returns (channels dict name -> (H, W) float32 array, attributes)."""
    if isinstance(path_or_bytes, (bytes, bytearray)):
        buf = bytes(path_or_bytes)
    else:
        with open(path_or_bytes, "rb") as f:
            buf = f.read()
    attrs, pos = _read_header(buf)
    for req in ("channels", "compression", "dataWindow"):
        if req not in attrs:
            raise ExrError(f"header lacks {req}")
    comp = attrs["compression"][1][0]
    if comp not in LINES_PER_BLOCK:
        raise ExrError(f"compression {COMPRESSION.get(comp, comp)} is not supported (NONE, RLE, ZIPS, ZIP are)")
    xmin, ymin, xmax, ymax = struct.unpack("<iiii", attrs["dataWindow"][1])
    W, H = xmax - xmin + 1, ymax - ymin + 1
    if W <= 0 or H <= 0:
        raise ExrError("empty data window")
    chans = _channels(attrs["channels"][1])
    for _, t in chans:
        if t not in PIXEL_TYPES:
            raise ExrError(f"unknown pixel type {t}")
    lpb = LINES_PER_BLOCK[comp]
    nblocks = (H + lpb - 1) // lpb
    offsets = struct.unpack_from(f"<{nblocks}Q", buf, pos)
    row_bytes = sum(PIXEL_TYPES[t][1] for _, t in chans) * W
    out = {name: np.empty((H, W), np.float32) for name, _ in chans}
    for off in offsets:
        y, size = struct.unpack_from("<ii", buf, off)
        data = buf[off + 8:off + 8 + size]
        y0 = y - ymin
        if y0 < 0 or y0 >= H:
            raise ExrError("chunk outside the data window")
        lines = min(lpb, H - y0)
        raw_size = row_bytes * lines
        if size == raw_size or comp == 0:
            raw = data
        elif comp == 1:
            raw = _undo_predictor_reorder(_rle_decode(data, raw_size))
        else:
            raw = _undo_predictor_reorder(zlib.decompress(data))
        if len(raw) != raw_size:
            raise ExrError("corrupt block size")
        p = 0
        for ly in range(lines):
            for name, t in chans:
                dt, bpp = PIXEL_TYPES[t]
                out[name][y0 + ly] = np.frombuffer(raw, dt, W, p).astype(np.float32)
                p += bpp * W
    return out, attrs


def read_rgb(path_or_bytes):
    """(H, W, 3) float32 RGB; a single luminance channel Y is repeated."""
    ch, _ = read(path_or_bytes)
    names = {n.split(".")[-1]: n for n in ch}
    if all(k in names for k in "RGB"):
        return np.stack([ch[names["R"]], ch[names["G"]], ch[names["B"]]], -1)
    if "Y" in names:
        y = ch[names["Y"]]
        return np.stack([y, y, y], -1)
    raise ExrError(f"no RGB channels in {sorted(ch)}")


def _attr(name, typ, value):
    return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(value)) + value


def write(path, rgb, half=False, compression="ZIP"):
    """Writes an (H, W, 3) image as a scanline OpenEXR file (NONE or ZIP)."""
    rgb = np.ascontiguousarray(rgb, np.float32)
    H, W = rgb.shape[:2]
    comp = {"NONE": 0, "ZIP": 3}[compression]
    ptype = 1 if half else 2
    dt = np.float16 if half else np.float32
    chl = b"".join(n.encode() + b"\0" + struct.pack("<iB3xii", ptype, 0, 1, 1) for n in "BGR") + b"\0"
    hdr = struct.pack("<iI", MAGIC, 2)
    hdr += _attr("channels", "chlist", chl)
    hdr += _attr("compression", "compression", bytes([comp]))
    hdr += _attr("dataWindow", "box2i", struct.pack("<iiii", 0, 0, W - 1, H - 1))
    hdr += _attr("displayWindow", "box2i", struct.pack("<iiii", 0, 0, W - 1, H - 1))
    hdr += _attr("lineOrder", "lineOrder", bytes([0]))
    hdr += _attr("pixelAspectRatio", "float", struct.pack("<f", 1.0))
    hdr += _attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0))
    hdr += _attr("screenWindowWidth", "float", struct.pack("<f", 1.0))
    hdr += b"\0"
    lpb = LINES_PER_BLOCK[comp]
    nblocks = (H + lpb - 1) // lpb
    chunks = []
    for b in range(nblocks):
        y0 = b * lpb
        raw = b"".join(rgb[y, :, c].astype(dt).tobytes() for y in range(y0, min(H, y0 + lpb)) for c in (2, 1, 0))
        data = raw
        if comp == 3:
            z = zlib.compress(_apply_predictor_reorder(raw), 6)
            if len(z) < len(raw):
                data = z
        chunks.append(struct.pack("<ii", y0, len(data)) + data)
    pos = len(hdr) + 8 * nblocks
    offsets = []
    for c in chunks:
        offsets.append(pos)
        pos += len(c)
    with open(path, "wb") as f:
        f.write(hdr + struct.pack(f"<{nblocks}Q", *offsets) + b"".join(chunks))
