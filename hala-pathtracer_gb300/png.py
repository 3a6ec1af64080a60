"""PNG images: decoding of glTF texture images and writing of the 8-bit
final image (the reference saves PNGs through the `image` crate, 0.25.2).

Reads non-interlaced PNGs of every colour type (grey, RGB, palette, grey +
alpha, RGBA) at bit depths 1-16, with all five scanline filters; returns
float32 RGBA in [0, 1]. Writes 8-bit RGB / RGBA with filter 0.
"""
import struct
import zlib

import numpy as np

SIGNATURE = b"\x89PNG\r\n\x1a\n"
CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


class PngError(ValueError):
    pass


def _unfilter(data, height, stride, bpp):
    out = np.zeros((height, stride), np.uint8)
    prev = np.zeros(stride, np.uint8)
    pos = 0
    for y in range(height):
        ftype = data[pos]
        row = np.frombuffer(data, np.uint8, stride, pos + 1).copy()
        pos += 1 + stride
        if ftype == 0:
            pass
        elif ftype == 1:  # Sub: cumulative per byte lane of the pixel
            for k in range(bpp):
                row[k::bpp] = np.cumsum(row[k::bpp], dtype=np.uint8)
        elif ftype == 2:  # Up
            row = row + prev
        elif ftype == 3:  # Average
            r = row.astype(np.int32)
            p = prev.astype(np.int32)
            for i in range(stride):
                left = r[i - bpp] if i >= bpp else 0
                r[i] = (r[i] + ((left + p[i]) >> 1)) & 0xFF
            row = r.astype(np.uint8)
        elif ftype == 4:  # Paeth
            r = row.astype(np.int32)
            p = prev.astype(np.int32)
            for i in range(stride):
                a = r[i - bpp] if i >= bpp else 0
                b = p[i]
                c = p[i - bpp] if i >= bpp else 0
                pp = a + b - c
                pa, pb, pc = abs(pp - a), abs(pp - b), abs(pp - c)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                r[i] = (r[i] + pred) & 0xFF
            row = r.astype(np.uint8)
        else:
            raise PngError(f"unknown filter type {ftype}")
        out[y] = row
        prev = row
    return out


def read(path_or_bytes):
    """(H, W, 4) float32 RGBA in [0, 1]."""
    if isinstance(path_or_bytes, (bytes, bytearray)):
        buf = bytes(path_or_bytes)
    else:
        with open(path_or_bytes, "rb") as f:
            buf = f.read()
    if not buf.startswith(SIGNATURE):
        raise PngError("not a PNG file")
    pos = 8
    idat, plte, trns, hdr = [], None, None, None
    while pos < len(buf):
        n, typ = struct.unpack_from(">I4s", buf, pos)
        data = buf[pos + 8:pos + 8 + n]
        pos += 12 + n
        if typ == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", data)
        elif typ == b"PLTE":
            plte = np.frombuffer(data, np.uint8).reshape(-1, 3)
        elif typ == b"tRNS":
            trns = data
        elif typ == b"IDAT":
            idat.append(data)
        elif typ == b"IEND":
            break
    if hdr is None:
        raise PngError("missing IHDR")
    W, H, depth, ctype, _comp, _filt, interlace = hdr
    if interlace:
        raise PngError("interlaced PNGs are not supported")
    if ctype not in CHANNELS:
        raise PngError(f"unknown colour type {ctype}")
    nch = CHANNELS[ctype]
    bits = depth * nch
    stride = (W * bits + 7) // 8
    bpp = max(1, bits // 8)
    raw = zlib.decompress(b"".join(idat))
    rows = _unfilter(raw, H, stride, bpp)
    if depth == 16:
        vals = rows.view(">u2").reshape(H, W, nch).astype(np.float32) / 65535.0
    elif depth == 8:
        vals = rows.reshape(H, W, nch).astype(np.float32)
        vals = vals if ctype == 3 else vals / 255.0
    else:  # 1, 2, 4 bits: unpack
        bitsarr = np.unpackbits(rows, axis=1)[:, :W * depth].reshape(H, W, depth)
        weights = (1 << np.arange(depth - 1, -1, -1)).astype(np.uint16)
        v = (bitsarr * weights).sum(-1).astype(np.float32)[..., None]
        vals = v if ctype == 3 else v / float((1 << depth) - 1)
    if ctype == 3:
        if plte is None:
            raise PngError("palette image without PLTE")
        idx = vals[..., 0].astype(np.int64)
        rgb = plte[idx].astype(np.float32) / 255.0
        alpha = np.ones((H, W, 1), np.float32)
        if trns is not None:
            a = np.full(len(plte), 255, np.uint8)
            a[:len(trns)] = np.frombuffer(trns, np.uint8)
            alpha = (a[idx].astype(np.float32) / 255.0)[..., None]
        return np.concatenate([rgb, alpha], -1)
    if nch == 1:
        return np.concatenate([vals, vals, vals, np.ones_like(vals)], -1)
    if nch == 2:
        g = vals[..., :1]
        return np.concatenate([g, g, g, vals[..., 1:2]], -1)
    if nch == 3:
        return np.concatenate([vals, np.ones((H, W, 1), np.float32)], -1)
    return vals


def _chunk(typ, data):
    return struct.pack(">I", len(data)) + typ + data + struct.pack(">I", zlib.crc32(typ + data) & 0xFFFFFFFF)


def write(path, rgb8):
    """Writes an (H, W, 3|4) uint8 image."""
    a = np.ascontiguousarray(rgb8, np.uint8)
    H, W, C = a.shape
    ctype = {3: 2, 4: 6}[C]
    raw = b"".join(b"\0" + a[y].tobytes() for y in range(H))
    data = SIGNATURE + _chunk(b"IHDR", struct.pack(">IIBBBBB", W, H, 8, ctype, 0, 0, 0))
    data += _chunk(b"IDAT", zlib.compress(raw, 6)) + _chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(data)
