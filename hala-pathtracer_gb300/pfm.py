"""Portable float map (PFM) reader and writer.

save_images writes `<prefix>_color.pfm`, `_albedo.pfm` and `_normal.pfm`
(the three files denoise.py:11-19 of the reference reads): a text header
"PF\\n<width> <height>\\n<scale>\\n" and RGB float32 rows from the bottom of the
image to the top, little-endian when the scale is negative.
"""
import numpy as np


class PfmError(ValueError):
    pass


def read(path_or_bytes):
    """(H, W, 3) float32 with row 0 at the top of the image (or (H, W) for a
    greyscale "Pf" file)."""
    if isinstance(path_or_bytes, (bytes, bytearray)):
        buf = bytes(path_or_bytes)
    else:
        with open(path_or_bytes, "rb") as f:
            buf = f.read()
    fields, pos = [], 0
    while len(fields) < 4:
        while pos < len(buf) and buf[pos:pos + 1].isspace():
            pos += 1
        end = pos
        while end < len(buf) and not buf[end:end + 1].isspace():
            end += 1
        if end == pos:
            raise PfmError("truncated header")
        fields.append(buf[pos:end].decode("ascii"))
        pos = end
    pos += 1  # the single whitespace character after the scale
    kind, w, h, scale = fields[0], int(fields[1]), int(fields[2]), float(fields[3])
    if kind not in ("PF", "Pf"):
        raise PfmError(f"not a PFM file ({kind!r})")
    ch = 3 if kind == "PF" else 1
    dt = np.dtype("<f4") if scale < 0 else np.dtype(">f4")
    n = w * h * ch
    if len(buf) - pos < 4 * n:
        raise PfmError("truncated pixel data")
    px = np.frombuffer(buf, dt, n, pos).astype(np.float32)
    img = px.reshape(h, w, ch)[::-1]
    return np.ascontiguousarray(img if ch == 3 else img[..., 0])


def write(path, img):
    """Writes (H, W, 3) (or (H, W, 4): alpha dropped) float data as a
    little-endian PFM, rows bottom to top."""
    a = np.asarray(img, np.float32)
    if a.ndim != 3 or a.shape[2] < 3:
        raise PfmError("expected an (H, W, 3) image")
    h, w = a.shape[:2]
    with open(path, "wb") as f:
        f.write(f"PF\n{w} {h}\n-1.0\n".encode("ascii"))
        f.write(np.ascontiguousarray(a[::-1, :, :3]).astype("<f4").tobytes())
