"""Render export as vkrt writes it (src/core/utility/export/image.c, exr.cpp): the linear image from the
accumulation and the display image from the linear one, written as EXR (linear RGBA32F) or 16-bit PNG (display).

* linear (image.c:907-951): RGB mode keeps the accumulation's linear sRGB; spectral mode converts its CIE XYZ with a
  Bradford adaptation from the equal-energy white to D65 and the XYZ -> linear sRGB matrix; non-finite values -> 0;
  alpha 1.
* display (image.c:641-699): exposure, ACES fit when the tone-mapping mode is ACES, sRGB transfer function, each
  channel clamped to [0, 1] and stored as round(v * 65535); alpha 65535.
* EXR: scanline, uncompressed, four FLOAT channels (vkrt writes FP32 through tinyexr's SaveEXR).
* PNG: 16 bits per channel RGBA (vkrt writes 16-bit RGBA through libspng). JPEG is not written (no encoder here).

Readers for both formats (the subset written here) serve the tests.
"""
from __future__ import annotations

import struct
import zlib
from pathlib import Path

import numpy as np

from . import abi

_BRADFORD = np.array([[0.8951, 0.2664, -0.1614], [-0.7502, 1.7135, 0.0367], [0.0389, -0.0685, 1.0296]], np.float32)
_BRADFORD_INV = np.array([[0.9869929, -0.1470543, 0.1599627], [0.4323053, 0.5183603, 0.0492912],
                          [-0.0085287, 0.0400428, 0.9684867]], np.float32)
_E_TO_D65 = np.array([0.9413344, 1.0404175, 1.0895327], np.float32)
_XYZ_TO_SRGB = np.array([[3.2404542, -1.5371385, -0.4985314], [-0.9692660, 1.8760108, 0.0415560],
                         [0.0556434, -0.2040259, 1.0572252]], np.float32)
TONE_MAPPING_ACES = 1


def _settings(scene_data):
    sd = np.asarray(scene_data).reshape(-1)[0]
    tone, mode, _ = abi.unpack_render_settings(int(sd["packedRenderSettings"]))
    return sd, tone, mode


def linear_rgba(accumulation: np.ndarray, scene_data) -> np.ndarray:
    """(H, W, 4) float32 linear sRGB with alpha 1, from an accumulation image (RGB or spectral XYZ)."""
    _, _, mode = _settings(scene_data)
    a = np.asarray(accumulation, np.float32)
    out = np.ones(a.shape[:2] + (4,), np.float32)
    rgb = a[..., :3].astype(np.float32)
    if mode == abi.RENDER_MODE_SPECTRAL:
        lms = rgb @ _BRADFORD.T
        rgb = ((lms * _E_TO_D65) @ _BRADFORD_INV.T) @ _XYZ_TO_SRGB.T
    out[..., :3] = np.where(np.isfinite(rgb), rgb, 0.0)
    return out


def _srgb_encode(v):
    v = np.clip(v, 0.0, 1.0)
    return np.where(v <= 0.0031308, 12.92 * v, 1.055 * np.power(v, np.float32(1.0 / 2.4)) - 0.055).astype(np.float32)


def display_rgba16(linear: np.ndarray, scene_data) -> np.ndarray:
    """(H, W, 4) uint16 display image from a linear image."""
    sd, tone, _ = _settings(scene_data)
    exposure = np.float32(sd["exposure"])
    if not np.isfinite(exposure) or exposure < 0:
        exposure = np.float32(1.0)
    c = np.asarray(linear, np.float32)[..., :3] * exposure
    if tone == TONE_MAPPING_ACES:
        c = (c * (np.float32(2.51) * c + np.float32(0.03))) / (c * (np.float32(2.43) * c + np.float32(0.59))
                                                                + np.float32(0.14))
    enc = _srgb_encode(c)
    out = np.full(c.shape[:2] + (4,), 65535, np.uint16)
    out[..., :3] = (np.clip(enc, 0.0, 1.0) * np.float32(65535.0) + np.float32(0.5)).astype(np.uint16)
    return out


# ---- PNG --------------------------------------------------------------------------------------------------------------
def _chunk(kind: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)


def write_png16(path, rgba16: np.ndarray) -> None:
    img = np.ascontiguousarray(rgba16, np.uint16)
    h, w = img.shape[:2]
    rows = img.astype(">u2").reshape(h, w * 4).view(np.uint8)
    raw = np.zeros((h, 1 + w * 8), np.uint8)  # filter type 0 per scanline
    raw[:, 1:] = rows
    data = (b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 16, 6, 0, 0, 0))
            + _chunk(b"IDAT", zlib.compress(raw.tobytes(), 6)) + _chunk(b"IEND", b""))
    Path(path).write_bytes(data)


def read_png16(path) -> np.ndarray:
    data = Path(path).read_bytes()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    off, idat, w = 8, b"", None
    while off < len(data):
        n = struct.unpack(">I", data[off:off + 4])[0]
        kind, body = data[off + 4:off + 8], data[off + 8:off + 8 + n]
        if kind == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            if depth != 16 or ctype != 6:
                raise ValueError("only 16-bit RGBA PNG files are read")
        elif kind == b"IDAT":
            idat += body
        off += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + w * 8)
    if np.any(raw[:, 0] != 0):
        raise ValueError("only unfiltered scanlines are read")
    return raw[:, 1:].copy().view(">u2").astype(np.uint16).reshape(h, w, 4)


# ---- OpenEXR (scanline, no compression, FLOAT) ------------------------------------------------------------------------
def _attr(name: str, kind: str, value: bytes) -> bytes:
    return name.encode() + b"\0" + kind.encode() + b"\0" + struct.pack("<i", len(value)) + value


def write_exr(path, rgba32f: np.ndarray) -> None:
    img = np.ascontiguousarray(rgba32f, np.float32)
    h, w = img.shape[:2]
    names = ["A", "B", "G", "R"]  # channels are stored in alphabetical order
    chlist = b"".join(n.encode() + b"\0" + struct.pack("<iBBBBii", 2, 0, 0, 0, 0, 1, 1) for n in names) + b"\0"
    box = struct.pack("<iiii", 0, 0, w - 1, h - 1)
    header = (struct.pack("<ii", 20000630, 2) + _attr("channels", "chlist", chlist)
              + _attr("compression", "compression", b"\0") + _attr("dataWindow", "box2i", box)
              + _attr("displayWindow", "box2i", box) + _attr("lineOrder", "lineOrder", b"\0")
              + _attr("pixelAspectRatio", "float", struct.pack("<f", 1.0))
              + _attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0))
              + _attr("screenWindowWidth", "float", struct.pack("<f", 1.0)) + b"\0")
    line = 4 * 4 * w
    table_end = len(header) + 8 * h
    offsets = [table_end + y * (8 + line) for y in range(h)]
    chans = [img[..., 3], img[..., 2], img[..., 1], img[..., 0]]
    blocks = bytearray()
    for y in range(h):
        blocks += struct.pack("<ii", y, line)
        for c in chans:
            blocks += c[y].astype("<f4").tobytes()
    Path(path).write_bytes(header + struct.pack(f"<{h}Q", *offsets) + bytes(blocks))


def read_exr(path) -> np.ndarray:
    data = Path(path).read_bytes()
    magic, _ = struct.unpack_from("<ii", data, 0)
    if magic != 20000630:
        raise ValueError("not an OpenEXR file")
    off, attrs = 8, {}
    while data[off] != 0:
        end = data.index(b"\0", off)
        name = data[off:end].decode()
        tend = data.index(b"\0", end + 1)
        size = struct.unpack_from("<i", data, tend + 1)[0]
        attrs[name] = data[tend + 5:tend + 5 + size]
        off = tend + 5 + size
    off += 1
    if attrs.get("compression") != b"\0":
        raise ValueError("only uncompressed EXR files are read")
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    names, p, cl = [], 0, attrs["channels"]
    while cl[p] != 0:
        e = cl.index(b"\0", p)
        names.append(cl[p:e].decode())
        if struct.unpack_from("<i", cl, e + 1)[0] != 2:
            raise ValueError("only FLOAT channels are read")
        p = e + 17
    offsets = struct.unpack_from(f"<{h}Q", data, off)
    planes = {n: np.zeros((h, w), np.float32) for n in names}
    for o in offsets:
        y = struct.unpack_from("<i", data, o)[0] - y0
        q = o + 8
        for n in names:
            planes[n][y] = np.frombuffer(data, "<f4", w, q)
            q += 4 * w
    return np.stack([planes.get(c, np.ones((h, w), np.float32)) for c in "RGBA"], -1)


def export_render(path, accumulation: np.ndarray, scene_data) -> None:
    """vkrt's render export: .exr -> linear RGBA32F, .png -> 16-bit display image."""
    suffix = Path(path).suffix.lower()
    lin = linear_rgba(accumulation, scene_data)
    if suffix == ".exr":
        write_exr(path, lin)
    elif suffix == ".png":
        write_png16(path, display_rgba16(lin, scene_data))
    else:
        raise ValueError(f"unsupported export format {suffix!r} (.png or .exr)")
