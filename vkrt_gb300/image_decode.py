"""Texture image decoding for imported scenes, following vkrt's image loading (src/core/utility/image.c:86-192,
368-396): the codec is chosen by MIME type, else by the file signature; PNG images decode to RGBA8, or to RGBA16 when
their bit depth is 16 (vkrt decodes through libspng with SPNG_FMT_RGBA8 / SPNG_FMT_RGBA16), and a 16-bit image that
is to be read as sRGB is converted to linear 16-bit values on the host (convertSRGB16PNGToLinearRGBA16).

The PNG decoder is written from the PNG specification (2nd edition): chunk layout with CRC-32 checks, IHDR / PLTE /
tRNS / IDAT, zlib inflation (Python's zlib), the five scanline filters (reversed by vkrt_host_png_unfilter in the host
library), Adam7 interlacing, every colour type and bit depth, and the expansion to RGBA that libspng's RGBA formats
define: grey and palette samples below 8 bits are scaled to the full range (palette indices select PLTE entries),
tRNS supplies palette alpha or the transparent colour key, and missing alpha is opaque. Ancillary chunks (gAMA, iCCP,
sRGB, ...) do not change the samples, as in a decode without gamma correction. JPEG and EXR images, which vkrt
decodes with libjpeg-turbo and tinyexr, are refused with UnsupportedImage.

`texture_texels` turns a decoded image into the linear RGBA32F texels the backend stores, as vkrt's sampler reads
them: R8G8B8A8_SRGB images through the exact sRGB transfer function (colour channels; alpha is linear), UNORM
images divided by 255 or 65535.
"""
from __future__ import annotations

import ctypes as C
import struct
import zlib
from dataclasses import dataclass

import numpy as np

from . import abi

PNG_SIGNATURE = b"\x89PNG\r\n\x1a\n"
JPEG_SIGNATURE = b"\xff\xd8\xff"
EXR_SIGNATURE = b"\x76\x2f\x31\x01"
# Adam7 passes: (x start, y start, x step, y step)
_ADAM7 = ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2))
_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}
_DEPTHS = {0: (1, 2, 4, 8, 16), 2: (8, 16), 3: (1, 2, 4, 8), 4: (8, 16), 6: (8, 16)}


class UnsupportedImage(ValueError):
    """An image this package does not decode (JPEG, EXR, or not an image)."""


class ImageDecodeError(ValueError):
    """A damaged or non-conforming PNG stream."""


@dataclass
class DecodedImage:
    pixels: np.ndarray   # (H, W, 4) uint8 (RGBA8) or uint16 (RGBA16)
    color_space: int     # abi.COLOR_SPACE_* the samples are stored in

    @property
    def format(self) -> int:
        return abi.TEXTURE_FORMAT_RGBA16_UNORM if self.pixels.dtype == np.uint16 else abi.TEXTURE_FORMAT_RGBA8_UNORM


def _chunks(data: bytes):
    if not data.startswith(PNG_SIGNATURE):
        raise ImageDecodeError("not a PNG stream")
    pos = len(PNG_SIGNATURE)
    while pos + 12 <= len(data):
        (length,) = struct.unpack(">I", data[pos:pos + 4])
        kind = data[pos + 4:pos + 8]
        end = pos + 12 + length
        if end > len(data):
            raise ImageDecodeError(f"chunk {kind!r} runs past the end of the stream")
        body = data[pos + 8:pos + 8 + length]
        (crc,) = struct.unpack(">I", data[pos + 8 + length:end])
        if zlib.crc32(kind + body) & 0xFFFFFFFF != crc:
            raise ImageDecodeError(f"chunk {kind!r}: CRC mismatch")
        yield kind, body
        pos = end
        if kind == b"IEND":
            return
    raise ImageDecodeError("no IEND chunk")


def _unfilter(raw: bytes, height: int, row_bytes: int, bpp: int) -> np.ndarray:
    if len(raw) < height * (row_bytes + 1):
        raise ImageDecodeError("image data is shorter than its scanlines")
    src = np.frombuffer(raw, np.uint8, count=height * (row_bytes + 1))
    dst = np.empty(height * row_bytes, np.uint8)
    r = abi.load().vkrt_host_png_unfilter(C.c_void_p(src.ctypes.data), height, row_bytes, bpp,
                                          C.c_void_p(dst.ctypes.data))
    if r != 0:
        raise ImageDecodeError("unknown scanline filter type")
    return dst.reshape(height, row_bytes)


def _samples(rows: np.ndarray, width: int, channels: int, depth: int) -> np.ndarray:
    """Reconstructed scanlines -> (h, width, channels) integer samples."""
    h = rows.shape[0]
    if depth == 16:  # big-endian sample pairs
        hi = rows[:, 0:width * channels * 2:2].astype(np.uint16)
        lo = rows[:, 1:width * channels * 2:2].astype(np.uint16)
        return ((hi << 8) | lo).reshape(h, width, channels)
    if depth == 8:
        return rows[:, :width * channels].reshape(h, width, channels)
    bits = np.unpackbits(rows, axis=1)  # MSB first, as PNG packs sub-byte samples
    per = depth
    n = width * channels
    bits = bits[:, :n * per].reshape(h, n, per)
    weights = (1 << np.arange(per - 1, -1, -1)).astype(np.uint8)
    return (bits * weights).sum(-1).astype(np.uint8).reshape(h, width, channels)


def decode_png(data: bytes) -> DecodedImage:
    """PNG stream -> RGBA8 (bit depth <= 8) or RGBA16 (bit depth 16) pixels, colour space left to the caller."""
    ihdr = plte = trns = None
    idat = []
    for kind, body in _chunks(data):
        if kind == b"IHDR":
            if len(body) != 13:
                raise ImageDecodeError("IHDR has the wrong size")
            ihdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"tRNS":
            trns = body
        elif kind == b"IDAT":
            idat.append(body)
    if ihdr is None or not idat:
        raise ImageDecodeError("missing IHDR or IDAT")
    width, height, depth, ctype, comp, filt, interlace = ihdr
    if ctype not in _CHANNELS or depth not in _DEPTHS[ctype] or comp != 0 or filt != 0 or interlace > 1:
        raise ImageDecodeError(f"unsupported IHDR (colour type {ctype}, bit depth {depth})")
    if width == 0 or height == 0:
        raise ImageDecodeError("empty image")
    if ctype == 3 and plte is None:
        raise ImageDecodeError("palette image without PLTE")
    try:
        raw = zlib.decompress(b"".join(idat))
    except zlib.error as e:
        raise ImageDecodeError(f"zlib: {e}") from e
    ch = _CHANNELS[ctype]
    bits_pp = ch * depth
    bpp = max(1, bits_pp // 8)
    if interlace == 0:
        rb = (width * bits_pp + 7) // 8
        samp = _samples(_unfilter(raw, height, rb, bpp), width, ch, depth)
    else:
        samp = np.zeros((height, width, ch), np.uint16 if depth == 16 else np.uint8)
        pos = 0
        for x0, y0, dx, dy in _ADAM7:
            pw, ph = (width - x0 + dx - 1) // dx, (height - y0 + dy - 1) // dy
            if pw <= 0 or ph <= 0:
                continue
            rb = (pw * bits_pp + 7) // 8
            n = ph * (rb + 1)
            samp[y0::dy, x0::dx] = _samples(_unfilter(raw[pos:pos + n], ph, rb, bpp), pw, ch, depth)
            pos += n
    return DecodedImage(_to_rgba(samp, ctype, depth, plte, trns), abi.COLOR_SPACE_SRGB)


def _to_rgba(s: np.ndarray, ctype: int, depth: int, plte, trns) -> np.ndarray:
    h, w = s.shape[:2]
    wide = depth == 16
    out = np.empty((h, w, 4), np.uint16 if wide else np.uint8)
    full = 65535 if wide else 255
    if ctype == 3:
        idx = s[..., 0].astype(np.int64)
        if (idx >= len(plte)).any():
            raise ImageDecodeError("palette index out of range")
        out[..., :3] = plte[idx]
        alpha = np.full(len(plte), 255, np.uint8)
        if trns is not None:
            a = np.frombuffer(trns, np.uint8)[:len(plte)]
            alpha[:len(a)] = a
        out[..., 3] = alpha[idx]
        return out
    if ctype in (0, 4):
        g = s[..., 0]
        if depth < 8:
            g = (g.astype(np.uint32) * 255 // ((1 << depth) - 1)).astype(np.uint8)
        out[..., 0] = out[..., 1] = out[..., 2] = g
        if ctype == 4:
            out[..., 3] = s[..., 1]
        else:
            out[..., 3] = full
            if trns is not None and len(trns) >= 2:
                (key,) = struct.unpack(">H", trns[:2])
                out[..., 3][s[..., 0] == key] = 0
        return out
    out[..., :3] = s[..., :3]
    if ctype == 6:
        out[..., 3] = s[..., 3]
    else:
        out[..., 3] = full
        if trns is not None and len(trns) >= 6:
            key = np.array(struct.unpack(">HHH", trns[:6]))
            out[..., 3][(s[..., :3] == key).all(-1)] = 0
    return out


def decode_image(data: bytes, mime_type: str | None = None, color_space: int = abi.COLOR_SPACE_SRGB) -> DecodedImage:
    """decodeImageBytes: the codec from the MIME type, else from the signature; color_space is the colour space the
    caller reads the image in (sRGB for base colour and emission, linear for data textures)."""
    mime = (mime_type or "").lower()
    if mime.startswith("image/png") or (not mime and data.startswith(PNG_SIGNATURE)):
        img = decode_png(data)
    elif mime.startswith("image/jpeg") or data.startswith(JPEG_SIGNATURE):
        raise UnsupportedImage("JPEG images are not decoded by this package")
    elif mime.startswith(("image/exr", "image/x-exr")) or data.startswith(EXR_SIGNATURE):
        raise UnsupportedImage("EXR images are not decoded by this package")
    else:
        raise UnsupportedImage(f"unknown image format ({mime_type or 'no MIME type'})")
    img.color_space = color_space
    if img.pixels.dtype == np.uint16 and color_space == abi.COLOR_SPACE_SRGB:
        # convertSRGB16PNGToLinearRGBA16 (image.c:70-84): colour channels to linear 16-bit, alpha kept (FP64 here)
        v = img.pixels[..., :3].astype(np.float32) / np.float32(65535.0)
        lin = np.where(v <= np.float32(0.04045), v / 12.92, ((v + 0.055) / 1.055) ** 2.4)
        img.pixels[..., :3] = np.clip(np.rint(lin * 65535.0), 0, 65535).astype(np.uint16)
        img.color_space = abi.COLOR_SPACE_LINEAR
    return img


_SRGB8_LUT = None


def texture_texels(img: DecodedImage) -> np.ndarray:
    """(H, W, 4) float32 linear RGBA texels of a decoded image, as the sampler reads them (sRGB 8-bit colour through
    the exact transfer function, correctly rounded to FP32)."""
    global _SRGB8_LUT
    p = img.pixels
    if p.dtype == np.uint16:
        t = p.astype(np.float32) / np.float32(65535.0)
        if img.color_space == abi.COLOR_SPACE_SRGB:  # only reached for images built by hand
            c = t[..., :3].astype(np.float64)
            t[..., :3] = np.where(c <= 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4).astype(np.float32)
        return t
    t = p.astype(np.float32) / np.float32(255.0)
    if img.color_space == abi.COLOR_SPACE_SRGB:
        if _SRGB8_LUT is None:
            c = np.arange(256, dtype=np.float64) / 255.0
            _SRGB8_LUT = np.where(c <= 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4).astype(np.float32)
        t[..., :3] = _SRGB8_LUT[p[..., :3]]
    return t
