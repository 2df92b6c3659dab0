"""PNG decoding of imported textures (vkrt_gb300/image_decode.py, vkrt_host_png_unfilter) against an independent
encoder: every colour type and bit depth, all five scanline filters, Adam7, palettes with tRNS alpha, grey and RGB
colour keys, and the RGBA expansion vkrt's libspng formats define; damaged streams are refused; the sRGB texel
conversion is the exact transfer function."""
import os
import struct
from pathlib import Path

import numpy as np
import pytest

from png_writer import encode_png
from vkrt_gb300 import abi
from vkrt_gb300.image_decode import (ImageDecodeError, UnsupportedImage, decode_image, decode_png,
                                     texture_texels)

CASES = [(0, 1), (0, 2), (0, 4), (0, 8), (0, 16), (2, 8), (2, 16), (3, 1), (3, 2), (3, 4), (3, 8), (4, 8), (4, 16),
         (6, 8), (6, 16)]
CH = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _expected(samples, ctype, depth, palette=None, trns=None):
    h, w = samples.shape[:2]
    wide = depth == 16
    out = np.zeros((h, w, 4), np.uint16 if wide else np.uint8)
    full = 65535 if wide else 255
    if ctype == 3:
        out[..., :3] = palette[samples[..., 0]]
        alpha = np.full(len(palette), 255)
        if trns is not None:
            alpha[:len(trns)] = list(trns)
        out[..., 3] = alpha[samples[..., 0]]
        return out
    if ctype in (0, 4):
        g = samples[..., 0].astype(np.int64)
        if depth < 8:
            g = np.array([int(round(v * 255 / ((1 << depth) - 1))) for v in g.ravel()]).reshape(g.shape)
        out[..., 0] = out[..., 1] = out[..., 2] = g
        out[..., 3] = samples[..., 1] if ctype == 4 else full
        return out
    out[..., :3] = samples[..., :3]
    out[..., 3] = samples[..., 3] if ctype == 6 else full
    return out


@pytest.mark.parametrize("interlace", [False, True], ids=["progressive", "adam7"])
@pytest.mark.parametrize("ctype,depth", CASES)
def test_png_round_trip(built, ctype, depth, interlace):
    rng = np.random.default_rng(ctype * 100 + depth + (7 if interlace else 0))
    h, w = 13, 29  # odd sizes: partial Adam7 passes, sub-byte row padding
    palette = None
    if ctype == 3:
        n = min(1 << depth, 37)
        palette = rng.integers(0, 256, (n, 3)).astype(np.uint8)
        samples = rng.integers(0, n, (h, w, 1))
    else:
        samples = rng.integers(0, 1 << depth, (h, w, CH[ctype]))
    data = encode_png(samples, depth, ctype, palette=palette, interlace=interlace, seed=depth)
    img = decode_png(data)
    np.testing.assert_array_equal(img.pixels, _expected(samples, ctype, depth, palette))
    assert img.pixels.dtype == (np.uint16 if depth == 16 else np.uint8)


@pytest.mark.parametrize("kind", range(5))
def test_each_filter_type_alone(built, kind):
    rng = np.random.default_rng(kind)
    s = rng.integers(0, 256, (9, 17, 4))
    img = decode_png(encode_png(s, 8, 6, filters=kind))
    np.testing.assert_array_equal(img.pixels, s)


def test_transparency_chunks(built):
    # palette alpha from tRNS (shorter than the palette: the rest opaque)
    pal = np.array([[10, 20, 30], [40, 50, 60], [70, 80, 90]], np.uint8)
    idx = np.array([[[0], [1], [2]]])
    img = decode_png(encode_png(idx, 8, 3, palette=pal, trns=bytes([0, 128])))
    np.testing.assert_array_equal(img.pixels[0, :, 3], [0, 128, 255])
    # grey and RGB colour keys make matching pixels transparent
    g = np.array([[[5], [7]]])
    img = decode_png(encode_png(g, 8, 0, trns=struct.pack(">H", 7)))
    np.testing.assert_array_equal(img.pixels[0, :, 3], [255, 0])
    rgb = np.array([[[1, 2, 3], [4, 5, 6]]])
    img = decode_png(encode_png(rgb, 16, 2, trns=struct.pack(">HHH", 1, 2, 3)))
    np.testing.assert_array_equal(img.pixels[0, :, 3], [0, 65535])


def test_damaged_streams_are_refused(built):
    data = bytearray(encode_png(np.zeros((4, 4, 4), np.uint8), 8, 6))
    with pytest.raises(ImageDecodeError):
        decode_png(bytes(data[:-20]))            # truncated
    bad = bytearray(data)
    bad[40] ^= 0xFF                              # inside a chunk: CRC mismatch
    with pytest.raises(ImageDecodeError):
        decode_png(bytes(bad))
    with pytest.raises(UnsupportedImage):
        decode_image(b"\xff\xd8\xff\xe0" + b"\x00" * 16)   # JPEG
    with pytest.raises(UnsupportedImage):
        decode_image(b"GIF89a" + b"\x00" * 16)


def test_texels_and_16_bit_srgb_conversion(built):
    s = np.arange(256, dtype=np.uint8).reshape(16, 16, 1).repeat(4, -1)
    img = decode_image(encode_png(s, 8, 6), "image/png", abi.COLOR_SPACE_SRGB)
    t = texture_texels(img)
    c = np.arange(256) / 255.0
    want = np.where(c <= 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4).astype(np.float32)
    np.testing.assert_array_equal(t[..., 0].ravel(), want)
    np.testing.assert_array_equal(t[..., 3].ravel(), (np.arange(256) / np.float32(255)).astype(np.float32))
    lin = texture_texels(decode_image(encode_png(s, 8, 6), None, abi.COLOR_SPACE_LINEAR))
    np.testing.assert_array_equal(lin[..., 0].ravel(), (np.arange(256) / np.float32(255)).astype(np.float32))
    # 16-bit sRGB images become linear 16-bit values on decode (vkrt's convertSRGB16PNGToLinearRGBA16)
    s16 = np.array([[[0, 32768, 65535, 1000]]])
    img = decode_image(encode_png(s16, 16, 6), None, abi.COLOR_SPACE_SRGB)
    assert img.color_space == abi.COLOR_SPACE_LINEAR
    v = np.float32(32768) / np.float32(65535)
    mid = int(np.rint(((float(v) + 0.055) / 1.055) ** 2.4 * 65535.0))  # lrintf(srgbDecode(v) * 65535)
    np.testing.assert_array_equal(img.pixels[0, 0], [0, mid, 65535, 1000])


_REF = Path(os.environ["VKRT_REFERENCE"]) if os.environ.get("VKRT_REFERENCE") else None


@pytest.mark.skipif(_REF is None or not (_REF / "assets/images").exists(), reason="no vkrt checkout")
def test_decodes_vkrts_bundled_images(built):
    icon = decode_png((_REF / "assets/images/icon.png").read_bytes())  # 1-bit palette
    assert icon.pixels.shape == (256, 256, 4) and icon.pixels.dtype == np.uint8
    assert len(np.unique(icon.pixels.reshape(-1, 4), axis=0)) <= 2
    art = decode_png((_REF / "assets/images/dragon.png").read_bytes())  # 8-bit RGBA
    assert art.pixels.shape == (932, 1602, 4)
    # re-encoding the decoded pixels and decoding again is lossless
    again = decode_png(encode_png(art.pixels[:64, :96], 8, 6, seed=3))
    np.testing.assert_array_equal(again.pixels, art.pixels[:64, :96])
