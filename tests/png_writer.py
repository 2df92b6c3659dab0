"""A PNG encoder for the decoder tests, written from the PNG specification independently of the decoder: every
colour type and bit depth, a chosen or random filter type per scanline (the filters applied in the forward
direction), optional Adam7 interlacing, optional PLTE / tRNS."""
import struct
import zlib

import numpy as np

ADAM7 = ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2))
CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _chunk(kind: bytes, body: bytes) -> bytes:
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def _pack_row(samples: np.ndarray, depth: int) -> bytes:
    """One scanline of integer samples (flattened over pixels and channels) -> bytes."""
    if depth == 16:
        return samples.astype(">u2").tobytes()
    if depth == 8:
        return samples.astype(np.uint8).tobytes()
    bits = ((samples[:, None].astype(np.uint16) >> np.arange(depth - 1, -1, -1)) & 1).astype(np.uint8).reshape(-1)
    return np.packbits(bits).tobytes()


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def _filter(row: bytes, prev: bytes, bpp: int, kind: int) -> bytes:
    out = bytearray([kind])
    for i, x in enumerate(row):
        a = row[i - bpp] if i >= bpp else 0
        b = prev[i] if prev else 0
        c = prev[i - bpp] if (prev and i >= bpp) else 0
        pred = (0, a, b, (a + b) // 2, _paeth(a, b, c))[kind]
        out.append((x - pred) & 0xFF)
    return bytes(out)


def _image_bytes(samples: np.ndarray, depth: int, ctype: int, rng, filters) -> bytes:
    h, w = samples.shape[:2]
    ch = CHANNELS[ctype]
    bpp = max(1, ch * depth // 8)
    out, prev = b"", None
    for y in range(h):
        row = _pack_row(samples[y].reshape(-1), depth)
        kind = int(rng.integers(0, 5)) if filters is None else filters
        out += _filter(row, prev, bpp, kind)
        prev = row
    return out


def encode_png(samples: np.ndarray, depth: int, ctype: int, palette=None, trns: bytes | None = None,
               interlace: bool = False, filters: int | None = None, seed: int = 0) -> bytes:
    """samples: (H, W, channels) integers of the colour type (palette indices for type 3)."""
    rng = np.random.default_rng(seed)
    h, w = samples.shape[:2]
    if not interlace:
        raw = _image_bytes(samples, depth, ctype, rng, filters)
    else:
        raw = b""
        for x0, y0, dx, dy in ADAM7:
            sub = samples[y0::dy, x0::dx]
            if sub.shape[0] and sub.shape[1]:
                raw += _image_bytes(sub, depth, ctype, rng, filters)
    body = [_chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 1 if interlace else 0))]
    if palette is not None:
        body.append(_chunk(b"PLTE", np.asarray(palette, np.uint8).tobytes()))
    if trns is not None:
        body.append(_chunk(b"tRNS", trns))
    # IDAT split in two chunks to exercise concatenation
    z = zlib.compress(raw, 6)
    body += [_chunk(b"IDAT", z[: len(z) // 2]), _chunk(b"IDAT", z[len(z) // 2:]), _chunk(b"IEND", b"")]
    return b"\x89PNG\r\n\x1a\n" + b"".join(body)
