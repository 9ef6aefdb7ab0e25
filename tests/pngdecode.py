"""A small PNG reader for the tests: any non-interlaced PNG of bit depth <= 8 (greyscale, RGB, palette with or
without tRNS, grey + alpha, RGBA) to an (H, W, 4) uint8 RGBA array.  The PNG format is the W3C/ISO 15948
specification; decompression is Python's zlib.  Chunk CRCs are checked."""
from __future__ import annotations

import struct
import zlib

import numpy as np

SIGNATURE = b"\x89PNG\r\n\x1a\n"
CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def read_chunks(data: bytes):
    if data[:8] != SIGNATURE:
        raise ValueError("not a PNG file")
    pos = 8
    while pos < len(data):
        (length,) = struct.unpack(">I", data[pos:pos + 4])
        ctype = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + length]
        (crc,) = struct.unpack(">I", data[pos + 8 + length:pos + 12 + length])
        if zlib.crc32(ctype + body) & 0xFFFFFFFF != crc:
            raise ValueError("bad CRC in chunk %r" % ctype)
        yield ctype, body
        pos += 12 + length
        if ctype == b"IEND":
            break


def _unfilter(raw: bytes, height: int, stride: int, bpp: int) -> np.ndarray:
    buf = np.frombuffer(raw, dtype=np.uint8)
    if len(buf) < height * (stride + 1):
        raise ValueError("image data too short")
    rows = buf[: height * (stride + 1)].reshape(height, stride + 1)
    out = np.zeros((height, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int32)
    for y in range(height):
        f = int(rows[y, 0])
        line = rows[y, 1:].astype(np.int32)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 255
        elif f in (1, 3, 4):
            cur = np.zeros(stride, dtype=np.int32)
            for x in range(stride):  # sequential in x: depends on the byte bpp to the left
                a = cur[x - bpp] if x >= bpp else 0
                b = prev[x]
                c = prev[x - bpp] if x >= bpp else 0
                if f == 1:
                    pred = a
                elif f == 3:
                    pred = (a + b) >> 1
                else:
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (line[x] + pred) & 255
        else:
            raise ValueError("bad filter type %d" % f)
        out[y] = cur
        prev = cur
    return out


def decode(data: bytes) -> np.ndarray:
    ihdr = None
    plte = None
    trns = None
    idat = []
    for ctype, body in read_chunks(data):
        if ctype == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif ctype == b"PLTE":
            plte = np.frombuffer(body, dtype=np.uint8).reshape(-1, 3)
        elif ctype == b"tRNS":
            trns = body
        elif ctype == b"IDAT":
            idat.append(body)
    if ihdr is None:
        raise ValueError("no IHDR")
    W, H, depth, ctype, comp, filt, interlace = ihdr
    if comp != 0 or filt != 0 or interlace != 0 or depth > 8 or ctype not in CHANNELS:
        raise ValueError("unsupported PNG: %r" % (ihdr,))
    ch = CHANNELS[ctype]
    bits = depth * ch
    stride = (W * bits + 7) // 8
    bpp = max(1, bits // 8)
    raw = zlib.decompress(b"".join(idat))
    rows = _unfilter(raw, H, stride, bpp)
    if depth < 8:
        per = 8 // depth
        shifts = np.array([8 - depth * (i + 1) for i in range(per)], dtype=np.uint8)
        samples = ((rows[:, :, None] >> shifts[None, None, :]) & ((1 << depth) - 1)).reshape(H, -1)[:, :W * ch]
    else:
        samples = rows[:, :W * ch]
    samples = samples.reshape(H, W, ch).astype(np.uint8)
    out = np.zeros((H, W, 4), dtype=np.uint8)
    if ctype == 3:
        idx = samples[:, :, 0].astype(np.int64)
        if plte is None or idx.max(initial=0) >= len(plte):
            raise ValueError("palette index out of range")
        out[:, :, :3] = plte[idx]
        alpha = np.full(len(plte), 255, dtype=np.uint8)
        if trns is not None:
            alpha[: len(trns)] = np.frombuffer(trns, dtype=np.uint8)
        out[:, :, 3] = alpha[idx]
        return out
    scale = 255 // ((1 << depth) - 1)
    s = samples.astype(np.int32) * scale
    if ctype == 0:
        out[:, :, 0] = out[:, :, 1] = out[:, :, 2] = s[:, :, 0]
        out[:, :, 3] = 255
    elif ctype == 4:
        out[:, :, 0] = out[:, :, 1] = out[:, :, 2] = s[:, :, 0]
        out[:, :, 3] = s[:, :, 1]
    elif ctype == 2:
        out[:, :, :3] = s
        out[:, :, 3] = 255
    else:
        out[:, :, :] = s
    return out


def read(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        return decode(f.read())
