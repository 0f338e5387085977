"""Image files for the command line, without OpenCV.

Mirrors fpie/io.py (read_image / write_image / read_images): images come back
as HxWx3 uint8 (a gray image is repeated over three channels, an alpha
channel is dropped) and a missing mask file means "use the whole source"
(all 255).  Formats: PNG (8-bit gray, gray+alpha, RGB, RGBA; non-interlaced),
binary PPM/PGM, and .npy arrays.  Channel order is the file's (RGB); the
solver treats channels independently, so reading and writing in the same
order gives the same pictures as the reference's BGR round trip.
"""

from __future__ import annotations

import os
import struct
import warnings
import zlib

import numpy as np

_PNG_SIG = b"\x89PNG\r\n\x1a\n"


def _unfilter(raw: np.ndarray, h: int, w: int, bpp: int) -> np.ndarray:
    stride = w * bpp
    rows = raw.reshape(h, stride + 1)
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        ft = int(rows[y, 0])
        line = rows[y, 1:].astype(np.int32)
        if ft == 0:
            cur = line
        elif ft == 1:  # Sub: running sum per channel
            cur = line.reshape(w, bpp).cumsum(axis=0).reshape(-1) & 0xFF
        elif ft == 2:  # Up
            cur = (line + prev) & 0xFF
        elif ft == 3:  # Average (sequential in x)
            cur = np.empty(stride, np.int32)
            left = np.zeros(bpp, np.int32)
            for x in range(w):
                s = slice(x * bpp, (x + 1) * bpp)
                left = (line[s] + ((left + prev[s]) >> 1)) & 0xFF
                cur[s] = left
        elif ft == 4:  # Paeth (sequential in x)
            cur = np.empty(stride, np.int32)
            a = np.zeros(bpp, np.int32)
            c = np.zeros(bpp, np.int32)
            for x in range(w):
                s = slice(x * bpp, (x + 1) * bpp)
                b = prev[s]
                p = a + b - c
                pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
                pred = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))
                a = (line[s] + pred) & 0xFF
                cur[s] = a
                c = b
        else:
            raise ValueError(f"bad PNG filter type {ft}")
        out[y] = cur
        prev = cur
    return out


def read_png(path: str) -> np.ndarray:
    data = open(path, "rb").read()
    if data[:8] != _PNG_SIG:
        raise ValueError(f"{path} is not a PNG file")
    pos, idat, hdr = 8, [], None
    while pos < len(data):
        (length,) = struct.unpack(">I", data[pos:pos + 4])
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + length]
        pos += 12 + length
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    if hdr is None:
        raise ValueError(f"{path}: no IHDR chunk")
    w, h, depth, ctype, _, _, interlace = hdr
    if depth != 8 or interlace != 0 or ctype not in (0, 2, 4, 6):
        raise ValueError(f"{path}: only 8-bit non-interlaced gray/RGB(A) PNGs are supported")
    bpp = {0: 1, 2: 3, 4: 2, 6: 4}[ctype]
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), np.uint8)
    return _unfilter(raw, h, w, bpp).reshape(h, w, bpp)


def write_png(path: str, img: np.ndarray) -> None:
    img = np.ascontiguousarray(img, np.uint8)
    if img.ndim == 2:
        img = img[..., None]
    h, w, c = img.shape
    ctype = {1: 0, 2: 4, 3: 2, 4: 6}[c]
    raw = np.concatenate([np.zeros((h, 1), np.uint8), img.reshape(h, w * c)], axis=1)

    def chunk(kind: bytes, body: bytes) -> bytes:
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body))

    out = _PNG_SIG + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0))
    out += chunk(b"IDAT", zlib.compress(raw.tobytes(), 6)) + chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(out)


def _read_pnm(path: str) -> np.ndarray:
    data = open(path, "rb").read()
    tokens, pos = [], 0
    while len(tokens) < 4:
        while data[pos:pos + 1].isspace():
            pos += 1
        if data[pos:pos + 1] == b"#":
            pos = data.index(b"\n", pos) + 1
            continue
        end = pos
        while not data[end:end + 1].isspace():
            end += 1
        tokens.append(data[pos:end])
        pos = end
    magic, w, h, mx = tokens[0], int(tokens[1]), int(tokens[2]), int(tokens[3])
    if mx != 255 or magic not in (b"P5", b"P6"):
        raise ValueError(f"{path}: only 8-bit binary PGM/PPM are supported")
    c = 3 if magic == b"P6" else 1
    return np.frombuffer(data[pos + 1:pos + 1 + w * h * c], np.uint8).reshape(h, w, c)


def read_image(name: str) -> np.ndarray:
    """HxWx3 uint8 (gray repeated, alpha dropped), as fpie/io.py:10-19."""
    if not os.path.exists(name):
        raise FileNotFoundError(f"Failed to read image: {name}")
    ext = os.path.splitext(name)[1].lower()
    if ext == ".npy":
        img = np.load(name)
    elif ext in (".ppm", ".pgm", ".pnm"):
        img = _read_pnm(name)
    else:
        img = read_png(name)
    img = np.asarray(img, np.uint8)
    if img.ndim == 2:
        img = img[..., None]
    if img.shape[-1] in (1, 2):
        img = np.repeat(img[..., :1], 3, axis=-1)
    elif img.shape[-1] == 4:
        img = img[..., :3]
    return np.ascontiguousarray(img)


def write_image(name: str, image: np.ndarray) -> None:
    ext = os.path.splitext(name)[1].lower()
    if ext == ".npy":
        np.save(name, image)
    elif ext in (".ppm", ".pnm"):
        img = np.ascontiguousarray(image, np.uint8)
        h, w = img.shape[:2]
        with open(name, "wb") as f:
            f.write(b"P6\n%d %d\n255\n" % (w, h) + img.reshape(h, w, 3).tobytes())
    else:
        write_png(name, image)


def read_images(src_name: str, mask_name: str, tgt_name: str):
    """(src, mask, tgt); a missing mask file means the whole source (fpie/io.py:27-39)."""
    src, tgt = read_image(src_name), read_image(tgt_name)
    if mask_name and os.path.exists(mask_name):
        mask = read_image(mask_name)
    else:
        warnings.warn("No mask file found, use default setting", stacklevel=2)
        mask = np.zeros_like(src) + 255
    return src, mask, tgt
