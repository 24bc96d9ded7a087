"""8-bit images to PNG files and back (zlib only; no imaging library).

Milton writes its tone-mapped output through Qt's image writer; this module gives the same
kind of file for an (H, W, 4) uint8 array from pathtracer.Film.tonemap, and reads the PNG and
PPM / PGM files a scene's materials name as image maps.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np


def _chunk(tag: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)


def png_bytes(rgba: np.ndarray) -> bytes:
    a = np.ascontiguousarray(rgba, np.uint8)
    if a.ndim != 3 or a.shape[2] != 4:
        raise ValueError("expected an (H, W, 4) uint8 array")
    h, w, _ = a.shape
    raw = np.zeros((h, 1 + 4 * w), np.uint8)  # filter type 0 per row
    raw[:, 1:] = a.reshape(h, 4 * w)
    ihdr = struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)
    return b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", ihdr) + _chunk(b"IDAT", zlib.compress(raw.tobytes(), 6)) + \
        _chunk(b"IEND", b"")


def write_png(path: str, rgba: np.ndarray) -> None:
    with open(path, "wb") as f:
        f.write(png_bytes(rgba))


_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}  # PNG colour type -> samples per pixel


def _unfilter(raw: np.ndarray, h: int, stride: int, bpp: int) -> np.ndarray:
    """Undoes the PNG row filters (None, Sub, Up, Average, Paeth) of h rows of stride bytes."""
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        f, line = int(raw[y, 0]), raw[y, 1:].astype(np.int32)
        if f == 0:
            cur = line
        elif f == 1:  # Sub: a running sum per byte position within the pixel
            cur = np.cumsum(line.reshape(-1, bpp), axis=0).reshape(-1) & 0xFF
        elif f == 2:
            cur = (line + prev) & 0xFF
        elif f in (3, 4):
            cur = np.zeros(stride, np.int32)
            for x in range(0, stride, bpp):
                a = cur[x - bpp:x] if x >= bpp else np.zeros(bpp, np.int32)
                b = prev[x:x + bpp]
                if f == 3:
                    p = (a + b) // 2
                else:
                    c = prev[x - bpp:x] if x >= bpp else np.zeros(bpp, np.int32)
                    pa, pb, pc = np.abs(b - c), np.abs(a - c), np.abs(a + b - 2 * c)
                    p = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))
                cur[x:x + bpp] = (line[x:x + bpp] + p) & 0xFF
        else:
            raise ValueError(f"bad PNG row filter {f}")
        out[y] = cur
        prev = cur.astype(np.int32)
    return out


def read_png(path: str, rgb: bool = False) -> np.ndarray:
    """Reads an 8-bit, non-interlaced PNG of any colour type (grey, RGB, palette, grey + alpha,
    RGBA).  Returns (H, W, 4) uint8 RGBA, or with rgb=True (H, W, 3) with the alpha dropped, as
    Qt's conversion to Format_RGB32 does."""
    data = open(path, "rb").read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, idat, w, h, ctype, plte, trns = 8, b"", 0, 0, 6, None, None
    while pos < len(data):
        n, tag = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if tag == b"IHDR":
            w, h, depth, ctype, _, _, inter = struct.unpack(">IIBBBBB", body)
            if depth != 8 or inter != 0 or ctype not in _CHANNELS:
                raise ValueError("only 8-bit, non-interlaced PNGs are read")
        elif tag == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif tag == b"tRNS":
            trns = np.frombuffer(body, np.uint8)
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    ch = _CHANNELS[ctype]
    raw = np.frombuffer(zlib.decompress(idat), np.uint8)[:h * (1 + ch * w)].reshape(h, 1 + ch * w)
    px = _unfilter(raw, h, ch * w, ch).reshape(h, w, ch)
    out = np.full((h, w, 4), 255, np.uint8)
    if ctype == 0:
        out[..., :3] = px[..., :1]
    elif ctype == 2:
        out[..., :3] = px
    elif ctype == 3:
        if plte is None or px.max(initial=0) >= len(plte):
            raise ValueError("palette PNG without a palette entry for some pixel")
        out[..., :3] = plte[px[..., 0]]
        if trns is not None:
            alpha = np.full(len(plte), 255, np.uint8)
            alpha[:len(trns)] = trns[:len(plte)]
            out[..., 3] = alpha[px[..., 0]]
    elif ctype == 4:
        out[..., :3] = px[..., :1]
        out[..., 3] = px[..., 1]
    else:
        out[...] = px
    return out[..., :3].copy() if rgb else out


def read_pnm(path: str) -> np.ndarray:
    """Reads a binary or ASCII PPM / PGM (P6, P3, P5, P2) with maxval 255 as (H, W, 3) uint8."""
    data = open(path, "rb").read()
    toks, pos = [], 0
    while len(toks) < 4:
        while pos < len(data) and data[pos:pos + 1].isspace():
            pos += 1
        if data[pos:pos + 1] == b"#":
            while pos < len(data) and data[pos:pos + 1] not in (b"\n", b"\r"):
                pos += 1
            continue
        start = pos
        while pos < len(data) and not data[pos:pos + 1].isspace():
            pos += 1
        if start == pos:
            raise ValueError("truncated PNM header")
        toks.append(data[start:pos])
    magic, w, h, maxval = toks[0], int(toks[1]), int(toks[2]), int(toks[3])
    if magic not in (b"P2", b"P3", b"P5", b"P6") or maxval != 255:
        raise ValueError("only P2 / P3 / P5 / P6 images with maxval 255 are read")
    ch = 3 if magic in (b"P3", b"P6") else 1
    if magic in (b"P5", b"P6"):
        px = np.frombuffer(data[pos + 1:pos + 1 + w * h * ch], np.uint8)
    else:
        px = np.array(data[pos:].split()[:w * h * ch], np.int64).astype(np.uint8)
    if px.size != w * h * ch:
        raise ValueError("truncated PNM data")
    px = px.reshape(h, w, ch)
    return np.repeat(px, 3, axis=2) if ch == 1 else px.copy()


def read_hdr(path: str) -> np.ndarray:
    """Reads a Radiance RGBE (.hdr) image, flat or run-length encoded scanlines, '-Y h +X w'
    orientation: (H, W, 3) float32, row 0 on top.  A pixel is mantissa * 2^(e - 136), 0 for e = 0
    (HDRUtils::loadHDR with rgbe2float, HDRUtils.cpp:36-70, rgbe.cpp:116-131)."""
    data = open(path, "rb").read()
    pos, fmt_ok, first = 0, False, True
    while True:
        nl = data.find(b"\n", pos)
        if nl < 0:
            raise ValueError("truncated HDR header")
        line = data[pos:nl].strip()
        pos = nl + 1
        if first and not line.startswith(b"#?"):
            raise ValueError("not a Radiance HDR file")
        first = False
        if line.startswith(b"FORMAT="):
            fmt_ok = line == b"FORMAT=32-bit_rle_rgbe"
            if not fmt_ok:
                raise ValueError("only 32-bit_rle_rgbe HDR files are read")
        if line.startswith(b"-Y "):
            p = line.split()
            if len(p) != 4 or p[2] != b"+X":
                raise ValueError("only '-Y h +X w' HDR orientation is read")
            h, w = int(p[1]), int(p[3])
            break
    if w <= 0 or h <= 0:
        raise ValueError("bad HDR size")
    buf = np.frombuffer(data, np.uint8)
    rgbe = np.zeros((h, w, 4), np.uint8)
    for y in range(h):
        if w < 8 or w > 0x7FFF or pos + 4 > len(buf) or buf[pos] != 2 or buf[pos + 1] != 2 or (buf[pos + 2] & 0x80):
            rest = buf[pos:pos + 4 * w * (h - y)]  # flat (uncompressed) pixels from here on
            if rest.size != 4 * w * (h - y):
                raise ValueError("truncated HDR data")
            rgbe[y:] = rest.reshape(h - y, w, 4)
            break
        if (int(buf[pos + 2]) << 8 | int(buf[pos + 3])) != w:
            raise ValueError("wrong HDR scanline width")
        pos += 4
        for c in range(4):
            x = 0
            while x < w:
                if pos >= len(buf):
                    raise ValueError("truncated HDR data")
                n = int(buf[pos])
                if n > 128:  # a run
                    n -= 128
                    if n == 0 or x + n > w or pos + 1 >= len(buf):
                        raise ValueError("bad HDR run")
                    rgbe[y, x:x + n, c] = buf[pos + 1]
                    pos += 2
                else:  # n literal bytes
                    if n == 0 or x + n > w or pos + 1 + n > len(buf):
                        raise ValueError("bad HDR run")
                    rgbe[y, x:x + n, c] = buf[pos + 1:pos + 1 + n]
                    pos += 1 + n
                x += n
    e = rgbe[..., 3].astype(np.int32)
    f = np.where(e > 0, np.ldexp(np.float32(1.0), e - 136), 0.0).astype(np.float32)
    return rgbe[..., :3].astype(np.float32) * f[..., None]


def read_image(path: str) -> np.ndarray:
    """An image file as Milton's Image::load gives it to materials (Image.cpp:67-100, through
    Qt's Format_RGB32 and Rgba32 -> RgbaHDR, Rgba.inl:32-40): (H, W, 3) float32 byte / 255, row 0
    on top.  PNG, PPM / PGM and Radiance HDR (float values as stored) are read; other formats
    raise ValueError (the reference reads PFM as not implemented and EXR only with OpenEXR)."""
    suffix = path[path.rfind(".") + 1:].lower()
    if suffix in ("hdr", "rgbe"):
        return read_hdr(path)
    if suffix == "png":
        px = read_png(path, rgb=True)
    elif suffix in ("ppm", "pgm", "pnm"):
        px = read_pnm(path)
    else:
        raise ValueError(f"unsupported image format '{suffix}' (PNG, PPM, PGM and Radiance HDR are read)")
    return px.astype(np.float32) / np.float32(255.0)
