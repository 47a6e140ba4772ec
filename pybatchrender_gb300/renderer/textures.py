"""Texture images: PNG decoding/encoding and the texel layout the kernels read.

The reference loads a node's texture with Panda3D (``loader.loadTexture``,
``renderer/node.py:277-287``) and samples it in ``shaders/basic.frag:31-32``
with the sampler defaults Panda3D gives a loaded texture: linear filtering
without mipmaps and repeat wrap.  Panda3D stores an image with its bottom row
first, so ``v = 0`` is the bottom edge of the picture.  Here a texture is a
``[h, w, 4]`` uint8 RGBA array in image order (row 0 = top, as in the file);
:func:`gl_rows` flips it into the kernels' layout (row 0 = ``v = 0``).

PIL is not available, so PNG is decoded and encoded here with ``zlib``: 8- and
16-bit greyscale, grey+alpha, RGB, RGBA and palette images, non-interlaced.
"""
from __future__ import annotations

import os
import struct
import zlib

import numpy as np
import torch

_PNG_SIG = b"\x89PNG\r\n\x1a\n"
_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _unfilter(raw: bytes, h: int, stride: int, bpp: int) -> np.ndarray:
    """Undo the per-row PNG filters (None, Sub, Up, Average, Paeth)."""
    data = np.frombuffer(raw, dtype=np.uint8)
    if data.size != h * (stride + 1):
        raise ValueError("PNG image data has the wrong size")
    rows = data.reshape(h, stride + 1)
    out = np.zeros((h, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int32)
    for y in range(h):
        f = int(rows[y, 0])
        line = rows[y, 1:].astype(np.int32)
        if f == 0:
            cur = line
        elif f == 1:  # Sub: running sum along the row, per byte of a pixel
            pad = (-stride) % bpp
            lp = np.concatenate([line, np.zeros(pad, np.int32)]).reshape(-1, bpp)
            cur = (np.cumsum(lp, axis=0) & 255).reshape(-1)[:stride]
        elif f == 2:  # Up
            cur = (line + prev) & 255
        elif f in (3, 4):  # Average / Paeth: sequential along the row
            cur = np.zeros(stride, dtype=np.int32)
            for x in range(0, stride, bpp):
                a = cur[x - bpp:x] if x >= bpp else np.zeros(min(bpp, stride - x), np.int32)
                b = prev[x:x + bpp]
                if f == 3:
                    pred = (a + b) >> 1
                else:
                    c = prev[x - bpp:x] if x >= bpp else np.zeros(min(bpp, stride - x), np.int32)
                    p = a + b - c
                    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
                    pred = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))
                cur[x:x + bpp] = (line[x:x + bpp] + pred) & 255
        else:
            raise ValueError(f"unknown PNG filter type {f}")
        out[y] = cur
        prev = cur
    return out


def decode_png(data: bytes) -> np.ndarray:
    """PNG bytes -> ``[h, w, 4]`` uint8 RGBA, row 0 = top of the image."""
    if not data.startswith(_PNG_SIG):
        raise ValueError("not a PNG file")
    pos = len(_PNG_SIG)
    ihdr, idat, plte, trns = None, [], None, None
    while pos + 8 <= len(data):
        (length,) = struct.unpack(">I", data[pos:pos + 4])
        ctype = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + length]
        pos += 12 + length
        if ctype == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif ctype == b"PLTE":
            plte = np.frombuffer(body, dtype=np.uint8).reshape(-1, 3)
        elif ctype == b"tRNS":
            trns = body
        elif ctype == b"IDAT":
            idat.append(body)
        elif ctype == b"IEND":
            break
    if ihdr is None:
        raise ValueError("PNG without IHDR")
    w, h, depth, ctype_, _, _, interlace = ihdr
    if interlace != 0:
        raise ValueError("interlaced PNG is not supported")
    if ctype_ not in _CHANNELS or depth not in ((1, 2, 4, 8) if ctype_ == 3 else (8, 16)):
        raise ValueError(f"unsupported PNG format (colour type {ctype_}, bit depth {depth})")
    ch = _CHANNELS[ctype_]
    raw = zlib.decompress(b"".join(idat))
    bits = ch * depth
    stride = (w * bits + 7) // 8
    bpp = max(1, bits // 8)
    px = _unfilter(raw, h, stride, bpp)
    if depth == 16:
        arr = px.reshape(h, w, ch, 2)[..., 0]  # the high byte of each big-endian sample
    elif depth == 8:
        arr = px.reshape(h, w, ch)
    else:  # packed palette indices
        per = 8 // depth
        shifts = (8 - depth * (1 + np.arange(per))).astype(np.uint8)
        arr = ((px[:, :, None] >> shifts) & ((1 << depth) - 1)).reshape(h, -1)[:, :w, None]
    out = np.empty((h, w, 4), dtype=np.uint8)
    if ctype_ == 3:
        if plte is None:
            raise ValueError("palette PNG without PLTE")
        idx = arr[..., 0].astype(np.int64)
        if idx.max(initial=0) >= len(plte):
            raise ValueError("PNG palette index out of range")
        out[..., :3] = plte[idx]
        alpha = np.full(len(plte), 255, np.uint8)
        if trns is not None:
            t = np.frombuffer(trns, dtype=np.uint8)[:len(plte)]
            alpha[:len(t)] = t
        out[..., 3] = alpha[idx]
    elif ch in (1, 2):
        out[..., 0] = out[..., 1] = out[..., 2] = arr[..., 0]
        out[..., 3] = arr[..., 1] if ch == 2 else 255
    else:
        out[..., :3] = arr[..., :3]
        out[..., 3] = arr[..., 3] if ch == 4 else 255
    return out


def _chunk(tag: bytes, body: bytes) -> bytes:
    return struct.pack(">I", len(body)) + tag + body + struct.pack(">I", zlib.crc32(tag + body) & 0xFFFFFFFF)


def encode_png(img: np.ndarray, level: int = 6) -> bytes:
    """``[h, w]`` / ``[h, w, 1|2|3|4]`` uint8 (row 0 = top) -> PNG bytes (Up filter)."""
    a = np.asarray(img)
    if a.dtype != np.uint8:
        raise TypeError("encode_png needs uint8 pixels")
    if a.ndim == 2:
        a = a[:, :, None]
    h, w, c = a.shape
    ctype = {1: 0, 2: 4, 3: 2, 4: 6}.get(c)
    if ctype is None:
        raise ValueError("encode_png needs 1 to 4 channels")
    rows = np.ascontiguousarray(a).reshape(h, w * c).astype(np.int16)
    up = (rows - np.vstack([np.zeros((1, w * c), np.int16), rows[:-1]])) & 255
    body = np.concatenate([np.full((h, 1), 2, np.uint8), up.astype(np.uint8)], axis=1).tobytes()
    return (_PNG_SIG + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0))
            + _chunk(b"IDAT", zlib.compress(body, level)) + _chunk(b"IEND", b""))


def load_image(path: str) -> np.ndarray:
    """An image file as ``[h, w, 4]`` uint8 RGBA (PNG, or a ``.npy`` array)."""
    if path.lower().endswith(".npy"):
        return as_rgba8(np.load(path))
    with open(path, "rb") as f:
        data = f.read()
    if data.startswith(_PNG_SIG):
        return decode_png(data)
    raise ValueError(f"unsupported texture image '{os.path.basename(path)}' (PNG or .npy only)")


def as_rgba8(img) -> np.ndarray:
    """``[h, w]`` / ``[h, w, 1|3|4]`` uint8 (or float in [0, 1]) array or tensor
    -> contiguous ``[h, w, 4]`` uint8 RGBA, row 0 = top."""
    if isinstance(img, torch.Tensor):
        img = img.detach().cpu().numpy()
    a = np.asarray(img)
    if a.ndim == 2:
        a = a[:, :, None]
    if a.ndim != 3 or a.shape[2] not in (1, 3, 4) or a.shape[0] < 1 or a.shape[1] < 1:
        raise ValueError("a texture image must be [h, w] or [h, w, 1|3|4]")
    if a.dtype != np.uint8:
        a = np.floor(np.clip(a.astype(np.float64), 0.0, 1.0) * 255.0 + 0.5).astype(np.uint8)
    h, w, c = a.shape
    out = np.empty((h, w, 4), dtype=np.uint8)
    if c == 1:
        out[..., :3] = a
        out[..., 3] = 255
    elif c == 3:
        out[..., :3] = a
        out[..., 3] = 255
    else:
        out[...] = a
    return out


def gl_rows(img: np.ndarray) -> np.ndarray:
    """Image-order RGBA8 -> the kernels' texel layout (row 0 at ``v = 0``).
    Always a fresh array with positive strides: numpy counts a one-row view
    with a negative row stride as contiguous, which ``torch.from_numpy``
    rejects."""
    return img[::-1].copy(order="C")


WHITE = np.full((1, 1, 4), 255, dtype=np.uint8)
