"""Image files for batch snapshots: grids of scenes as PNG and animated GIF.

The reference writes them with PIL (``env.py:97-358``); PIL is not available
here, so PNG goes through :func:`renderer.textures.encode_png` and GIF through
the GIF89a writer below (global palette, LZW-compressed frames, looping
animation).
"""
from __future__ import annotations

import math
import struct

import numpy as np
import torch

from .renderer.textures import encode_png

__all__ = ["make_grid", "encode_png", "encode_gif", "palette_quantize"]


def make_grid(pixels: torch.Tensor, indices: list[int] | None = None, num: int = 16,
              scale: int = 1) -> np.ndarray:
    """``[B,C,H,W]`` (or ``[T,B,C,H,W]``) scenes -> one ``[rows*H, cols*W, C]``
    uint8 grid, as ``PBREnv._make_grid_frame`` (``env.py:186-241``): the
    first ``num`` scenes (or ``indices``), ``rows = ceil(sqrt(k))``,
    ``cols = ceil(k / rows)``, scene n at (n // cols, n % cols), nearest-
    neighbour upscaling by ``scale``."""
    if pixels.dim() == 5:
        pixels = torch.flatten(pixels, start_dim=0, end_dim=1)
    B, C, H, W = pixels.shape
    k = min(max(1, int(num)), int(B))
    if indices is not None and len(indices) > 0:
        sel = [int(i) for i in indices if 0 <= int(i) < B][:k]
    else:
        sel = list(range(k))
    imgs = pixels[sel].detach()
    if imgs.dtype != torch.uint8:
        imgs = imgs.clamp(0, 255).to(torch.uint8)
    imgs = imgs.permute(0, 2, 3, 1).cpu().numpy()  # [k,H,W,C]
    rows = int(math.ceil(math.sqrt(k)))
    cols = int(math.ceil(k / rows))
    canvas = np.zeros((rows * H, cols * W, C), dtype=np.uint8)
    for n in range(len(sel)):
        r, c = n // cols, n % cols
        canvas[r * H:(r + 1) * H, c * W:(c + 1) * W] = imgs[n]
    if scale > 1:
        canvas = np.repeat(np.repeat(canvas, int(scale), axis=0), int(scale), axis=1)
    return canvas


# ---------------------------------------------------------------------------
# GIF

def _median_cut(colors: np.ndarray, counts: np.ndarray, n: int) -> np.ndarray:
    """Palette of at most n colours: split the box with the widest channel
    range at its (count-weighted) median until n boxes remain."""
    boxes = [(colors, counts)]
    while len(boxes) < n:
        best, best_range = -1, -1
        for i, (c, _) in enumerate(boxes):
            if len(c) > 1:
                rng = int((c.max(axis=0) - c.min(axis=0)).max())
                if rng > best_range:
                    best, best_range = i, rng
        if best < 0 or best_range == 0:
            break
        c, w = boxes.pop(best)
        ch = int(np.argmax(c.max(axis=0) - c.min(axis=0)))
        order = np.argsort(c[:, ch], kind="stable")
        c, w = c[order], w[order]
        cum = np.cumsum(w)
        cut = int(np.searchsorted(cum, cum[-1] / 2.0)) + 1
        cut = min(max(cut, 1), len(c) - 1)
        boxes += [(c[:cut], w[:cut]), (c[cut:], w[cut:])]
    pal = [np.round((c.astype(np.float64) * w[:, None]).sum(axis=0) / w.sum()) for c, w in boxes]
    return np.clip(np.array(pal), 0, 255).astype(np.uint8)


def palette_quantize(frames: list[np.ndarray]) -> tuple[np.ndarray, list[np.ndarray]]:
    """RGB frames -> (palette ``[P,3]``, index frames).  Exact when all frames
    together use at most 256 colours, else a median-cut palette with
    nearest-colour mapping."""
    rgb = [np.ascontiguousarray(f[..., :3]) for f in frames]
    keys = [(f[..., 0].astype(np.uint32) << 16) | (f[..., 1].astype(np.uint32) << 8) | f[..., 2] for f in rgb]
    uniq, counts = np.unique(np.concatenate([k.reshape(-1) for k in keys]), return_counts=True)
    if len(uniq) <= 256:
        pal = np.stack([(uniq >> 16) & 255, (uniq >> 8) & 255, uniq & 255], axis=1).astype(np.uint8)
        return pal, [np.searchsorted(uniq, k).astype(np.uint8) for k in keys]
    cols = np.stack([(uniq >> 16) & 255, (uniq >> 8) & 255, uniq & 255], axis=1).astype(np.int32)
    pal = _median_cut(cols, counts, 256)
    # nearest palette entry for every distinct colour, then a lookup per pixel
    p = pal.astype(np.int32)
    nearest = np.empty(len(cols), np.uint8)
    for s in range(0, len(cols), 4096):
        d = ((cols[s:s + 4096, None, :] - p[None]) ** 2).sum(axis=2)
        nearest[s:s + 4096] = np.argmin(d, axis=1)
    return pal, [nearest[np.searchsorted(uniq, k)] for k in keys]


def _lzw(indices: np.ndarray, min_code: int = 8) -> bytes:
    """GIF LZW: variable-width codes (min_code + 1 .. 12 bits), LSB first,
    clear code at the start and whenever the 4096-entry table is full."""
    clear, eoi = 1 << min_code, (1 << min_code) + 1
    out = bytearray()
    acc, nbits = 0, 0
    width = min_code + 1

    def emit(code, w):
        nonlocal acc, nbits
        acc |= code << nbits
        nbits += w
        while nbits >= 8:
            out.append(acc & 255)
            acc >>= 8
            nbits -= 8

    data = indices.reshape(-1).tobytes()
    emit(clear, width)
    table: dict[int, int] = {}
    next_code = eoi + 1
    if data:
        prefix = data[0]
        for b in data[1:]:
            key = (prefix << 8) | b
            code = table.get(key)
            if code is not None:
                prefix = code
                continue
            emit(prefix, width)
            if next_code < 4096:
                table[key] = next_code
                if next_code == (1 << width) and width < 12:
                    width += 1
                next_code += 1
            else:
                emit(clear, width)
                table.clear()
                next_code = eoi + 1
                width = min_code + 1
            prefix = b
        emit(prefix, width)
        # the decoder adds one more entry on reading that code and may widen before the end code
        if next_code == (1 << width) and width < 12:
            width += 1
    emit(eoi, width)
    if nbits:
        out.append(acc & 255)
    return bytes(out)


def _sub_blocks(data: bytes) -> bytes:
    parts = [bytes([len(data[i:i + 255])]) + data[i:i + 255] for i in range(0, len(data), 255)]
    return b"".join(parts) + b"\x00"


def encode_gif(frames: list[np.ndarray], duration_ms: int = 100, loop: int = 0) -> bytes:
    """``[H,W,3|4]`` uint8 frames (same size) -> animated GIF89a bytes."""
    if not frames:
        raise ValueError("encode_gif needs at least one frame")
    H, W = frames[0].shape[:2]
    if any(f.shape[:2] != (H, W) for f in frames):
        raise ValueError("all GIF frames must have the same size")
    if W > 65535 or H > 65535:
        raise ValueError("GIF frames are limited to 65535 x 65535")
    pal, idx = palette_quantize(frames)
    size_bits = max(1, int(math.ceil(math.log2(max(2, len(pal))))))
    table = np.zeros((1 << size_bits, 3), np.uint8)
    table[:len(pal)] = pal
    out = bytearray(b"GIF89a")
    out += struct.pack("<HHBBB", W, H, 0x80 | 0x70 | (size_bits - 1), 0, 0)
    out += table.tobytes()
    out += b"\x21\xff\x0bNETSCAPE2.0\x03\x01" + struct.pack("<H", int(loop)) + b"\x00"
    delay = max(0, int(round(duration_ms / 10.0)))
    for f in idx:
        out += b"\x21\xf9\x04\x00" + struct.pack("<H", delay) + b"\x00\x00"
        out += b"\x2c" + struct.pack("<HHHHB", 0, 0, W, H, 0)
        out += bytes([8]) + _sub_blocks(_lzw(f, 8))
    out += b"\x3b"
    return bytes(out)
