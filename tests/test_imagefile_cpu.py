"""Batch snapshots on the CPU: the scene grid, the GIF writer (checked with an
independent GIF decoder written here from the GIF89a specification), and
``save_batch_examples`` / ``save_batch_gif`` file output."""
import struct

import numpy as np
import pytest
import torch

from pybatchrender_gb300 import envs, imagefile
from pybatchrender_gb300.renderer import textures


def _lzw_decode(data: bytes, min_code: int) -> list[int]:
    clear, eoi = 1 << min_code, (1 << min_code) + 1
    width = min_code + 1
    table = [[i] for i in range(1 << min_code)] + [[], []]
    out: list[int] = []
    prev = None
    pos = 0
    nbits = len(data) * 8
    while pos + width <= nbits:
        code = 0
        for k in range(width):
            bit = (data[(pos + k) >> 3] >> ((pos + k) & 7)) & 1
            code |= bit << k
        pos += width
        if code == clear:
            table = table[:eoi + 1]
            width = min_code + 1
            prev = None
            continue
        if code == eoi:
            break
        if prev is None:
            entry = table[code]
        elif code < len(table):
            entry = table[code]
            table.append(prev + [entry[0]])
        else:
            assert code == len(table), "invalid LZW code"
            entry = prev + [prev[0]]
            table.append(entry)
        out += entry
        prev = entry
        if len(table) == (1 << width) and width < 12:
            width += 1
    return out


def _gif_decode(data: bytes):
    assert data[:6] == b"GIF89a"
    W, H, flags, _, _ = struct.unpack("<HHBBB", data[6:13])
    pos = 13
    pal = None
    if flags & 0x80:
        n = 2 << (flags & 7)
        pal = np.frombuffer(data[pos:pos + 3 * n], np.uint8).reshape(n, 3)
        pos += 3 * n
    frames, delays, loop = [], [], None
    while True:
        b = data[pos]
        if b == 0x3B:
            break
        if b == 0x21:
            label = data[pos + 1]
            pos += 2
            blocks = []
            while data[pos]:
                blocks.append(data[pos + 1:pos + 1 + data[pos]])
                pos += 1 + data[pos]
            pos += 1
            if label == 0xF9:
                delays.append(struct.unpack("<H", blocks[0][1:3])[0])
            elif label == 0xFF and blocks[0] == b"NETSCAPE2.0":
                loop = struct.unpack("<H", blocks[1][1:3])[0]
            continue
        assert b == 0x2C
        x, y, w, h, fl = struct.unpack("<HHHHB", data[pos + 1:pos + 10])
        assert (x, y, w, h, fl) == (0, 0, W, H, 0)
        pos += 10
        min_code = data[pos]
        pos += 1
        raw = bytearray()
        while data[pos]:
            raw += data[pos + 1:pos + 1 + data[pos]]
            pos += 1 + data[pos]
        pos += 1
        idx = np.array(_lzw_decode(bytes(raw), min_code), np.uint8)
        assert idx.size == W * H
        frames.append(pal[idx.reshape(H, W)])
    return frames, delays, loop


def test_grid_layout():
    B, H, W = 5, 3, 4
    px = torch.arange(B, dtype=torch.uint8).reshape(B, 1, 1, 1).expand(B, 3, H, W) * 40
    g = imagefile.make_grid(px, num=16, scale=2)
    assert g.shape == (3 * H * 2, 2 * W * 2, 3)  # rows = ceil(sqrt(5)) = 3, cols = ceil(5 / 3) = 2
    for n in range(B):
        r, c = n // 2, n % 2
        assert np.all(g[r * 2 * H:(r + 1) * 2 * H, c * 2 * W:(c + 1) * 2 * W] == 40 * n)
    assert np.all(g[2 * 2 * H:, 2 * W:] == 0)  # the sixth cell is empty
    sel = imagefile.make_grid(px, indices=[4, 1, 99], num=2)
    assert sel.shape == (2 * H, W, 3) and sel[0, 0, 0] == 160 and sel[H, 0, 0] == 40


@pytest.mark.parametrize("colours", [5, 255, 5000])
def test_gif_roundtrip(colours):
    rng = np.random.default_rng(colours)
    pal = rng.integers(0, 256, size=(colours, 3), dtype=np.uint8)
    frames = [pal[rng.integers(0, colours, size=(37, 53))] for _ in range(3)]
    frames.append(np.repeat(np.repeat(frames[0][:10, :10], 4, 0), 4, 1)[:37, :40].copy())
    frames[-1] = np.pad(frames[-1], ((0, 0), (0, 13), (0, 0)))
    data = imagefile.encode_gif(frames, duration_ms=70)
    got, delays, loop = _gif_decode(data)
    assert len(got) == len(frames) and delays == [7] * len(frames) and loop == 0
    if colours < 256:  # with the black padding of the last frame: at most 256 colours
        for a, b in zip(got, frames):
            assert np.array_equal(a, b)
    else:
        p, idx = imagefile.palette_quantize(frames)
        for a, i in zip(got, idx):
            assert np.array_equal(a, p[i])
        err = np.abs(got[0].astype(int) - frames[0].astype(int)).mean()
        assert err < 24


def test_gif_lzw_long_runs_and_table_resets():
    # long single-colour runs and high-entropy data both cross the 4096-code table size
    rng = np.random.default_rng(1)
    for idx in (np.zeros((300, 300), np.uint8), rng.integers(0, 256, size=(150, 170), dtype=np.uint8),
                np.arange(65536, dtype=np.uint32).astype(np.uint8).reshape(256, 256)):
        assert _lzw_decode(imagefile._lzw(idx, 8), 8) == idx.reshape(-1).tolist()
    for n in range(1, 40):  # every short length, including the width change before the end code
        idx = rng.integers(0, 4, size=n, dtype=np.uint8)
        assert _lzw_decode(imagefile._lzw(idx, 8), 8) == idx.tolist()


def test_save_batch_examples_and_gif_files(tmp_path):
    env = envs.make("CartPole-v0", num_scenes=6, device="cpu", render=False)
    px = torch.randint(0, 255, (6, 3, 8, 8), dtype=torch.uint8)
    path, data = env.save_batch_examples(pixels=px, num=4, scale=3, out_dir=str(tmp_path), return_bytes=True)
    assert path.endswith(".png") and open(path, "rb").read() == data
    img = textures.decode_png(data)
    assert img.shape == (2 * 24, 2 * 24, 4)
    assert np.array_equal(img[:24, 24:48, :3], px[1].permute(1, 2, 0).numpy().repeat(3, 0).repeat(3, 1))
    # a worker other than 0 of a parallel env writes nothing
    env.cfg.num_workers, env.cfg.worker_index = 2, 1
    assert env.save_batch_examples(pixels=px, out_dir=str(tmp_path)) is None
    env.cfg.num_workers, env.cfg.worker_index = 1, 0

    # save_batch_gif with the render replaced by a synthetic one (no GPU here)
    calls = []

    def fake_render(obs):
        calls.append(1)
        return torch.full((6, 3, 8, 8), 10 * len(calls), dtype=torch.uint8)

    env.render_pixels = fake_render
    path, data = env.save_batch_gif(num_steps=6, frame_interval=2, num=4, scale=1, duration_ms=50,
                                    out_dir=str(tmp_path), return_bytes=True)
    frames, delays, loop = _gif_decode(data)
    assert len(frames) == 1 + 3 and delays == [5] * 4 and loop == 0
    assert [int(f[0, 0, 0]) for f in frames] == [10, 20, 30, 40]
