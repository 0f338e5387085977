"""Image IO without OpenCV, and the command line (reference tests/test_smoke.py:68-86)."""

from __future__ import annotations

import struct
import subprocess
import sys
import zlib

import numpy as np
import pytest

from conftest import ROOT
from fpie_gb300 import io


def _encode_filtered(img: np.ndarray, ft: int) -> bytes:
    """PNG with every row using filter type ft (a plain reimplementation for the test)."""
    h, w, c = img.shape
    a = img.astype(np.int32).reshape(h, w * c)
    rows = []
    for y in range(h):
        cur = a[y]
        prev = a[y - 1] if y else np.zeros_like(cur)
        left = np.concatenate([np.zeros(c, np.int32), cur[:-c]])
        upleft = np.concatenate([np.zeros(c, np.int32), prev[:-c]])
        if ft == 0:
            f = cur
        elif ft == 1:
            f = cur - left
        elif ft == 2:
            f = cur - prev
        elif ft == 3:
            f = cur - ((left + prev) >> 1)
        else:
            p = left + prev - upleft
            pa, pb, pc = np.abs(p - left), np.abs(p - prev), np.abs(p - upleft)
            pred = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, upleft))
            f = cur - pred
        rows.append(bytes([ft]) + (f & 0xFF).astype(np.uint8).tobytes())
    ctype = {1: 0, 3: 2, 4: 6}[c]

    def chunk(k, b):
        return struct.pack(">I", len(b)) + k + b + struct.pack(">I", zlib.crc32(k + b))

    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0))
            + chunk(b"IDAT", zlib.compress(b"".join(rows))) + chunk(b"IEND", b""))


@pytest.mark.parametrize("ft", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("channels", [1, 3, 4])
def test_png_filters_decode(tmp_path, ft, channels):
    rng = np.random.default_rng(ft * 10 + channels)
    img = rng.integers(0, 256, (13, 17, channels), dtype=np.uint8)
    p = tmp_path / "f.png"
    p.write_bytes(_encode_filtered(img, ft))
    np.testing.assert_array_equal(io.read_png(str(p)), img)


def test_round_trips_and_channel_rules(tmp_path):
    rng = np.random.default_rng(0)
    rgb = rng.integers(0, 256, (20, 30, 3), dtype=np.uint8)
    for ext in (".png", ".ppm", ".npy"):
        f = str(tmp_path / f"a{ext}")
        io.write_image(f, rgb)
        np.testing.assert_array_equal(io.read_image(f), rgb)
    gray = rng.integers(0, 256, (9, 8), dtype=np.uint8)
    io.write_png(str(tmp_path / "g.png"), gray)
    np.testing.assert_array_equal(io.read_image(str(tmp_path / "g.png")), np.repeat(gray[..., None], 3, -1))
    rgba = rng.integers(0, 256, (9, 8, 4), dtype=np.uint8)
    io.write_png(str(tmp_path / "r.png"), rgba)
    np.testing.assert_array_equal(io.read_image(str(tmp_path / "r.png")), rgba[..., :3])
    with pytest.raises(FileNotFoundError):
        io.read_image(str(tmp_path / "missing.png"))
    with pytest.warns(UserWarning):
        s, m, t = io.read_images(str(tmp_path / "a.png"), str(tmp_path / "nomask.png"), str(tmp_path / "a.png"))
    assert (m == 255).all() and m.shape == s.shape


def test_cli_check_backend():
    r = subprocess.run([sys.executable, "-m", "fpie_gb300.cli", "--check-backend"], cwd=ROOT,
                       check=True, capture_output=True, text=True)
    assert "gb300" in r.stdout
    # the reference's list on the first line, then when to pick each backend
    first, *notes = r.stdout.strip().splitlines()
    assert first.startswith("[") and len(notes) == first.count(",") + 1
    assert any(n.strip().startswith("gb300-rb:") for n in notes)


def test_cli_missing_source_exits_1(tmp_path):
    r = subprocess.run([sys.executable, "-m", "fpie_gb300.cli", "-s", str(tmp_path / "x.png"),
                        "-t", str(tmp_path / "y.png"), "-o", str(tmp_path / "o.png")],
                       cwd=ROOT, capture_output=True, text=True)
    assert r.returncode == 1 and "not found" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("method,backend", [("grid", "gb300"), ("equ", "gb300"), ("equ", "gb300-rb")])
def test_cli_end_to_end(tmp_path, method, backend, monkeypatch):
    from fpie_gb300 import cli, workloads
    from fpie_gb300.process import EquProcessor, GridProcessor

    pb = workloads.circle256()
    for name, arr in (("s.png", pb.src), ("m.png", pb.mask), ("t.png", pb.tgt)):
        io.write_image(str(tmp_path / name), arr)
    monkeypatch.chdir(tmp_path)
    cli.main(["-s", "s.png", "-m", "m.png", "-t", "t.png", "-o", "o.png", "-n", "300", "-p", "100",
              "-g", "src", "--method", method, "-b", backend])
    out = io.read_image(str(tmp_path / "o.png"))
    assert (tmp_path / "iter00100.png").exists() and (tmp_path / "iter00200.png").exists()
    mask3 = np.repeat(pb.mask[..., None], 3, -1)  # PNG round trip of a gray mask gives 3 channels
    proc = (GridProcessor if method == "grid" else EquProcessor)(gradient="src", backend=backend)
    proc.reset(pb.src, mask3, pb.tgt, (0, 0), (0, 0))
    ref, _ = proc.step(300)
    np.testing.assert_array_equal(out, ref)
