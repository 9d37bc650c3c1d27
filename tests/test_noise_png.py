"""Ingestion of the reference's noise textures (noise_from_pngs): a PNG
written here with every filter type decodes exactly; the reference's own
textures, when the reference tree is present, decode to four 256 x 256 planes
in (0, 1]."""
import os
import struct
import sys
import zlib

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "fft-ocean-waves_gb300"))
sys.path.insert(0, ROOT)
import ocean_gb300 as og  # noqa: E402


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)


def _write_png(path, img, chans):
    h, w = img.shape[:2]
    flat = img.reshape(h, w * chans).astype(np.int32)
    rows = []
    prev = np.zeros(w * chans, dtype=np.int32)
    for y in range(h):
        f = y % 5
        line = flat[y]
        enc = np.empty_like(line)
        for i in range(len(line)):
            left = line[i - chans] if i >= chans else 0
            up, ul = prev[i], (prev[i - chans] if i >= chans else 0)
            pr = [0, left, up, (left + up) >> 1, _paeth(left, up, ul)][f]
            enc[i] = (line[i] - pr) & 255
        rows.append(bytes([f]) + enc.astype(np.uint8).tobytes())
        prev = line
    ctype = {1: 0, 3: 2, 4: 6}[chans]
    chunk = lambda t, b: struct.pack(">I", len(b)) + t + b + struct.pack(">I", zlib.crc32(t + b) & 0xFFFFFFFF)
    data = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0))
    data += chunk(b"IDAT", zlib.compress(b"".join(rows))) + chunk(b"IEND", b"")
    with open(path, "wb") as fh:
        fh.write(data)


@pytest.mark.parametrize("chans", [1, 3, 4])
def test_png_roundtrip_all_filters(tmp_path, chans):
    rng = np.random.default_rng(chans)
    imgs = [rng.integers(0, 256, (23, 17, chans), dtype=np.uint8) for _ in range(4)]
    paths = []
    for k, im in enumerate(imgs):
        p = str(tmp_path / f"n{k}.png")
        _write_png(p, im, chans)
        paths.append(p)
    nz = og.noise_from_pngs(paths, N=17)
    assert nz.shape == (4, 17, 17) and nz.dtype == np.float32
    ys = (np.arange(17) * 23) // 17
    for k in range(4):
        assert np.array_equal(nz[k], imgs[k][ys, :, 0].astype(np.float32) / np.float32(255.0))


def test_reference_noise_textures():
    from oracle import build_ref
    base = os.path.join(build_ref.REF, "data", "noise")
    paths = [os.path.join(base, f"LDR_LLL1_{k}.png") for k in range(4)]
    if not all(os.path.exists(p) for p in paths):
        pytest.skip("the reference tree is not present")
    nz = og.noise_from_pngs(paths)
    assert nz.shape == (4, 256, 256)
    assert 0.0 <= nz.min() and nz.max() <= 1.0
    assert 0.3 < nz.mean() < 0.7
