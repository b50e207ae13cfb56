"""PNG encoder pieces that run without a GPU: the deflate block format of the
encoder (its shared arithmetic compiled for the host and driven the way the
deflate kernel drives it, then inflated by Python's zlib), the oracle's filter
restatement against a direct one, and the size bound of the C ABI."""

import os
import shutil
import subprocess
import zlib

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SEG = 32768


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path_factory.mktemp("deflate") / "deflate_host"
    subprocess.run([cxx, "-O2", "-std=c++17", "-Wall", "-o", str(exe),
                    os.path.join(ROOT, "tests", "native", "deflate_host.cpp")], check=True)
    return exe


def _deflate(harness, tmp_path, data: bytes):
    src, dst = tmp_path / "in.bin", tmp_path / "out.z"
    src.write_bytes(data)
    out = subprocess.run([str(harness), str(src), str(dst)], capture_output=True, text=True, check=True)
    crc, adler, segments, stored = (int(v) for v in out.stdout.split())
    return dst.read_bytes(), crc, adler, segments, stored


def _smooth_image(rng, h, w, dtype=np.uint8):
    top = 255 if dtype == np.uint8 else 65535
    y, x = np.mgrid[0:h, 0:w]
    base = (np.sin(x / 37.0) + np.cos(y / 23.0) + 2.0) / 4.0 * top
    img = np.stack([base, base * 0.7, top - base], axis=-1) + rng.normal(0, top / 200.0, (h, w, 3))
    return np.clip(img, 0, top).astype(dtype)


def _cases(oracle):
    rng = np.random.default_rng(7)
    runs = b"".join(bytes([i % 256]) * (i % 700 + 1) for i in range(700))
    return {
        "one_byte": b"\x2a",
        "random": rng.integers(0, 256, 3 * SEG + 17, dtype=np.uint8).tobytes(),
        "zeros": bytes(5 * SEG),
        "exact_segment": rng.integers(0, 3, SEG, dtype=np.uint8).tobytes(),
        "segment_plus_one": rng.integers(0, 3, SEG + 1, dtype=np.uint8).tobytes(),
        "runs_across_258": runs,
        "filtered_photo": oracle.png_filter(_smooth_image(rng, 211, 307)),
        "filtered_photo16": oracle.png_filter(_smooth_image(rng, 97, 131, np.uint16)),
    }


def test_segments_inflate_with_zlib(harness, tmp_path, oracle):
    for name, data in _cases(oracle).items():
        z, crc, adler, segments, stored = _deflate(harness, tmp_path, data)
        assert zlib.decompress(z) == data, name
        assert crc == zlib.crc32(data), name
        assert adler == zlib.adler32(data), name
        assert segments == (len(data) + SEG - 1) // SEG
        if name == "random":
            assert stored == segments  # incompressible: every segment stored
        if name in ("zeros", "runs_across_258", "filtered_photo"):
            assert stored == 0 and len(z) < len(data) // 2, name


def _filter_direct(image: np.ndarray) -> bytes:
    """PNG filter type 0 with minimum-sum-of-absolute-differences selection, in plain Python."""
    depth = 16 if image.dtype == np.uint16 else 8
    h, w = image.shape[:2]
    rows = image.reshape(h, 3 * w)
    rows = rows.astype(">u2").view(np.uint8).reshape(h, -1) if depth == 16 else rows
    bpp = 3 * depth // 8
    out = bytearray()
    prev = [0] * rows.shape[1]
    for r in range(h):
        line = [int(v) for v in rows[r]]

        def pred(t, i):
            a = line[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            if t == 0:
                return 0
            if t == 1:
                return a
            if t == 2:
                return b
            if t == 3:
                return (a + b) // 2
            p = a + b - c
            pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
            return a if pa <= pb and pa <= pc else (b if pb <= pc else c)

        filtered = [[(line[i] - pred(t, i)) & 0xFF for i in range(len(line))] for t in range(5)]
        sums = [sum(v if v < 128 else 256 - v for v in f) for f in filtered]
        best = sums.index(min(sums))
        out.append(best)
        out.extend(filtered[best])
        prev = line
    return bytes(out)


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16])
def test_oracle_filter_matches_a_direct_restatement(oracle, dtype):
    rng = np.random.default_rng(3)
    top = np.iinfo(dtype).max
    for h, w in ((1, 1), (4, 5), (9, 13)):
        for image in (rng.integers(0, top + 1, (h, w, 3)).astype(dtype), _smooth_image(rng, h, w, dtype),
                      np.full((h, w, 3), top // 3, dtype=dtype)):
            stream = oracle.png_filter(image)
            assert stream == _filter_direct(image)
            depth = 16 if dtype == np.uint16 else 8
            assert np.array_equal(oracle.png_unfilter(stream, w, h, depth), image)


def test_png_bound_is_the_stored_worst_case():
    from rohditor_gb300 import PngEncoder

    for w, h, depth, icc, exif in ((1, 1, 8, 0, 0), (6048, 4024, 8, 0, 0), (6048, 4024, 16, 3144, 210),
                                   (5, 70000, 16, 70000, 1)):
        stream = h * (1 + w * 3 * depth // 8)
        segments = (stream + SEG - 1) // SEG
        header = 8 + 25
        if icc:
            blocks = (icc + 65534) // 65535
            header += 12 + len(b"ICC profile") + 2 + 2 + 5 * blocks + icc + 4
        if exif:
            header += 12 + exif
        assert PngEncoder.bound(w, h, depth, icc, exif) == header + stream + 17 * segments + 6 + 12
    assert PngEncoder.bound(10, 10, 12) == 0
    assert PngEncoder.bound(0, 10, 8) == 0
    assert PngEncoder.bound(10, 10, 8, 1 << 40, 0) == 0  # metadata past a chunk's 31-bit length
    assert PngEncoder.bound(10, 10, 8, 0, 1 << 40) == 0


def test_jpeg_bound_limits():
    from rohditor_gb300 import JpegEncoder

    assert JpegEncoder.bound(6048, 4024) > 0
    assert JpegEncoder.bound(65535, 1) > 0 and JpegEncoder.bound(65536, 1) == 0
    assert JpegEncoder.bound(16, 16, 0, 65527) > 0 and JpegEncoder.bound(16, 16, 0, 65528) == 0  # one APP1
    assert JpegEncoder.bound(16, 16, 255 * 65519, 0) > 0 and JpegEncoder.bound(16, 16, 255 * 65519 + 1, 0) == 0


def test_runs_across_chunk_and_segment_boundaries(harness, tmp_path):
    # A thread's tokens depend on runs that start or end in other threads'
    # 32-byte chunks and stop at segment ends: runs of every length from 1 to
    # 600 placed at every offset around a chunk boundary and a segment boundary.
    rng = np.random.default_rng(11)
    for anchor in (4 * 32, SEG - 40):
        pieces = []
        for length in list(range(1, 40)) + [255, 256, 257, 258, 259, 260, 261, 515, 516, 517, 600]:
            for shift in range(0, 36, 5):
                noise = rng.integers(0, 256, anchor - shift, dtype=np.uint8)
                pieces.append(noise.tobytes() + bytes([rng.integers(0, 256)]) * length)
        data = b"".join(pieces)
        z, crc, adler, segments, _ = _deflate(harness, tmp_path, data)
        assert zlib.decompress(z) == data
        assert crc == zlib.crc32(data) and adler == zlib.adler32(data)

