"""JPEG pieces that run without a GPU: the encoder's own integer arithmetic
(rohditor_gb300/csrc/jpeg.cuh compiled for the host) against the oracle's
independent restatement, the oracle's integer coefficients against the
floating-point FDCT of T.81 (A.3.3), and the oracle's baseline decoder on a
file written here in plain Python (fixed Huffman tables, restart markers, byte
stuffing), so that the decoder the GPU tests rely on is itself checked."""

import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def jpeg_harness(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path_factory.mktemp("jpeg") / "jpeg_host"
    subprocess.run([cxx, "-O2", "-std=c++17", "-Wall", "-o", str(exe),
                    os.path.join(ROOT, "tests", "native", "jpeg_host.cpp")], check=True)
    return exe


@pytest.mark.parametrize("quality", [1, 25, 50, 75, 90, 100])
def test_encoder_arithmetic_matches_the_oracle(jpeg_harness, oracle, tmp_path, quality):
    rng = np.random.default_rng(quality)
    for h, w, kind in ((1, 1, "random"), (13, 21, "random"), (40, 56, "smooth"), (64, 64, "extreme")):
        if kind == "random":
            img = rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
        elif kind == "extreme":
            img = np.where(rng.random((h, w, 3)) < 0.5, 0, 255).astype(np.uint8)
        else:
            img = _smooth(rng, h, w)
        src, dst = tmp_path / "in.rgb", tmp_path / "out.coef"
        src.write_bytes(img.tobytes())
        subprocess.run([str(jpeg_harness), str(src), str(dst), str(w), str(h), str(quality)], check=True)
        got = np.fromfile(dst, dtype=np.int16).reshape(-1, 3, 64)
        assert np.array_equal(got, oracle.jpeg_coefficients(img, quality)), (h, w, kind)

ANNEX_K_LUMA = [16, 11, 10, 16, 24, 40, 51, 61, 12, 12, 14, 19, 26, 58, 60, 55, 14, 13, 16, 24, 40, 57, 69, 56,
                14, 17, 22, 29, 51, 87, 80, 62, 18, 22, 37, 56, 68, 109, 103, 77, 24, 35, 55, 64, 81, 104, 113, 92,
                49, 64, 78, 87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99]


def _smooth(rng, h, w):
    y, x = np.mgrid[0:h, 0:w]
    base = (np.sin(x / 9.0) + np.cos(y / 7.0) + 2.0) / 4.0 * 255
    img = np.stack([base, 0.5 * base + 60, 255 - base], axis=-1) + rng.normal(0, 2.0, (h, w, 3))
    return np.clip(img, 0, 255).astype(np.uint8)


def test_quantisation_reciprocals_divide_exactly():
    # floor(n / q) == (n * ceil(2^31 / q)) >> 31 for every step and every
    # numerator the encoder can meet (|coefficient| + q / 2 stays below 2^11).
    n = np.arange(0, 1 << 14, dtype=np.uint64)
    for q in range(1, 256):
        m = np.uint64(((1 << 31) + q - 1) // q)
        assert np.array_equal((n * m) >> np.uint64(31), n // np.uint64(q)), q


def test_oracle_coefficients_follow_the_float_fdct(oracle):
    rng = np.random.default_rng(1)
    img = _smooth(rng, 16, 24)
    q = 100  # every table entry 1: the coefficient itself, rounded
    coef = oracle.jpeg_coefficients(img, q)
    nat = oracle._zigzag_natural()
    u = np.arange(8)
    basis = np.cos((2 * u[None, :] + 1) * u[:, None] * np.pi / 16) * np.where(u == 0, np.sqrt(0.5), 1.0)[:, None] / 2
    r, g, b = (img[..., k].astype(np.int64) for k in range(3))
    ycc = [(19595 * r + 38470 * g + 7471 * b + 32768) >> 16,
           np.minimum(255, (-11059 * r - 21709 * g + 32768 * b + (128 << 16) + 32768) >> 16),
           np.minimum(255, (32768 * r - 27439 * g - 5329 * b + (128 << 16) + 32768) >> 16)]
    worst = 0.0
    for by in range(2):
        for bx in range(3):
            for c in range(3):
                s = ycc[c][by * 8:by * 8 + 8, bx * 8:bx * 8 + 8].astype(np.float64) - 128
                f = basis @ s @ basis.T  # F[v][u]
                got = np.zeros(64)
                got[nat] = coef[by * 3 + bx, c]
                worst = max(worst, float(np.max(np.abs(got.reshape(8, 8) - f))))
    assert worst <= 1.0  # the 13-bit integer DCT stays within one unit of the exact one


def _huffman_fixed(symbols, bits):
    """A canonical table giving every symbol a `bits`-bit code, in ascending symbol order."""
    counts = [0] * 16
    counts[bits - 1] = len(symbols)
    codes = {s: (i, bits) for i, s in enumerate(sorted(symbols))}
    return counts, sorted(symbols), codes


class _Bits:
    def __init__(self):
        self.out, self.acc, self.n = bytearray(), 0, 0

    def put(self, value, bits):
        for i in range(bits - 1, -1, -1):
            self.acc = (self.acc << 1) | ((value >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc, self.n = 0, 0

    def flush(self):
        while self.n:
            self.put(1, 1)


def _write_jpeg(coef, w, h, quant_nat, restart):
    def seg(m, body):
        return bytes([0xFF, m]) + (len(body) + 2).to_bytes(2, "big") + bytes(body)

    zz = _zigzag_positions()
    dc_syms = list(range(12))
    ac_syms = [0x00, 0xF0] + [(r << 4) | s for r in range(16) for s in range(1, 11)]
    dc_counts, dc_vals, dc_codes = _huffman_fixed(dc_syms, 4)
    ac_counts, ac_vals, ac_codes = _huffman_fixed(ac_syms, 8)
    out = bytearray([0xFF, 0xD8])
    out += seg(0xDB, [0] + [quant_nat[zz[k]] for k in range(64)])
    out += seg(0xC0, [8, h >> 8, h & 255, w >> 8, w & 255, 3, 1, 0x11, 0, 2, 0x11, 0, 3, 0x11, 0])
    for tid, counts, vals in ((0x00, dc_counts, dc_vals), (0x10, ac_counts, ac_vals)):
        out += seg(0xC4, [tid] + counts + vals)
    out += seg(0xDD, [0, restart])
    out += seg(0xDA, [3, 1, 0x00, 2, 0x00, 3, 0x00, 0, 63, 0])

    def cat(v):
        return int(abs(int(v))).bit_length()

    def extra(v, c):
        return (v if v >= 0 else v + (1 << c) - 1) & ((1 << c) - 1)

    bits = _Bits()
    pred = [0, 0, 0]
    for m in range(coef.shape[0]):
        if m and m % restart == 0:
            bits.flush()
            out += bits.out
            out += bytes([0xFF, 0xD0 + ((m // restart - 1) & 7)])
            bits = _Bits()
            pred = [0, 0, 0]
        for c in range(3):
            z = [int(v) for v in coef[m, c]]
            d = z[0] - pred[c]
            pred[c] = z[0]
            k = cat(d)
            bits.put(*dc_codes[k])
            bits.put(extra(d, k), k)
            run = 0
            for v in z[1:]:
                if v == 0:
                    run += 1
                    continue
                while run > 15:
                    bits.put(*ac_codes[0xF0])
                    run -= 16
                k = cat(v)
                bits.put(*ac_codes[(run << 4) | k])
                bits.put(extra(v, k), k)
                run = 0
            if run:
                bits.put(*ac_codes[0x00])
    bits.flush()
    out += bits.out + bytes([0xFF, 0xD9])
    return bytes(out)


def _zigzag_positions():
    from oracle import oracle as o

    return list(o._zigzag_natural())


@pytest.mark.parametrize("restart", [1, 2, 5])
def test_oracle_decoder_reads_a_baseline_file(oracle, restart):
    rng = np.random.default_rng(restart)
    img = _smooth(rng, 21, 37)
    img[:8, :8] = 255  # saturated blocks: 0xFF bytes in the entropy-coded data
    coef = oracle.jpeg_coefficients(img, 100)
    coef[3, 1, 5:30] = 0  # long zero runs (ZRL)
    coef[3, 1, 40] = -7
    data = _write_jpeg(coef, 37, 21, [1] * 64, restart)
    got = oracle.jpeg_decode(data)
    assert (got["width"], got["height"], got["restart"]) == (37, 21, restart)
    assert np.array_equal(got["coef"], coef)
    assert np.all(got["quant"] == 1)


def test_decoded_pixels_match_the_image(oracle):
    # Quality 100 quantises by 1: only the rounding of the DCT and of the
    # colour conversions separates the decoded pixels from the image.
    rng = np.random.default_rng(4)
    img = _smooth(rng, 40, 56)
    coef = oracle.jpeg_coefficients(img, 100)
    got = oracle.jpeg_decode(_write_jpeg(coef, 56, 40, [1] * 64, 3))
    pixels = oracle.jpeg_pixels(got)
    err = pixels.astype(np.int32) - img.astype(np.int32)
    assert np.abs(err).max() <= 3
    psnr = 10 * np.log10(255.0 ** 2 / np.mean(err.astype(np.float64) ** 2))
    assert psnr > 45.0
