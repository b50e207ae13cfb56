"""JPEG encode on the GPU through the C ABI (rd_encode_jpeg, rd_encode_jpeg_device)
against the oracle.

The reference's encoder (the image crate's JpegEncoder) is not vendored, so
its bytes cannot be compared. Checked instead:
  * the file decodes (the oracle's T.81 baseline decoder: markers, Huffman
    tables, restart intervals, byte stuffing) to exactly the quantised
    coefficients the oracle computes from the same rows and quality;
  * the quantisation tables are the Annex K tables scaled by quality;
  * a higher quality gives a larger file with different decoded pixels, as
    the reference's export test holds (crates/core/tests/export.rs:152-179);
  * the ICC profile and EXIF come back from APP2 / APP1;
  * padded rows, qualities outside 1..100 and sides above 65535 are refused.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ANNEX_K = [
    [16, 11, 10, 16, 24, 40, 51, 61, 12, 12, 14, 19, 26, 58, 60, 55, 14, 13, 16, 24, 40, 57, 69, 56,
     14, 17, 22, 29, 51, 87, 80, 62, 18, 22, 37, 56, 68, 109, 103, 77, 24, 35, 55, 64, 81, 104, 113, 92,
     49, 64, 78, 87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99],
    [17, 18, 24, 47, 99, 99, 99, 99, 18, 21, 26, 66, 99, 99, 99, 99, 24, 26, 56, 99, 99, 99, 99, 99,
     47, 66] + [99] * 38,
]


@pytest.fixture(scope="module")
def encoder(device):
    from rohditor_gb300 import JpegEncoder

    return JpegEncoder(device)


def _image(kind, h, w, seed=0):
    rng = np.random.default_rng(seed)
    if kind == "random":
        return rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
    if kind == "flat":
        return np.full((h, w, 3), 77, dtype=np.uint8)
    y, x = np.mgrid[0:h, 0:w]
    base = (np.sin(x / 23.0) + np.cos(y / 17.0) + 2.0) / 4.0 * 255
    img = np.stack([base, 0.6 * base + 40, 255 - base], axis=-1) + rng.normal(0, 3.0, (h, w, 3))
    return np.clip(img, 0, 255).astype(np.uint8)


def _segments(data: bytes):
    """(marker, body) of every segment before the scan."""
    pos, out = 2, []
    while data[pos + 1] != 0xDA:
        n = int.from_bytes(data[pos + 2:pos + 4], "big")
        out.append((data[pos + 1], data[pos + 4:pos + 2 + n]))
        pos += 2 + n
    return out


def _check(encoder, oracle, image, quality, icc=b"", exif=None):
    data = encoder.encode(image, quality, icc, exif)
    h, w = image.shape[:2]
    assert len(data) <= encoder.bound(w, h, len(icc), len(exif or b""))
    got = oracle.jpeg_decode(data)
    assert (got["width"], got["height"], got["restart"]) == (w, h, 32)
    assert np.array_equal(got["coef"], oracle.jpeg_coefficients(image, quality))
    scale = 5000 // quality if quality < 50 else 200 - 2 * quality
    for c in range(3):
        want = [max(1, min(255, (v * scale + 50) // 100)) for v in ANNEX_K[0 if c == 0 else 1]]
        assert list(got["quant"][c]) == want
    return data, got


@pytest.mark.parametrize("h,w", [(1, 1), (5, 7), (8, 8), (33, 17), (200, 300), (517, 1033)])
@pytest.mark.parametrize("quality", [1, 50, 90, 100])
@pytest.mark.parametrize("kind", ["random", "smooth", "flat"])
def test_jpeg_carries_the_oracle_coefficients(encoder, oracle, h, w, quality, kind):
    _check(encoder, oracle, _image(kind, h, w, seed=h + w), quality)


def test_jpeg_full_frame(encoder, oracle):
    image = _image("smooth", 4024, 6048, seed=2)
    data, got = _check(encoder, oracle, image, 90)
    pixels = oracle.jpeg_pixels(got)
    err = pixels.astype(np.float64) - image
    assert 10 * np.log10(255.0 ** 2 / np.mean(err ** 2)) > 33.0
    assert len(data) < image.nbytes // 4


def test_higher_quality_is_larger_and_decodes_differently(encoder, oracle):
    # crates/core/tests/export.rs:152-179
    image = _image("smooth", 96, 128, seed=3)
    low, high = encoder.encode(image, 40), encoder.encode(image, 95)
    assert len(high) > len(low)
    assert not np.array_equal(oracle.jpeg_pixels(oracle.jpeg_decode(low)),
                              oracle.jpeg_pixels(oracle.jpeg_decode(high)))


def test_jpeg_embeds_the_profile_and_exif(encoder, oracle):
    rng = np.random.default_rng(12)
    icc = rng.integers(0, 256, 70000, dtype=np.uint8).tobytes()  # two APP2 segments
    exif = b"II*\x00" + bytes(range(100))
    data, _ = _check(encoder, oracle, _image("smooth", 40, 64), 85, icc, exif)
    segs = _segments(data)
    app1 = [b for m, b in segs if m == 0xE1]
    assert app1 == [b"Exif\x00\x00" + exif]
    app2 = [b for m, b in segs if m == 0xE2]
    assert [b[:12] for b in app2] == [b"ICC_PROFILE\x00"] * 2
    assert [(b[12], b[13]) for b in app2] == [(1, 2), (2, 2)]
    assert b"".join(b[14:] for b in app2) == icc
    assert segs[0][0] == 0xE0 and segs[0][1][:5] == b"JFIF\x00"


def test_jpeg_refuses_bad_arguments(encoder, device):
    from rohditor_gb300 import GpuPreviewError

    image = _image("smooth", 16, 20)
    for q in (0, 101):
        with pytest.raises(GpuPreviewError) as err:
            encoder.encode(image, q)
        assert err.value.code == 8
    padded = np.zeros((16, 66), dtype=np.uint8)
    with pytest.raises(GpuPreviewError) as err:
        encoder.encode(padded, 90, row_stride=66, width=20)
    assert err.value.code == 8
    with pytest.raises(GpuPreviewError) as err:
        encoder.encode(np.zeros((1, 65536, 3), dtype=np.uint8), 90)
    assert err.value.code == 4
    encoder.encode(image, 90)  # the context stays usable


def test_device_entry_point_writes_the_same_file(encoder, device):
    import torch

    image = _image("smooth", 300, 451, seed=9)
    host = encoder.encode(image, 80)
    d_rgb = torch.from_numpy(image.copy()).cuda()
    cap = encoder.bound(451, 300)
    d_out = torch.zeros(cap, dtype=torch.uint8, device="cuda")
    d_size = torch.zeros(1, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    device.check(device.lib.rd_encode_jpeg_device(device.handle, ctypes.c_void_p(d_rgb.data_ptr()), 451, 300,
                                                  3 * 451, 80, None, 0, None, 0, ctypes.c_void_p(d_out.data_ptr()),
                                                  cap, ctypes.c_void_p(d_size.data_ptr())))
    n = int(d_size.cpu()[0])
    assert d_out[:n].cpu().numpy().tobytes() == host
