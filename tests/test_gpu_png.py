"""PNG encode on the GPU through the C ABI (rd_encode_png, rd_encode_png_device)
against the oracle.

The reference encodes with the image crate's PngEncoder (not vendored), so
the file's compressed bytes are not comparable; what is checked is what the
reference's own export tests hold (crates/core/tests/export.rs:19-64, 115-148,
228-246) plus the encoder's internals:
  * every chunk's CRC-32, the IHDR fields and chunk order;
  * the inflated IDAT stream (Python's zlib also checks its Adler-32) equals
    the oracle's filtered scanlines byte for byte;
  * decoding gives back exactly the input samples, 8 and 16 bits;
  * the ICC profile and EXIF come back unchanged from iCCP / eXIf;
  * padded rows and other bit depths are refused.
"""

import zlib

import numpy as np
import pytest

from pngfile import decode, read_chunks

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def encoder(device):
    from rohditor_gb300 import PngEncoder

    return PngEncoder(device)


def _image(kind, h, w, dtype, seed=0):
    rng = np.random.default_rng(seed)
    top = np.iinfo(dtype).max
    if kind == "random":
        return rng.integers(0, top + 1, (h, w, 3)).astype(dtype)
    if kind == "flat":
        return np.full((h, w, 3), top // 5, dtype=dtype)
    if kind == "bands":
        rows = rng.integers(0, top + 1, (h, 1, 3))
        return np.broadcast_to(rows, (h, w, 3)).astype(dtype)
    y, x = np.mgrid[0:h, 0:w]
    base = (np.sin(x / 41.0) + np.cos(y / 29.0) + 2.0) / 4.0 * top
    img = np.stack([base, 0.6 * base, top - base], axis=-1) + rng.normal(0, top / 300.0, (h, w, 3))
    return np.clip(img, 0, top).astype(dtype)


def _check(encoder, oracle, image, icc=b"", exif=None):
    png = encoder.encode(image, icc, exif)
    h, w = image.shape[:2]
    depth = 16 if image.dtype == np.uint16 else 8
    assert len(png) <= encoder.bound(w, h, depth, len(icc), len(exif or b""))
    got = decode(png, oracle)
    assert (got["width"], got["height"], got["depth"]) == (w, h, depth)
    assert got["stream"] == oracle.png_filter(image)
    assert np.array_equal(got["pixels"], image)
    return png, got


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16])
@pytest.mark.parametrize("h,w", [(1, 1), (5, 7), (200, 300), (517, 1033), (40, 6000)])
@pytest.mark.parametrize("kind", ["random", "smooth", "flat", "bands"])
def test_png_decodes_to_the_input_and_the_oracle_stream(encoder, oracle, dtype, h, w, kind):
    _check(encoder, oracle, _image(kind, h, w, dtype, seed=h * 31 + w))


def test_png16_keeps_native_sixteen_bit_samples(encoder, oracle):
    # crates/core/tests/export.rs:115-148: samples that are not multiples of 257 survive.
    image = _image("random", 64, 96, np.uint16, seed=5)
    assert np.any(image % 257 != 0)
    _, got = _check(encoder, oracle, image)
    assert got["pixels"].dtype == np.uint16


def test_png_embeds_the_profile_and_exif(encoder, oracle):
    rng = np.random.default_rng(11)
    icc = rng.integers(0, 256, 70000, dtype=np.uint8).tobytes()  # two stored blocks in the iCCP stream
    exif = b"Exif\x00\x00II*\x00" + bytes(range(200))
    _, got = _check(encoder, oracle, _image("smooth", 64, 96, np.uint8), icc, exif)
    kinds = [k for k, _ in got["chunks"]]
    assert kinds[:3] == [b"IHDR", b"iCCP", b"eXIf"] and kinds[3] == b"IDAT"
    body = got["chunks"][1][1]
    name, rest = body.split(b"\x00", 1)
    assert name == b"ICC profile" and rest[0] == 0
    assert zlib.decompress(rest[1:]) == icc
    assert got["chunks"][2][1] == exif
    png = encoder.encode(_image("smooth", 8, 8, np.uint8))
    assert [k for k, _ in read_chunks(png)][:2] == [b"IHDR", b"IDAT"]


def test_png_refuses_padded_rows_and_other_depths(encoder, device):
    from rohditor_gb300 import GpuPreviewError

    image = _image("smooth", 16, 20, np.uint8)
    padded = np.zeros((16, 3 * 20 + 6), dtype=np.uint8)
    padded[:, :60] = image.reshape(16, 60)
    with pytest.raises(GpuPreviewError) as err:
        encoder.encode(padded, row_stride=66, width=20)
    assert err.value.code == 8  # RD_INVALID_INPUT
    out = np.zeros(1 << 16, dtype=np.uint8)
    size = np.zeros(1, dtype=np.uint64)
    import ctypes

    rc = device.lib.rd_encode_png(device.handle, image.ctypes.data_as(ctypes.c_void_p), 20, 16, 60, 12, None, 0,
                                  None, 0, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), out.nbytes,
                                  size.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), None)
    assert rc == 8
    rc = device.lib.rd_encode_png(device.handle, image.ctypes.data_as(ctypes.c_void_p), 20, 16, 60, 8, None, 0,
                                  None, 0, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), 10,
                                  size.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), None)
    assert rc == 4 and 10 < int(size[0]) <= out.nbytes  # RD_INVALID_DIMENSIONS with the needed size
    # The context stays usable.
    encoder.encode(image)


def test_device_entry_point_writes_the_same_file(encoder, device, oracle):
    import ctypes

    import torch

    image = _image("smooth", 300, 451, np.uint16, seed=9)
    host = encoder.encode(image)
    d_rgb = torch.from_numpy(image.view(np.int16).copy()).cuda()
    cap = encoder.bound(451, 300, 16)
    d_png = torch.zeros(cap, dtype=torch.uint8, device="cuda")
    d_size = torch.zeros(1, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    rc = device.lib.rd_encode_png_device(device.handle, ctypes.c_void_p(d_rgb.data_ptr()), 451, 300, 3 * 451, 16,
                                         None, 0, None, 0, ctypes.c_void_p(d_png.data_ptr()), cap,
                                         ctypes.c_void_p(d_size.data_ptr()))
    device.check(rc)
    n = int(d_size.cpu()[0])
    assert d_png[:n].cpu().numpy().tobytes() == host


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16])
def test_png_full_frame(encoder, oracle, dtype):
    # The bench frame's size: 6048x4024 (24.3 MP), 1.6k segments per 8-bit file.
    image = _image("smooth", 4024, 6048, dtype, seed=1)
    png, _ = _check(encoder, oracle, image)
    assert len(png) < image.nbytes
