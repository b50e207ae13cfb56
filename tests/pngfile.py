"""Minimal PNG reader for the encoder tests: chunk walk with CRC checks, zlib
inflate of the IDAT stream (Python's zlib checks the Adler-32), and the
oracle's inverse filters for the samples."""

from __future__ import annotations

import zlib

SIGNATURE = b"\x89PNG\r\n\x1a\n"


def read_chunks(data: bytes) -> list[tuple[bytes, bytes]]:
    assert data[:8] == SIGNATURE, "not a PNG signature"
    pos, chunks = 8, []
    while pos < len(data):
        n = int.from_bytes(data[pos:pos + 4], "big")
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc = int.from_bytes(data[pos + 8 + n:pos + 12 + n], "big")
        assert len(body) == n, f"{kind!r} chunk runs past the end of the file"
        assert zlib.crc32(kind + body) == crc, f"{kind!r} chunk at {pos} has a bad CRC"
        chunks.append((kind, body))
        pos += 12 + n
    assert pos == len(data)
    assert chunks[0][0] == b"IHDR" and chunks[-1] == (b"IEND", b"")
    return chunks


def decode(data: bytes, oracle) -> dict:
    chunks = read_chunks(data)
    ihdr = chunks[0][1]
    width, height = int.from_bytes(ihdr[0:4], "big"), int.from_bytes(ihdr[4:8], "big")
    depth, colour, method, filtering, interlace = ihdr[8:13]
    assert (colour, method, filtering, interlace) == (2, 0, 0, 0)
    kinds = [k for k, _ in chunks]
    first_idat = kinds.index(b"IDAT")
    assert all(k == b"IDAT" for k in kinds[first_idat:-1]), "IDAT chunks must be consecutive"
    stream = zlib.decompress(b"".join(b for k, b in chunks if k == b"IDAT"))
    return {
        "width": width, "height": height, "depth": depth, "chunks": chunks, "stream": stream,
        "pixels": oracle.png_unfilter(stream, width, height, depth),
    }
