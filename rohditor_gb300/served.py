"""Served preview loop (the engine's preview worker and caches on the GPU).

`PreviewServer` wraps the C ABI's `rd_server_*` entry points
(include/rd_gpu.h), which replace crates/engine/src/coordinator/scheduler.rs
(newest-wins mailbox), coordinator/worker.rs (develop_preview) and the preview
caches for many open images: images stay resident, edits are newest-wins per
image and render in cross-image batches ahead of develops, and the least
recently used images lose their device layers when the budget is reached.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _ffi
from .processor import (CaptureContract, ColorContract, GpuPreviewError, OpticsExecution, OutputSpec,
                        SensorDescription, _f32, _ptr)

EDIT, DEVELOP, EXPORT = 0, 1, 2


class PreviewServer:
    """A served loop on GPU `device`, or a dry server (device < 0) that models
    develop and render times on the host, for tests of the policy."""

    def __init__(self, device: int = 0, budget_bytes: int = 0):
        self.lib = _ffi.load()
        h = ctypes.c_void_p()
        rc = self.lib.rd_server_create(device, budget_bytes, ctypes.byref(h))
        if rc != 0:
            raise GpuPreviewError(rc, f"could not create a preview server on device {device}")
        self.handle = h
        self._sizes: dict[int, tuple[int, int]] = {}
        self._crops: dict[int, tuple[int, int]] = {}
        self._export_buffers: dict[int, list] = {}

    @classmethod
    def dry(cls, budget_bytes: int = 0, develop_us: int = 2000, render_us: int = 200) -> "PreviewServer":
        s = cls(-1, budget_bytes)
        s._check(s.lib.rd_server_set_dry_timing(s.handle, develop_us, render_us))
        return s

    def _check(self, rc: int):
        if rc != 0:
            raise GpuPreviewError(rc, self.lib.rd_status_name(rc).decode())

    def open(self, image_id: int, mosaic: np.ndarray, sensor: SensorDescription, capture: CaptureContract,
             optics: OpticsExecution, target: tuple[int, int], wb_gains, camera_to_rec2020) -> int:
        mosaic = np.ascontiguousarray(mosaic, dtype=np.uint16)
        wb = _f32(wb_gains)
        cam = _f32(camera_to_rec2020)
        rid = ctypes.c_uint64()
        s, d, o = sensor.to_c(), capture.to_c(), optics.to_c()
        self._check(self.lib.rd_server_open(self.handle, image_id, _ptr(mosaic, ctypes.c_uint16), mosaic.shape[1],
                                            ctypes.byref(s), ctypes.byref(d), ctypes.byref(o), target[0], target[1],
                                            _ptr(wb, ctypes.c_float), _ptr(cam, ctypes.c_float), ctypes.byref(rid)))
        self._sizes[image_id] = target
        self._crops[image_id] = sensor.crop_size
        return int(rid.value)

    def close_image(self, image_id: int):
        self._check(self.lib.rd_server_close_image(self.handle, image_id))

    def submit_edit(self, image_id: int, revision: int, color: ColorContract | _ffi.ColorDesc) -> int:
        c = color if isinstance(color, _ffi.ColorDesc) else color.to_c()
        rid = ctypes.c_uint64()
        self._check(self.lib.rd_server_submit_edit(self.handle, image_id, revision, ctypes.byref(c), ctypes.byref(rid)))
        return int(rid.value)

    def submit_develop(self, image_id: int, revision: int, capture: CaptureContract, optics: OpticsExecution) -> int:
        d, o = capture.to_c(), optics.to_c()
        rid = ctypes.c_uint64()
        self._check(self.lib.rd_server_submit_develop(self.handle, image_id, revision, ctypes.byref(d),
                                                      ctypes.byref(o), ctypes.byref(rid)))
        return int(rid.value)

    def submit_export(self, image_id: int, revision: int, color: ColorContract,
                      outputs: list[OutputSpec]) -> tuple[int, list[np.ndarray]]:
        """Full-resolution export of an open image; returns the request id and the
        output arrays, which the server fills before the export's result is polled."""
        cw, ch = self._crops[image_id]
        arrays = []
        for spec in outputs:
            ow, oh = spec.dimensions(cw, ch)
            arrays.append(np.empty((oh, 3 * ow), dtype=spec.dtype))
        descs = (_ffi.OutputDesc * len(outputs))(*[spec.to_c() for spec in outputs])
        dst = (ctypes.c_void_p * len(outputs))(*[a.ctypes.data for a in arrays])
        caps = (ctypes.c_size_t * len(outputs))(*[a.nbytes for a in arrays])
        c = color.to_c()
        rid = ctypes.c_uint64()
        self._check(self.lib.rd_server_submit_export(self.handle, image_id, revision, ctypes.byref(c), descs,
                                                     len(outputs), dst, caps, ctypes.byref(rid)))
        self._export_buffers[int(rid.value)] = arrays  # alive until the result is polled
        return int(rid.value), arrays

    def submit_export_files(self, image_id: int, revision: int, color: ColorContract, outputs: list[OutputSpec],
                            files: list[dict]) -> tuple[int, list[np.ndarray], np.ndarray]:
        """Export whose outputs are encoded as files (export::encode): files[k] is
        {"format": "png" | "jpeg" | "rows", "quality": q, "icc": bytes, "exif": bytes}.
        Returns the request id, one byte buffer per output and the array that
        receives each file's size; file k is buffers[k][:sizes[k]] once the
        export's result is polled."""
        cw, ch = self._crops[image_id]
        arrays, descs_c, files_c = [], [], []
        sizes = np.zeros(len(outputs), dtype=np.uint64)
        keep = []
        for k, (spec, f) in enumerate(zip(outputs, files)):
            ow, oh = spec.dimensions(cw, ch)
            fmt = _ffi.FILE_FORMAT[f.get("format", "rows")]
            icc, exif = f.get("icc") or b"", f.get("exif") or b""
            if fmt == 1:
                cap = int(self.lib.rd_png_bound(ow, oh, 16 if spec.format == "srgb16" else 8, len(icc), len(exif)))
                arrays.append(np.empty(max(cap, 1), dtype=np.uint8))
            elif fmt == 2:
                arrays.append(np.empty(max(int(self.lib.rd_jpeg_bound(ow, oh, len(icc), len(exif))), 1), dtype=np.uint8))
            else:
                arrays.append(np.empty((oh, 3 * ow), dtype=spec.dtype))
            icc_a = np.frombuffer(icc, dtype=np.uint8) if icc else None
            exif_a = np.frombuffer(exif, dtype=np.uint8) if exif else None
            keep += [icc_a, exif_a]
            files_c.append(_ffi.ExportFile(
                fmt, int(f.get("quality", 90)),
                icc_a.ctypes.data_as(_ffi.U8P) if icc_a is not None else None, len(icc),
                exif_a.ctypes.data_as(_ffi.U8P) if exif_a is not None else None, len(exif),
                ctypes.cast(sizes.ctypes.data + 8 * k, _ffi.U64P)))
            descs_c.append(spec.to_c())
        descs = (_ffi.OutputDesc * len(outputs))(*descs_c)
        fc = (_ffi.ExportFile * len(outputs))(*files_c)
        dst = (ctypes.c_void_p * len(outputs))(*[a.ctypes.data for a in arrays])
        caps = (ctypes.c_size_t * len(outputs))(*[a.nbytes for a in arrays])
        c = color.to_c()
        rid = ctypes.c_uint64()
        self._check(self.lib.rd_server_submit_export_files(self.handle, image_id, revision, ctypes.byref(c), descs,
                                                           fc, len(outputs), dst, caps, ctypes.byref(rid)))
        self._export_buffers[int(rid.value)] = (arrays, sizes)  # alive until the result is polled
        return int(rid.value), arrays, sizes

    def poll(self, max_results: int = 256, wait_ms: int = 0) -> list[dict]:
        buf = (_ffi.ServerResult * max_results)()
        n = self.lib.rd_server_poll(self.handle, buf, max_results, wait_ms)
        out = [{f: getattr(buf[i], f) for f, _ in _ffi.ServerResult._fields_} for i in range(n)]
        for r in out:
            if r["kind"] == EXPORT:
                self._export_buffers.pop(r["request_id"], None)
        return out

    def read_output(self, image_id: int) -> tuple[np.ndarray, np.ndarray, int]:
        w, h = self._sizes[image_id]
        out = np.empty((h, 3 * w), dtype=np.uint8)
        hist = np.zeros(1024, dtype=np.uint64)
        rev = ctypes.c_uint64()
        self._check(self.lib.rd_server_read_output(self.handle, image_id, _ptr(out, ctypes.c_uint8),
                                                   _ptr(hist, ctypes.c_uint64), ctypes.byref(rev)))
        return out, hist, int(rev.value)

    def stats(self) -> dict:
        st = _ffi.ServerStats()
        self._check(self.lib.rd_server_get_stats(self.handle, ctypes.byref(st)))
        return {f: int(getattr(st, f)) for f, _ in _ffi.ServerStats._fields_}

    def drain(self, wait_ms: int = 60000):
        self._check(self.lib.rd_server_drain(self.handle, wait_ms))

    def close(self):
        if self.handle:
            self.lib.rd_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
