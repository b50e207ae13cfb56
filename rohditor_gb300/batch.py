"""Batched develop of many mosaics (include/rd_gpu.h rd_develop_batch,
rd_develop_batch_graph).

Each image goes through the whole path (develop, spatial pass, render) with
host buffers. With `graph=False`, `lanes` contexts on their own streams work
through a shared queue concurrently so their kernels overlap on the GPU. With
`graph=True` the whole batch is captured into one CUDA graph of `lanes`
parallel branches and runs as a single launch. With `flat=True` the batch
runs stage by stage, with one AMaZE launch over the tiles of every image and
one launch per RL iteration over the batch; `flat=True` with `graph=True`
captures that stage-by-stage batch into one CUDA graph.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _ffi
from .processor import (CaptureContract, ColorContract, GpuPreviewError, OpticsExecution, SensorDescription, _f32,
                        _ptr)


@dataclass
class BatchImage:
    mosaic: np.ndarray
    sensor: SensorDescription
    capture: CaptureContract
    optics: OpticsExecution
    target: tuple[int, int]
    wb_gains: tuple
    camera_to_rec2020: tuple
    color: ColorContract


def _fill_item(it, im: BatchImage):
    it.sensor = im.sensor.to_c()
    it.detail = im.capture.to_c()
    it.optics = im.optics.to_c()
    it.target_width, it.target_height = im.target
    for c in range(3):
        it.wb_gains[c] = im.wb_gains[c]
    for c in range(9):
        it.camera_to_rec2020[c] = im.camera_to_rec2020[c]
    it.color = im.color.to_c()


class PinnedBatch:
    """A batch whose mosaics and outputs live in pinned host memory
    (rd_host_alloc), as a pipeline that decodes into pinned buffers holds them;
    the buffers are reused by every run, with lanes or as one graph."""

    def __init__(self, images: list[BatchImage], device: int = 0):
        self.lib = _ffi.load()
        self.device = device
        self.items = (_ffi.BatchItem * len(images))()
        self.buffers = []
        self.outs = []
        for k, im in enumerate(images):
            mosaic = np.ascontiguousarray(im.mosaic, dtype=np.uint16)
            sizes = (mosaic.nbytes, 3 * im.target[0] * im.target[1], 1024 * 8)
            ptrs = []
            for n in sizes:
                p = ctypes.c_void_p()
                rc = self.lib.rd_host_alloc(n, ctypes.byref(p))
                if rc != 0:
                    raise GpuPreviewError(rc, "pinned allocation failed")
                ptrs.append(p.value)
                self.buffers.append(p.value)
            ctypes.memmove(ptrs[0], mosaic.ctypes.data, mosaic.nbytes)
            it = self.items[k]
            it.mosaic = ctypes.cast(ptrs[0], ctypes.POINTER(ctypes.c_uint16))
            it.row_stride = mosaic.shape[1]
            _fill_item(it, im)
            it.srgb_out = ctypes.cast(ptrs[1], ctypes.POINTER(ctypes.c_uint8))
            it.hist = ctypes.cast(ptrs[2], ctypes.POINTER(ctypes.c_uint64))
            self.outs.append((ptrs[1], ptrs[2], im.target))

    def run(self, lanes: int = 3, graph: bool = False, flat: bool = False) -> dict:
        """Times of one run: wall_ms, and for a graph capture_ms and launch_ms."""
        wall, cap, launch = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        n = len(self.items)
        if flat and graph:
            rc = self.lib.rd_develop_batch_flat_graph(self.device, self.items, n, lanes, 1, ctypes.byref(wall),
                                                      ctypes.byref(cap), ctypes.byref(launch))
        elif flat:
            rc = self.lib.rd_develop_batch_flat(self.device, self.items, n, lanes, ctypes.byref(wall))
        elif graph:
            rc = self.lib.rd_develop_batch_graph(self.device, self.items, n, lanes, 1, ctypes.byref(wall),
                                                 ctypes.byref(cap), ctypes.byref(launch))
        else:
            rc = self.lib.rd_develop_batch(self.device, self.items, n, lanes, ctypes.byref(wall))
        if rc != 0:
            raise GpuPreviewError(rc, f"batched develop failed: {self.lib.rd_status_name(rc).decode()}")
        out = {"wall_ms": wall.value}
        if graph:
            out.update(capture_ms=cap.value, launch_ms=launch.value)
        return out

    def outputs(self) -> list[tuple[np.ndarray, np.ndarray]]:
        res = []
        for srgb_p, hist_p, (tw, th) in self.outs:
            srgb = np.empty((th, 3 * tw), dtype=np.uint8)
            hist = np.empty(1024, dtype=np.uint64)
            ctypes.memmove(srgb.ctypes.data, srgb_p, srgb.nbytes)
            ctypes.memmove(hist.ctypes.data, hist_p, hist.nbytes)
            res.append((srgb, hist))
        return res

    def close(self):
        for p in self.buffers:
            self.lib.rd_host_free(ctypes.c_void_p(p))
        self.buffers = []


def develop_batch(images: list[BatchImage], lanes: int = 3, device: int = 0, graph: bool = False,
                  flat: bool = False):
    """Returns (outputs [(srgb8, hist)], per-image ms, wall ms); with `graph`,
    the per-image ms are 0 and the capture + instantiation ms is the last
    element of the returned tuple. With `flat` the batch runs stage by stage
    with one AMaZE launch over every image's tiles and one launch per RL
    iteration over the batch (rd_develop_batch_flat; with `graph` too, the
    same captured into one CUDA graph, rd_develop_batch_flat_graph)."""
    lib = _ffi.load()
    items = (_ffi.BatchItem * len(images))()
    keep = []
    outs = []
    for k, im in enumerate(images):
        mosaic = np.ascontiguousarray(im.mosaic, dtype=np.uint16)
        srgb = np.empty((im.target[1], 3 * im.target[0]), dtype=np.uint8)
        hist = np.zeros(1024, dtype=np.uint64)
        keep.append(mosaic)
        outs.append((srgb, hist))
        it = items[k]
        it.mosaic = _ptr(mosaic, ctypes.c_uint16)
        it.row_stride = mosaic.shape[1]
        _fill_item(it, im)
        it.srgb_out = _ptr(srgb, ctypes.c_uint8)
        it.hist = _ptr(hist, ctypes.c_uint64)
    wall = ctypes.c_double()
    if graph:
        capture = ctypes.c_double()
        run = lib.rd_develop_batch_flat_graph if flat else lib.rd_develop_batch_graph
        rc = run(device, items, len(images), lanes, 0, ctypes.byref(wall), ctypes.byref(capture), None)
        if rc != 0:
            raise GpuPreviewError(rc, f"batched graph develop failed: {lib.rd_status_name(rc).decode()}")
        return outs, [0.0] * len(images), wall.value, capture.value
    if flat:
        rc = lib.rd_develop_batch_flat(device, items, len(images), lanes, ctypes.byref(wall))
    else:
        rc = lib.rd_develop_batch(device, items, len(images), lanes, ctypes.byref(wall))
    if rc != 0:
        raise GpuPreviewError(rc, f"batched develop failed: {lib.rd_status_name(rc).decode()}")
    return outs, [items[k].ms for k in range(len(images))], wall.value
