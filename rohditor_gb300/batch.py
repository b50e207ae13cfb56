"""Batched develop of many mosaics (include/rd_gpu.h rd_develop_batch).

Each image goes through the whole path (develop, spatial pass, render) with
host buffers; `lanes` contexts on their own streams work through the queue
concurrently so their kernels overlap on the GPU.
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


def develop_batch(images: list[BatchImage], lanes: int = 3, device: int = 0):
    """Returns (outputs [(srgb8, hist)], per-image ms, wall ms)."""
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
        it.sensor = im.sensor.to_c()
        it.detail = im.capture.to_c()
        it.optics = im.optics.to_c()
        it.target_width, it.target_height = im.target
        for c in range(3):
            it.wb_gains[c] = im.wb_gains[c]
        for c in range(9):
            it.camera_to_rec2020[c] = im.camera_to_rec2020[c]
        it.color = im.color.to_c()
        it.srgb_out = _ptr(srgb, ctypes.c_uint8)
        it.hist = _ptr(hist, ctypes.c_uint64)
    wall = ctypes.c_double()
    rc = lib.rd_develop_batch(device, items, len(images), lanes, ctypes.byref(wall))
    if rc != 0:
        raise GpuPreviewError(rc, f"batched develop failed: {lib.rd_status_name(rc).decode()}")
    return outs, [items[k].ms for k in range(len(images))], wall.value
