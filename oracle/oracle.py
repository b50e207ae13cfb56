"""ctypes loader for the CPU oracle (test infrastructure).

Only the test-suite, the smoke check and the bench's CPU-baseline leg import
this module; the product library never does. `load()` builds the shared
library with the Makefile beside this file when it is missing or stale.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "librd_oracle.so")
_lock = threading.Lock()
_lib = None

F32P = ctypes.POINTER(ctypes.c_float)
U16P = ctypes.POINTER(ctypes.c_uint16)
U8P = ctypes.POINTER(ctypes.c_uint8)
U32P = ctypes.POINTER(ctypes.c_uint32)
U64P = ctypes.POINTER(ctypes.c_uint64)


def build() -> str:
    """Compile the oracle (make is incremental) and return the library path."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _stale() -> bool:
    if not os.path.exists(_LIB_PATH):
        return True
    built = os.path.getmtime(_LIB_PATH)
    for name in os.listdir(_HERE):
        if name.endswith((".cpp", ".h")) and os.path.getmtime(os.path.join(_HERE, name)) > built:
            return True
    return False


class SensorDesc(ctypes.Structure):
    _fields_ = [
        ("sensor_w", ctypes.c_int), ("sensor_h", ctypes.c_int), ("row_stride", ctypes.c_int),
        ("crop_x", ctypes.c_int), ("crop_y", ctypes.c_int), ("crop_w", ctypes.c_int), ("crop_h", ctypes.c_int),
        ("pattern", ctypes.c_int), ("black_w", ctypes.c_int), ("black_h", ctypes.c_int),
        ("black", F32P), ("white_count", ctypes.c_int), ("white", F32P),
    ]


class OpticsDesc(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int), ("height", ctypes.c_int),
        ("norm_scale", ctypes.c_double), ("norm_unscale", ctypes.c_double),
        ("center_x", ctypes.c_double), ("center_y", ctypes.c_double),
        ("scale", ctypes.c_float),
        ("distortion_model", ctypes.c_int), ("distortion", ctypes.c_float * 3),
        ("tca_model", ctypes.c_int), ("tca_red", ctypes.c_float * 3), ("tca_blue", ctypes.c_float * 3),
        ("vignetting_model", ctypes.c_int), ("vignetting", ctypes.c_float * 3),
    ]


class AdjustDesc(ctypes.Structure):
    _fields_ = [
        ("exposure_ev", ctypes.c_float), ("base_lut", F32P), ("tone_lut", F32P),
        ("saturation", ctypes.c_float), ("vibrance", ctypes.c_float),
        ("has_hsl", ctypes.c_int), ("hsl", (ctypes.c_float * 3) * 8),
        ("has_grading", ctypes.c_int), ("grading", (ctypes.c_float * 3) * 3),
    ]


def load():
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if _stale():
            build()
        lib = ctypes.CDLL(_LIB_PATH)
        sig = {
            "ro_fixture_amaze_golden": (None, [ctypes.c_int, ctypes.c_int, F32P]),
            "ro_fixture_amaze_probe": (None, [F32P]),
            "ro_fnv1a_f32": (ctypes.c_uint64, [F32P, ctypes.c_size_t]),
            "ro_demosaic": (ctypes.c_int, [F32P, ctypes.c_int, ctypes.c_int, ctypes.c_int, F32P, ctypes.c_int, F32P]),
            "ro_amaze_probe_tile": (ctypes.c_int, [F32P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                   ctypes.c_float, ctypes.c_char_p, F32P]),
        }
        optional = {
            "ro_normalize": (ctypes.c_int, [U16P, ctypes.POINTER(SensorDesc), F32P]),
            "ro_clip": (ctypes.c_int, [F32P, ctypes.c_int, ctypes.c_int, ctypes.c_int, F32P, U64P]),
            "ro_opposed": (ctypes.c_int, [F32P, ctypes.c_int, ctypes.c_int, ctypes.c_int, F32P, F32P, U64P,
                                          U32P, U32P]),
            "ro_label_components": (ctypes.c_uint32, [U32P, ctypes.c_int, ctypes.c_int]),
            "ro_gaussian_kernel": (ctypes.c_int, [ctypes.c_float, F32P, ctypes.c_int]),
            "ro_capture_sharpen": (ctypes.c_int, [F32P, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                                  ctypes.c_float, F32P, ctypes.c_int]),
            "ro_optics_plan": (ctypes.c_int, [ctypes.POINTER(OpticsDesc), ctypes.c_float, ctypes.c_float,
                                              ctypes.c_float, ctypes.c_float]),
            "ro_optics_apply": (ctypes.c_int, [ctypes.POINTER(OpticsDesc), F32P, F32P]),
            "ro_optics_map": (ctypes.c_int, [ctypes.POINTER(OpticsDesc), ctypes.c_int, ctypes.c_int, F32P]),
            "ro_area_reduce": (ctypes.c_int, [F32P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, F32P]),
            "ro_white_balance": (None, [F32P, ctypes.c_size_t, F32P]),
            "ro_camera_matrix": (None, [F32P, ctypes.c_size_t, F32P]),
            "ro_adjust_apply": (None, [F32P, ctypes.c_size_t, ctypes.POINTER(AdjustDesc)]),
            "ro_standard_base_lut": (None, [F32P]),
            "ro_display_srgb8": (None, [F32P, ctypes.c_size_t, U8P]),
            "ro_histogram": (None, [U8P, ctypes.c_size_t, U64P, U64P]),
        }
        for name, (res, args) in list(sig.items()) + list(optional.items()):
            if not hasattr(lib, name):
                if name in sig:
                    raise RuntimeError(f"oracle symbol {name} missing")
                continue
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def ptr(array: np.ndarray, ctype=ctypes.c_float):
    assert array.flags["C_CONTIGUOUS"]
    return array.ctypes.data_as(ctypes.POINTER(ctype))


def f32(array: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(array, dtype=np.float32)


def demosaic(mosaic: np.ndarray, pattern: int, balance, algorithm: int) -> np.ndarray:
    lib = load()
    mosaic = f32(mosaic)
    h, w = mosaic.shape
    out = np.zeros((h, 3 * w), dtype=np.float32)
    bal = f32(np.asarray(balance))
    rc = lib.ro_demosaic(ptr(mosaic), w, h, pattern, ptr(bal), algorithm, ptr(out))
    if rc != 0:
        raise RuntimeError(f"oracle demosaic failed: {rc}")
    return out


def fnv1a(values: np.ndarray) -> int:
    values = f32(values).reshape(-1)
    return int(load().ro_fnv1a_f32(ptr(values), values.size))


def amaze_golden_fixture(width: int = 513, height: int = 389) -> np.ndarray:
    out = np.zeros((height, width), dtype=np.float32)
    load().ro_fixture_amaze_golden(width, height, ptr(out))
    return out


def amaze_probe_fixture() -> np.ndarray:
    out = np.zeros((47, 53), dtype=np.float32)
    load().ro_fixture_amaze_probe(ptr(out))
    return out


def amaze_probe_plane(mosaic: np.ndarray, pattern: int, clip_point: float, plane: str) -> np.ndarray:
    mosaic = f32(mosaic)
    h, w = mosaic.shape
    out = np.zeros(256 * 256, dtype=np.float32)
    rc = load().ro_amaze_probe_tile(ptr(mosaic), w, h, w, pattern, clip_point, plane.encode(), ptr(out))
    if rc != 0:
        raise KeyError(plane)
    full = {"cfa", "green", "delhvsqsum", "dirwts0", "dirwts1", "vcd", "hcd", "vcdalt", "hcdalt", "cddiffsq",
            "dgintv", "dginth"}
    return out.reshape(256, 256) if plane in full else out[: 256 * 128].reshape(256, 128)


os.environ.setdefault("OMP_WAIT_POLICY", "PASSIVE")
