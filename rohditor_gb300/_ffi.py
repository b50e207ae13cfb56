"""ctypes declarations of include/rd_gpu.h and the library loader.

The library is the product: if `_lib/librd_gpu.so` is missing it is built from
csrc/ with nvcc, and if that fails the import error propagates. There is no
CPU fallback.
"""

from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

F32P = ctypes.POINTER(ctypes.c_float)
U16P = ctypes.POINTER(ctypes.c_uint16)
U8P = ctypes.POINTER(ctypes.c_uint8)
U64P = ctypes.POINTER(ctypes.c_uint64)
VOIDP = ctypes.c_void_p
MAX_LEVEL_PATTERN = 64

CFA = {"RGGB": 0, "BGGR": 1, "GRBG": 2, "GBRG": 3}
HIGHLIGHT = {"off": 0, "clip": 1, "opposed": 2}
DEMOSAIC = {"bilinear": 0, "mhc": 1, "rcd": 2, "amaze": 3}
DISTORTION = {"none": 0, "poly3": 1, "poly5": 2, "ptlens": 3}
TCA = {"none": 0, "linear": 1, "poly3": 2}

STATUS_NAMES = [
    "Ok", "Cancelled", "Unsupported", "OverBudget", "InvalidDimensions", "BaseMismatch",
    "UnsupportedEdits", "Synchronization", "InvalidInput", "Readback",
]


class SensorDesc(ctypes.Structure):
    _fields_ = [
        ("sensor_width", ctypes.c_uint32), ("sensor_height", ctypes.c_uint32),
        ("crop_x", ctypes.c_uint32), ("crop_y", ctypes.c_uint32),
        ("crop_width", ctypes.c_uint32), ("crop_height", ctypes.c_uint32),
        ("cfa", ctypes.c_int32),
        ("black_repeat_w", ctypes.c_uint32), ("black_repeat_h", ctypes.c_uint32),
        ("black", ctypes.c_float * MAX_LEVEL_PATTERN),
        ("white_count", ctypes.c_uint32),
        ("white", ctypes.c_float * MAX_LEVEL_PATTERN),
        ("highlight", ctypes.c_int32),
        ("clip_levels", ctypes.c_float * 3),
        ("detection_levels", ctypes.c_float * 3),
        ("has_neutral_ceiling", ctypes.c_int32),
        ("neutral_ceiling", ctypes.c_float * 3),
        ("demosaic", ctypes.c_int32),
        ("demosaic_balance", ctypes.c_float * 3),
    ]


class DetailDesc(ctypes.Structure):
    _fields_ = [
        ("enabled", ctypes.c_int32), ("amount", ctypes.c_float), ("radius", ctypes.c_float),
        ("noise_protection", ctypes.c_float), ("ceilings", ctypes.c_float * 3), ("iterations", ctypes.c_int32),
    ]


class OpticsDesc(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
        ("norm_scale", ctypes.c_double), ("norm_unscale", ctypes.c_double),
        ("center_x", ctypes.c_double), ("center_y", ctypes.c_double),
        ("scale", ctypes.c_float),
        ("distortion_model", ctypes.c_int32), ("distortion", ctypes.c_float * 3),
        ("tca_model", ctypes.c_int32), ("tca_red", ctypes.c_float * 3), ("tca_blue", ctypes.c_float * 3),
        ("vignetting", ctypes.c_int32), ("vignetting_k", ctypes.c_float * 3),
    ]


class ColorDesc(ctypes.Structure):
    _fields_ = [
        ("wb_gains", ctypes.c_float * 3),
        ("camera_to_rec2020", ctypes.c_float * 9),
        ("exposure_ev", ctypes.c_float),
        ("has_base_lut", ctypes.c_int32), ("base_lut", ctypes.c_float * 4096),
        ("has_light_tone_lut", ctypes.c_int32), ("light_tone_lut", ctypes.c_float * 4096),
        ("has_tone_lut", ctypes.c_int32), ("tone_lut", ctypes.c_float * 4096),
        ("saturation", ctypes.c_float), ("vibrance", ctypes.c_float),
        ("has_hsl", ctypes.c_int32), ("hsl", (ctypes.c_float * 3) * 8),
        ("has_grading", ctypes.c_int32), ("grading", (ctypes.c_float * 3) * 3),
    ]


class Metrics(ctypes.Structure):
    _fields_ = [
        ("normalize_highlight_ms", ctypes.c_float), ("demosaic_ms", ctypes.c_float),
        ("capture_ms", ctypes.c_float), ("optics_ms", ctypes.c_float), ("reduce_ms", ctypes.c_float),
        ("color_ms", ctypes.c_float), ("total_ms", ctypes.c_float),
        ("highlight_stats", ctypes.c_uint64 * 9),
        ("kernel_launches", ctypes.c_uint64), ("device_bytes", ctypes.c_uint64),
    ]


class SynthDesc(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("cfa", ctypes.c_int32),
        ("bits", ctypes.c_uint32), ("black", ctypes.c_float), ("white", ctypes.c_float),
        ("clip_fraction", ctypes.c_float), ("gains", ctypes.c_float * 3), ("seed", ctypes.c_uint64),
        ("highlight_blobs", ctypes.c_int32), ("hot_pixel_fraction", ctypes.c_float),
    ]


class BatchItem(ctypes.Structure):
    _fields_ = [
        ("mosaic", ctypes.POINTER(ctypes.c_uint16)), ("row_stride", ctypes.c_size_t), ("sensor", SensorDesc),
        ("detail", DetailDesc), ("optics", OpticsDesc), ("target_width", ctypes.c_uint32),
        ("target_height", ctypes.c_uint32), ("wb_gains", ctypes.c_float * 3), ("camera_to_rec2020", ctypes.c_float * 9),
        ("color", ColorDesc), ("srgb_out", ctypes.POINTER(ctypes.c_uint8)), ("hist", ctypes.POINTER(ctypes.c_uint64)),
        ("status", ctypes.c_int32), ("ms", ctypes.c_double),
    ]


class ServerResult(ctypes.Structure):
    _fields_ = [
        ("request_id", ctypes.c_uint64), ("image_id", ctypes.c_uint32), ("kind", ctypes.c_int32),
        ("status", ctypes.c_int32), ("batch_size", ctypes.c_uint32), ("revision", ctypes.c_uint64),
        ("queue_ms", ctypes.c_double), ("service_ms", ctypes.c_double), ("latency_ms", ctypes.c_double),
    ]


class ExportFile(ctypes.Structure):
    _fields_ = [
        ("format", ctypes.c_int32), ("quality", ctypes.c_int32),
        ("icc", U8P), ("icc_len", ctypes.c_uint64), ("exif", U8P), ("exif_len", ctypes.c_uint64),
        ("file_bytes", U64P),
    ]


FILE_FORMAT = {"rows": 0, "png": 1, "jpeg": 2}


class ServerStats(ctypes.Structure):
    _fields_ = [(name, ctypes.c_uint64) for name in (
        "requested", "completed", "coalesced", "failed", "redeveloped", "evictions", "batches", "batched_edits",
        "resident_bytes", "peak_resident_bytes", "budget_bytes", "exports")]


class OutputDesc(ctypes.Structure):
    _fields_ = [
        ("format", ctypes.c_int32), ("primaries", ctypes.c_int32), ("policy", ctypes.c_int32),
        ("dither", ctypes.c_int32), ("orientation", ctypes.c_int32), ("has_crop", ctypes.c_int32),
        ("crop", ctypes.c_double * 4), ("headroom", ctypes.c_float),
    ]


OUTPUT_FORMAT = {"srgb8": 0, "srgb16": 1, "extended_f32": 2, "extended_f16": 3}
PRIMARIES = {"srgb": 0, "display_p3": 1}
OUTPUT_POLICY = {"clip": 0, "chroma_compress": 1}
DITHER = {"none": 0, "ordered8x8": 1}
ORIENTATION = {"normal": 0, "horizontal_flip": 1, "rotate180": 2, "vertical_flip": 3, "transpose": 4,
               "rotate90": 5, "transverse": 6, "rotate270": 7, "unknown": 8}
GAMUT_STATUS = ("in_gamut", "compressed", "limited", "clipped_fallback", "invalid")

# Every exported symbol of include/rd_gpu.h with its ctypes signature.
SIGNATURES = {
    "rd_status_is_routing": (ctypes.c_int, [ctypes.c_int]),
    "rd_status_name": (ctypes.c_char_p, [ctypes.c_int]),
    "rd_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(VOIDP)]),
    "rd_ctx_destroy": (None, [VOIDP]),
    "rd_ctx_set_budget": (ctypes.c_int, [VOIDP, ctypes.c_uint64]),
    "rd_ctx_last_error": (ctypes.c_char_p, [VOIDP]),
    "rd_ctx_synchronize": (ctypes.c_int, [VOIDP]),
    "rd_ctx_kernel_launches": (ctypes.c_uint64, [VOIDP]),
    "rd_ctx_set_wait_test": (ctypes.c_int, [VOIDP, ctypes.c_uint32, ctypes.c_int32]),
    "rd_supports": (ctypes.c_int, [ctypes.POINTER(SensorDesc)]),
    "rd_develop": (ctypes.c_int, [VOIDP, U16P, ctypes.c_size_t, ctypes.POINTER(SensorDesc),
                                  ctypes.POINTER(DetailDesc), ctypes.POINTER(ctypes.c_uint32),
                                  ctypes.POINTER(VOIDP), ctypes.POINTER(Metrics)]),
    "rd_develop_device": (ctypes.c_int, [VOIDP, VOIDP, ctypes.c_size_t, ctypes.POINTER(SensorDesc),
                                         ctypes.POINTER(DetailDesc), ctypes.POINTER(ctypes.c_uint32),
                                         ctypes.POINTER(VOIDP), ctypes.POINTER(Metrics)]),
    "rd_spatial": (ctypes.c_int, [VOIDP, VOIDP, ctypes.POINTER(OpticsDesc), ctypes.c_uint32, ctypes.c_uint32,
                                  F32P, F32P, ctypes.POINTER(VOIDP), ctypes.POINTER(Metrics)]),
    "rd_render": (ctypes.c_int, [VOIDP, VOIDP, ctypes.POINTER(ColorDesc), U8P, U64P, U64P,
                                 ctypes.POINTER(Metrics)]),
    "rd_render_device": (ctypes.c_int, [VOIDP, VOIDP, ctypes.POINTER(ColorDesc), ctypes.POINTER(Metrics)]),
    "rd_render_device_noalloc": (ctypes.c_int, [VOIDP, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ColorDesc),
                                                VOIDP, VOIDP, VOIDP]),
    "rd_output_dimensions": (ctypes.c_int, [ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(OutputDesc),
                                            ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32),
                                            ctypes.POINTER(ctypes.c_uint32)]),
    "rd_render_output": (ctypes.c_int, [VOIDP, VOIDP, ctypes.POINTER(ColorDesc), ctypes.POINTER(OutputDesc), VOIDP,
                                        ctypes.c_size_t, U64P, U64P, ctypes.POINTER(Metrics)]),
    "rd_render_output_device": (ctypes.c_int, [VOIDP, VOIDP, ctypes.POINTER(ColorDesc), ctypes.POINTER(OutputDesc),
                                               VOIDP, VOIDP, VOIDP, ctypes.POINTER(Metrics)]),
    "rd_png_bound": (ctypes.c_uint64, [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int32, ctypes.c_uint64,
                                       ctypes.c_uint64]),
    "rd_encode_png": (ctypes.c_int, [VOIDP, VOIDP, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32,
                                     U8P, ctypes.c_uint64, U8P, ctypes.c_uint64, U8P, ctypes.c_uint64, U64P,
                                     ctypes.POINTER(Metrics)]),
    "rd_encode_png_device": (ctypes.c_int, [VOIDP, VOIDP, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64,
                                            ctypes.c_int32, U8P, ctypes.c_uint64, U8P, ctypes.c_uint64, VOIDP,
                                            ctypes.c_uint64, VOIDP]),
    "rd_jpeg_bound": (ctypes.c_uint64, [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64]),
    "rd_encode_jpeg": (ctypes.c_int, [VOIDP, VOIDP, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32,
                                      U8P, ctypes.c_uint64, U8P, ctypes.c_uint64, U8P, ctypes.c_uint64, U64P,
                                      ctypes.POINTER(Metrics)]),
    "rd_encode_jpeg_device": (ctypes.c_int, [VOIDP, VOIDP, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64,
                                             ctypes.c_int32, U8P, ctypes.c_uint64, U8P, ctypes.c_uint64, VOIDP,
                                             ctypes.c_uint64, VOIDP]),
    "rd_check_math": (ctypes.c_int, [VOIDP, ctypes.c_int32, U64P]),
    "rd_rl_launch_shape": (ctypes.c_int, [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float,
                                          ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
                                          ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "rd_launch_shape": (ctypes.c_int, [ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float,
                                       ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
                                       ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "rd_stage_output": (ctypes.c_int, [VOIDP, F32P, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ColorDesc),
                                       ctypes.POINTER(OutputDesc), VOIDP, ctypes.c_size_t, U64P, U64P]),
    "rd_source_dimensions": (ctypes.c_int, [VOIDP, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32)]),
    "rd_source_download": (ctypes.c_int, [VOIDP, VOIDP, F32P]),
    "rd_base_dimensions": (ctypes.c_int, [VOIDP, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32)]),
    "rd_base_download": (ctypes.c_int, [VOIDP, VOIDP, F32P]),
    "rd_source_release": (None, [VOIDP]),
    "rd_base_release": (None, [VOIDP]),
    "rd_stage_highlight": (ctypes.c_int, [VOIDP, U16P, ctypes.c_size_t, ctypes.POINTER(SensorDesc), F32P, U64P]),
    "rd_stage_opposed": (ctypes.c_int, [VOIDP, F32P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int32, F32P, F32P,
                                        F32P, U64P, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32)]),
    "rd_stage_demosaic": (ctypes.c_int, [VOIDP, F32P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int32,
                                         ctypes.c_int32, F32P, F32P]),
    "rd_stage_capture": (ctypes.c_int, [VOIDP, F32P, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(DetailDesc)]),
    "rd_stage_optics": (ctypes.c_int, [VOIDP, ctypes.POINTER(OpticsDesc), F32P, F32P]),
    "rd_stage_area_reduce": (ctypes.c_int, [VOIDP, F32P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                            ctypes.c_uint32, F32P]),
    "rd_stage_color": (ctypes.c_int, [VOIDP, F32P, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ColorDesc),
                                      U8P, U64P, U64P]),
    "rd_optics_radial_table": (ctypes.c_int, [ctypes.POINTER(OpticsDesc), F32P, F32P, ctypes.POINTER(ctypes.c_int32)]),
    "rd_optics_plan": (ctypes.c_int, [ctypes.POINTER(OpticsDesc), ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_float]),
    "rd_standard_base_lut": (None, [F32P]),
    "rd_light_tone_lut": (None, [ctypes.c_float] * 5 + [F32P]),
    "rd_synth_mosaic_device": (ctypes.c_int, [VOIDP, ctypes.POINTER(SynthDesc), VOIDP]),
    "rd_develop_batch": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(BatchItem), ctypes.c_int32, ctypes.c_int32,
                                        ctypes.POINTER(ctypes.c_double)]),
    "rd_develop_batch_graph": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(BatchItem), ctypes.c_int32, ctypes.c_int32,
                                              ctypes.c_int32, ctypes.POINTER(ctypes.c_double),
                                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "rd_develop_batch_flat": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(BatchItem), ctypes.c_int32, ctypes.c_int32,
                                             ctypes.POINTER(ctypes.c_double)]),
    "rd_develop_batch_flat_graph": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(BatchItem), ctypes.c_int32,
                                                   ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_double),
                                                   ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "rd_server_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(VOIDP)]),
    "rd_server_set_dry_timing": (ctypes.c_int, [VOIDP, ctypes.c_uint32, ctypes.c_uint32]),
    "rd_server_destroy": (None, [VOIDP]),
    "rd_server_open": (ctypes.c_int, [VOIDP, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint16), ctypes.c_size_t,
                                      ctypes.POINTER(SensorDesc), ctypes.POINTER(DetailDesc),
                                      ctypes.POINTER(OpticsDesc), ctypes.c_uint32, ctypes.c_uint32, F32P, F32P, U64P]),
    "rd_server_close_image": (ctypes.c_int, [VOIDP, ctypes.c_uint32]),
    "rd_server_submit_edit": (ctypes.c_int, [VOIDP, ctypes.c_uint32, ctypes.c_uint64, ctypes.POINTER(ColorDesc), U64P]),
    "rd_server_submit_develop": (ctypes.c_int, [VOIDP, ctypes.c_uint32, ctypes.c_uint64, ctypes.POINTER(DetailDesc),
                                                ctypes.POINTER(OpticsDesc), U64P]),
    "rd_server_submit_export": (ctypes.c_int, [VOIDP, ctypes.c_uint32, ctypes.c_uint64, ctypes.POINTER(ColorDesc),
                                               ctypes.POINTER(OutputDesc), ctypes.c_int32, ctypes.POINTER(VOIDP),
                                               ctypes.POINTER(ctypes.c_size_t), U64P]),
    "rd_server_submit_export_files": (ctypes.c_int, [VOIDP, ctypes.c_uint32, ctypes.c_uint64,
                                                     ctypes.POINTER(ColorDesc), ctypes.POINTER(OutputDesc),
                                                     ctypes.POINTER(ExportFile), ctypes.c_int32,
                                                     ctypes.POINTER(VOIDP), ctypes.POINTER(ctypes.c_size_t), U64P]),
    "rd_server_poll": (ctypes.c_int32, [VOIDP, ctypes.POINTER(ServerResult), ctypes.c_int32, ctypes.c_int32]),
    "rd_server_read_output": (ctypes.c_int, [VOIDP, ctypes.c_uint32, U8P, U64P, U64P]),
    "rd_server_get_stats": (ctypes.c_int, [VOIDP, ctypes.POINTER(ServerStats)]),
    "rd_server_drain": (ctypes.c_int, [VOIDP, ctypes.c_int32]),
    "rd_synth_mosaic": (ctypes.c_int, [VOIDP, ctypes.POINTER(SynthDesc), U16P]),
    "rd_ctx_event_record": (ctypes.c_int, [VOIDP, ctypes.c_int]),
    "rd_ctx_event_elapsed": (ctypes.c_int, [VOIDP, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]),
    "rd_ctx_flush_l2": (ctypes.c_int, [VOIDP]),
    "rd_ctx_enable_kernel_timing": (ctypes.c_int, [VOIDP, ctypes.c_int]),
    "rd_ctx_kernel_timing": (ctypes.c_int, [VOIDP, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                            ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint64)]),
    "rd_ctx_reset_kernel_timing": (ctypes.c_int, [VOIDP]),
    "rd_host_alloc": (ctypes.c_int, [ctypes.c_size_t, ctypes.POINTER(VOIDP)]),
    "rd_host_free": (None, [VOIDP]),
    "rd_device_alloc": (ctypes.c_int, [VOIDP, ctypes.c_size_t, ctypes.POINTER(VOIDP)]),
    "rd_device_free": (ctypes.c_int, [VOIDP, VOIDP]),
    "rd_copy_to_device": (ctypes.c_int, [VOIDP, VOIDP, VOIDP, ctypes.c_size_t]),
    "rd_copy_to_host": (ctypes.c_int, [VOIDP, VOIDP, VOIDP, ctypes.c_size_t]),
}

_lock = threading.Lock()
_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load librd_gpu.so (building it first when missing) and declare every symbol."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise OSError(f"{path} is missing; run rohditor_gb300.build.build()")
            _build.build()
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)  # AttributeError: the library lacks a declared symbol
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib
