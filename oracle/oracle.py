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


class SynthDesc(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("cfa", ctypes.c_int32), ("bits", ctypes.c_uint32),
        ("black", ctypes.c_float), ("white", ctypes.c_float), ("clip_fraction", ctypes.c_float),
        ("gains", ctypes.c_float * 3), ("seed", ctypes.c_uint64), ("highlight_blobs", ctypes.c_int32),
        ("hot_pixel_fraction", ctypes.c_float),
    ]


class AdjustDesc(ctypes.Structure):
    _fields_ = [
        ("exposure_ev", ctypes.c_float), ("base_lut", F32P), ("light_lut", F32P), ("extended", ctypes.c_int),
        ("tone_lut", F32P),
        ("saturation", ctypes.c_float), ("vibrance", ctypes.c_float),
        ("has_hsl", ctypes.c_int), ("hsl", (ctypes.c_float * 3) * 8),
        ("has_grading", ctypes.c_int), ("grading", (ctypes.c_float * 3) * 3),
    ]


class OutputDesc(ctypes.Structure):
    _fields_ = [
        ("format", ctypes.c_int), ("primaries", ctypes.c_int), ("policy", ctypes.c_int), ("dither", ctypes.c_int),
        ("orientation", ctypes.c_int), ("has_crop", ctypes.c_int), ("crop", ctypes.c_double * 4),
        ("headroom", ctypes.c_float),
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
            "ro_optics_radial": (ctypes.c_int, [ctypes.POINTER(OpticsDesc), F32P, F32P, ctypes.POINTER(ctypes.c_int),
                                                F32P, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
            "ro_optics_map_lut": (ctypes.c_int, [ctypes.POINTER(OpticsDesc), ctypes.c_int, ctypes.c_int, F32P]),
            "ro_area_reduce": (ctypes.c_int, [F32P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, F32P]),
            "ro_white_balance": (None, [F32P, ctypes.c_size_t, F32P]),
            "ro_camera_matrix": (None, [F32P, ctypes.c_size_t, F32P]),
            "ro_adjust_apply": (None, [F32P, ctypes.c_size_t, ctypes.POINTER(AdjustDesc)]),
            "ro_standard_base_lut": (None, [F32P]),
            "ro_light_tone_lut": (None, [ctypes.c_float] * 5 + [F32P]),
            "ro_synth_mosaic": (ctypes.c_int, [ctypes.POINTER(SynthDesc), U16P]),
            "ro_display_srgb8": (None, [F32P, ctypes.c_size_t, U8P]),
            "ro_histogram": (None, [U8P, ctypes.c_size_t, U64P, U64P]),
            "ro_set_exact_math": (None, [ctypes.c_int]),
            "ro_cbrt": (ctypes.c_float, [ctypes.c_float]),
            "ro_cbrt_correctly_rounded": (ctypes.c_float, [ctypes.c_float]),
            "ro_output_geometry": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(OutputDesc),
                                                  ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                                  ctypes.POINTER(ctypes.c_int)]),
            "ro_source_coordinate": (None, [ctypes.c_int] * 5 + [ctypes.POINTER(ctypes.c_int)] * 2),
            "ro_gamut_map": (ctypes.c_int, [F32P, ctypes.c_int, ctypes.c_int, ctypes.c_float, F32P]),
            "ro_oklab": (None, [ctypes.c_int, F32P, F32P]),
            "ro_oklab_inverse": (None, [ctypes.c_int, F32P, F32P]),
            "ro_render_output": (ctypes.c_int, [F32P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(OutputDesc),
                                                ctypes.c_void_p, U64P]),
            "ro_png_filter": (None, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, U8P]),
            "ro_jpeg_coefficients": (None, [U8P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.POINTER(ctypes.c_int16)]),
            "ro_jpeg_decode": (ctypes.c_int, [U8P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_int),
                                              ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), U8P,
                                              ctypes.POINTER(ctypes.c_int16), ctypes.c_size_t]),
            "ro_png_unfilter": (ctypes.c_int, [U8P, ctypes.c_int, ctypes.c_int, ctypes.c_int, U8P]),
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


_flops_lib = None
FLOP_CLASSES = ("add_sub", "mul", "div", "compare", "abs", "min_max")


def load_flops():
    """The operation-counting AMaZE build (oracle/flops/amaze_flops.cpp)."""
    global _flops_lib
    with _lock:
        if _flops_lib is None:
            path = os.path.join(_HERE, "_build", "librd_oracle_flops.so")
            if _stale() or not os.path.exists(path):
                build()
            lib = ctypes.CDLL(path)
            lib.ro_amaze_reconstruct.restype = ctypes.c_int
            lib.ro_amaze_reconstruct.argtypes = [F32P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, F32P,
                                                 ctypes.c_float, F32P, ctypes.c_int]
            lib.ro_flops_reset.restype = None
            lib.ro_flops_read.argtypes = [U64P]
            lib.ro_flops_read.restype = None
            _flops_lib = lib
        return _flops_lib


def amaze_counted(mosaic: np.ndarray, pattern: int, balance) -> tuple[np.ndarray, dict]:
    """AMaZE as ro_demosaic runs it (channel balance first), with its operation counts."""
    lib = load_flops()
    mosaic = f32(mosaic)
    h, w = mosaic.shape
    bal = np.asarray(balance, dtype=np.float32)
    fwd = bal / bal.max()
    gains = np.ones(3, dtype=np.float32)
    clip_point = np.float32(1.0)
    src = mosaic
    if not np.all(fwd == 1.0):
        ch = np.zeros((h, w), dtype=np.int64)
        for y in range(2):
            for x in range(2):
                ch[y::2, x::2] = _CFA_TABLE[pattern][(y << 1) | x]
        src = (mosaic * fwd[ch]).astype(np.float32)
        gains = (np.float32(1.0) / fwd).astype(np.float32)
        clip_point = np.float32(fwd.min())
    src = np.ascontiguousarray(src)
    out = np.zeros((h, 3 * w), dtype=np.float32)
    lib.ro_flops_reset()
    rc = lib.ro_amaze_reconstruct(ptr(src), w, h, w, pattern, ptr(gains), float(clip_point), ptr(out), 3 * w)
    if rc != 0:
        raise RuntimeError(f"counted AMaZE failed: {rc}")
    ops = np.zeros(6, dtype=np.uint64)
    lib.ro_flops_read(ptr(ops, ctypes.c_uint64))
    return out, dict(zip(FLOP_CLASSES, (int(v) for v in ops)))


# color_at (crates/image/src/lib.rs:88-116): channel of (x & 1, y & 1) per CFA code.
_CFA_TABLE = ((0, 1, 1, 2), (2, 1, 1, 0), (1, 0, 2, 1), (1, 2, 0, 1))


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


# ---------------------------------------------------------------- stage wrappers
def sensor_desc(sensor_w, sensor_h, row_stride, crop, pattern, black, black_repeat, white):
    """Build the oracle's sensor struct; keeps the level arrays alive on the struct."""
    d = SensorDesc()
    d.sensor_w, d.sensor_h, d.row_stride = sensor_w, sensor_h, row_stride
    d.crop_x, d.crop_y, d.crop_w, d.crop_h = crop
    d.pattern = pattern
    d.black_w, d.black_h = black_repeat
    d._black = f32(np.asarray(black))
    d._white = f32(np.asarray(white))
    d.black = ptr(d._black)
    d.white_count = d._white.size
    d.white = ptr(d._white)
    return d


def normalize(mosaic_u16: np.ndarray, desc: SensorDesc) -> tuple[np.ndarray, int]:
    mosaic_u16 = np.ascontiguousarray(mosaic_u16, dtype=np.uint16)
    out = np.zeros((desc.crop_h, desc.crop_w), dtype=np.float32)
    pattern = load().ro_normalize(ptr(mosaic_u16, ctypes.c_uint16), ctypes.byref(desc), ptr(out))
    return out, pattern


def clip(mosaic: np.ndarray, pattern: int, levels) -> tuple[np.ndarray, np.ndarray]:
    m = f32(mosaic).copy()
    h, w = m.shape
    stats = np.zeros(6, dtype=np.uint64)
    lv = f32(np.asarray(levels))
    if load().ro_clip(ptr(m), w, h, pattern, ptr(lv), ptr(stats, ctypes.c_uint64)) != 0:
        raise ValueError("non-finite sample")
    return m, stats


def opposed(mosaic: np.ndarray, pattern: int, levels, ceiling=None):
    m = f32(mosaic).copy()
    h, w = m.shape
    stats = np.zeros(9, dtype=np.uint64)
    lv = f32(np.asarray(levels))
    ce = f32(np.asarray(ceiling)) if ceiling is not None else None
    labels = np.zeros(((h + 1) // 2, (w + 1) // 2), dtype=np.uint32)
    count = ctypes.c_uint32()
    rc = load().ro_opposed(ptr(m), w, h, pattern, ptr(lv), ptr(ce) if ce is not None else None,
                           ptr(stats, ctypes.c_uint64), ptr(labels, ctypes.c_uint32), ctypes.byref(count))
    if rc == -2:
        raise ValueError("invalid level: levels must be finite and positive")
    if rc != 0:
        raise ValueError("non-finite sample")
    return m, stats, labels, count.value


def label_components(grid: np.ndarray) -> tuple[np.ndarray, int]:
    g = np.ascontiguousarray(grid, dtype=np.uint32).copy()
    h, w = g.shape
    count = load().ro_label_components(ptr(g, ctypes.c_uint32), w, h)
    return g, int(count)


def capture(rgb: np.ndarray, amount, radius, noise, ceilings, iterations) -> np.ndarray:
    out = f32(rgb).copy()
    h, w3 = out.shape
    ce = f32(np.asarray(ceilings))
    if load().ro_capture_sharpen(ptr(out), w3 // 3, h, amount, radius, noise, ptr(ce), iterations) != 0:
        raise ValueError("capture failed")
    return out


def optics_desc_from(c) -> OpticsDesc:
    """Copy a product optics descriptor (same field meaning) into the oracle struct."""
    d = OpticsDesc()
    d.width, d.height = c.width, c.height
    d.norm_scale, d.norm_unscale, d.center_x, d.center_y = c.norm_scale, c.norm_unscale, c.center_x, c.center_y
    d.scale = c.scale
    d.distortion_model = c.distortion_model
    d.tca_model = c.tca_model
    d.vignetting_model = c.vignetting
    for k in range(3):
        d.distortion[k] = c.distortion[k]
        d.tca_red[k] = c.tca_red[k]
        d.tca_blue[k] = c.tca_blue[k]
        d.vignetting[k] = c.vignetting_k[k]
    return d


def optics_plan(width, height, distortion_model, distortion, tca_model, tca_red, tca_blue, crop=1.0,
                focal=35.0, center=(0.0, 0.0)) -> OpticsDesc:
    d = OpticsDesc()
    d.width, d.height = width, height
    d.distortion_model, d.tca_model = distortion_model, tca_model
    for k in range(3):
        d.distortion[k] = distortion[k]
        d.tca_red[k] = tca_red[k]
        d.tca_blue[k] = tca_blue[k]
    if load().ro_optics_plan(ctypes.byref(d), crop, focal, center[0], center[1]) != 0:
        raise ValueError("no safe scale")
    return d


RADIAL_GUARDS = {-1: "no table", 0: "accepted", 1: "non-finite", 2: "tripwire", 3: "break collision",
                 4: "freeze ambiguity", 5: "unexplained jump"}


def optics_radial(desc: OpticsDesc):
    """RadialMultipliers::build: (guard name, step, table [1024, 3], pinned segments [(index, radius)])."""
    table = np.zeros((1024, 3), dtype=np.float32)
    step = np.zeros(1, dtype=np.float32)
    idx = (ctypes.c_int * 64)()
    rad = np.zeros(64, dtype=np.float32)
    n = ctypes.c_int(0)
    g = load().ro_optics_radial(ctypes.byref(desc), ptr(table), ptr(step), idx, ptr(rad), 64, ctypes.byref(n))
    segs = [(idx[i], float(rad[i])) for i in range(min(n.value, 64))]
    return RADIAL_GUARDS[g], float(step[0]), table, segs


def optics_map_lut(desc: OpticsDesc, x: int, y: int) -> np.ndarray:
    """The table branch's six source coordinates at output pixel (x, y)."""
    out = np.zeros(6, dtype=np.float32)
    if load().ro_optics_map_lut(ctypes.byref(desc), x, y, ptr(out)) != 0:
        raise ValueError("no radial table")
    return out


def optics_apply(desc: OpticsDesc, rgb: np.ndarray) -> np.ndarray:
    rgb = f32(rgb)
    out = np.zeros_like(rgb)
    rc = load().ro_optics_apply(ctypes.byref(desc), ptr(rgb), ptr(out))
    if rc != 0:
        raise ValueError(f"optics failed: {rc}")
    return out


def area_reduce(rgb: np.ndarray, target) -> np.ndarray:
    rgb = f32(rgb)
    h, w3 = rgb.shape
    out = np.zeros((target[1], 3 * target[0]), dtype=np.float32)
    if load().ro_area_reduce(ptr(rgb), w3 // 3, h, target[0], target[1], ptr(out)) != 0:
        raise ValueError("bad reduction")
    return out


def white_balance(rgb: np.ndarray, gains) -> np.ndarray:
    out = f32(rgb).copy()
    g = f32(np.asarray(gains))
    load().ro_white_balance(ptr(out), out.size // 3, ptr(g))
    return out


def camera_matrix(rgb: np.ndarray, m) -> np.ndarray:
    out = f32(rgb).copy()
    mm = f32(np.asarray(m)).reshape(-1)
    load().ro_camera_matrix(ptr(out), out.size // 3, ptr(mm))
    return out


def adjust(rgb: np.ndarray, exposure_ev=0.0, base_lut=None, tone_lut=None, saturation=1.0, vibrance=0.0,
           hsl=None, grading=None, light_lut=None, extended=False) -> np.ndarray:
    out = f32(rgb).copy()
    a = AdjustDesc()
    a.exposure_ev = exposure_ev
    a.extended = 1 if extended else 0
    keep = []
    if base_lut is not None:
        b = f32(base_lut)
        keep.append(b)
        a.base_lut = ptr(b)
    if light_lut is not None:
        lt = f32(light_lut)
        keep.append(lt)
        a.light_lut = ptr(lt)
    if tone_lut is not None:
        t = f32(tone_lut)
        keep.append(t)
        a.tone_lut = ptr(t)
    a.saturation, a.vibrance = saturation, vibrance
    if hsl is not None:
        a.has_hsl = 1
        ctypes.memmove(a.hsl, f32(hsl).ctypes.data, 24 * 4)
    if grading is not None:
        a.has_grading = 1
        ctypes.memmove(a.grading, f32(grading).ctypes.data, 9 * 4)
    load().ro_adjust_apply(ptr(out), out.size // 3, ctypes.byref(a))
    return out


def standard_base_lut() -> np.ndarray:
    out = np.zeros(4096, dtype=np.float32)
    load().ro_standard_base_lut(ptr(out))
    return out


def synth_mosaic(width, height, cfa=0, bits=14, black=512.0, white=16383.0, clip_fraction=0.05,
                 gains=(0.5, 1.0, 0.625), seed=2, highlight_blobs=True, hot_pixel_fraction=0.0) -> np.ndarray:
    """The seeded synthetic Bayer mosaic [height][width] u16 (synth.cpp), equal bit for bit to the
    library's device generator for the same description."""
    d = SynthDesc()
    d.width, d.height, d.cfa, d.bits = width, height, cfa, bits
    d.black, d.white, d.clip_fraction = black, white, clip_fraction
    for c in range(3):
        d.gains[c] = gains[c]
    d.seed = seed
    d.highlight_blobs = 1 if highlight_blobs else 0
    d.hot_pixel_fraction = hot_pixel_fraction
    out = np.empty((height, width), dtype=np.uint16)
    if load().ro_synth_mosaic(ctypes.byref(d), out.ctypes.data_as(U16P)) != 0:
        raise ValueError("synthetic mosaic must be at least 2x2")
    return out


def light_tone_lut(contrast=0.0, highlights=0.0, shadows=0.0, whites=0.0, blacks=0.0) -> np.ndarray:
    """LightToneLut::new (crates/edit/src/light.rs:27-47) values."""
    out = np.zeros(4096, dtype=np.float32)
    f = ctypes.c_float
    load().ro_light_tone_lut(f(contrast), f(highlights), f(shadows), f(whites), f(blacks), ptr(out))
    return out


def display_srgb8(rgb: np.ndarray) -> np.ndarray:
    rgb = f32(rgb)
    out = np.zeros(rgb.shape, dtype=np.uint8)
    load().ro_display_srgb8(ptr(rgb), rgb.size // 3, ptr(out, ctypes.c_uint8))
    return out


def histogram(rgb8: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    rgb8 = np.ascontiguousarray(rgb8, dtype=np.uint8)
    hist = np.zeros(1024, dtype=np.uint64)
    clipped = np.zeros(6, dtype=np.uint64)
    load().ro_histogram(ptr(rgb8, ctypes.c_uint8), rgb8.size // 3, ptr(hist, ctypes.c_uint64),
                        ptr(clipped, ctypes.c_uint64))
    return hist, clipped


# ---- display / extended output (output.cpp) ----
FORMATS = {"srgb8": 0, "srgb16": 1, "extended_f32": 2}
ORIENTATIONS = ("normal", "horizontal_flip", "rotate180", "vertical_flip", "transpose", "rotate90", "transverse",
                "rotate270", "unknown")


def output_desc(fmt="srgb8", primaries="srgb", policy="clip", dither="none", orientation="normal", crop=None,
                headroom=1.0) -> OutputDesc:
    d = OutputDesc()
    d.format = FORMATS[fmt]
    d.primaries = {"srgb": 0, "display_p3": 1}[primaries]
    d.policy = {"clip": 0, "chroma_compress": 1}[policy]
    d.dither = {"none": 0, "ordered8x8": 1}[dither]
    d.orientation = ORIENTATIONS.index(orientation)
    if crop is not None:
        d.has_crop = 1
        for k in range(4):
            d.crop[k] = crop[k]
    d.headroom = headroom
    return d


def set_exact_math(on: bool) -> None:
    """True: correctly rounded cube root and transfer power; False: the platform libm."""
    load().ro_set_exact_math(1 if on else 0)


def output_geometry(width: int, height: int, desc: OutputDesc):
    """(out_width, out_height, (left, top, right, bottom)) or None for an invalid geometry."""
    ow, oh = ctypes.c_int(), ctypes.c_int()
    crop = (ctypes.c_int * 4)()
    if load().ro_output_geometry(width, height, ctypes.byref(desc), ctypes.byref(ow), ctypes.byref(oh), crop) != 0:
        return None
    return ow.value, oh.value, tuple(crop)


def render_output(rgb: np.ndarray, desc: OutputDesc):
    """Adjusted linear Rec.2020 [h][3w] -> (image, gamut counts[5]); None for invalid geometry/headroom."""
    rgb = f32(rgb)
    h, w3 = rgb.shape
    geo = output_geometry(w3 // 3, h, desc)
    if geo is None:
        return None
    ow, oh, _ = geo
    dtype = {0: np.uint8, 1: np.uint16, 2: np.float32}[desc.format]
    out = np.zeros((oh, 3 * ow), dtype=dtype)
    gamut = np.zeros(5, dtype=np.uint64)
    if load().ro_render_output(ptr(rgb), w3 // 3, h, ctypes.byref(desc), out.ctypes.data_as(ctypes.c_void_p),
                               ptr(gamut, ctypes.c_uint64)) != 0:
        return None
    return out, gamut


GAMUT_STATUS = ("in_gamut", "compressed", "limited", "clipped_fallback", "invalid")


def gamut_map(rgb, primaries="srgb", policy="chroma_compress", ceiling=1.0):
    """(mapped linear rgb, status name) of one pixel in the target primaries."""
    v = np.asarray(rgb, dtype=np.float32).copy()
    out = np.zeros(3, dtype=np.float32)
    st = load().ro_gamut_map(ptr(v), 1 if primaries == "display_p3" else 0, 1 if policy == "chroma_compress" else 0,
                             ceiling, ptr(out))
    return out, GAMUT_STATUS[st]


def oklab(rgb, primaries="srgb", inverse=False) -> np.ndarray:
    v = np.asarray(rgb, dtype=np.float32).copy()
    out = np.zeros(3, dtype=np.float32)
    fn = load().ro_oklab_inverse if inverse else load().ro_oklab
    fn(1 if primaries == "display_p3" else 0, ptr(v), ptr(out))
    return out


def png_filter(image: np.ndarray) -> bytes:
    """Filtered PNG scanlines (filter byte + bytes per line) of RGB rows [h][w][3], u8 or u16."""
    image = np.ascontiguousarray(image)
    depth = 16 if image.dtype == np.uint16 else 8
    h, w = image.shape[:2]
    stream = np.zeros(h * (1 + w * 3 * depth // 8), dtype=np.uint8)
    load().ro_png_filter(image.ctypes.data_as(ctypes.c_void_p), w, h, depth, ptr(stream, ctypes.c_uint8))
    return stream.tobytes()


def png_unfilter(stream: bytes, width: int, height: int, depth: int) -> np.ndarray:
    """Samples [h][w][3] (u8, or u16 from the file's big-endian bytes) of a filtered stream."""
    line = 1 + width * 3 * depth // 8
    if len(stream) != height * line:
        raise ValueError(f"stream holds {len(stream)} bytes, expected {height * line}")
    src = np.frombuffer(stream, dtype=np.uint8).copy()
    out = np.zeros(height * (line - 1), dtype=np.uint8)
    if load().ro_png_unfilter(ptr(src, ctypes.c_uint8), width, height, depth, ptr(out, ctypes.c_uint8)) != 0:
        raise ValueError("unknown PNG filter type")
    if depth == 16:
        return out.view(">u2").astype(np.uint16).reshape(height, width, 3)
    return out.reshape(height, width, 3)


def jpeg_coefficients(rgb: np.ndarray, quality: int) -> np.ndarray:
    """Quantised coefficients [blocks][3][64] (zigzag order) of 8-bit RGB rows [h][w][3]."""
    rgb = np.ascontiguousarray(rgb, dtype=np.uint8)
    h, w = rgb.shape[:2]
    out = np.zeros((((w + 7) // 8) * ((h + 7) // 8), 3, 64), dtype=np.int16)
    load().ro_jpeg_coefficients(ptr(rgb, ctypes.c_uint8), w, h, quality, ptr(out, ctypes.c_int16))
    return out


def jpeg_decode(data: bytes) -> dict:
    """Baseline JPEG back to its coefficients: width, height, restart interval, quant tables, coef."""
    src = np.frombuffer(data, dtype=np.uint8).copy()
    w, h, ri = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    quant = np.zeros((3, 64), dtype=np.uint8)
    # The coefficient buffer is sized from the frame header's dimensions.
    pos = 2
    while pos + 9 < len(data) and not (data[pos] == 0xFF and data[pos + 1] == 0xC0):
        pos += 2 + int.from_bytes(data[pos + 2:pos + 4], "big")
    fh, fw = int.from_bytes(data[pos + 5:pos + 7], "big"), int.from_bytes(data[pos + 7:pos + 9], "big")
    coef = np.zeros((((fw + 7) // 8) * ((fh + 7) // 8), 3, 64), dtype=np.int16)
    rc = load().ro_jpeg_decode(ptr(src, ctypes.c_uint8), len(data), ctypes.byref(w), ctypes.byref(h),
                               ctypes.byref(ri), ptr(quant, ctypes.c_uint8), ptr(coef, ctypes.c_int16), coef.size)
    if rc != 0:
        raise ValueError(f"JPEG decode failed ({rc})")
    return {"width": w.value, "height": h.value, "restart": ri.value, "quant": quant, "coef": coef}


def jpeg_pixels(decoded: dict) -> np.ndarray:
    """RGB u8 [h][w][3] from decoded coefficients: dequantisation, the inverse DCT and
    the JFIF colour conversion in floating point."""
    w, h = decoded["width"], decoded["height"]
    bw, bh = (w + 7) // 8, (h + 7) // 8
    nat = _zigzag_natural()
    coef = decoded["coef"].astype(np.float64)
    blocks = np.zeros((bw * bh, 3, 64))
    blocks[:, :, nat] = coef * decoded["quant"][None, :, nat]
    blocks = blocks.reshape(bw * bh, 3, 8, 8)
    u = np.arange(8)
    basis = np.cos((2 * u[None, :] + 1) * u[:, None] * np.pi / 16) * np.where(u == 0, np.sqrt(0.5), 1.0)[:, None] / 2
    spatial = np.einsum("vy,bcvu,ux->bcyx", basis, blocks, basis) + 128.0
    img = spatial.reshape(bh, bw, 3, 8, 8).transpose(0, 3, 1, 4, 2).reshape(bh * 8, bw * 8, 3)[:h, :w]
    y, cb, cr = img[..., 0], img[..., 1] - 128.0, img[..., 2] - 128.0
    rgb = np.stack([y + 1.402 * cr, y - 0.344136 * cb - 0.714136 * cr, y + 1.772 * cb], axis=-1)
    return np.clip(np.rint(rgb), 0, 255).astype(np.uint8)


def _zigzag_natural() -> np.ndarray:
    order = sorted(((r + c, r if (r + c) % 2 else c, r, c) for r in range(8) for c in range(8)))
    return np.array([r * 8 + c for _, _, r, c in order])

