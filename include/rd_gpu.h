/* rd_gpu.h - C ABI of the GB300 sensor-development library.
 *
 * This is the drop-in boundary that replaces the wgpu executors of the
 * reference's `rohditor-gpu` crate (crates/gpu). Only plain-old-data, opaque
 * handles and plain pointers cross it; no exception and no C++ or torch type.
 * Every call is ordered on the context's CUDA stream. Host pointers are
 * borrowed only for the duration of the call. Device objects (rd_source,
 * rd_base) are owned by their handles and must be released.
 *
 * Reference interface each entry point stands in for (file:line in the
 * reference project):
 *   rd_status                GpuPreviewError            crates/gpu/src/lib.rs:55-111
 *   rd_ctx_create            GpuSensorProcessor::new    crates/gpu/src/sensor/normalize.rs:91
 *   rd_ctx_set_budget        GpuSensorProcessor::set_budget  crates/gpu/src/sensor/normalize.rs:157
 *   rd_supports              GpuSensorProcessor::supports    crates/gpu/src/sensor/develop.rs:55
 *   rd_develop               GpuSensorProcessor::develop     crates/gpu/src/sensor/develop.rs:68
 *   rd_spatial               GpuSpatialProcessor::reduce_preview crates/gpu/src/spatial/reduction.rs:15
 *   rd_render                GpuPreviewProcessor::render + begin_histogram
 *                                                       crates/gpu/src/preview/processor.rs:1011,1518
 *   rd_render_output         GpuExportProcessor::render's output conversion
 *                            crates/gpu/src/export/mod.rs:218, matching the CPU renders render_display8_cancellable,
 *                            render_display_srgb16_with_geometry, render_extended_linear_with_geometry
 *                            crates/core/src/cpu/stages.rs:1028-1195, crates/core/src/cpu/extended.rs:27
 *   stage entry points       the crates' stage APIs the CPU pipeline calls:
 *     rd_stage_normalize     NormalizationContract::normalize crates/core/src/pipeline/sensor.rs:221
 *     rd_stage_highlight     HighlightExecution::apply_cancellable crates/highlight/src/lib.rs:172
 *     rd_stage_demosaic      demosaic_cancellable        crates/demosaic/src/lib.rs:302
 *     rd_stage_capture       sharpening::apply_cancellable crates/core/src/sharpening.rs:87
 *     rd_stage_optics        OpticsExecution::apply_cancellable crates/optics/src/correction.rs:49
 *     rd_stage_area_reduce   resize_area_with_plan_cancellable crates/core/src/resample.rs:235
 *     rd_stage_color         apply_white_balance + apply_camera_color_transform +
 *                            apply_adjustments_with_local + render_display8 + Histogram
 *                            crates/core/src/cpu/stages.rs:250-308,380-528,1028-1094;
 *                            crates/core/src/analysis/histogram.rs:92-128
 *     rd_stage_output        apply_adjustments_with_local + the output conversions above
 *   rd_encode_png            export::encode, PNG arms     crates/core/src/export.rs:155-219
 *   rd_encode_jpeg           export::encode, JPEG arm     crates/core/src/export.rs:166-175
 */
#ifndef RD_GPU_H
#define RD_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* GpuPreviewError variants (crates/gpu/src/lib.rs:55-111). */
typedef enum rd_status {
  RD_OK = 0,
  RD_CANCELLED = 1,
  RD_UNSUPPORTED = 2,
  RD_OVER_BUDGET = 3,
  RD_INVALID_DIMENSIONS = 4,
  RD_BASE_MISMATCH = 5,
  RD_UNSUPPORTED_EDITS = 6,
  RD_SYNCHRONIZATION = 7,
  RD_INVALID_INPUT = 8,
  RD_READBACK = 9
} rd_status;

/* 1 for the routing answers that keep the device usable (UnsupportedEdits,
 * OverBudget; GpuPreviewError::is_routing), else 0. */
int rd_status_is_routing(rd_status status);
const char* rd_status_name(rd_status status);

typedef struct rd_ctx rd_ctx;
typedef struct rd_source rd_source; /* full-resolution camera RGB resident on the device */
typedef struct rd_base rd_base;     /* reduced Rec.2020 base resident on the device */

/* ---- descriptors: the CPU-resolved contracts, never raw recipe fields ---- */

enum { RD_CFA_RGGB = 0, RD_CFA_BGGR = 1, RD_CFA_GRBG = 2, RD_CFA_GBRG = 3 };
enum { RD_HIGHLIGHT_OFF = 0, RD_HIGHLIGHT_CLIP = 1, RD_HIGHLIGHT_OPPOSED = 2 };
enum { RD_DEMOSAIC_BILINEAR = 0, RD_DEMOSAIC_MHC = 1, RD_DEMOSAIC_RCD = 2, RD_DEMOSAIC_AMAZE = 3 };
#define RD_MAX_LEVEL_PATTERN 64

/* NormalizationContract + SensorDevelopmentDescription
 * (crates/core/src/pipeline/sensor.rs:56-67, 280-298). Levels are indexed at
 * SENSOR coordinates; the crop's CFA phase is derived from `cfa` by the shift. */
typedef struct rd_sensor_desc {
  uint32_t sensor_width, sensor_height;
  uint32_t crop_x, crop_y, crop_width, crop_height;
  int32_t cfa;                       /* pattern at sensor (0,0): RD_CFA_* */
  uint32_t black_repeat_w, black_repeat_h;
  float black[RD_MAX_LEVEL_PATTERN]; /* black_repeat_w*black_repeat_h values */
  uint32_t white_count;              /* 1, 3 (per channel) or black_repeat_w*black_repeat_h */
  float white[RD_MAX_LEVEL_PATTERN];
  int32_t highlight;                 /* RD_HIGHLIGHT_* */
  float clip_levels[3];              /* Clip: per-channel ceilings */
  float detection_levels[3];         /* Opposed: detection levels */
  int32_t has_neutral_ceiling;
  float neutral_ceiling[3];          /* Opposed: WB-aware neutral ceiling */
  int32_t demosaic;                  /* RD_DEMOSAIC_* */
  float demosaic_balance[3];         /* as-shot gains the demosaic reconstructs under */
} rd_sensor_desc;

/* CaptureSharpeningContract (crates/core/src/sharpening.rs:17-68). The
 * iteration count is explicit (the reference fixes it at 8). */
typedef struct rd_detail_desc {
  int32_t enabled;
  float amount, radius, noise_protection;
  float ceilings[3];
  int32_t iterations;
} rd_detail_desc;

enum { RD_DISTORTION_NONE = 0, RD_DISTORTION_POLY3 = 1, RD_DISTORTION_POLY5 = 2, RD_DISTORTION_PTLENS = 3 };
enum { RD_TCA_NONE = 0, RD_TCA_LINEAR = 1, RD_TCA_POLY3 = 2 };

/* OpticsExecution (crates/optics/src/plan.rs:37-50): the resolved, lensfun-free
 * correction contract. */
typedef struct rd_optics_desc {
  uint32_t width, height;
  double norm_scale, norm_unscale, center_x, center_y;
  float scale;
  int32_t distortion_model;
  float distortion[3];
  int32_t tca_model;
  float tca_red[3], tca_blue[3];
  int32_t vignetting;     /* 0 none, 1 PA */
  float vignetting_k[3];
} rd_optics_desc;

/* White balance, camera matrix and the global adjustment chain
 * (crates/core/src/cpu/stages.rs:380-528) with LUTs resolved on the host.
 * The chain runs exposure, base rendering, Light tone, tone curve,
 * saturation / vibrance, HSL and grading, each step only when its has_ flag
 * is set (stages.rs:434-452 decides the same per recipe). */
typedef struct rd_color_desc {
  float wb_gains[3];
  float camera_to_rec2020[9];   /* row-major */
  float exposure_ev;
  int32_t has_base_lut;
  float base_lut[4096];         /* BaseRenderingLut values */
  int32_t has_light_tone_lut;   /* set when contrast, highlights, shadows, whites or blacks is non-zero */
  float light_tone_lut[4096];   /* LightToneLut values (crates/edit/src/light.rs:27-47), see rd_light_tone_lut */
  int32_t has_tone_lut;
  float tone_lut[4096];         /* ToneCurveLut values */
  float saturation, vibrance;
  int32_t has_hsl;
  float hsl[8][3];              /* hue, saturation, luminance per band */
  int32_t has_grading;
  float grading[3][3];          /* shadows, midtones, highlights x RGB */
} rd_color_desc;

/* StageTimings-style device timings (ms) and counters. */
typedef struct rd_metrics {
  float normalize_highlight_ms, demosaic_ms, capture_ms, optics_ms, reduce_ms, color_ms, total_ms;
  uint64_t highlight_stats[9]; /* Clip: affected, changed, over_white, aff_r,g,b.
                                  Opposed: suspected, reconstructed, changed, fallback,
                                  unsupported, neutralised, susp_r,g,b */
  uint64_t kernel_launches;
  uint64_t device_bytes;
} rd_metrics;

/* ---- context ---- */
rd_status rd_ctx_create(int device, uint64_t budget_bytes, rd_ctx** out);
/* Every rd_source and rd_base of the context must be released first. */
void rd_ctx_destroy(rd_ctx* ctx);
rd_status rd_ctx_set_budget(rd_ctx* ctx, uint64_t budget_bytes);
const char* rd_ctx_last_error(const rd_ctx* ctx);
rd_status rd_ctx_synchronize(rd_ctx* ctx);
/* Number of this library's kernels launched on the context so far. */
uint64_t rd_ctx_kernel_launches(const rd_ctx* ctx);
/* Test facility for the bounded device waits (no reference counterpart).
 * Every spin-wait of this library's kernels gives up after an iteration
 * limit, records why in the context's error word and returns, so the call
 * fails with RD_INVALID_INPUT and the context stays usable. This setting
 * makes a wait run out on purpose: `wait_limit` (0: the built-in limits)
 * shortens every wait, and `withhold` names a completion the next calls
 * never deliver: RD_WAIT_AMAZE_TILE (phase A of AMaZE tile 0 does not
 * publish its slab, so its phase B waits), RD_WAIT_RL_COPY (every block
 * of the capture-sharpening kernels skips its first tensor copy but waits
 * for it, then drains its other copies in flight), RD_WAIT_DEMOSAIC_COPY
 * (every block of the bilinear / MHC and RCD kernels skips the tensor copy
 * of its tile but waits for it; sources that TMA cannot address, and RCD
 * windows that cross the image edge, are staged by plain loads and have no
 * such wait) or RD_WAIT_AMAZE_COPY (AMaZE issues none of its mosaic-row
 * tensor copies but waits for the first of each block, then loads the rows
 * directly). RD_WAIT_NONE restores normal operation. */
enum {
  RD_WAIT_NONE = 0,
  RD_WAIT_AMAZE_TILE = 1,
  RD_WAIT_RL_COPY = 2,
  RD_WAIT_DEMOSAIC_COPY = 3,
  RD_WAIT_AMAZE_COPY = 4
};
rd_status rd_ctx_set_wait_test(rd_ctx* ctx, uint32_t wait_limit, int32_t withhold);

/* ---- routing ---- */
int rd_supports(const rd_sensor_desc* sensor);

/* ---- processor API (resident objects) ----
 * `cancel` (optional) is a host word polled between stages; non-zero ends the
 * call with RD_CANCELLED and returns no device state. */
rd_status rd_develop(rd_ctx* ctx, const uint16_t* mosaic, size_t row_stride, const rd_sensor_desc* sensor,
                     const rd_detail_desc* detail, const volatile uint32_t* cancel, rd_source** out,
                     rd_metrics* metrics);
/* Same, with the mosaic already resident on the device (d_mosaic is a device
 * pointer of sensor_height*row_stride u16). */
rd_status rd_develop_device(rd_ctx* ctx, const uint16_t* d_mosaic, size_t row_stride,
                            const rd_sensor_desc* sensor, const rd_detail_desc* detail,
                            const volatile uint32_t* cancel, rd_source** out, rd_metrics* metrics);
rd_status rd_spatial(rd_ctx* ctx, const rd_source* source, const rd_optics_desc* optics, uint32_t target_width,
                     uint32_t target_height, const float wb_gains[3], const float camera_to_rec2020[9],
                     rd_base** out, rd_metrics* metrics);
/* srgb_out: host [h][3w] u8, or NULL. hist: 4*256 u64 (R, G, B, luma) or NULL.
 * clipped: 6 u64 (shadow r,g,b, highlight r,g,b) or NULL. */
rd_status rd_render(rd_ctx* ctx, const rd_base* base, const rd_color_desc* color, uint8_t* srgb_out,
                    uint64_t* hist, uint64_t* clipped, rd_metrics* metrics);
/* Device-resident render: writes u8 output and histogram into device memory
 * owned by the base; nothing is copied to the host. */
rd_status rd_render_device(rd_ctx* ctx, rd_base* base, const rd_color_desc* color, rd_metrics* metrics);
/* Allocation-free render. No counterpart in the reference: it exists for
 * callers that cannot allocate device memory on the render path (an
 * interactive loop re-rendering the preview per slider event under a fixed,
 * pre-reserved device budget). Same arithmetic as rd_render_device.
 *   d_base      planar Rec.2020 f32 [3][height][width] on the current device
 *               (the white-balanced, camera-matrixed base)
 *   d_srgb_out  device [height][3*width] u8
 *   d_hist      device 4*256 u64 (R, G, B, luma); cleared by this call
 *   stream      cudaStream_t the work is enqueued on (NULL: legacy default)
 * Returns after enqueueing; results are ready when `stream` completes. No
 * context, no device allocation: the three 4096-entry LUTs (48 KB, the only
 * scratch; LUT length is fixed by rd_color_desc, image size is not limited)
 * are staged in a static device array of this library, copied there from
 * `color` on every call. The first call on a device resolves that array's
 * address and may load the module there. Calls overlapping in time on one
 * device (any streams, any threads) share the array and race: serialise them.
 * RD_INVALID_INPUT for null pointers, zero or > INT32_MAX sizes, device
 * ordinals >= 64, or a stream that is being captured into a CUDA graph (the
 * call enqueues nothing then); RD_SYNCHRONIZATION when a CUDA call fails. */
rd_status rd_render_device_noalloc(const float* d_base, uint32_t width, uint32_t height,
                                   const rd_color_desc* color, uint8_t* d_srgb_out, uint64_t* d_hist,
                                   void* stream);

/* ---- display and extended-range output ----
 * The output conversions of the reference's renders: the adjustment chain of
 * rd_color_desc, then orientation + crop (OutputGeometry), gamut mapping into
 * the target primaries and the output encoding:
 *   RD_OUTPUT_SRGB8         render_display8_cancellable   crates/core/src/cpu/stages.rs:1028-1094
 *   RD_OUTPUT_SRGB16        render_display_srgb16_with_geometry_and_diagnostics  stages.rs:1124-1195
 *   RD_OUTPUT_EXTENDED_F32  render_extended_linear_with_geometry  crates/core/src/cpu/extended.rs:27-106
 *   RD_OUTPUT_EXTENDED_F16  the same, each channel rounded to binary16 (round to nearest even)
 * All outputs are interleaved [out_h][3*out_w]: u8, u16, f32, or binary16 bits
 * in u16. 8- and 16-bit values are sRGB-transfer encoded; extended values are
 * linear in 0..headroom with diffuse white at 1. The cube root of OkLab and the
 * transfer power are correctly rounded (the reference takes both from the
 * platform libm). */
typedef enum rd_output_format {
  RD_OUTPUT_SRGB8 = 0,
  RD_OUTPUT_SRGB16 = 1,
  RD_OUTPUT_EXTENDED_F32 = 2,
  RD_OUTPUT_EXTENDED_F16 = 3
} rd_output_format;
/* RgbPrimaries (crates/image), OutputPolicy (crates/core/src/pipeline/orchestration.rs:53),
 * DitherMode (crates/core/src/export/types.rs:99), Orientation (crates/image/src/orientation.rs). */
enum { RD_PRIMARIES_SRGB = 0, RD_PRIMARIES_DISPLAY_P3 = 1 };
enum { RD_POLICY_CLIP = 0, RD_POLICY_CHROMA_COMPRESS = 1 };
enum { RD_DITHER_NONE = 0, RD_DITHER_ORDERED_8X8 = 1 };
enum {
  RD_ORIENTATION_NORMAL = 0, RD_ORIENTATION_HORIZONTAL_FLIP = 1, RD_ORIENTATION_ROTATE180 = 2,
  RD_ORIENTATION_VERTICAL_FLIP = 3, RD_ORIENTATION_TRANSPOSE = 4, RD_ORIENTATION_ROTATE90 = 5,
  RD_ORIENTATION_TRANSVERSE = 6, RD_ORIENTATION_ROTATE270 = 7, RD_ORIENTATION_UNKNOWN = 8
};
typedef struct rd_output_desc {
  int32_t format;       /* rd_output_format */
  int32_t primaries;    /* RD_PRIMARIES_* */
  int32_t policy;       /* RD_POLICY_*: clip_linear_rgb or compress_chroma */
  int32_t dither;       /* RD_DITHER_*: 8- and 16-bit outputs only */
  int32_t orientation;  /* RD_ORIENTATION_* */
  int32_t has_crop;
  double crop[4];       /* NormalizedCropRect left, top, right, bottom on the oriented canvas */
  float headroom;       /* extended outputs: the ceiling, finite and >= 1 */
} rd_output_desc;
/* Output size of a width x height base (OutputGeometry::output_dimensions,
 * crates/core/src/geometry.rs:111-114); RD_INVALID_INPUT for an invalid
 * description (unknown enum, crop outside 0..1, unordered or below one pixel,
 * extended headroom not finite or < 1). bytes_per_pixel may be NULL. */
rd_status rd_output_dimensions(uint32_t width, uint32_t height, const rd_output_desc* output, uint32_t* out_width,
                               uint32_t* out_height, uint32_t* bytes_per_pixel);
/* out: host buffer of at least out_capacity = out_w*out_h*bytes_per_pixel bytes.
 * hist: 4*256 u64 of the 8-bit output (R, G, B, luma), or NULL (must be NULL
 * for the other formats). gamut: 5 u64 GamutMappingDiagnostics (in_gamut,
 * compressed, limited, clipped_fallback, invalid), or NULL. */
rd_status rd_render_output(rd_ctx* ctx, const rd_base* base, const rd_color_desc* color, const rd_output_desc* output,
                           void* out, size_t out_capacity, uint64_t* hist, uint64_t* gamut, rd_metrics* metrics);
/* Same into device buffers (d_out of out_w*out_h*bytes_per_pixel bytes; d_hist
 * 1024 u64 or NULL; d_gamut 5 u64 or NULL), ordered on the context's stream. */
rd_status rd_render_output_device(rd_ctx* ctx, const rd_base* base, const rd_color_desc* color,
                                  const rd_output_desc* output, void* d_out, uint64_t* d_hist, uint64_t* d_gamut,
                                  rd_metrics* metrics);
/* ---- PNG encode: the PNG arms of export::encode (crates/core/src/export.rs:176-211),
 * which hand tightly packed RGB rows, the output colour space's ICC profile and
 * optional EXIF to the image crate's PngEncoder.
 * Samples are 8-bit (bit_depth 8, u8 rows) or 16-bit (bit_depth 16, u16 rows in
 * host byte order; the file stores them most significant byte first). rgb is
 * interleaved [height][3*width]; row_stride is in samples and must equal
 * 3*width, as the reference rejects padded rows (ExportError::InvalidImageLayout,
 * export.rs:136-150): RD_INVALID_INPUT otherwise, and for another bit depth. icc
 * (icc_len bytes) becomes an iCCP chunk and exif an eXIf chunk; either may be
 * NULL with length 0. Decoding the file gives back exactly the input samples.
 * rd_png_bound: the largest file for these sizes (0 for invalid arguments). */
uint64_t rd_png_bound(uint32_t width, uint32_t height, int32_t bit_depth, uint64_t icc_len, uint64_t exif_len);
/* Host rows in, host file out: png receives *png_bytes bytes. When capacity is
 * smaller than the file, RD_INVALID_DIMENSIONS with *png_bytes set to its size.
 * metrics->total_ms: device time of the encode (copies excluded). */
rd_status rd_encode_png(rd_ctx* ctx, const void* rgb, uint32_t width, uint32_t height, uint64_t row_stride,
                        int32_t bit_depth, const uint8_t* icc, uint64_t icc_len, const uint8_t* exif,
                        uint64_t exif_len, uint8_t* png, uint64_t capacity, uint64_t* png_bytes,
                        rd_metrics* metrics);
/* Device rows in, device file out, ordered on the context's stream: d_png (4-byte
 * aligned, capacity >= rd_png_bound) receives the file and *d_png_bytes (device
 * u64) its size. */
rd_status rd_encode_png_device(rd_ctx* ctx, const void* d_rgb, uint32_t width, uint32_t height, uint64_t row_stride,
                               int32_t bit_depth, const uint8_t* icc, uint64_t icc_len, const uint8_t* exif,
                               uint64_t exif_len, uint8_t* d_png, uint64_t capacity, uint64_t* d_png_bytes);
/* ---- JPEG encode: the JPEG arm of export::encode (crates/core/src/export.rs:166-175),
 * which hands tightly packed 8-bit RGB rows and a quality of 1..100, with the ICC
 * profile and optional EXIF, to the image crate's JpegEncoder.
 * The file is a baseline JPEG (ITU-T T.81): JFIF, Y/Cb/Cr at 4:4:4, the Annex K
 * quantisation tables scaled by quality, Huffman tables built for the image,
 * a restart marker every 32 MCUs, the profile in APP2 ICC_PROFILE segments and
 * the EXIF block (a TIFF structure) in an APP1 Exif segment. rgb is interleaved
 * u8 [height][3*width]; row_stride (samples) must equal 3*width. RD_INVALID_INPUT
 * for padded rows or a quality outside 1..100, RD_INVALID_DIMENSIONS above 65535
 * pixels a side. The encoder reads the image's symbol counts back once to build
 * its tables (one synchronisation of the context's stream).
 * rd_jpeg_bound: the largest file for these sizes (0 for invalid sizes). */
uint64_t rd_jpeg_bound(uint32_t width, uint32_t height, uint64_t icc_len, uint64_t exif_len);
/* Host rows in, host file out; as rd_encode_png for the buffer and metrics. */
rd_status rd_encode_jpeg(rd_ctx* ctx, const uint8_t* rgb, uint32_t width, uint32_t height, uint64_t row_stride,
                         int32_t quality, const uint8_t* icc, uint64_t icc_len, const uint8_t* exif,
                         uint64_t exif_len, uint8_t* jpeg, uint64_t capacity, uint64_t* jpeg_bytes,
                         rd_metrics* metrics);
/* Device rows in, device file out (capacity >= rd_jpeg_bound; *d_jpeg_bytes a device u64). */
rd_status rd_encode_jpeg_device(rd_ctx* ctx, const uint8_t* d_rgb, uint32_t width, uint32_t height,
                                uint64_t row_stride, int32_t quality, const uint8_t* icc, uint64_t icc_len,
                                const uint8_t* exif, uint64_t exif_len, uint8_t* d_jpeg, uint64_t capacity,
                                uint64_t* d_jpeg_bytes);
/* Self-check of the correctly rounded arithmetic on the device, for test
 * suites (no reference counterpart). which = 0: the number of positive finite
 * f32 whose cube root is not correctly rounded (or not odd-symmetric), exact
 * integer comparison, expected 0. which = 1: the largest distance in ulps of
 * powf(x, 1/2.4) from the correctly rounded power over (0.0031308, 1], which
 * must not exceed the bound the 8- and 16-bit quantisation relies on (1).
 * which = 2: the number of f32 in (0.0031308, 1] whose transfer power (as the
 * quantisation computes it) differs from the correctly rounded one, expected 0.
 * which = 3: the number of (f32 in that domain, 8- or 16-bit, three dither
 * offsets) whose quantised code differs from the code of the correctly
 * rounded power, expected 0. which = 4: the number of sampled f32 pairs (x
 * over every f32 in [2^-12, 2), y hashed with 2^-18 <= |y| < 2, and y = 0)
 * whose hypot in the optics remap differs from f32::hypot as glibc computes
 * it (the double square root of the double sum of squares, narrowed once),
 * expected 0. */
rd_status rd_check_math(rd_ctx* ctx, int32_t which, uint64_t* result);
/* Launch shape of the capture-sharpening iteration chosen for one image shape
 * (no reference counterpart). The first develop of a (width, height, kernel
 * radius) shape times its iterations under a few row-segment counts around the
 * occupancy heuristic's; the fastest is kept process-wide and used by later
 * develops of that shape. The results are the same under every count.
 * segments: the chosen count; default_segments: the heuristic's; best_ms and
 * default_ms: their fastest timed iteration (0 when not timed). Any output may
 * be NULL except segments. RD_UNSUPPORTED when the shape has not been tuned. */
rd_status rd_rl_launch_shape(uint32_t width, uint32_t height, float radius, int32_t* segments,
                             int32_t* default_segments, float* best_ms, float* default_ms);
/* Launch shapes tuned across calls (no reference counterpart): the RL guide /
 * mask kernel's row segments per strip (stage RD_SHAPE_RL_MASK, `radius` the
 * capture radius), the colour kernel's CTAs per SM (RD_SHAPE_COLOR, `radius`
 * ignored) and the rows of the optics gather's 32-column tiles
 * (RD_SHAPE_OPTICS, `radius` ignored). The first calls for an image shape each launch one
 * candidate, timed; once every candidate has been timed twice the fastest is
 * used for that shape by every context of the process. Results never depend
 * on the shape. RD_UNSUPPORTED until the shape is tuned. */
enum { RD_SHAPE_RL_MASK = 0, RD_SHAPE_COLOR = 1, RD_SHAPE_OPTICS = 2 };
rd_status rd_launch_shape(int32_t stage, uint32_t width, uint32_t height, float radius, int32_t* value,
                          int32_t* default_value, float* best_ms, float* default_ms);

rd_status rd_source_dimensions(const rd_source* source, uint32_t* width, uint32_t* height);
rd_status rd_source_download(rd_ctx* ctx, const rd_source* source, float* rgb_interleaved);
rd_status rd_base_dimensions(const rd_base* base, uint32_t* width, uint32_t* height);
rd_status rd_base_download(rd_ctx* ctx, const rd_base* base, float* rgb_interleaved);
void rd_source_release(rd_source* source);
void rd_base_release(rd_base* base);

/* ---- stage entry points (host buffers in and out) ---- */
/* Normalize + highlight at full crop size. out: crop_h*crop_w f32. stats: 9 u64. */
rd_status rd_stage_highlight(rd_ctx* ctx, const uint16_t* mosaic, size_t row_stride, const rd_sensor_desc* sensor,
                             float* out, uint64_t* stats);
/* Opposed reconstruction of a normalized mosaic (crop-local CFA `cfa`), as
 * reconstruct_opposed (crates/highlight/src/opposed.rs:63). ceiling may be
 * NULL. stats: 9 u64 (OpposedStats order). labels (optional): the compact
 * region label of every 2x2 cell, ceil(w/2)*ceil(h/2) u32. */
rd_status rd_stage_opposed(rd_ctx* ctx, const float* mosaic, uint32_t width, uint32_t height, int32_t cfa,
                           const float levels[3], const float* ceiling, float* out, uint64_t* stats,
                           uint32_t* labels, uint32_t* region_count);
/* Demosaic a normalized mosaic (crop-local CFA `cfa`). out: interleaved [h][3w]. */
rd_status rd_stage_demosaic(rd_ctx* ctx, const float* mosaic, uint32_t width, uint32_t height, int32_t cfa,
                            int32_t algorithm, const float balance[3], float* out);
rd_status rd_stage_capture(rd_ctx* ctx, float* rgb_interleaved, uint32_t width, uint32_t height,
                           const rd_detail_desc* detail);
rd_status rd_stage_optics(rd_ctx* ctx, const rd_optics_desc* optics, const float* rgb_in, float* rgb_out);
rd_status rd_stage_area_reduce(rd_ctx* ctx, const float* rgb_in, uint32_t width, uint32_t height,
                               uint32_t target_width, uint32_t target_height, float* rgb_out);
/* Camera-native RGB -> WB -> matrix -> adjustments -> sRGB8 + histogram. */
rd_status rd_stage_color(rd_ctx* ctx, const float* rgb_in, uint32_t width, uint32_t height,
                         const rd_color_desc* color, uint8_t* srgb_out, uint64_t* hist, uint64_t* clipped);
/* Linear Rec.2020 (interleaved [h][3w]) -> adjustments -> display / extended
 * output, as rd_render_output. */
rd_status rd_stage_output(rd_ctx* ctx, const float* rgb_in, uint32_t width, uint32_t height,
                          const rd_color_desc* color, const rd_output_desc* output, void* out, size_t out_capacity,
                          uint64_t* hist, uint64_t* gamut);

/* ---- host-side contract helpers ---- */
/* build_plan geometry + automatic scale (crates/optics/src/plan.rs:173-231,521-559)
 * for a lens given crop factor, real focal length and lens centre offsets. */
rd_status rd_optics_plan(rd_optics_desc* optics, float crop_factor, float real_focal, float lens_center_x,
                         float lens_center_y);
/* RadialMultipliers::build (crates/optics/src/radial.rs:172-208, 400-491): the
 * table rd_spatial remaps through when its build accepts it. guard: -1 no
 * table (no distortion and no TCA, or a degenerate grid), 0 accepted, else the
 * refusing rule: 1 non-finite knot, 2 radiality tripwire, 3 two freeze flips in
 * one segment, 4 ambiguous freeze band, 5 unexplained jump. knots (1024 x 4,
 * optional) receives [m_red, m_green, m_blue, pin] per knot, pin being the
 * break radius of a freeze boundary pinned in the segment that starts at the
 * knot, or NaN; step the radius between knots. Host only. */
rd_status rd_optics_radial_table(const rd_optics_desc* optics, float* knots, float* step, int32_t* guard);
/* BaseRenderingLut::standard_v1 (crates/core/src/rendering.rs:36-50). */
void rd_standard_base_lut(float* lut4096);
/* LightToneLut::new (crates/edit/src/light.rs:27-47, evaluate_light_tone
 * :90-137): the 4096-entry Light transfer table for the contrast, highlights,
 * shadows, whites and blacks sliders, made monotone, into lut4096. Host only;
 * uses the platform exp2f / powf as the reference's f32::exp2 / f32::powf do. */
void rd_light_tone_lut(float contrast, float highlights, float shadows, float whites, float blacks, float* lut4096);

/* ---- batched develop ----
 * Many mosaics of uneven sizes, CFA phases and settings through the whole path
 * (rd_develop -> rd_spatial -> rd_render, host buffers in and out) on one GPU:
 * `lanes` host threads with their own contexts and streams take images from a
 * shared queue, so their kernels overlap on the device. The reference runs one
 * image per call (SpatialCache::prepare_sensor,
 * crates/engine/src/preview_cache/spatial.rs:475-600). Each item reports its
 * status and time; the return value is the first failing status (RD_OK when
 * all succeed); wall_ms (optional) is the elapsed time of the whole batch. */
typedef struct rd_batch_item {
  const uint16_t* mosaic;  /* host, sensor_height rows of row_stride samples */
  size_t row_stride;
  rd_sensor_desc sensor;
  rd_detail_desc detail;
  rd_optics_desc optics;
  uint32_t target_width, target_height;
  float wb_gains[3];
  float camera_to_rec2020[9];
  rd_color_desc color;
  uint8_t* srgb_out;       /* host [target_height][3*target_width] */
  uint64_t* hist;          /* host 1024 bins, or NULL */
  int32_t status;          /* out */
  double ms;               /* out: this item's time in its lane */
} rd_batch_item;
rd_status rd_develop_batch(int device, rd_batch_item* items, int32_t count, int32_t lanes, double* wall_ms);
/* The same batch captured into one CUDA graph (uneven develops in one
 * captured launch graph). `chains` parallel branches each run their share of
 * the images (k % chains) through develop -> spatial -> render, with every
 * device buffer allocated and freed inside the graph; the batch is one graph
 * launch. With host_pinned != 0 the items' mosaic, srgb_out and hist are
 * pinned host memory (rd_host_alloc) and the graph reads and writes them in
 * place; otherwise they are staged through pinned copies. Optional timings:
 * capture_ms (capture + instantiation), launch_ms (launch to completion),
 * wall_ms (launch plus staging copies). Per-item `ms` is 0. */
rd_status rd_develop_batch_graph(int device, rd_batch_item* items, int32_t count, int32_t chains,
                                 int32_t host_pinned, double* wall_ms, double* capture_ms, double* launch_ms);
/* The same batch stage by stage: `lanes` lanes upload their images
 * (k % lanes) and normalize / highlight them, then one AMaZE launch works
 * through the half-tile items of every image from a shared queue (images of
 * other demosaic algorithms, or of 32 px or less, are demosaiced one by
 * one), then each capture-sharpening iteration is one launch over the work
 * items of every image that shares its taps (the guide / mask pass and the
 * gain run image by image; images below 256x64 take the per-image path),
 * then the lanes finish their images (spatial pass, render). Outputs equal
 * rd_develop + rd_spatial + rd_render per image bit for bit; device memory
 * holds every image's intermediates at once. Per-item `ms` covers the
 * finishing stage only. */
rd_status rd_develop_batch_flat(int device, rd_batch_item* items, int32_t count, int32_t lanes, double* wall_ms);
/* The stage-by-stage batch captured into one CUDA graph and run as a single
 * launch: `chains` branches upload and normalize / highlight the images
 * (k % chains), then one branch runs the AMaZE launch over every image's
 * tiles and the capture sharpening with one launch per RL iteration over the
 * batch, then the branches finish their images (spatial pass, render). Host
 * buffers and timings as rd_develop_batch_graph; outputs equal the per-image
 * path bit for bit. */
rd_status rd_develop_batch_flat_graph(int device, rd_batch_item* items, int32_t count, int32_t chains,
                                      int32_t host_pinned, double* wall_ms, double* capture_ms, double* launch_ms);

/* ---- served preview loop ----
 * Replaces the engine's preview worker and caches
 * (crates/engine/src/coordinator/scheduler.rs:44-180 newest-wins mailbox,
 * coordinator/worker.rs:1597-1703 develop_preview, preview_cache/spatial.rs:475-600,
 * crates/gpu/src/memory.rs:44-60 reservations) for many open images on one GPU:
 * images stay resident (decoded mosaic, 2560-px Rec.2020 base, render outputs),
 * requests are newest-wins per image by (revision, submission order), pending
 * edits of all images render in one batched launch ahead of develops, and the
 * least recently used images lose their layers when the budget is reached.
 * A worker thread serves requests; results are polled. Device < 0 creates a
 * dry server that models service times without a GPU (policy tests). */
typedef struct rd_server rd_server;
typedef struct rd_server_result {
  uint64_t request_id;
  uint32_t image_id;
  int32_t kind;      /* 0 edit (render), 1 develop, 2 export */
  int32_t status;    /* rd_status; RD_CANCELLED: replaced by a newer request or closed */
  uint32_t batch_size;
  uint64_t revision;
  double queue_ms, service_ms, latency_ms;  /* submit->start, start->done, submit->done */
} rd_server_result;
typedef struct rd_server_stats {
  uint64_t requested, completed, coalesced, failed, redeveloped, evictions, batches, batched_edits;
  uint64_t resident_bytes, peak_resident_bytes, budget_bytes;
  uint64_t exports;  /* exports served (completed or failed) */
} rd_server_stats;
rd_status rd_server_create(int device, uint64_t budget_bytes, rd_server** out);
/* Dry servers only: modelled develop and render times. */
rd_status rd_server_set_dry_timing(rd_server* server, uint32_t develop_us, uint32_t render_us);
void rd_server_destroy(rd_server* server);
/* Copies the mosaic and the contracts; queues the first develop (revision 0). */
rd_status rd_server_open(rd_server* server, uint32_t image_id, const uint16_t* mosaic, size_t row_stride,
                         const rd_sensor_desc* sensor, const rd_detail_desc* detail, const rd_optics_desc* optics,
                         uint32_t target_width, uint32_t target_height, const float wb_gains[3],
                         const float camera_to_rec2020[9], uint64_t* request_id);
rd_status rd_server_close_image(rd_server* server, uint32_t image_id);
rd_status rd_server_submit_edit(rd_server* server, uint32_t image_id, uint64_t revision, const rd_color_desc* color,
                                uint64_t* request_id);
rd_status rd_server_submit_develop(rd_server* server, uint32_t image_id, uint64_t revision,
                                   const rd_detail_desc* detail, const rd_optics_desc* optics, uint64_t* request_id);
/* Up to max_results completed requests (waiting up to wait_ms for the first); returns the count. */
int32_t rd_server_poll(rd_server* server, rd_server_result* out, int32_t max_results, int32_t wait_ms);
/* Export of an open image at full resolution (GpuExportProcessor::render,
 * crates/gpu/src/export/mod.rs:218): a develop from the resident mosaic with
 * the image's current settings, the spatial pass at the crop size, then each
 * of the n_outputs descriptions rendered into the client's host buffer dst[k]
 * (capacity[k] bytes, at least rd_output_dimensions' size). Runs on the
 * develop lane, its working set charged against the budget; completes with a
 * result of kind 2. The buffers must stay valid until that result is polled.
 * A later revision replaces a pending export of the same image (RD_CANCELLED). */
rd_status rd_server_submit_export(rd_server* server, uint32_t image_id, uint64_t revision, const rd_color_desc* color,
                                  const rd_output_desc* outputs, int32_t n_outputs, void* const* dst,
                                  const size_t* capacities, uint64_t* request_id);
/* Files of a served export (export::encode, crates/core/src/export.rs:155-219):
 * output k of rd_server_submit_export_files is encoded as described by files[k]
 * and dst[k] receives the file's bytes (capacity: rd_png_bound / rd_jpeg_bound of
 * the output's dimensions and the metadata lengths). PNG takes an RD_OUTPUT_SRGB8
 * or RD_OUTPUT_SRGB16 output, JPEG an RD_OUTPUT_SRGB8 one; RD_FILE_ROWS keeps the
 * rows as rd_server_submit_export does. The profile and EXIF bytes are copied at
 * submission; *file_bytes (may be NULL) receives the size when the export ends. */
enum { RD_FILE_ROWS = 0, RD_FILE_PNG = 1, RD_FILE_JPEG = 2 };
typedef struct rd_export_file {
  int32_t format;          /* RD_FILE_* */
  int32_t quality;         /* JPEG: 1..100 */
  const uint8_t* icc;      /* ICC profile, or NULL */
  uint64_t icc_len;
  const uint8_t* exif;     /* EXIF block (a TIFF structure), or NULL */
  uint64_t exif_len;
  uint64_t* file_bytes;
} rd_export_file;
rd_status rd_server_submit_export_files(rd_server* server, uint32_t image_id, uint64_t revision,
                                        const rd_color_desc* color, const rd_output_desc* outputs,
                                        const rd_export_file* files, int32_t n_outputs, void* const* dst,
                                        const size_t* capacities, uint64_t* request_id);
/* The latest rendered output of an image: sRGB8 [h][3w], 1024 histogram bins, its revision. */
rd_status rd_server_read_output(rd_server* server, uint32_t image_id, uint8_t* srgb, uint64_t* hist,
                                uint64_t* revision);
rd_status rd_server_get_stats(rd_server* server, rd_server_stats* out);
/* Waits up to wait_ms until no request is pending or running. */
rd_status rd_server_drain(rd_server* server, int32_t wait_ms);

/* ---- synthetic scene generator (seeded, counter-based; identical on CPU and GPU) ---- */
typedef struct rd_synth_desc {
  uint32_t width, height;
  int32_t cfa;
  uint32_t bits;          /* 12, 14 or 16 */
  float black;            /* DN */
  float white;            /* DN */
  float clip_fraction;    /* target fraction of clipped sites (0..1) */
  float gains[3];         /* camera channel response (as-shot WB is its inverse) */
  uint64_t seed;
  int32_t highlight_blobs; /* 1: clipped regions are Gaussian blobs */
  float hot_pixel_fraction;
} rd_synth_desc;
/* Generate on the device into d_out (height*width u16, row stride = width). */
rd_status rd_synth_mosaic_device(rd_ctx* ctx, const rd_synth_desc* desc, uint16_t* d_out);
/* Generate into host memory (runs on the device, then copies). */
rd_status rd_synth_mosaic(rd_ctx* ctx, const rd_synth_desc* desc, uint16_t* out);

/* ---- measurement ---- */
/* Record CUDA event `slot` (0..63) on the context stream; elapsed ms between two slots. */
rd_status rd_ctx_event_record(rd_ctx* ctx, int slot);
rd_status rd_ctx_event_elapsed(rd_ctx* ctx, int start_slot, int stop_slot, float* ms);
/* Overwrite a buffer larger than L2 on the context stream (cold-cache timing). */
rd_status rd_ctx_flush_l2(rd_ctx* ctx);
/* Per-kernel-family device time: when enabled, every launch of the library is
 * bracketed by CUDA events; totals are resolved at each call's final sync. */
rd_status rd_ctx_enable_kernel_timing(rd_ctx* ctx, int enable);
/* family: index 0..RD_KERNEL_FAMILIES-1; returns its name, total ms and launch count. */
#define RD_KERNEL_FAMILIES 16
rd_status rd_ctx_kernel_timing(const rd_ctx* ctx, int family, const char** name, double* total_ms,
                               uint64_t* launches);
rd_status rd_ctx_reset_kernel_timing(rd_ctx* ctx);

/* ---- device memory helpers for callers without a CUDA runtime of their own ---- */
/* Page-locked host memory for fast host<->device copies. */
rd_status rd_host_alloc(size_t bytes, void** out);
void rd_host_free(void* ptr);
rd_status rd_device_alloc(rd_ctx* ctx, size_t bytes, void** out);
rd_status rd_device_free(rd_ctx* ctx, void* ptr);
rd_status rd_copy_to_device(rd_ctx* ctx, void* dst, const void* src, size_t bytes);
rd_status rd_copy_to_host(rd_ctx* ctx, void* dst, const void* src, size_t bytes);

#ifdef __cplusplus
}
#endif
#endif /* RD_GPU_H */
