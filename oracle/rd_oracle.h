/* C interface of the CPU oracle (test infrastructure; see oracle_common.h).
 *
 * Layouts: mosaics are row-major f32 or u16 with an explicit row stride in
 * samples; RGB images are interleaved f32 [h][3*w]. CFA codes: 0 RGGB, 1 BGGR,
 * 2 GRBG, 3 GBRG. Every function is a restatement of one reference stage; the
 * file that implements it cites the reference file:line it follows.
 */
#ifndef RD_ORACLE_H
#define RD_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- demosaic (demosaic.cpp, amaze.cpp) ---- */
void ro_bilinear_reconstruct(const float* mosaic, int w, int h, int stride, int pattern, const float gains[3],
                             float* out, int out_stride);
void ro_mhc_reconstruct(const float* mosaic, int w, int h, int stride, int pattern, const float gains[3],
                        float* out, int out_stride);
int ro_rcd_reconstruct(const float* mosaic, int w, int h, int stride, int pattern, const float gains[3],
                       float* out, int out_stride);
int ro_amaze_reconstruct(const float* mosaic, int w, int h, int stride, int pattern, const float gains[3],
                         float clip_point, float* out, int out_stride);
int ro_amaze_probe_tile(const float* mosaic, int w, int h, int stride, int pattern, float clip_point,
                        const char* plane, float* out);
/* algorithm: 0 bilinear, 1 MHC, 2 RCD, 3 AMaZE; balance = as-shot gains. */
int ro_demosaic(const float* mosaic, int w, int h, int pattern, const float balance[3], int algorithm,
                float* out);

/* ---- sensor contract + highlight (sensor.cpp) ---- */
typedef struct ro_sensor {
  int sensor_w, sensor_h, row_stride;
  int crop_x, crop_y, crop_w, crop_h;
  int pattern;                /* sensor CFA pattern at sensor (0,0) */
  int black_w, black_h;       /* black repeat pattern */
  const float* black;         /* black_w*black_h values */
  int white_count;            /* 1, 3 or black_w*black_h */
  const float* white;
} ro_sensor;

/* NormalizationContract::normalize at full crop size. Returns crop pattern. */
int ro_normalize(const uint16_t* mosaic, const ro_sensor* s, float* out);
/* clip_cancellable: stats = {affected, changed, over_white, aff_r, aff_g, aff_b}. */
int ro_clip(float* mosaic, int w, int h, int pattern, const float levels[3], uint64_t stats[6]);
/* reconstruct_opposed_cancellable. ceiling may be NULL. stats = {suspected, reconstructed,
 * changed, fallback, unsupported, neutralised, susp_r, susp_g, susp_b}. labels_out (optional,
 * ceil(w/2)*ceil(h/2) u32) receives the compact region labels. */
int ro_opposed(float* mosaic, int w, int h, int pattern, const float levels[3], const float* ceiling,
               uint64_t stats[9], uint32_t* labels_out, uint32_t* region_count);
/* label_components on a 0/1 grid (regions.rs:188-281); returns count. */
uint32_t ro_label_components(uint32_t* labels, int w, int h);

/* ---- capture sharpening (capture.cpp) ---- */
/* Gaussian kernel weights (crates/detail/src/gaussian.rs:9-17); returns tap count. */
int ro_gaussian_kernel(float sigma, float* weights, int max_taps);
int ro_capture_sharpen(float* rgb, int w, int h, float amount, float radius, float noise,
                       const float ceilings[3], int iterations);

/* ---- optics (optics.cpp) ---- */
typedef struct ro_optics {
  int width, height;
  double norm_scale, norm_unscale, center_x, center_y;
  float scale;
  int distortion_model; /* 0 none, 1 poly3, 2 poly5, 3 ptlens */
  float distortion[3];
  int tca_model;        /* 0 none, 1 linear, 2 poly3 */
  float tca_red[3], tca_blue[3];
  int vignetting_model; /* 0 none, 1 pa */
  float vignetting[3];
} ro_optics;
/* build_plan's geometry for a 36x24-normalised sensor: fills norm/center/scale. */
int ro_optics_plan(ro_optics* plan, float crop_factor, float real_focal, float lens_center_x,
                   float lens_center_y);
int ro_optics_apply(const ro_optics* plan, const float* rgb_in, float* rgb_out);
int ro_optics_map(const ro_optics* plan, int x, int y, float coords[6]);
/* RadialMultipliers::build: -1 no table, 0 accepted, 1 non-finite, 2 tripwire,
 * 3 break collision, 4 freeze ambiguity, 5 unexplained jump. table gets
 * 1024 x 3 multipliers, the pinned segments up to max_segments. */
int ro_optics_radial(const ro_optics* plan, float* table, float* step, int* seg_index, float* seg_radius,
                     int max_segments, int* n_segments);
/* The table branch's source coordinates (whatever the guard says). */
int ro_optics_map_lut(const ro_optics* plan, int x, int y, float coords[6]);

/* ---- area reduction (spatial.cpp) ---- */
int ro_area_reduce(const float* rgb, int w, int h, int tw, int th, float* out);

/* ---- colour + output (color.cpp) ---- */
void ro_white_balance(float* rgb, size_t pixels, const float gains[3]);
void ro_camera_matrix(float* rgb, size_t pixels, const float m[9]);
typedef struct ro_adjust {
  float exposure_ev;
  const float* base_lut;    /* 4096 entries or NULL */
  const float* light_lut;   /* LightToneLut, 4096 entries or NULL */
  int extended;             /* 1: extended rendition (LightToneLut::sample_extended) */
  const float* tone_lut;    /* 4096 entries or NULL */
  float saturation, vibrance;
  int has_hsl;
  float hsl[8][3];          /* hue, saturation, luminance per band */
  int has_grading;
  float grading[3][3];      /* shadows, midtones, highlights x RGB */
} ro_adjust;
void ro_adjust_apply(float* rgb, size_t pixels, const ro_adjust* a);
void ro_standard_base_lut(float* lut4096);
void ro_light_tone_lut(float contrast, float highlights, float shadows, float whites, float blacks, float* lut4096);
void ro_display_srgb8(const float* rgb, size_t pixels, uint8_t* out);
void ro_histogram(const uint8_t* rgb8, size_t pixels, uint64_t hist[4 * 256], uint64_t clipped[6]);

/* ---- display / extended output (output.cpp) ---- */
typedef struct ro_output {
  int format;       /* 0 display u8, 1 sRGB u16, 2 extended linear f32 */
  int primaries;    /* 0 sRGB, 1 Display P3 */
  int policy;       /* 0 clip, 1 chroma compress */
  int dither;       /* 0 none, 1 ordered 8x8 */
  int orientation;  /* 0 Normal, 1 HorizontalFlip, 2 Rotate180, 3 VerticalFlip, 4 Transpose,
                       5 Rotate90, 6 Transverse, 7 Rotate270, 8 Unknown */
  int has_crop;
  double crop[4];   /* normalized left, top, right, bottom on the oriented canvas */
  float headroom;   /* extended output ceiling, finite and >= 1 */
} ro_output;
/* 1: correctly rounded cube root and transfer power; 0 (default): platform libm. */
void ro_set_exact_math(int on);
float ro_cbrt(float x);
float ro_cbrt_correctly_rounded(float x);
/* gamut.rs mappers on linear RGB in the target primaries; returns the status index. */
int ro_gamut_map(const float rgb[3], int p3, int policy, float ceiling, float out[3]);
void ro_oklab(int p3, const float rgb[3], float lab[3]);
void ro_oklab_inverse(int p3, const float lab[3], float rgb[3]);
int ro_output_geometry(int w, int h, const ro_output* o, int* out_w, int* out_h, int crop[4]);
void ro_source_coordinate(int w, int h, int orientation, int x, int y, int* sx, int* sy);
/* rgb: adjusted linear Rec.2020, interleaved. gamut = {in_gamut, compressed, limited,
 * clipped_fallback, invalid}. Returns 0, or -1 for an invalid geometry or headroom. */
int ro_render_output(const float* rgb, int w, int h, const ro_output* o, void* out, uint64_t gamut[5]);

/* ---- seeded synthetic scenes (synth.cpp) ---- */
typedef struct ro_synth {
  uint32_t width, height;
  int32_t cfa;
  uint32_t bits;
  float black, white;
  float clip_fraction;
  float gains[3];
  uint64_t seed;
  int32_t highlight_blobs;
  float hot_pixel_fraction;
} ro_synth;
/* out: [height][width] u16. Returns 0, or -1 below 2x2. */
int ro_synth_mosaic(const ro_synth* desc, uint16_t* out);

/* ---- PNG scanlines (encode.cpp) ----
 * ro_png_filter: image is interleaved RGB [h][3w], u8 (depth 8) or u16 in host
 * byte order (depth 16); stream receives h scanlines of 1 + w*3*depth/8 bytes
 * (filter type, filtered bytes). ro_png_unfilter inverts a stream into the
 * file's sample bytes (16-bit most significant byte first); -1 for a filter
 * type above 4. */
void ro_png_filter(const uint8_t* image, int w, int h, int depth, uint8_t* stream);
int ro_png_unfilter(const uint8_t* stream, int w, int h, int depth, uint8_t* out);

/* ---- JPEG (jpeg.cpp) ----
 * ro_jpeg_coefficients: the quantised coefficients of 8-bit RGB rows [h][3w] at
 * quality 1..100, [block (raster order)][Y, Cb, Cr][64 in zigzag order].
 * ro_jpeg_decode: a baseline JPEG (three 1x1 components, restart intervals) back
 * into its coefficients in the same layout; quant receives each component's
 * table (3 x 64, natural order). 0 on success, negative for a malformed file. */
void ro_jpeg_coefficients(const uint8_t* rgb, int w, int h, int quality, int16_t* coef);
int ro_jpeg_decode(const uint8_t* data, size_t n, int* width, int* height, int* restart, uint8_t* quant,
                   int16_t* coef, size_t coef_capacity);

#ifdef __cplusplus
}
#endif
#endif
