/*
 * jxg_oracle.c -- CPU oracle for the VarDCT front end.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C, the scalar path
 * of the Rust JPEG XL encoder jixel 0.5.14 for the UltraFast VarDCT front end
 * (XYB, frame statistics, adaptive quant field, chroma-from-luma tiles,
 * DCT8 + quantisation, tokens and per-context histograms).  It exists to check
 * the CUDA path and to be timed as the CPU baseline; the product library never
 * links, loads or calls it.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py use it.
 *
 * Semantics fixed here (the reference's result depends on CPU dispatch):
 *   - the scalar twins of every kernel;
 *   - `fmla` is a fused multiply-add (src/dct.rs:31-41, aarch64 semantic);
 *   - `round` rounds half away from zero (Rust f32::round);
 *   - float -> int casts saturate and send NaN to 0 (Rust `as`);
 *   - num_threads does not change any result (each unit owns its outputs).
 *
 * Every function names the reference file:line it follows.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_OK 0
#define ORC_ERR_EMPTY 1
#define ORC_ERR_INPUT 2
#define ORC_ERR_DISTANCE 4
#define ORC_ERR_UNSUPPORTED 8
#define ORC_ERR_ALLOC 9

#define BLOCK 8
#define TILE 64
#define GROUP 256
#define DC_GROUP 2048
#define GROUP_BLOCKS 32
#define TILE_BLOCKS 8

#define NUM_FINE_BLOCK_CTXS 30
#define NON_ZERO_BUCKETS 37
#define ZERO_DENSITY_CONTEXTS 458
#define NUM_FINE_AC_CONTEXTS (NUM_FINE_BLOCK_CTXS * (NON_ZERO_BUCKETS + ZERO_DENSITY_CONTEXTS))
#define ALPHABET 128

/* ------------------------------------------------------------------ */
/* Rust scalar semantics                                               */
/* ------------------------------------------------------------------ */

/* transform kinds of orc_dct (rows x columns, as the reference names them) */
enum {
  JXG_ORC_DCT8X8 = 0, JXG_ORC_DCT8X16 = 1, JXG_ORC_DCT16X8 = 2, JXG_ORC_DCT16X16 = 3,
  JXG_ORC_DCT16X32 = 4, JXG_ORC_DCT32X16 = 5, JXG_ORC_DCT32X32 = 6, JXG_ORC_DCT32X8 = 7,
  JXG_ORC_DCT8X32 = 8, JXG_ORC_DCT64X64 = 9, JXG_ORC_DCT64X32 = 10, JXG_ORC_DCT32X64 = 11,
  JXG_ORC_DCT128X128 = 12, JXG_ORC_DCT128X64 = 13, JXG_ORC_DCT64X128 = 14
};

static inline float fmla(float a, float b, float c) { return fmaf(a, b, c); }

static inline int32_t sat_i32(float v) {
  if (v != v) return 0;
  if (v >= 2147483647.0f) return INT32_MAX;
  if (v <= -2147483648.0f) return INT32_MIN;
  return (int32_t)v;
}

static inline int16_t sat_i16(float v) {
  if (v != v) return 0;
  if (v >= 32767.0f) return 32767;
  if (v <= -32768.0f) return -32768;
  return (int16_t)v;
}

static inline float clampf(float v, float lo, float hi) {
  return v < lo ? lo : (v > hi ? hi : v);
}

static inline float rmin(float a, float b) { return fminf(a, b); }
static inline float rmax(float a, float b) { return fmaxf(a, b); }

static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* IEEE binary16 conversion with round-to-nearest-even
 * (src/util.rs:382-411 and its hardware twins). */
static uint16_t f32_to_f16(float v) {
  uint32_t bits = f2u(v);
  uint16_t sign = (uint16_t)((bits >> 16) & 0x8000u);
  int32_t exp = (int32_t)((bits >> 23) & 0xFF);
  uint32_t mant = bits & 0x7FFFFFu;
  int32_t e16 = exp - 112;
  if (e16 >= 31) return sign | 0x7BFF;
  if (e16 <= 0) {
    if (e16 < -10) return sign;
    uint32_t m = mant | 0x800000u;
    uint32_t shift = (uint32_t)(14 - e16);
    uint32_t rounded = (m + (1u << (shift - 1)) - 1 + ((m >> shift) & 1)) >> shift;
    return sign | (uint16_t)rounded;
  }
  uint32_t m = mant + 0xFFFu + ((mant >> 13) & 1);
  uint32_t e = (uint32_t)e16;
  uint32_t m16 = m >> 13;
  if (m16 == 0x400) {
    m16 = 0;
    e += 1;
    if (e >= 31) return sign | 0x7BFF;
  }
  return sign | (uint16_t)(e << 10) | (uint16_t)m16;
}

static float f16_to_f32(uint16_t b) {
  uint32_t sign = b >> 15;
  uint32_t e = (b >> 10) & 0x1F;
  uint32_t m = b & 0x3FF;
  float v;
  if (e == 0) {
    v = (1.0f / 16384.0f) * ((float)m * (1.0f / 1024.0f));
  } else if (e == 31) {
    v = m ? NAN : INFINITY;
  } else {
    v = u2f(((e + 112u) << 23) | (m << 13));
  }
  return sign ? -v : v;
}

static inline float f16_round(float v) { return f16_to_f32(f32_to_f16(v)); }

/* ------------------------------------------------------------------ */
/* Quality and distance parameters                                      */
/* ------------------------------------------------------------------ */

/* src/encode_image.rs:1321-1338 */
float orc_distance_from_quality(float quality) {
  float q = clampf(quality, 0.0f, 100.0f);
  float d;
  if (q >= 99.0f) d = 0.05f * powf(2.0f, 100.0f - q);
  else if (q >= 90.0f) d = powf(10.0f, (99.0f - q) / 9.0f - 1.0f);
  else if (q >= 30.0f) d = 0.1f + (100.0f - q) * 0.09f;
  else d = 6.24f + powf(2.5f, (30.0f - q) / 5.0f) / 6.25f;
  return rmin(d, 25.0f);
}

/* src/frame/quantization.rs:56-66 */
static float dc_refinement(float d) {
  if (d <= 3.0f) return 1.35f;
  if (d >= 5.0f) return 1.0f;
  const float recip = 1.0f / (5.0f - 3.0f);
  float t = (d - 3.0f) * recip;
  return fmla(1.0f - 1.35f, t, 1.35f);
}

/* src/frame/quantization.rs:72-75 */
static float dcepf_vlq_t(float d) {
  return clampf((d - 8.0f) / (15.0f - 8.0f), 0.0f, 1.0f);
}

/* src/frame/quantization.rs:77-86 */
static float quant_dc_of(float d) {
  float refine = dc_refinement(d);
  float vlq = fmla(dcepf_vlq_t(d), 0.7f - 1.0f, 1.0f);
  float effective = 2.9f * powf(d / 2.9f, 0.57f);
  effective = clampf(effective, 0.5f * d, d);
  return rmin(1.12f / effective, 50.0f) * refine * vlq;
}

/* src/frame/quantization.rs:163-178 */
static float luma_dc_coarsening(float d) {
  const float a = 1.25f, b = 1.75f, c = 4.25f, e = 5.0f;
  float t;
  if (d <= a || d >= e) t = 0.0f;
  else if (d < b) t = (d - a) / (b - a);
  else if (d <= c) t = 1.0f;
  else t = (e - d) / (e - c);
  return fmla(t, 1.15f - 1.0f, 1.0f);
}

/* src/color_correlation.rs:1835-1844 */
static float signaled_dc_step(int c, float mul) {
  static const float dc_quant[3] = {1.0f / 4096.0f, 1.0f / 512.0f, 1.0f / 256.0f};
  float wire = dc_quant[c] * 128.0f * mul;
  return f16_round(wire) / (dc_quant[c] * 128.0f);
}

/* src/frame/quantization.rs:196-216 */
static float epf_pass0_scale(float d, int* some) {
  *some = 0;
  if (d < 2.5f) return 0.0f;
  float t = dcepf_vlq_t(d);
  if (t >= 0.5f) return 0.0f;
  *some = 1;
  return fmla(2.0f * t, 0.9f - 3.6f, 3.6f);
}

typedef struct {
  float distance;
  int32_t global_scale;
  int32_t quant_dc;
  float scale;
  float scale_dc;
  uint32_t x_qm_scale;
  uint32_t b_qm_scale;
  uint32_t epf_iters;
  float dc_step[3];
  float x_qm_mul;
  float b_qm_mul;
} orc_params;

/* src/frame/quantization.rs:89-156 plus the XYB floors of
 * src/frame/vardct_encoder.rs:834-840 and src/frame/chroma.rs:410-413
 * (UltraFast: no pixel-chromacity steps, so both floors are 2). */
int orc_params_for(float distance, orc_params* p) {
  if (!(distance > 0.0f) || isinf(distance)) return ORC_ERR_DISTANCE;
  float d = rmax(distance, 0.05f);
  memset(p, 0, sizeof(*p));
  float qdc_fine = quant_dc_of(d);
  float coarsen = luma_dc_coarsening(d);
  float qdc = qdc_fine / coarsen;
  float scale = 65536.0f * 0.8f / (d * 10.0f);
  int32_t gs = sat_i32(roundf(scale));
  if (gs < 1) gs = 1;
  if (gs > (1 << 15)) gs = 1 << 15;
  float scale_f = (float)gs / 65536.0f;
  int32_t qd = sat_i32((qdc / scale_f) + 0.5f);
  if (qd < 1) qd = 1;
  if (qd > (1 << 16)) qd = 1 << 16;
  p->distance = d;
  p->global_scale = gs;
  p->quant_dc = qd;
  p->scale = scale_f;
  p->scale_dc = (float)qd * scale_f;
  uint32_t x = 2;
  if (d >= 1.25f) x += 1;
  if (d > 9.0f) x += 1;
  if (d < 0.299f) x += 1;
  p->x_qm_scale = x; /* max(x, floor=2) */
  p->b_qm_scale = 2;
  uint32_t iters = 0;
  if (d >= 0.7f) iters++;
  if (d >= 1.5f) iters++;
  int some;
  (void)epf_pass0_scale(d, &some);
  if (some || dcepf_vlq_t(d) >= 0.5f) iters = 3;
  p->epf_iters = iters;
  /* src/frame/quantization.rs:188-194 */
  float growth = rmax(quant_dc_of(3.5f) / qdc_fine, 1.0f);
  float steps[3] = {2.0f * powf(growth, 0.75f - 1.0f), 1.0f, powf(growth, 0.5f - 1.0f)};
  float in[3] = {steps[0] / coarsen, steps[1], steps[2] / coarsen};
  for (int c = 0; c < 3; c++) p->dc_step[c] = signaled_dc_step(c, in[c]);
  p->x_qm_mul = powf(1.25f, (float)p->x_qm_scale - 2.0f);
  static const float b_mul[6] = {1.0f, 1.25f, 1.5625f, 1.953125f, 2.4414062f, 3.0517578f};
  p->b_qm_mul = b_mul[p->b_qm_scale - 2];
  return ORC_OK;
}

/* src/frame/quantization.rs:218-239 */
int32_t orc_epf_sharpness_id(float distance, int screen_content) {
  float t = dcepf_vlq_t(distance);
  if (t >= 0.75f) return 1;
  if (t >= 0.5f) return 2;
  if (t >= 0.25f) return 3;
  if (distance < 1.4f || (screen_content && distance < 5.0f)) return 7;
  if (distance < 1.75f) return 6;
  if (distance < 3.5f) return 5;
  return 4;
}

/* ------------------------------------------------------------------ */
/* DCT8 quant table (src/quant_weights.rs)                              */
/* ------------------------------------------------------------------ */

static const float DCT8_BANDS[3][6] = {
    {3150.0f, 0.0f, -0.4f, -0.4f, -0.4f, -2.0f},
    {560.0f, 0.0f, -0.3f, -0.3f, -0.3f, -0.3f},
    {512.0f, -2.0f, -1.0f, 0.0f, -1.0f, -2.0f},
};
static const float FLAT_B8_HQ[6] = {512.0f, -0.5f, -0.25f, 0.0f, -0.25f, -0.5f};
static const float FLAT_B8_MID[6] = {512.0f, -0.13f, -0.235f, -0.276f, -0.609f, -0.339f};

/* src/quant_weights.rs:1002-1004 */
static float band_mult(float v) { return v > 0.0f ? 1.0f + v : 1.0f / (1.0f - v); }

/* src/quant_weights.rs:1372-1379 */
static float interpolate_bands(float pos, const float* bands) {
  float idx_f = floorf(pos);
  float frac = pos - idx_f;
  size_t idx = (size_t)idx_f;
  float a = bands[idx];
  float b = bands[idx + 1];
  return powf(b / a, frac) * a;
}

/* src/quant_weights.rs:140-200: default / coarse DCT8 override, B row
 * replaced by `flat`, every parameter F16 round-tripped. */
static void dct8_override(int coarse, const float* flat, float out[3][6]) {
  for (int c = 0; c < 3; c++)
    for (int i = 0; i < 6; i++) out[c][i] = DCT8_BANDS[c][i];
  if (coarse) {
    float hf_step = powf(1.25f, 1.0f / 5.0f);
    for (int i = 1; i < 6; i++) {
      float ratio = band_mult(DCT8_BANDS[1][i]) * hf_step;
      out[1][i] = ratio > 1.0f ? ratio - 1.0f : 1.0f - 1.0f / ratio;
    }
    for (int c = 0; c < 3; c++)
      for (int i = 0; i < 6; i++)
        out[c][i] = i == 0 ? f16_round(out[c][i] / 64.0f) * 64.0f : f16_round(out[c][i]);
  }
  for (int i = 0; i < 6; i++) out[2][i] = flat[i];
  for (int c = 0; c < 3; c++)
    for (int i = 0; i < 6; i++)
      out[c][i] = i == 0 ? f16_round(out[c][i] / 64.0f) * 64.0f : f16_round(out[c][i]);
}

/* src/quant_weights.rs:1564-1586 and fill_ac_reciprocals :3136-3141 */
static void dct8_matrix_from(const float bands_in[3][6], float* matrix, float* inv) {
  for (int c = 0; c < 3; c++) {
    float bands[6];
    bands[0] = bands_in[c][0];
    for (int i = 1; i < 6; i++) bands[i] = bands[i - 1] * band_mult(bands_in[c][i]);
    float scale = (6.0f - 1.0f) / (1.41421356237309505f + 1e-6f);
    float rcp = scale / 7.0f;
    for (int y = 0; y < 8; y++) {
      float dy = (float)y * rcp;
      float dy2 = dy * dy;
      for (int x = 0; x < 8; x++) {
        float dx = (float)x * rcp;
        float dist = sqrtf(fmla(dx, dx, dy2));
        matrix[c * 64 + y * 8 + x] = 1.0f / interpolate_bands(dist, bands);
      }
    }
    inv[c * 64] = 0.0f;
    for (int k = 1; k < 64; k++) inv[c * 64 + k] = 1.0f / matrix[c * 64 + k];
  }
}

void orc_dct8_matrix_from_bands(const float* bands18, float* matrix, float* inv) {
  float b[3][6];
  for (int c = 0; c < 3; c++)
    for (int i = 0; i < 6; i++) b[c][i] = bands18[c * 6 + i];
  dct8_matrix_from(b, matrix, inv);
}

void orc_dct8_default_bands(float* bands18) {
  for (int c = 0; c < 3; c++)
    for (int i = 0; i < 6; i++) bands18[c * 6 + i] = DCT8_BANDS[c][i];
}

#include "library_dct8.inc"

/* DequantMatrices::new_fast (src/quant_weights.rs:2294-2339) restricted to
 * its DCT8 table; arbiter SSIMULACRA2 (qm_ss2_distance 2.25).  Below 0.3 it
 * falls to DequantMatrices::new -> the library table (src/quant_weights.rs:
 * 2261-2291, shared_tables :1986-1992). */
int orc_dct8_tables(float distance, float* matrix, float* inv) {
  float d = rmax(distance, 0.05f);
  if (d < 0.3f) {
    for (int c = 0; c < 3; c++) {
      for (int k = 0; k < 64; k++) matrix[c * 64 + k] = u2f(LIBRARY_DCT8_BITS[c][k]);
      inv[c * 64] = 0.0f;
      for (int k = 1; k < 64; k++) inv[c * 64 + k] = 1.0f / matrix[c * 64 + k];
    }
    return ORC_OK;
  }
  float bands[3][6];
  if (d >= 2.25f) dct8_override(d >= 3.5f, FLAT_B8_MID, bands);
  else if (d >= 1.25f) dct8_override(0, FLAT_B8_MID, bands);
  else dct8_override(0, FLAT_B8_HQ, bands);
  dct8_matrix_from(bands, matrix, inv);
  return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* sRGB -> linear and XYB                                               */
/* ------------------------------------------------------------------ */

/* src/color.rs:35-42 */
void orc_srgb_lut(float* lut) {
  for (int v = 0; v < 256; v++) {
    double x = (double)v * (1.0 / 255.0);
    lut[v] = (float)(x <= 0.04045 ? x / 12.92 : pow((x + 0.055) / 1.055, 2.4));
  }
}

/* Transfer functions of integer samples (src/color.rs:44-222), as the
 * H.273 transfer-characteristics codes of TransferFunction
 * (src/color_encoding.rs:99-160).  Each takes the sample over the largest
 * code value and returns linear light. */
static float clamp01(float v) { return v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v); }
/* srgb_to_linear_f32 (:44-52) */
static float tf_srgb(float v) {
  v = clamp01(v);
  return v <= 0.04045f ? v / 12.92f : powf((v + 0.055f) / 1.055f, 2.4f);
}
/* linear_to_linear (:57-59) */
static float tf_linear(float v) { return clamp01(v); }
/* bt709_to_linear (:164-174) */
static float tf_bt709(float v) {
  v = clamp01(v);
  const float alpha = 1.0992968f, beta = 0.01805397f;
  return v < 4.5f * beta ? v / 4.5f : powf((v + alpha - 1.0f) / alpha, 1.0f / 0.45f);
}
/* bt470m_to_linear (:176-179), bt470bg_to_linear (:181-184),
 * smpte428_to_linear (:196-199) */
static float tf_bt470m(float v) { return powf(clamp01(v), 2.2f); }
static float tf_bt470bg(float v) { return powf(clamp01(v), 2.8f); }
static float tf_smpte428(float v) { return powf(clamp01(v), 2.6f); }
/* smpte240_to_linear (:186-194) */
static float tf_smpte240(float v) {
  v = clamp01(v);
  return v < 0.0912f ? v / 4.0f : powf((v + 0.1115f) / 1.1115f, 1.0f / 0.45f);
}

typedef float (*transfer_fn)(float);

/* select_transfer (src/color.rs:201-222) for the codes the front end takes:
 * 0 is the default encoding's sRGB (13); PQ (16) and HLG (18) need the
 * display model and are not built (NULL); anything else is invalid. */
static int select_transfer(int code, transfer_fn* fn) {
  switch (code) {
    case 1: case 6: case 14: case 15: *fn = tf_bt709; return 0;
    case 4: *fn = tf_bt470m; return 0;
    case 5: *fn = tf_bt470bg; return 0;
    case 7: *fn = tf_smpte240; return 0;
    case 8: *fn = tf_linear; return 0;
    case 17: *fn = tf_smpte428; return 0;
    case 0: case 2: case 9: case 10: case 11: case 12: case 13: *fn = tf_srgb; return 0;
    case 16: case 18: *fn = NULL; return ORC_ERR_INPUT;
    default: *fn = NULL; return ORC_ERR_INPUT;
  }
}

/* TransferLut::build (src/color.rs:297-333) for `bits` 8, 10, 12 or 16:
 * 256 entries for 8-bit samples, else 65536 (codes above the largest are 0).
 * 8-bit sRGB takes the f64 table of srgb_to_linear_u8_ref. */
int orc_transfer_lut(int bits, int transfer, float* lut) {
  transfer_fn fn;
  if (bits != 8 && bits != 10 && bits != 12 && bits != 16) return ORC_ERR_INPUT;
  int st = select_transfer(transfer, &fn);
  if (st) return st;
  const int size = 1 << bits, domain = bits <= 8 ? 256 : 65536;
  if (bits == 8 && (transfer == 13 || transfer == 0)) {
    orc_srgb_lut(lut);
    return 0;
  }
  const float max = (float)(size - 1);
  for (int v = 0; v < domain; v++) lut[v] = v < size ? fn((float)v / max) : 0.0f;
  return 0;
}

#define OPSIN_BIAS 0.0037930734f
#define NEG_BIAS_CBRT (-0.1559542f)

/* src/xyb.rs:145-150 */
static inline float halley(float x, float a) {
  float tx = x * x * x;
  return x * fmla(2.0f, a, tx) / fmla(2.0f, tx, a);
}

/* src/xyb.rs:152-167: bit-hack seed (B1 = 709958130) + two Halley steps */
static inline float xyb_cbrtf(float x) {
  if (x == 0.0f) return x;
  uint32_t ui = f2u(x);
  uint32_t hx = ui & 0x7fffffffu;
  hx = hx / 3u + 709958130u;
  ui &= 0x80000000u;
  ui |= hx;
  float t = u2f(ui);
  t = halley(t, x);
  return halley(t, x);
}

/* XybMatrix::SPEC (src/xyb.rs:35-48, :81-85) */
static void opsin_matrix(float m[9]) {
  const float m00 = 0.30f, m02 = 0.078f;
  const float m01 = 1.0f - m02 - m00;
  const float m10 = 0.23f, m12 = 0.078f;
  const float m11 = 1.0f - m12 - m10;
  const float b_bias = 0.55180986f;
  const float ratio = 0.24342269f / (0.24342269f + 0.20476745f);
  const float m20 = ratio * (1.0f - b_bias);
  const float m21 = (1.0f - ratio) * (1.0f - b_bias);
  const float m22 = 1.0f - m20 - m21;
  m[0] = m00; m[1] = m01; m[2] = m02;
  m[3] = m10; m[4] = m11; m[5] = m12;
  m[6] = m20; m[7] = m21; m[8] = m22;
}

void orc_opsin_matrix(float* m) { opsin_matrix(m); }

/* src/xyb.rs:172-185 */
static inline void rgb_to_xyb(const float m[9], float r, float g, float b, float* ox,
                              float* oy, float* ob) {
  float mixed0 = fmla(m[0], r, fmla(m[1], g, fmla(m[2], b, OPSIN_BIAS)));
  float mixed1 = fmla(m[3], r, fmla(m[4], g, fmla(m[5], b, OPSIN_BIAS)));
  float mixed2 = fmla(m[6], r, fmla(m[7], g, fmla(m[8], b, OPSIN_BIAS)));
  float tm0 = xyb_cbrtf(rmax(mixed0, 0.0f)) + NEG_BIAS_CBRT;
  float tm1 = xyb_cbrtf(rmax(mixed1, 0.0f)) + NEG_BIAS_CBRT;
  float tm2 = xyb_cbrtf(rmax(mixed2, 0.0f)) + NEG_BIAS_CBRT;
  *ox = 0.5f * (tm0 - tm1);
  *oy = 0.5f * (tm0 + tm1);
  *ob = tm2;
}

/* linearize_rgb (src/encode_image.rs:1498-1519) with the integer
 * ColorTransform of sRGB primaries (transform_identity, src/color.rs:498-509:
 * each sample through the transfer LUT) + to_xyb_in_place
 * (src/xyb.rs:439-470).  8-bit samples, or 10/12/16-bit samples in 16-bit
 * words; 3 or 4 channels, alpha ignored.  Returns 0, or ORC_ERR_INPUT for a
 * depth or transfer the front end does not take. */
int orc_to_xyb(const void* pixels, int bits, int transfer, int channels, size_t w, size_t h,
               float* xyb) {
  float* lut = (float*)malloc(65536 * sizeof(float));
  if (!lut) return ORC_ERR_ALLOC;
  int st = orc_transfer_lut(bits, transfer, lut);
  if (st) {
    free(lut);
    return st;
  }
  float m[9];
  opsin_matrix(m);
  size_t n = w * h;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (size_t i = 0; i < n; i++) {
    float r, g, b;
    /* grey (1 or 2 channels): R = G = B, linearize_gray (src/encode_image.rs:1571-1600) */
    const int cg = channels < 3 ? 0 : 1, cb = channels < 3 ? 0 : 2;
    if (bits == 8) {
      const uint8_t* p = (const uint8_t*)pixels + i * (size_t)channels;
      r = lut[p[0]];
      g = lut[p[cg]];
      b = lut[p[cb]];
    } else {
      const uint16_t* p = (const uint16_t*)pixels + i * (size_t)channels;
      r = lut[p[0]];
      g = lut[p[cg]];
      b = lut[p[cb]];
    }
    rgb_to_xyb(m, r, g, b, &xyb[i], &xyb[n + i], &xyb[2 * n + i]);
  }
  free(lut);
  return 0;
}

/* snap_achromatic_xyb (src/frame/encoder.rs:351-357): X = 0, B = Y */
void orc_snap_achromatic(float* xyb, size_t n) {
  for (size_t i = 0; i < n; i++) {
    xyb[i] = 0.0f;
    xyb[2 * n + i] = xyb[n + i];
  }
}

/* ------------------------------------------------------------------ */
/* Frame statistics (src/frame/chroma.rs)                               */
/* ------------------------------------------------------------------ */

/* constant_block_fraction numerator (src/frame/chroma.rs:48-68) */
uint64_t orc_constant_blocks(const float* xyb, size_t w, size_t h) {
  size_t bw = w / 8, bh = h / 8, n = w * h;
  uint64_t count = 0;
  for (size_t by = 0; by < bh; by++)
    for (size_t bx = 0; bx < bw; bx++) {
      int constant = 1;
      for (int c = 0; c < 3 && constant; c++) {
        const float* p = xyb + (size_t)c * n;
        float v = p[by * 8 * w + bx * 8];
        for (int iy = 0; iy < 8 && constant; iy++)
          for (int ix = 0; ix < 8; ix++)
            if (!(p[(by * 8 + iy) * w + bx * 8 + ix] == v)) { constant = 0; break; }
      }
      count += (uint64_t)constant;
    }
  return count;
}

/* is_screen_content (src/frame/chroma.rs:42-44) */
int orc_is_screen_content(uint64_t constant, size_t w, size_t h) {
  size_t bw = w / 8, bh = h / 8;
  if (bw == 0 || bh == 0) return 0;
  return (float)constant / (float)(bw * bh) >= 0.15f;
}

/* pixel_chromacity_steps (src/frame/chroma.rs:89-165): over every pixel
 * with a left and an upper neighbour, the counts of X steps reaching
 * 0.015 / 0.022 / 0.026, of B - Y steps above 0.28 / 0.33 / 0.38, and of
 * strongly exposed blue; then the extra X and B quant-scale steps, each level
 * needing 4 pixels.  counts = {x[3], b[3], exposed blue}, steps = {x, b}. */
void orc_pixel_chromacity(const float* xyb, size_t w, size_t h, uint32_t counts[7],
                          uint32_t steps[2]) {
  static const float x_levels[3] = {0.015f, 0.022f, 0.026f};
  static const float b_levels[3] = {0.28f, 0.33f, 0.38f};
  const size_t n = w * h;
  for (int k = 0; k < 7; k++) counts[k] = 0;
  steps[0] = steps[1] = 0;
  if (w < 2 || h < 2) return;
  const float *X = xyb, *Y = xyb + n, *B = xyb + 2 * n;
  for (size_t y = 1; y < h; y++) {
    const size_t r = y * w, u = (y - 1) * w;
    float left_x = X[r], left_b = B[r], left_diff = B[r] - Y[r];
    for (size_t x = 1; x < w; x++) {
      const float xv = X[r + x], yv = Y[r + x], bv = B[r + x];
      const float px = X[u + x], py = Y[u + x], pb = B[u + x];
      const float step_x = fmaxf(fabsf(xv - left_x), fabsf(xv - px));
      const float diff_b = bv - yv;
      const float step_b = fmaxf(fabsf(diff_b - left_diff), fabsf(diff_b - (pb - py)));
      for (int k = 0; k < 3; k++) {
        counts[k] += step_x >= x_levels[k];
        counts[3 + k] += step_b > b_levels[k];
      }
      const float step = fabsf(bv - left_b) + fabsf(bv - pb);
      counts[6] += (bv - yv * 1.2f) * step >= 0.13f;
      left_x = xv;
      left_b = bv;
      left_diff = diff_b;
    }
  }
  uint32_t lx = 0, lb = 0;
  for (int k = 0; k < 3; k++) {
    lx += counts[k] >= 4u;
    lb += counts[3 + k] >= 4u;
  }
  steps[0] = lx;
  steps[1] = lb == 0 ? 0 : lb - 1 + (counts[6] > 0);
}

/* ------------------------------------------------------------------ */
/* Adaptive quantisation (src/adaptive_quant.rs)                        */
/* ------------------------------------------------------------------ */

#define K_SG_MUL 226.77216153508914f
#define K_SG_MUL2 (1.0f / 73.377132366608819f)
#define K_LOG2 0.693147181f
#define K_SG_RET_MUL (K_SG_MUL2 * 18.6580932135f * K_LOG2)
#define K_SG_V_OFFSET 7.7825991679894591f

/* src/adaptive_quant.rs:53-64 (both INVERT forms) */
static inline float ratio_gamma(float v, int invert) {
  const float eps = 1e-2f;
  v = v < 0.0f ? 0.0f : v;
  const float num_mul = K_SG_RET_MUL * 3.0f * K_SG_MUL;
  const float v_offset = K_SG_V_OFFSET * K_LOG2 + eps;
  const float den_mul = K_LOG2 * K_SG_MUL;
  float v2 = v * v;
  float num = num_mul * v2 + eps;
  float den = (den_mul * v) * v2 + v_offset;
  return invert ? num / den : den / num;
}

/* src/adaptive_quant.rs:67-83 */
static inline float compute_mask(float out_val) {
  const float k_base = -0.699765f;
  const float k_mul4 = 9.4708735624378946f;
  const float k_mul2 = 17.35036561631863f;
  const float k_offset2 = 302.59587815579727f;
  const float k_mul3 = 6.7943250517376494f;
  const float k_offset3 = 3.7179635626140772f;
  const float k_offset4 = 0.25f * k_offset3;
  const float k_mul0 = 1.07267f;
  float v1 = rmax(out_val * k_mul0, 1e-3f);
  float v2 = 1.0f / (v1 + k_offset2);
  float v3 = 1.0f / (v1 * v1 + k_offset3);
  float v4 = 1.0f / (v1 * v1 + k_offset4);
  return fmla(k_mul4, v4, fmla(k_mul2, v2, fmla(k_mul3, v3, k_base)));
}

/* src/adaptive_quant.rs:86-92 */
static inline float masking_sqrt(float v) {
  const float k_log_offset = 27.505837037000106f;
  const float k_mul = 211.66567973503678f;
  const float mul_v = k_mul * 1e8f;
  return 0.25f * sqrtf(fmla(v, sqrtf(mul_v), k_log_offset));
}

static const float AQ_KNOTS[7] = {0.5f, 1.0f, 1.4f, 1.75f, 3.0f, 5.0f, 8.0f};
static const float AQ_STRENGTH[7] = {0.26565f, 0.275459f, 0.058287f, 0.0f, 0.0f, 0.0f, 0.0f};
static const float AQ_BASE[7] = {0.636493f, 0.648351f, 0.606759f, 0.48f, 0.48f, 0.48f, 0.48f};

/* src/adaptive_quant.rs:105-116 */
static float aq_schedule(const float* values, float d) {
  if (d <= AQ_KNOTS[0]) return values[0];
  for (int i = 1; i < 7; i++)
    if (d <= AQ_KNOTS[i]) {
      float f = (d - AQ_KNOTS[i - 1]) / (AQ_KNOTS[i] - AQ_KNOTS[i - 1]);
      return values[i - 1] + f * (values[i] - values[i - 1]);
    }
  return values[6];
}

/* src/adaptive_quant.rs:739-765 fast_exp2: 2^(i/64) table lookup, where the
 * table holds 2^((i - 32) / 64) rounded to f32 (FreeBSD exp2f method). */
static float exp2_table[64];
static int exp2_table_ready = 0;
static void init_exp2_table(void) {
  if (exp2_table_ready) return;
  for (int i = 0; i < 64; i++) exp2_table[i] = (float)exp2((double)(i - 32) / 64.0);
  exp2_table_ready = 1;
}
void orc_exp2_table(float* out) {
  init_exp2_table();
  memcpy(out, exp2_table, sizeof(exp2_table));
}

static inline float fast_exp2(float d) {
  const float redux = u2f(0x4b400000u) / 64.0f;
  uint32_t ui = f2u(d + redux);
  uint32_t i0 = ui + 32u;
  uint32_t k = i0 / 64u;
  i0 &= 63u;
  float uf = u2f(ui);
  uf -= redux;
  float z0 = exp2_table[i0];
  float f = d - uf;
  float u = 0.24022650695908768f;
  u = fmla(u, f, 0.69314718055994973f);
  u *= f;
  float i2 = u2f((uint32_t)((int32_t)k + 0x7f) << 23);
  return fmla(u, z0, z0) * i2;
}

/* src/adaptive_quant.rs:768-783 */
static inline float dirty_log2f(float d) {
  uint32_t ix = f2u(d);
  ix += 0x3f800000u - 0x3f3504f3u;
  int32_t n = (int32_t)(ix >> 23) - 0x7f;
  ix = (ix & 0x007fffffu) + 0x3f3504f3u;
  float a = u2f(ix);
  float x = (a - 1.0f) / (a + 1.0f);
  float x2 = x * x;
  float u = 0.4121985850084821691e+0f;
  u = fmla(u, x2, 0.5770780163490337802e+0f);
  u = fmla(u, x2, 0.9617966939259845749e+0f);
  return fmla(x2 * x, u, fmla(x, 0.2885390081777926802e+1f, (float)n));
}

float orc_fast_exp2(float d) { init_exp2_table(); return fast_exp2(d); }
float orc_dirty_log2f(float d) { return dirty_log2f(d); }

static inline size_t minz(size_t a, size_t b) { return a < b ? a : b; }

/* src/adaptive_quant.rs:410-433 */
static float gamma_modulation(size_t x, size_t y, const float* xyb, size_t w, size_t h,
                              float out_val) {
  const float k_bias = 0.16f;
  float overall = 0.0f;
  const float* px = xyb;
  const float* py = xyb + w * h;
  for (size_t dy = 0; dy < 8; dy++) {
    size_t ry = minz(y + dy, h - 1);
    for (size_t dx = 0; dx < 8; dx++) {
      size_t cx = minz(x + dx, w - 1);
      float iny = py[ry * w + cx] + k_bias;
      float inx = px[ry * w + cx];
      float r = iny - inx;
      float g = iny + inx;
      float rr = ratio_gamma(r, 1);
      float rg = ratio_gamma(g, 1);
      overall = fmla(0.5f, rr + rg, overall);
    }
  }
  overall *= 1.0f / 64.0f;
  const float k_gam = 0.119146f;
  return fmla(k_gam, dirty_log2f(overall), out_val);
}

/* src/adaptive_quant.rs:122-148 */
static float hf_modulation(size_t x, size_t y, const float* xyb, size_t w, size_t h,
                           float out_val, float strength) {
  const float* yp = xyb + w * h;
  const float valmin = 0.0206f;
  float sum = 0.0f;
  for (size_t dy = 0; dy < 8; dy++) {
    const float* row = yp + minz(y + dy, h - 1) * w;
    const float* next = dy == 7 ? row : yp + minz(y + dy + 1, h - 1) * w;
    for (size_t dx = 0; dx < 8; dx++) {
      size_t c0 = minz(x + dx, w - 1);
      float p = row[c0];
      if (dx < 7) sum += rmin(valmin, fabsf(p - row[minz(x + dx + 1, w - 1)]));
      sum += rmin(valmin, fabsf(p - next[c0]));
    }
  }
  float k_mul = -0.506626f * strength;
  const float k_offset = 0.655866f;
  return fmla(sum, k_mul, k_offset) + out_val;
}

/* src/adaptive_quant.rs:153-183 */
static float blue_modulation(size_t x, size_t y, const float* xyb, size_t w, size_t h,
                             float out_val) {
  const float k_limit = 0.010474084867598155f;
  const float k_offset = 0.0031994768654636393f;
  const float* xp = xyb;
  const float* yp = xyb + w * h;
  const float* bp = xyb + 2 * w * h;
  float sum = 0.0f;
  for (size_t dy = 0; dy < 8; dy++) {
    size_t ry = minz(y + dy, h - 1);
    for (size_t dx = 0; dx < 8; dx++) {
      size_t cx = minz(x + dx, w - 1);
      float p_x = xp[ry * w + cx];
      float p_b = bp[ry * w + cx];
      float p_y = yp[ry * w + cx] + k_offset + fabsf(p_x);
      if (p_b > p_y) sum += rmin(p_b - p_y, k_limit);
    }
  }
  const float k_mul = 0.127191f;
  float s = sum;
  if (s >= 32.0f * k_limit) s = 64.0f * k_limit - s;
  const float k_max_limit = 15.463398341612438f;
  if (s >= k_max_limit * k_limit) s = k_max_limit * k_limit;
  s *= k_mul;
  return s + out_val;
}

static inline void sort4(float a[4]) {
#define CSWAP(i, j) if (a[i] > a[j]) { float t_ = a[i]; a[i] = a[j]; a[j] = t_; }
  CSWAP(0, 1) CSWAP(2, 3) CSWAP(0, 2) CSWAP(1, 3) CSWAP(1, 2)
#undef CSWAP
}

static inline void store_min4(float v, float m[4]) {
  if (v < m[3]) {
    if (v < m[0]) { m[3] = m[2]; m[2] = m[1]; m[1] = m[0]; m[0] = v; }
    else if (v < m[1]) { m[3] = m[2]; m[2] = m[1]; m[1] = v; }
    else if (v < m[2]) { m[3] = m[2]; m[2] = v; }
    else m[3] = v;
  }
}

/* fill_quant_field_scalar (src/adaptive_quant.rs:547-727) for the DC group
 * whose pixel origin is (x0, y0) and whose block extent is xb x yb.  Writes
 * the raw field into `qf` (image block raster, stride `qf_stride`). */
static void fill_quant_field(const float* xyb, size_t w, size_t h, size_t x0, size_t y0,
                             size_t xb, size_t yb, float distance, float inv_scale,
                             uint8_t* qf, size_t qf_stride) {
  const float* yp = xyb + w * h;
  float scale = 0.8294f / distance;
  size_t rw = xb * 8, rh = yb * 8;
  size_t pw = rw / 4, ph = rh / 4;
  float* acc = (float*)malloc(rw * sizeof(float));
  float* pre = (float*)malloc(pw * ph * sizeof(float));
  float* aq = (float*)malloc(xb * yb * sizeof(float));
  for (size_t ry = 0; ry < rh; ry++) {
    long gy = (long)(y0 + ry);
    size_t gyc = (size_t)(gy < (long)h - 1 ? gy : (long)h - 1);
    size_t gy1 = (size_t)(gy - 1 < 0 ? 0 : (gy - 1 > (long)h - 1 ? (long)h - 1 : gy - 1));
    size_t gy2 = (size_t)(gy + 1 > (long)h - 1 ? (long)h - 1 : gy + 1);
    const float* row = yp + gyc * w;
    const float* row1 = yp + gy1 * w;
    const float* row2 = yp + gy2 * w;
    for (size_t rx = 0; rx < rw; rx++) {
      long gx = (long)(x0 + rx);
      size_t gxc = (size_t)(gx < (long)w - 1 ? gx : (long)w - 1);
      size_t gx1 = (size_t)(gx - 1 < 0 ? 0 : (gx - 1 > (long)w - 1 ? (long)w - 1 : gx - 1));
      size_t gx2 = (size_t)(gx + 1 > (long)w - 1 ? (long)w - 1 : gx + 1);
      float in_y = row[gxc];
      float base = 0.25f * (row2[gxc] + row1[gxc] + row[gx1] + row[gx2]);
      float gammac = ratio_gamma(in_y + 0.019f, 0);
      float diff = gammac * (in_y - base);
      diff *= diff;
      if (diff >= 0.2f) diff = 0.2f;
      diff = masking_sqrt(diff);
      if ((ry & 3) != 0) acc[rx] += diff;
      else acc[rx] = diff;
    }
    if (ry % 4 == 3) {
      float* prow = pre + (ry / 4) * pw;
      for (size_t px = 0; px < pw; px++)
        prow[px] = (acc[px * 4] + acc[px * 4 + 1] + acc[px * 4 + 2] + acc[px * 4 + 3]) * 0.25f;
    }
  }
  float fe_mul = distance < 2.0f ? (2.0f - distance) * 0.5f : 0.0f;
  const float fe_base[4] = {0.125f, 0.1f, 0.09f, 0.06f};
  const float fe_add[4] = {0.0f, -0.1f, -0.09f, -0.06f};
  float kmul[4];
  float norm = 0.0f;
  for (int i = 0; i < 4; i++) {
    kmul[i] = fe_base[i] + fe_mul * fe_add[i];
    norm += kmul[i];
  }
  const float k_total = 0.29959705784054957f;
  for (int i = 0; i < 4; i++) kmul[i] *= k_total / norm;
  for (size_t fy = 0; fy < ph; fy++) {
    size_t ym1 = fy >= 1 ? fy - 1 : fy;
    size_t yp1 = fy + 1 < ph ? fy + 1 : fy;
    const float* rt = pre + ym1 * pw;
    const float* r = pre + fy * pw;
    const float* rb = pre + yp1 * pw;
    for (size_t fx = 0; fx < pw; fx++) {
      size_t xm1 = fx >= 1 ? fx - 1 : fx;
      size_t xp1 = fx + 1 < pw ? fx + 1 : fx;
      float m[4] = {r[fx], r[xm1], r[xp1], rt[xm1]};
      sort4(m);
      store_min4(rt[fx], m);
      store_min4(rt[xp1], m);
      store_min4(rb[xm1], m);
      store_min4(rb[fx], m);
      store_min4(rb[xp1], m);
      float v = kmul[0] * m[0] + kmul[1] * m[1] + kmul[2] * m[2] + kmul[3] * m[3];
      size_t idx = (fy / 2) * xb + fx / 2;
      if (fx % 2 == 0 && fy % 2 == 0) aq[idx] = v;
      else aq[idx] += v;
    }
  }
  float base_level = aq_schedule(AQ_BASE, distance) * scale;
  float dampen = clampf(aq_schedule(AQ_STRENGTH, distance), 0.0f, 1.0f);
  float mul = scale * dampen;
  float add = (1.0f - dampen) * base_level;
  float strength = clampf(1.06836f * distance, 0.1f, 0.890398f);
  for (size_t by = 0; by < yb; by++) {
    size_t py = y0 + by * 8;
    for (size_t bx = 0; bx < xb; bx++) {
      size_t px = x0 + bx * 8;
      uint8_t* out = qf + (y0 / 8 + by) * qf_stride + x0 / 8 + bx;
      if (px >= w || py >= h) { *out = 1; continue; }
      size_t bxp = minz(px, w >= 8 ? w - 8 : 0);
      size_t byp = minz(py, h >= 8 ? h - 8 : 0);
      float mask = compute_mask(aq[by * xb + bx]);
      mask = gamma_modulation(bxp, byp, xyb, w, h, mask);
      float out_val = hf_modulation(bxp, byp, xyb, w, h, mask, strength);
      out_val = rmin(out_val, blue_modulation(bxp, byp, xyb, w, h, mask));
      float q = fast_exp2(out_val * 1.442695041f) * mul + add;
      int32_t qi = sat_i32(fmla(q, inv_scale, 0.5f));
      *out = (uint8_t)(qi < 1 ? 1 : (qi > 255 ? 255 : qi));
    }
  }
  free(acc);
  free(pre);
  free(aq);
}

/* ------------------------------------------------------------------ */
/* DCT8 (src/dct.rs:55-133, :631-659)                                   */
/* ------------------------------------------------------------------ */

static const float WC4_0 = 0.5411961f, WC4_1 = 1.306563f;
static const float WC8[4] = {0.5097956f, 0.6013449f, 0.8999762f, 2.5629156f};
#define SQRT2F 1.41421356237309505f

static inline void dct1d_4(float* b) {
  float t0 = b[0] + b[3];
  float t1 = b[1] + b[2];
  float a = t0, c = t1;
  t0 = a + c;
  t1 = a - c;
  float t2 = b[0] - b[3];
  float t3 = b[1] - b[2];
  t2 *= WC4_0;
  t3 *= WC4_1;
  a = t2;
  c = t3;
  t2 = a + c;
  t3 = a - c;
  t2 = fmla(t2, SQRT2F, t3);
  b[0] = t0;
  b[2] = t1;
  b[1] = t2;
  b[3] = t3;
}

static inline void dct1d_8(float* b) {
  float t[8];
  for (int i = 0; i < 4; i++) t[i] = b[i] + b[7 - i];
  dct1d_4(t);
  for (int i = 0; i < 4; i++) t[4 + i] = (b[i] - b[7 - i]) * WC8[i];
  dct1d_4(t + 4);
  t[4] = fmla(t[4], SQRT2F, t[5]);
  t[5] += t[6];
  t[6] += t[7];
  for (int i = 0; i < 4; i++) {
    b[2 * i] = t[i];
    b[2 * i + 1] = t[4 + i];
  }
}

/* dct8x8_scalar_input: rows, then columns stored transposed, scaled 1/64. */
static void dct8x8(const float* in, size_t stride, float* out) {
  float tmp[64];
  for (int y = 0; y < 8; y++) {
    float row[8];
    for (int x = 0; x < 8; x++) row[x] = in[y * stride + x];
    dct1d_8(row);
    for (int x = 0; x < 8; x++) tmp[y * 8 + x] = row[x];
  }
  for (int x = 0; x < 8; x++) {
    float col[8];
    for (int y = 0; y < 8; y++) col[y] = tmp[y * 8 + x];
    dct1d_8(col);
    for (int y = 0; y < 8; y++) out[x * 8 + y] = col[y] * (1.0f / 64.0f);
  }
}

void orc_dct8x8(const float* in, float* out) { dct8x8(in, 8, out); }

/* ---- transforms of the larger DCT blocks (src/dct.rs) ---------------- */

static const float WC16[8] = {0.5024193f, 0.5224986f, 0.566944f,  0.6468218f,
                              0.7881546f, 1.0606777f, 1.7224471f, 5.1011486f};
static const float WC32[16] = {0.50060298f, 0.50547096f, 0.5154473f, 0.5310426f,
                               0.5531039f,  0.582935f,   0.6225041f, 0.67480834f,
                               0.7445363f,  0.83934965f, 0.97256825f, 1.16944f,
                               1.4841646f,  2.057781f,   3.4076084f, 10.190008f};

/* dct1d_16 (src/dct.rs:687-716): mirrored sums and differences, the sums
 * through dct1d_8, the differences scaled by WC16 and through dct1d_8, the
 * odd half's running sums, interleaved. */
static inline void dct1d_16(float* b) {
  float t[16];
  for (int i = 0; i < 8; i++) {
    t[i] = b[i] + b[15 - i];
    t[8 + i] = b[i] - b[15 - i];
  }
  dct1d_8(t);
  for (int i = 0; i < 8; i++) t[8 + i] *= WC16[i];
  dct1d_8(t + 8);
  t[8] = fmla(t[8], SQRT2F, t[9]);
  for (int i = 9; i < 15; i++) t[i] += t[i + 1];
  for (int i = 0; i < 8; i++) {
    b[2 * i] = t[i];
    b[2 * i + 1] = t[8 + i];
  }
}

/* dct1d_32 (src/dct.rs:1477-1496), the same recursion over dct1d_16. */
static inline void dct1d_32(float* b) {
  float t[32];
  for (int i = 0; i < 16; i++) {
    t[i] = b[i] + b[31 - i];
    t[16 + i] = b[i] - b[31 - i];
  }
  dct1d_16(t);
  for (int i = 0; i < 16; i++) t[16 + i] *= WC32[i];
  dct1d_16(t + 16);
  t[16] = fmla(t[16], SQRT2F, t[17]);
  for (int i = 17; i < 31; i++) t[i] += t[i + 1];
  for (int i = 0; i < 16; i++) {
    b[2 * i] = t[i];
    b[2 * i + 1] = t[16 + i];
  }
}

/* WC64 (src/dct.rs:2404-2437), the reference's literals rounded to float. */
static const float WC64[32] = {
    0x1.0013bep-1f, 0x1.00b20ep-1f, 0x1.01f098p-1f, 0x1.03d342p-1f,
    0x1.06600ap-1f, 0x1.099f32p-1f, 0x1.0d9b8ap-1f, 0x1.1262c6p-1f,
    0x1.1805f4p-1f, 0x1.1e9a26p-1f, 0x1.263934p-1f, 0x1.2f02d6p-1f,
    0x1.391e0cp-1f, 0x1.44baf8p-1f, 0x1.52157p-1f, 0x1.617874p-1f,
    0x1.7343p-1f, 0x1.87eedap-1f, 0x1.a01a7ep-1f, 0x1.bc97aep-1f,
    0x1.de81bep-1f, 0x1.03b042p+0f, 0x1.1cb0bap+0f, 0x1.3bdc76p+0f,
    0x1.63a8c4p+0f, 0x1.980e92p+0f, 0x1.dfeac4p+0f, 0x1.241a36p+1f,
    0x1.765a3ap+1f, 0x1.056a44p+2f, 0x1.b2fdf6p+2f, 0x1.45fb68p+4f,
};

/* dct1d_64 (src/dct.rs:2529-2546), the same recursion over dct1d_32. */
static inline void dct1d_64(float* b) {
  float t[64];
  for (int i = 0; i < 32; i++) {
    t[i] = b[i] + b[63 - i];
    t[32 + i] = (b[i] - b[63 - i]) * WC64[i];
  }
  dct1d_32(t);
  dct1d_32(t + 32);
  t[32] = fmla(t[32], SQRT2F, t[33]);
  for (int i = 33; i < 63; i++) t[i] += t[i + 1];
  for (int i = 0; i < 32; i++) {
    b[2 * i] = t[i];
    b[2 * i + 1] = t[32 + i];
  }
}

/* WC128 (src/dct128.rs:76-141), the reference's literals rounded to float. */
static const float WC128[64] = {
    0x1.0004fp-1f, 0x1.002c7p-1f, 0x1.007b9p-1f, 0x1.00f28ep-1f,
    0x1.0191c2p-1f, 0x1.0259aep-1f, 0x1.034aecp-1f, 0x1.04663ap-1f,
    0x1.05ac7cp-1f, 0x1.071ebap-1f, 0x1.08be24p-1f, 0x1.0a8c1p-1f,
    0x1.0c8a06p-1f, 0x1.0eb9bap-1f, 0x1.111d12p-1f, 0x1.13b632p-1f,
    0x1.168776p-1f, 0x1.19937ep-1f, 0x1.1cdd2ep-1f, 0x1.2067c4p-1f,
    0x1.2436ccp-1f, 0x1.284e3cp-1f, 0x1.2cb272p-1f, 0x1.31684ap-1f,
    0x1.367524p-1f, 0x1.3bdfp-1f, 0x1.41ac88p-1f, 0x1.47e52cp-1f,
    0x1.4e914p-1f, 0x1.55ba12p-1f, 0x1.5d6a1ap-1f, 0x1.65ad26p-1f,
    0x1.6e9088p-1f, 0x1.78235ep-1f, 0x1.8276d8p-1f, 0x1.8d9e9ap-1f,
    0x1.99b12ep-1f, 0x1.a6c88cp-1f, 0x1.b502c4p-1f, 0x1.c482ep-1f,
    0x1.d571ep-1f, 0x1.e8001ep-1f, 0x1.fc66f4p-1f, 0x1.09757ep+0f,
    0x1.15ef74p+0f, 0x1.23d3aep+0f, 0x1.335ffap+0f, 0x1.44e132p+0f,
    0x1.58b8p+0f, 0x1.6f5fc6p+0f, 0x1.897872p+0f, 0x1.a7d52cp+0f,
    0x1.cb9292p+0f, 0x1.f639b2p+0f, 0x1.14fc92p+1f, 0x1.350332p+1f,
    0x1.5da68cp+1f, 0x1.92e00ap+1f, 0x1.db8d12p+1f, 0x1.225298p+2f,
    0x1.74f8d8p+2f, 0x1.04ec54p+3f, 0x1.b2b282p+3f, 0x1.45f52p+5f,
};

/* dct1d_128 (src/dct128.rs:330-350), the recursion over dct1d_64. */
static inline void dct1d_128(float* b) {
  float t[128];
  for (int i = 0; i < 64; i++) {
    t[i] = b[i] + b[127 - i];
    t[64 + i] = (b[i] - b[127 - i]) * WC128[i];
  }
  dct1d_64(t);
  dct1d_64(t + 64);
  t[64] = fmla(t[64], SQRT2F, t[65]);
  for (int i = 65; i < 127; i++) t[i] += t[i + 1];
  for (int i = 0; i < 64; i++) {
    b[2 * i] = t[i];
    b[2 * i + 1] = t[64 + i];
  }
}

static inline void dct1d_n(float* b, int n) {
  if (n == 8) dct1d_8(b);
  else if (n == 16) dct1d_16(b);
  else if (n == 32) dct1d_32(b);
  else if (n == 64) dct1d_64(b);
  else dct1d_128(b);
}

/* An H x W block (H rows of W samples), columns first: each column through
 * the H-point transform, then each row through the W-point one, stored
 * out[u * H + v] scaled by 1 / (W H) -- dct16x8 (src/dct.rs:904),
 * dct16x16 (:1010), dct32x32 (:1980), dct32x16 (:2251), dct32x8 (:1742),
 * dct64x64 (:2576), dct64x32 (:2659); src/dct128.rs dct128x128 :385,
 * dct128x64 :416. */
static void dct_cols_first(const float* in, int W, int H, float* out) {
  float* after = malloc(sizeof(float) * (size_t)(W * H));
  float col[128], row[128];
  for (int u = 0; u < W; u++) {
    for (int i = 0; i < H; i++) col[i] = in[i * W + u];
    dct1d_n(col, H);
    for (int v = 0; v < H; v++) after[v * W + u] = col[v];
  }
  const float scale = 1.0f / (float)(W * H);
  for (int v = 0; v < H; v++) {
    for (int u = 0; u < W; u++) row[u] = after[v * W + u];
    dct1d_n(row, W);
    for (int u = 0; u < W; u++) out[u * H + v] = row[u] * scale;
  }
  free(after);
}

/* Rows first, then columns, stored out[v * W + u] -- dct8x16
 * (src/dct.rs:823), dct16x32 (:2340), dct8x32 (:1777), dct32x64 (:2689);
 * dct64x128 (src/dct128.rs:446). */
static void dct_rows_first(const float* in, int W, int H, float* out) {
  float* after = malloc(sizeof(float) * (size_t)(W * H));
  float col[128], row[128];
  for (int i = 0; i < H; i++) {
    for (int u = 0; u < W; u++) row[u] = in[i * W + u];
    dct1d_n(row, W);
    for (int u = 0; u < W; u++) after[i * W + u] = row[u];
  }
  const float scale = 1.0f / (float)(W * H);
  for (int u = 0; u < W; u++) {
    for (int i = 0; i < H; i++) col[i] = after[i * W + u];
    dct1d_n(col, H);
    for (int v = 0; v < H; v++) out[v * W + u] = col[v] * scale;
  }
  free(after);
}

/* idct1d_4 of the DC extraction (src/dct.rs:2144-2167). */
static void idct1d_4(const float v[4], float out[4]) {
  float t0 = v[0], t1 = v[2], t2 = v[1], t3 = v[3];
  const float e0 = t0 + t1, e1 = t0 - t1;
  t0 = e0;
  t1 = e1;
  t3 += t2;
  t2 *= SQRT2F;
  const float o0 = t2 + t3, o1 = t2 - t3;
  t2 = o0;
  t3 = o1;
  out[0] = fmla(WC4_0, t2, t0);
  out[3] = fmla(-WC4_0, t2, t0);
  out[1] = fmla(WC4_1, t3, t1);
  out[2] = fmla(-WC4_1, t3, t1);
}

static inline void inv_dct1d_8(float* b);
static inline void inv_dct1d_16(float* b);
static void idct_square(const float* c, int n, float* out);

static const float R16_2[2] = {1.0f, 0.9017642f};                         /* :927 */
static const float R32_4[4] = {1.0f, 0.9748868f, 0.9017642f, 0.7870549f};  /* :2018 */
/* RESAMPLE_SCALE_64_TO_8 (:2005-2014) */
static const float R64_8[8] = {
    0x1p+0f, 0x1.fcc47ep-1f, 0x1.f3245ep-1f, 0x1.e35656p-1f,
    0x1.cdb40ap-1f, 0x1.b2b7aap-1f, 0x1.92f8dcp-1f, 0x1.6f28ccp-1f,
};

/* RESAMPLE_SCALE_128_TO_16 (src/dct128.rs:48-65) */
static const float R128_16[16] = {
    0x1p+0f, 0x1.ff30d6p-1f, 0x1.fcc47ep-1f, 0x1.f8be6cp-1f,
    0x1.f3245ep-1f, 0x1.ebfe48p-1f, 0x1.e35656p-1f, 0x1.d938d2p-1f,
    0x1.cdb40ap-1f, 0x1.c0d848p-1f, 0x1.b2b7aap-1f, 0x1.a3660ap-1f,
    0x1.92f8dcp-1f, 0x1.81870ap-1f, 0x1.6f28ccp-1f, 0x1.5bf786p-1f,
};

/* dc_from_dct128x64_normalized (src/dct128.rs:580-609): along the 64-point
 * axis a, the 128-point axis' 16 lowest coefficients scaled by r8[a]
 * r16[b] and 16 through the 16-point inverse; then per position, scaled by
 * 8, the 8-point inverse across a.  norm[i][j]: i along the 64-point axis,
 * j along the 128-point one. */
static void dc_128x64_normalized(const float* c, float norm[8][16]) {
  float rows[8][16];
  for (int a = 0; a < 8; a++) {
    for (int b = 0; b < 16; b++) rows[a][b] = c[a * 128 + b] * (R64_8[a] * R128_16[b]) * 16.0f;
    inv_dct1d_16(rows[a]);
  }
  for (int x = 0; x < 16; x++) {
    float col[8];
    for (int y = 0; y < 8; y++) col[y] = rows[y][x] * 8.0f;
    inv_dct1d_8(col);
    for (int y = 0; y < 8; y++) norm[y][x] = col[y];
  }
}

/* dc_from_dct64x32_normalized (:2767-2786): per low horizontal-or-vertical
 * frequency a of the 32-point axis, the 8-point axis' lowest coefficients
 * scaled by r4[a] r8[b] through the unnormalised 8-point inverse; then per
 * position the 4-point inverse across a.  norm[i][j]: i along the 4-point
 * axis, j along the 8-point one. */
static void dc_64x32_normalized(const float* c, float norm[4][8]) {
  float rows[4][8];
  for (int a = 0; a < 4; a++) {
    for (int b = 0; b < 8; b++) rows[a][b] = c[a * 64 + b] * (R32_4[a] * R64_8[b]) * 8.0f;
    inv_dct1d_8(rows[a]);
  }
  for (int x = 0; x < 8; x++) {
    const float col[4] = {rows[0][x], rows[1][x], rows[2][x], rows[3][x]};
    float o[4];
    idct1d_4(col, o);
    for (int y = 0; y < 4; y++) norm[y][x] = o[y];
  }
}

/* The DC values a transform's lowest coefficients resample to, one per
 * covered 8x8 block (dc_from_dct16x8 :930, dc_from_dct8x16 :939,
 * dc_from_dct16x16 :1033, dc_from_dct32x32 :2170, dc_from_dct32x16 :2356,
 * dc_from_dct16x32 :2381); an 8x8 block's DC is its first coefficient. */
static void dc_from(int kind, const float* c, float* dc) {
  switch (kind) {
    case JXG_ORC_DCT8X8:
      dc[0] = c[0];
      break;
    case JXG_ORC_DCT8X16:
    case JXG_ORC_DCT16X8: {
      const float s0 = c[0] * R16_2[0], s1 = c[1] * R16_2[1];
      dc[0] = s0 + s1;
      dc[1] = s0 - s1;
      break;
    }
    case JXG_ORC_DCT16X16: {
      /* the products of the resample scales, as f32 */
      const float r00 = 1.0f, r01 = 0.9017642f, r11 = 0x1.a058f6p-1f;
      const float s00 = c[0] * r00, s01 = c[1] * r01, s10 = c[16] * r01, s11 = c[17] * r11;
      const float a00 = s00 + s01, a01 = s00 - s01, a10 = s10 + s11, a11 = s10 - s11;
      dc[0] = a00 + a10;
      dc[1] = a00 - a10;
      dc[2] = a01 + a11;
      dc[3] = a01 - a11;
      break;
    }
    case JXG_ORC_DCT16X32:
    case JXG_ORC_DCT32X16: {
      float rr[2][4];
      for (int a = 0; a < 2; a++) {
        float s[4];
        for (int b = 0; b < 4; b++) s[b] = c[a * 32 + b] * R16_2[a] * R32_4[b];
        idct1d_4(s, rr[a]);
      }
      for (int bb = 0; bb < 4; bb++) {
        const float c0 = rr[0][bb], c1 = rr[1][bb];
        if (kind == JXG_ORC_DCT32X16) {
          dc[bb * 2] = c0 + c1;
          dc[bb * 2 + 1] = c0 - c1;
        } else {
          dc[bb] = c0 + c1;
          dc[4 + bb] = c0 - c1;
        }
      }
      break;
    }
    case JXG_ORC_DCT32X8:
    case JXG_ORC_DCT8X32: { /* dc_from_dct8x32 (:1864-1867) */
      float sv[4];
      for (int b = 0; b < 4; b++) sv[b] = c[b] * R32_4[b];
      idct1d_4(sv, dc);
      break;
    }
    case JXG_ORC_DCT64X64: { /* dc_from_dct64x64 (:2602-2612) */
      float low[64];
      for (int y = 0; y < 8; y++)
        for (int x = 0; x < 8; x++) low[y * 8 + x] = c[y * 64 + x] * (R64_8[x] * R64_8[y]);
      idct_square(low, 8, dc);
      break;
    }
    case JXG_ORC_DCT64X32:
    case JXG_ORC_DCT32X64: { /* dc_from_dct64x32 (:2789), dc_from_dct32x64 (:2800) */
      float norm[4][8];
      dc_64x32_normalized(c, norm);
      for (int y = 0; y < 4; y++)
        for (int x = 0; x < 8; x++) {
          if (kind == JXG_ORC_DCT64X32) dc[x * 4 + y] = norm[y][x];
          else dc[y * 8 + x] = norm[y][x];
        }
      break;
    }
    case JXG_ORC_DCT128X128: { /* dc_from_dct128x128 (src/dct128.rs:561-573) */
      float low[256];
      for (int y = 0; y < 16; y++)
        for (int x = 0; x < 16; x++)
          low[y * 16 + x] = c[y * 128 + x] * (R128_16[x] * R128_16[y]);
      idct_square(low, 16, dc);
      break;
    }
    case JXG_ORC_DCT128X64:
    case JXG_ORC_DCT64X128: { /* dc_from_dct128x64 (:612), dc_from_dct64x128 (:629) */
      float norm[8][16];
      dc_128x64_normalized(c, norm);
      for (int y = 0; y < 8; y++)
        for (int x = 0; x < 16; x++) {
          if (kind == JXG_ORC_DCT128X64) dc[x * 8 + y] = norm[y][x];
          else dc[y * 16 + x] = norm[y][x];
        }
      break;
    }
    default: { /* 32x32 */
      float rr[4][4];
      for (int a = 0; a < 4; a++) {
        float s[4];
        for (int b = 0; b < 4; b++) s[b] = c[a * 32 + b] * R32_4[a] * R32_4[b];
        idct1d_4(s, rr[a]);
      }
      for (int bb = 0; bb < 4; bb++) {
        const float col[4] = {rr[0][bb], rr[1][bb], rr[2][bb], rr[3][bb]};
        float o[4];
        idct1d_4(col, o);
        for (int r = 0; r < 4; r++) dc[bb * 4 + r] = o[r];
      }
    }
  }
}

/* DctFn<W, H, N> of one block (row-major H x W samples) and its DC values;
 * `kind` as JXG_ORC_DCT*.  Returns 0, or -1 for an unknown kind. */
int orc_dct(int kind, const float* in, float* out, float* dc) {
  switch (kind) {
    case JXG_ORC_DCT8X8: dct8x8(in, 8, out); break;
    case JXG_ORC_DCT8X16: dct_rows_first(in, 16, 8, out); break;
    case JXG_ORC_DCT16X8: dct_cols_first(in, 8, 16, out); break;
    case JXG_ORC_DCT16X16: dct_cols_first(in, 16, 16, out); break;
    case JXG_ORC_DCT16X32: dct_rows_first(in, 32, 16, out); break;
    case JXG_ORC_DCT32X16: dct_cols_first(in, 16, 32, out); break;
    case JXG_ORC_DCT32X32: dct_cols_first(in, 32, 32, out); break;
    case JXG_ORC_DCT32X8: dct_cols_first(in, 8, 32, out); break;
    case JXG_ORC_DCT8X32: dct_rows_first(in, 32, 8, out); break;
    case JXG_ORC_DCT64X64: dct_cols_first(in, 64, 64, out); break;
    case JXG_ORC_DCT64X32: dct_cols_first(in, 32, 64, out); break;
    case JXG_ORC_DCT32X64: dct_rows_first(in, 64, 32, out); break;
    case JXG_ORC_DCT128X128: dct_cols_first(in, 128, 128, out); break;
    case JXG_ORC_DCT128X64: dct_cols_first(in, 64, 128, out); break;
    case JXG_ORC_DCT64X128: dct_rows_first(in, 128, 64, out); break;
    default: return -1;
  }
  if (dc) dc_from(kind, out, dc);
  return 0;
}

/* ---- inverse transforms (src/dct.rs:1498-1730) ----------------------
 * The reciprocal tables are 1 / WC rounded to f32, written as their values;
 * IS2 is 1 / sqrt(2) as f32. */
static const float IS2F = 0x1.6a09e6p-1f;
static const float INV_WC4[2] = {0x1.d906bcp+0f, 0x1.87de2ap-1f};
static const float INV_WC8[4] = {0x1.f6297cp+0f, 0x1.a9b662p+0f, 0x1.1c73b4p+0f, 0x1.8f8b82p-2f};
static const float INV_WC16[8] = {0x1.fd88dap+0f, 0x1.e9f416p+0f, 0x1.c38b30p+0f, 0x1.8bc806p+0f,
                                  0x1.44cf32p+0f, 0x1.e2b5d4p-1f, 0x1.294062p-1f, 0x1.917a6cp-3f};
static const float INV_WC32[16] = {0x1.ff6220p+0f, 0x1.fa755ap+0f, 0x1.f0a7f0p+0f, 0x1.e21212p+0f,
                                   0x1.ced7aep+0f, 0x1.b72834p+0f, 0x1.9b3e04p+0f, 0x1.7b5df2p+0f,
                                   0x1.57d692p+0f, 0x1.30ff80p+0f, 0x1.073878p+0f, 0x1.b5d0fep-1f,
                                   0x1.58f9a8p-1f, 0x1.f19f98p-2f, 0x1.2c8106p-2f, 0x1.91f65ep-4f};

/* inv_dct1d_2 (:1500): the half sum and half difference. */
static inline void inv_dct1d_2(float* b) {
  const float s = b[0], d = b[1];
  b[0] = (s + d) * 0.5f;
  b[1] = (s - d) * 0.5f;
}

/* inv_dct1d_4 (:1508-1523). */
static inline void inv_dct1d_4(float* b) {
  float t[4] = {b[0], b[2], b[1], b[3]};
  t[2] = (t[2] - t[3]) * IS2F;
  inv_dct1d_2(t + 2);
  t[2] *= INV_WC4[0];
  t[3] *= INV_WC4[1];
  inv_dct1d_2(t);
  b[0] = (t[0] + t[2]) * 0.5f;
  b[3] = (t[0] - t[2]) * 0.5f;
  b[1] = (t[1] + t[3]) * 0.5f;
  b[2] = (t[1] - t[3]) * 0.5f;
}

/* inv_dct1d_8 (:1525-1542), inv_dct1d_16 (:1546-1566), inv_dct1d_32
 * (:1568-1588): de-interleave, undo the odd half's running sums from the
 * top, the odd half through the half-size inverse and 1 / WC, the even half
 * through the half-size inverse, half sums and differences mirrored. */
static inline void inv_dct1d_8(float* b) {
  float t[8];
  for (int i = 0; i < 4; i++) {
    t[i] = b[2 * i];
    t[4 + i] = b[2 * i + 1];
  }
  t[6] -= t[7];
  t[5] -= t[6];
  t[4] = (t[4] - t[5]) * IS2F;
  inv_dct1d_4(t + 4);
  for (int i = 0; i < 4; i++) t[4 + i] *= INV_WC8[i];
  inv_dct1d_4(t);
  for (int i = 0; i < 4; i++) {
    b[i] = (t[i] + t[4 + i]) * 0.5f;
    b[7 - i] = (t[i] - t[4 + i]) * 0.5f;
  }
}

static inline void inv_dct1d_16(float* b) {
  float t[16];
  for (int i = 0; i < 8; i++) {
    t[i] = b[2 * i];
    t[8 + i] = b[2 * i + 1];
  }
  for (int i = 14; i >= 9; i--) t[i] -= t[i + 1];
  t[8] = (t[8] - t[9]) * IS2F;
  inv_dct1d_8(t + 8);
  for (int i = 0; i < 8; i++) t[8 + i] *= INV_WC16[i];
  inv_dct1d_8(t);
  for (int i = 0; i < 8; i++) {
    b[i] = (t[i] + t[8 + i]) * 0.5f;
    b[15 - i] = (t[i] - t[8 + i]) * 0.5f;
  }
}

static inline void inv_dct1d_32(float* b) {
  float t[32];
  for (int i = 0; i < 16; i++) {
    t[i] = b[2 * i];
    t[16 + i] = b[2 * i + 1];
  }
  for (int i = 30; i >= 17; i--) t[i] -= t[i + 1];
  t[16] = (t[16] - t[17]) * IS2F;
  inv_dct1d_16(t + 16);
  for (int i = 0; i < 16; i++) t[16 + i] *= INV_WC32[i];
  inv_dct1d_16(t);
  for (int i = 0; i < 16; i++) {
    b[i] = (t[i] + t[16 + i]) * 0.5f;
    b[31 - i] = (t[i] - t[16 + i]) * 0.5f;
  }
}

/* INV_WC64 (src/dct.rs:2495-2527): 1 / WC64 as float. */
static const float INV_WC64[32] = {
    0x1.ffd888p+0f, 0x1.fe9cdcp+0f, 0x1.fc2648p+0f, 0x1.f87652p+0f,
    0x1.f38f3cp+0f, 0x1.ed741p+0f, 0x1.e6289p+0f, 0x1.ddb13ap+0f,
    0x1.d4134ep+0f, 0x1.c954b2p+0f, 0x1.bd7c0cp+0f, 0x1.b090a6p+0f,
    0x1.a29a7ap+0f, 0x1.93a224p+0f, 0x1.83b0ep+0f, 0x1.72d084p+0f,
    0x1.610b74p+0f, 0x1.4e6cacp+0f, 0x1.3affa2p+0f, 0x1.26d054p+0f,
    0x1.11eb36p+0f, 0x1.f8ba4ep-1f, 0x1.cc66eap-1f, 0x1.9ef794p-1f,
    0x1.708854p-1f, 0x1.4135c8p-1f, 0x1.111d26p-1f, 0x1.c0b828p-2f,
    0x1.5e2144p-2f, 0x1.f564e6p-3f, 0x1.2d520ap-3f, 0x1.92156p-5f,
};

/* inv_dct1d_64 (src/dct.rs:2548-2570). */
static inline void inv_dct1d_64(float* b) {
  float t[64];
  for (int i = 0; i < 32; i++) {
    t[i] = b[2 * i];
    t[32 + i] = b[2 * i + 1];
  }
  for (int i = 62; i >= 33; i--) t[i] -= t[i + 1];
  t[32] = (t[32] - t[33]) * IS2F;
  inv_dct1d_32(t + 32);
  for (int i = 0; i < 32; i++) t[32 + i] *= INV_WC64[i];
  inv_dct1d_32(t);
  for (int i = 0; i < 32; i++) {
    b[i] = (t[i] + t[32 + i]) * 0.5f;
    b[63 - i] = (t[i] - t[32 + i]) * 0.5f;
  }
}

/* INV_WC128 (src/dct128.rs:143-208): the reference's own literals, not all
 * equal to 1 / WC128 in float. */
static const float INV_WC128[64] = {
    0x1.fff622p+0f, 0x1.ffa72ep+0f, 0x1.ff0956p+0f, 0x1.fe1cbp+0f,
    0x1.fce16p+0f, 0x1.fb5798p+0f, 0x1.f97f92p+0f, 0x1.f7599ap+0f,
    0x1.f4e604p+0f, 0x1.f2253p+0f, 0x1.ef178ap+0f, 0x1.ebbd8cp+0f,
    0x1.e817bap+0f, 0x1.e426a4p+0f, 0x1.dfeae6p+0f, 0x1.db6526p+0f,
    0x1.d69618p+0f, 0x1.d17e78p+0f, 0x1.cc1f1p+0f, 0x1.c678b4p+0f,
    0x1.c08c42p+0f, 0x1.ba5aa6p+0f, 0x1.b3e4d4p+0f, 0x1.ad2bcap+0f,
    0x1.a63092p+0f, 0x1.9ef43ep+0f, 0x1.9777fp+0f, 0x1.8fbccap+0f,
    0x1.87c4p+0f, 0x1.7f8ecep+0f, 0x1.771e76p+0f, 0x1.6e7446p+0f,
    0x1.659192p+0f, 0x1.5c77bcp+0f, 0x1.53282ap+0f, 0x1.49a44ap+0f,
    0x1.3fed96p+0f, 0x1.36058cp+0f, 0x1.2bedb2p+0f, 0x1.21a79ap+0f,
    0x1.1734d6p+0f, 0x1.0c9704p+0f, 0x1.01cfc8p+0f, 0x1.edc196p-1f,
    0x1.d79776p-1f, 0x1.c1249ep-1f, 0x1.aa6c82p-1f, 0x1.9372a6p-1f,
    0x1.7c3a94p-1f, 0x1.64c7dep-1f, 0x1.4d1e24p-1f, 0x1.35410cp-1f,
    0x1.1d3444p-1f, 0x1.04fb8p-1f, 0x1.d934fep-2f, 0x1.a82a02p-2f,
    0x1.76dd9ep-2f, 0x1.45576cp-2f, 0x1.139f0cp-2f, 0x1.c3785cp-3f,
    0x1.5f6dp-3f, 0x1.f656e8p-4f, 0x1.2d8658p-4f, 0x1.921d2p-6f,
};

/* inv_dct1d_128 (src/dct128.rs:356-378). */
static inline void inv_dct1d_128(float* b) {
  float t[128];
  for (int i = 0; i < 64; i++) {
    t[i] = b[2 * i];
    t[64 + i] = b[2 * i + 1];
  }
  for (int i = 126; i >= 65; i--) t[i] -= t[i + 1];
  t[64] = (t[64] - t[65]) * IS2F;
  inv_dct1d_64(t + 64);
  for (int i = 0; i < 64; i++) t[64 + i] *= INV_WC128[i];
  inv_dct1d_64(t);
  for (int i = 0; i < 64; i++) {
    b[i] = (t[i] + t[64 + i]) * 0.5f;
    b[127 - i] = (t[i] - t[64 + i]) * 0.5f;
  }
}

static inline void inv_dct1d_n(float* b, int n) {
  if (n == 8) inv_dct1d_8(b);
  else if (n == 16) inv_dct1d_16(b);
  else if (n == 32) inv_dct1d_32(b);
  else if (n == 64) inv_dct1d_64(b);
  else inv_dct1d_128(b);
}

/* Inverse of a square transform (inv_dct_square, :1590-1620): coefficients
 * transposed and scaled by N, columns, then rows. */
static void idct_square(const float* c, int n, float* out) {
  float col[128];
  const float scale = (float)(n * n);
  for (int a = 0; a < n; a++)
    for (int b = 0; b < n; b++) out[b * n + a] = c[a * n + b] * scale;
  for (int u = 0; u < n; u++) {
    for (int v = 0; v < n; v++) col[v] = out[v * n + u];
    inv_dct1d_n(col, n);
    for (int v = 0; v < n; v++) out[v * n + u] = col[v];
  }
  for (int v = 0; v < n; v++) inv_dct1d_n(out + v * n, n);
}

/* Inverse of a rows-first transform (inv_dct8x16 :1634, inv_dct16x32
 * :1683, inv_dct8x32 :1804, inv_dct32x64 :2735, inv_dct64x128
 * src/dct128.rs:532): coefficients in place
 * scaled by N, columns (length H), rows. */
static void idct_rows_first(const float* c, int W, int H, float* out) {
  float col[128];
  const float scale = (float)(W * H);
  for (int k = 0; k < W * H; k++) out[k] = c[k] * scale;
  for (int u = 0; u < W; u++) {
    for (int v = 0; v < H; v++) col[v] = out[v * W + u];
    inv_dct1d_n(col, H);
    for (int v = 0; v < H; v++) out[v * W + u] = col[v];
  }
  for (int r = 0; r < H; r++) inv_dct1d_n(out + r * W, W);
}

/* Inverse of a columns-first transform (inv_dct16x8 :1658, inv_dct32x16
 * :1705, inv_dct32x8 :1833, inv_dct64x32 :2710, inv_dct128x64
 * src/dct128.rs:502): per pixel row v the
 * W-point inverse of coefficients c[u H + v] scaled by N, then per column
 * the H-point inverse. */
static void idct_cols_first(const float* c, int W, int H, float* out) {
  float* acd = malloc(sizeof(float) * (size_t)(W * H));
  float row[128], col[128];
  const float scale = (float)(W * H);
  for (int v = 0; v < H; v++) {
    for (int u = 0; u < W; u++) row[u] = c[u * H + v] * scale;
    inv_dct1d_n(row, W);
    for (int u = 0; u < W; u++) acd[v * W + u] = row[u];
  }
  for (int u = 0; u < W; u++) {
    for (int v = 0; v < H; v++) col[v] = acd[v * W + u];
    inv_dct1d_n(col, H);
    for (int i = 0; i < H; i++) out[i * W + u] = col[i];
  }
  free(acd);
}

/* The inverse of orc_dct's transform `kind`: W H coefficients back to a
 * row-major H x W block.  Returns 0, or -1 for an unknown kind. */
int orc_idct(int kind, const float* coeffs, float* out) {
  switch (kind) {
    case JXG_ORC_DCT8X8: idct_square(coeffs, 8, out); break;
    case JXG_ORC_DCT8X16: idct_rows_first(coeffs, 16, 8, out); break;
    case JXG_ORC_DCT16X8: idct_cols_first(coeffs, 8, 16, out); break;
    case JXG_ORC_DCT16X16: idct_square(coeffs, 16, out); break;
    case JXG_ORC_DCT16X32: idct_rows_first(coeffs, 32, 16, out); break;
    case JXG_ORC_DCT32X16: idct_cols_first(coeffs, 16, 32, out); break;
    case JXG_ORC_DCT32X32: idct_square(coeffs, 32, out); break;
    case JXG_ORC_DCT32X8: idct_cols_first(coeffs, 8, 32, out); break;
    case JXG_ORC_DCT8X32: idct_rows_first(coeffs, 32, 8, out); break;
    case JXG_ORC_DCT64X64: idct_square(coeffs, 64, out); break;
    case JXG_ORC_DCT64X32: idct_cols_first(coeffs, 32, 64, out); break;
    case JXG_ORC_DCT32X64: idct_rows_first(coeffs, 64, 32, out); break;
    case JXG_ORC_DCT128X128: idct_square(coeffs, 128, out); break;
    case JXG_ORC_DCT128X64: idct_cols_first(coeffs, 64, 128, out); break;
    case JXG_ORC_DCT64X128: idct_rows_first(coeffs, 128, 64, out); break;
    default: return -1;
  }
  return 0;
}

/* ---- the 8x8-sized transforms besides DCT8 (src/dct.rs) ------------- */

/* The 2x2 Hadamard of coefficients 0, 1, 8, 9, scaled 1/4. */
static void hadamard_0189(float* o) {
  const float b00 = o[0], b01 = o[1], b10 = o[8], b11 = o[9];
  o[0] = (b00 + b01 + b10 + b11) * 0.25f;
  o[1] = (b00 + b01 - b10 - b11) * 0.25f;
  o[8] = (b00 - b01 + b10 - b11) * 0.25f;
  o[9] = (b00 - b01 - b10 + b11) * 0.25f;
}

/* identity8x8 (:185-214): per 4x4 quadrant the residuals from its (1, 1)
 * anchor, the displaced top-left residual in the anchor's slot, the
 * quadrant mean in coefficient (qy, qx); then the Hadamard of the means. */
static void identity8x8(const float* in, float* o) {
  for (int qy = 0; qy < 2; qy++)
    for (int qx = 0; qx < 2; qx++) {
      const float anchor = in[(qy * 4 + 1) * 8 + qx * 4 + 1];
      float mean = 0.0f;
      for (int iy = 0; iy < 4; iy++)
        for (int ix = 0; ix < 4; ix++) {
          const float v = in[(qy * 4 + iy) * 8 + qx * 4 + ix];
          mean += v;
          if (ix == 1 && iy == 1) continue;
          o[(qy + iy * 2) * 8 + qx + ix * 2] = v - anchor;
        }
      o[(qy + 2) * 8 + qx + 2] = o[qy * 8 + qx];
      o[qy * 8 + qx] = mean * (1.0f / 16.0f);
    }
  hadamard_0189(o);
}

/* inv_identity8x8 (:225-264). */
static void inv_identity8x8(const float* c, float* o) {
  const float means[4] = {c[0] + c[1] + c[8] + c[9], c[0] + c[1] - c[8] - c[9],
                          c[0] - c[1] + c[8] - c[9], c[0] - c[1] - c[8] + c[9]};
  for (int qy = 0; qy < 2; qy++)
    for (int qx = 0; qx < 2; qx++) {
      float residual_sum = 0.0f;
      for (int iy = 0; iy < 4; iy++)
        for (int ix = 0; ix < 4; ix++) {
          if (ix == 1 && iy == 1) continue;
          residual_sum += (ix == 0 && iy == 0) ? c[(qy + 2) * 8 + qx + 2] : c[(qy + iy * 2) * 8 + qx + ix * 2];
        }
      const float anchor = means[qy * 2 + qx] - residual_sum * (1.0f / 16.0f);
      for (int iy = 0; iy < 4; iy++)
        for (int ix = 0; ix < 4; ix++) {
          const float r = (ix == 1 && iy == 1) ? 0.0f
                          : (ix == 0 && iy == 0) ? c[(qy + 2) * 8 + qx + 2]
                                                 : c[(qy + iy * 2) * 8 + qx + ix * 2];
          o[(qy * 4 + iy) * 8 + qx * 4 + ix] = anchor + r;
        }
    }
}

/* dct2_top_block::<S> (:274-299) and dct2x2_8x8 (:306-312). */
static void dct2_top_block(const float* in, int S, float* o) {
  float temp[64] = {0};
  const int half = S / 2;
  for (int y = 0; y < half; y++)
    for (int x = 0; x < half; x++) {
      const float c00 = in[(y * 2) * 8 + x * 2], c01 = in[(y * 2) * 8 + x * 2 + 1];
      const float c10 = in[(y * 2 + 1) * 8 + x * 2], c11 = in[(y * 2 + 1) * 8 + x * 2 + 1];
      temp[y * 8 + x] = (c00 + c01 + c10 + c11) * 0.25f;
      temp[y * 8 + half + x] = (c00 + c01 - c10 - c11) * 0.25f;
      temp[(y + half) * 8 + x] = (c00 - c01 + c10 - c11) * 0.25f;
      temp[(y + half) * 8 + half + x] = (c00 - c01 - c10 + c11) * 0.25f;
    }
  for (int y = 0; y < S; y++)
    for (int x = 0; x < S; x++) o[y * 8 + x] = temp[y * 8 + x];
}

static void dct2x2_8x8(const float* in, float* o) {
  float snap[64];
  dct2_top_block(in, 8, o);
  memcpy(snap, o, sizeof(snap));
  dct2_top_block(snap, 4, o);
  memcpy(snap, o, sizeof(snap));
  dct2_top_block(snap, 2, o);
}

/* inv_dct2_top_block::<S> (:322-341) and inv_dct2x2_8x8 (:345-354). */
static void inv_dct2_top_block(const float* in, int S, float* o) {
  const int half = S / 2;
  for (int y = 0; y < half; y++)
    for (int x = 0; x < half; x++) {
      const float r00 = in[y * 8 + x], r01 = in[y * 8 + half + x];
      const float r10 = in[(y + half) * 8 + x], r11 = in[(y + half) * 8 + half + x];
      o[(y * 2) * 8 + x * 2] = r00 + r01 + r10 + r11;
      o[(y * 2) * 8 + x * 2 + 1] = r00 + r01 - r10 - r11;
      o[(y * 2 + 1) * 8 + x * 2] = r00 - r01 + r10 - r11;
      o[(y * 2 + 1) * 8 + x * 2 + 1] = r00 - r01 - r10 + r11;
    }
}

static void inv_dct2x2_8x8(const float* c, float* o) {
  float a[64], snap[64];
  memcpy(a, c, sizeof(a));
  memcpy(snap, a, sizeof(snap));
  inv_dct2_top_block(snap, 2, a);
  memcpy(snap, a, sizeof(snap));
  inv_dct2_top_block(snap, 4, a);
  memcpy(snap, a, sizeof(snap));
  inv_dct2_top_block(snap, 8, o);
}

/* dct4x4_2d (:1061-1075) and dct4x4 (:1163-1190): each 4x4 quadrant through
 * rows then columns of dct1d_4 (transposed, 1/16), interleaved, then the
 * Hadamard of the quadrant DCs. */
static void dct4x4_2d(const float* in, float* out) {
  float tmp[16];
  memcpy(tmp, in, sizeof(tmp));
  for (int r = 0; r < 4; r++) dct1d_4(tmp + r * 4);
  for (int x = 0; x < 4; x++) {
    float col[4] = {tmp[x], tmp[4 + x], tmp[8 + x], tmp[12 + x]};
    dct1d_4(col);
    for (int i = 0; i < 4; i++) out[x * 4 + i] = col[i] * (1.0f / 16.0f);
  }
}

static void dct4x4(const float* in, float* o) {
  for (int qy = 0; qy < 2; qy++)
    for (int qx = 0; qx < 2; qx++) {
      float blk[16], d[16];
      for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) blk[r * 4 + c] = in[(qy * 4 + r) * 8 + qx * 4 + c];
      dct4x4_2d(blk, d);
      for (int iy = 0; iy < 4; iy++)
        for (int ix = 0; ix < 4; ix++) o[(qy + iy * 2) * 8 + qx + ix * 2] = d[iy * 4 + ix];
    }
  hadamard_0189(o);
}

/* dct4x8_2d (:1198-1220): a 4-row, 8-column block through column dct1d_4
 * then row dct1d_8 (1/32), frequencies [vertical][horizontal]. */
static void dct4x8_2d(const float* in, float* t) {
  memcpy(t, in, 32 * sizeof(float));
  for (int c = 0; c < 8; c++) {
    float col[4] = {t[c], t[8 + c], t[16 + c], t[24 + c]};
    dct1d_4(col);
    for (int vf = 0; vf < 4; vf++) t[vf * 8 + c] = col[vf];
  }
  for (int vf = 0; vf < 4; vf++) {
    dct1d_8(t + vf * 8);
    for (int k = 0; k < 8; k++) t[vf * 8 + k] *= 1.0f / 32.0f;
  }
}

/* dct4x8 (:1238-1262): each 4-row half through dct4x8_2d, rows
 * interleaved, the 2-point Hadamard of the half DCs. */
static void dct4x8(const float* in, float* o) {
  for (int y = 0; y < 2; y++) {
    float t[32];
    dct4x8_2d(in + y * 32, t);
    for (int iy = 0; iy < 4; iy++)
      for (int ix = 0; ix < 8; ix++) o[(y + iy * 2) * 8 + ix] = t[iy * 8 + ix];
  }
  const float b0 = o[0], b1 = o[8];
  o[0] = (b0 + b1) * 0.5f;
  o[8] = (b0 - b1) * 0.5f;
}

/* dct8x4_2d (:1267-1298) and dct8x4 (:1319-1340): each 4-column half
 * through column dct1d_8 then row dct1d_4 (transposed, 1/32). */
static void dct8x4(const float* in, float* o) {
  for (int x = 0; x < 2; x++) {
    float tmp[32], d[32];
    for (int c = 0; c < 4; c++) {
      float col[8];
      for (int r = 0; r < 8; r++) col[r] = in[r * 8 + x * 4 + c];
      dct1d_8(col);
      for (int vf = 0; vf < 8; vf++) tmp[vf * 4 + c] = col[vf];
    }
    for (int vf = 0; vf < 8; vf++) {
      float row[4] = {tmp[vf * 4], tmp[vf * 4 + 1], tmp[vf * 4 + 2], tmp[vf * 4 + 3]};
      dct1d_4(row);
      for (int hf = 0; hf < 4; hf++) d[hf * 8 + vf] = row[hf] * (1.0f / 32.0f);
    }
    for (int iy = 0; iy < 4; iy++)
      for (int ix = 0; ix < 8; ix++) o[(x + iy * 2) * 8 + ix] = d[iy * 8 + ix];
  }
  const float b0 = o[0], b1 = o[8];
  o[0] = (b0 + b1) * 0.5f;
  o[8] = (b0 - b1) * 0.5f;
}

/* The AFV basis of the JPEG XL standard (libjxl k4x4AFVBasisTranspose,
 * src/afv.rs:48-180), stored vector-major: AFV_BASIS[i][j] is basis vector
 * i sampled at pixel j of the mirrored 4x4 corner; the reference stores the
 * transpose.  Each value is the reference's decimal literal rounded to
 * float, written in hex. */
static const float AFV_BASIS[16][16] = {
    {// basis vector 0
     0x1p-2f, 0x1p-2f, 0x1p-2f, 0x1p-2f,
     0x1p-2f, 0x1p-2f, 0x1p-2f, 0x1p-2f,
     0x1p-2f, 0x1p-2f, 0x1p-2f, 0x1p-2f,
     0x1p-2f, 0x1p-2f, 0x1p-2f, 0x1p-2f},
    {// basis vector 1
     0x1.c0f96cp-1f, 0x1.c3e518p-3f, -0x1.9f5622p-4f, -0x1.9f5622p-4f,
     0x1.c3e518p-3f, -0x1.9f5622p-4f, -0x1.9f5622p-4f, -0x1.9f5622p-4f,
     -0x1.9f5622p-4f, -0x1.9f5622p-4f, -0x1.9f5622p-4f, -0x1.9f5622p-4f,
     -0x1.9f5622p-4f, -0x1.9f5622p-4f, -0x1.9f5622p-4f, -0x1.9f5622p-4f},
    {// basis vector 2
     0.0f, 0.0f, 0x1.a0762ap-2f, 0x1.c71d6cp-2f,
     0.0f, 0.0f, 0x1.90e23ap-3f, 0x1.2bf09ap-2f,
     -0x1.a0762ap-2f, -0x1.90e23ap-3f, 0.0f, 0x1.d2163ep-4f,
     -0x1.c71d6cp-2f, -0x1.2bf09ap-2f, -0x1.d2163ep-4f, 0.0f},
    {// basis vector 3
     0.0f, 0.0f, -0x1.b35156p-3f, 0x1.3bf474p-2f,
     0.0f, 0x1.e1f76p-2f, -0x1.4c05d8p-3f, 0.0f,
     -0x1.b35156p-3f, -0x1.4c05d8p-3f, -0x1.e1f76p-2f, -0x1.2be31p-3f,
     0x1.3bf474p-2f, 0.0f, -0x1.2be31p-3f, 0x1.b35156p-2f},
    {// basis vector 4
     0.0f, -0x1.6a09e6p-1f, 0.0f, 0.0f,
     0x1.6a09e6p-1f, 0.0f, 0.0f, 0.0f,
     0.0f, 0.0f, 0.0f, 0.0f,
     0.0f, 0.0f, 0.0f, 0.0f},
    {// basis vector 5
     -0x1.a46402p-2f, 0x1.3f41cp-1f, -0x1.07949ep-4f, -0x1.07949ep-4f,
     0x1.3f41cp-1f, -0x1.07949ep-4f, -0x1.07949ep-4f, -0x1.07949ep-4f,
     -0x1.07949ep-4f, -0x1.07949ep-4f, -0x1.07949ep-4f, -0x1.07949ep-4f,
     -0x1.07949ep-4f, -0x1.07949ep-4f, -0x1.07949ep-4f, -0x1.07949ep-4f},
    {// basis vector 6
     0.0f, 0.0f, -0x1.ce990ap-2f, 0x1.44b342p-3f,
     0.0f, -0x1.4ad5cep-5f, 0x1.e6293p-8f, 0x1.92f46p-2f,
     -0x1.ce990ap-2f, 0x1.e6293p-8f, 0x1.c5990cp-4f, 0x1.53e48cp-4f,
     0x1.44b342p-3f, 0x1.92f46p-2f, 0x1.53e48cp-4f, -0x1.ce990ap-2f},
    {// basis vector 7
     0.0f, 0.0f, -0x1.37ff48p-2f, 0x1.05c416p-1f,
     0.0f, 0.0f, -0x1.2973ap-2f, -0x1.0d76bp-4f,
     0x1.37ff48p-2f, 0x1.2973ap-2f, 0.0f, -0x1.e94338p-3f,
     -0x1.05c416p-1f, 0x1.0d76bp-4f, 0x1.e94338p-3f, 0.0f},
    {// basis vector 8
     0.0f, 0.0f, 0x1.350936p-2f, 0x1.081d22p-2f,
     0.0f, 0x1.4d41eep-3f, 0x1.85f0acp-4f, 0.0f,
     0x1.350936p-2f, 0x1.85f0acp-4f, -0x1.4d41eep-3f, -0x1.69994cp-2f,
     0x1.081d22p-2f, 0.0f, -0x1.69994cp-2f, -0x1.350936p-1f},
    {// basis vector 9
     0.0f, 0.0f, 0x1.a20bd8p-2f, 0.0f,
     0.0f, 0.0f, 0.0f, -0x1.a20bd8p-2f,
     -0x1.a20bd8p-2f, 0.0f, 0.0f, -0x1.a20bd8p-2f,
     0.0f, 0x1.a20bd8p-2f, 0x1.a20bd8p-2f, 0.0f},
    {// basis vector 10
     0.0f, 0.0f, 0x1.65f692p-3f, 0x1.4cd876p-4f,
     0.0f, 0.0f, -0x1.785c5ap-2f, -0x1.3b457ap-2f,
     -0x1.65f692p-3f, 0x1.785c5ap-2f, 0.0f, 0x1.ee40c2p-2f,
     -0x1.4cd876p-4f, 0x1.3b457ap-2f, -0x1.ee40c2p-2f, 0.0f},
    {// basis vector 11
     0.0f, 0.0f, -0x1.b03e22p-3f, 0x1.7c418p-3f,
     0.0f, 0.0f, 0x1.f7f86cp-2f, -0x1.8a7f04p-2f,
     0x1.b03e22p-3f, -0x1.f7f86cp-2f, 0.0f, 0x1.64bfe4p-3f,
     -0x1.7c418p-3f, 0x1.8a7f04p-2f, -0x1.64bfe4p-3f, 0.0f},
    {// basis vector 12
     0.0f, 0.0f, -0x1.242b5ep-3f, -0x1.5dd81ap-2f,
     0.0f, 0x1.793744p-1f, 0x1.f85cf8p-3f, -0x1.5f311cp-4f,
     -0x1.242b5ep-3f, 0x1.f85cf8p-3f, 0x1.30cfep-3f, -0x1.86a67ap-5f,
     -0x1.5dd81ap-2f, -0x1.5f311cp-4f, -0x1.86a67ap-5f, -0x1.242b5ep-3f},
    {// basis vector 13
     0.0f, 0.0f, -0x1.1ae6bcp-3f, 0x1.52275cp-2f,
     0.0f, 0x1.669c08p-4f, -0x1.457f42p-4f, -0x1.d868dap-2f,
     -0x1.1ae6bcp-3f, -0x1.457f42p-4f, 0x1.fd2e2ep-2f, 0x1.00c78ap-3f,
     0x1.52275cp-2f, -0x1.d868dap-2f, 0x1.00c78ap-3f, -0x1.1ae6bcp-3f},
    {// basis vector 14
     0.0f, 0.0f, -0x1.651f42p-3f, 0x1.1fdcf2p-4f,
     0.0f, -0x1.2b1cf6p-2f, 0x1.731432p-2f, 0.0f,
     -0x1.651f42p-3f, 0x1.731432p-2f, 0x1.2b1cf6p-2f, -0x1.bb0b6ep-2f,
     0x1.1fdcf2p-4f, 0.0f, -0x1.bb0b6ep-2f, 0x1.651f42p-2f},
    {// basis vector 15
     0.0f, 0.0f, 0x1.d119acp-4f, -0x1.2fd22cp-4f,
     0.0f, 0x1.8d5f0ap-3f, -0x1.bda294p-2f, 0x1.c0e508p-3f,
     0x1.d119acp-4f, -0x1.bda294p-2f, 0x1.1c2ec6p-1f, -0x1.04cb9p-2f,
     -0x1.2fd22cp-4f, 0x1.c0e508p-3f, -0x1.04cb9p-2f, 0x1.d119acp-4f},
};

void orc_afv_basis(float* out) { memcpy(out, AFV_BASIS, sizeof(AFV_BASIS)); }

/* The AFV parts' sub-transforms on their own, for the decoder-side round
 * trip: dct4x4_2d of a 4x4 block, dct4x8_2d of a 4-row, 8-column block. */
void orc_dct4x4_2d(const float* in, float* out) { dct4x4_2d(in, out); }
void orc_dct4x8_2d(const float* in, float* out) { dct4x8_2d(in, out); }

/* afv_dct4x4 (src/afv.rs:188-196): coefficient i is the fused dot product
 * of the corner's pixels with basis vector i, pixels in order. */
static void afv_dct4x4(const float* px, float* coeff) {
  for (int i = 0; i < 16; i++) {
    float acc = 0.0f;
    for (int j = 0; j < 16; j++) acc = fmla(px[j], AFV_BASIS[i][j], acc);
    coeff[i] = acc;
  }
}

/* afv_from_pixels (src/afv.rs:207-259): AFV of the mirrored corner quadrant
 * into the (even, even) positions, DCT4x4 of the horizontally adjacent
 * quadrant into (even, odd), DCT4x8 of the other vertical half into the odd
 * rows, then the three sub-part DCs rewritten so coefficient 0 is the block
 * mean.  kind bit 0 = right half, bit 1 = bottom half. */
static void afv_8x8(int kind, const float* in, float* o) {
  const int afv_x = kind & 1, afv_y = kind >> 1;
  float quad[16], coeff[16];
  for (int i = 0; i < 16; i++) {
    const int dy = i / 4, dx = i % 4;
    const int sy = afv_y ? 3 - dy : dy, sx = afv_x ? 3 - dx : dx;
    quad[i] = in[(sy + 4 * afv_y) * 8 + sx + 4 * afv_x];
  }
  afv_dct4x4(quad, coeff);
  for (int iy = 0; iy < 4; iy++)
    for (int ix = 0; ix < 4; ix++) o[iy * 16 + ix * 2] = coeff[iy * 4 + ix];
  const int qx = afv_x ? 0 : 4;
  for (int i = 0; i < 16; i++) quad[i] = in[(i / 4 + 4 * afv_y) * 8 + qx + i % 4];
  dct4x4_2d(quad, coeff);
  for (int iy = 0; iy < 4; iy++)
    for (int ix = 0; ix < 4; ix++) o[iy * 16 + ix * 2 + 1] = coeff[iy * 4 + ix];
  const int hy = afv_y ? 0 : 4;
  float half[32];
  dct4x8_2d(in + hy * 8, half);
  for (int iy = 0; iy < 4; iy++)
    for (int ix = 0; ix < 8; ix++) o[(1 + iy * 2) * 8 + ix] = half[iy * 8 + ix];
  const float block00 = o[0] * 0.25f, block01 = o[1], block10 = o[8];
  o[0] = (block00 + block01 + 2.0f * block10) * 0.25f;
  o[1] = (block00 - block01) * 0.5f;
  o[8] = (block00 + block01 - 2.0f * block10) * 0.25f;
}

/* The 8x8-sized transforms: 0 identity, 1 DCT2x2, 2 DCT4x4, 3 DCT4x8,
 * 4 DCT8x4 (forward), 5 / 6 the identity / DCT2x2 inverses, 7..10 AFV0..3
 * (forward).  Returns 0, or -1 for an unknown kind. */
int orc_small_transform(int kind, const float* in, float* out) {
  switch (kind) {
    case 0: identity8x8(in, out); break;
    case 1: dct2x2_8x8(in, out); break;
    case 2: dct4x4(in, out); break;
    case 3: dct4x8(in, out); break;
    case 4: dct8x4(in, out); break;
    case 5: inv_identity8x8(in, out); break;
    case 6: inv_dct2x2_8x8(in, out); break;
    case 7:
    case 8:
    case 9:
    case 10: afv_8x8(kind - 7, in, out); break;
    default: return -1;
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* Gaborish                                                             */
/* ------------------------------------------------------------------ */

/* K_GABORISH (src/gaborish.rs:32-38) */
static const float GAB_K[5] = {-0.09495815671340026f, -0.041031725066768575f, 0.013710004822696948f,
                               0.006510206083837737f, -0.0014789063378272242f};

/* reflect (src/gaborish.rs:78-90): mirror about the edges, repeated */
static size_t gab_reflect(long i, long len) {
  long j = i;
  while (j < 0 || j >= len) {
    if (j < 0) j = -j - 1;
    else j = 2 * len - j - 1;
  }
  return (size_t)j;
}

/* The normalised weights of gaborish_inverse (src/gaborish.rs:44-72):
 * c, r, d, R, L, D (centre, distance 1, sqrt 2, 2, sqrt 5, 2 sqrt 2). */
void orc_gaborish_inverse_weights(float mul, float* w6) {
  const float w_r = mul * GAB_K[0], w_d = mul * GAB_K[1], w_r2 = mul * GAB_K[2];
  const float w_l = mul * GAB_K[3], w_d2 = mul * GAB_K[4];
  float sum = 1.0f + mul * 4.0f * (GAB_K[0] + GAB_K[1] + GAB_K[2] + GAB_K[4] + 2.0f * GAB_K[3]);
  if (sum < 1e-5f) sum = 1e-5f;
  const float norm = 1.0f / sum;
  w6[0] = norm;
  w6[1] = norm * w_r;
  w6[2] = norm * w_d;
  w6[3] = norm * w_r2;
  w6[4] = norm * w_l;
  w6[5] = norm * w_d2;
}

/* gaborish_inverse (src/gaborish.rs:44-258): the symmetric 5x5 of every
 * channel with mirror-reflected neighbours, each output from source pixels
 * only (the reference delays its writes by two rows).  `in` and `out` are 3
 * planes of w*h floats. */
void orc_gaborish_inverse(const float* in, float* out, size_t w, size_t h, float mul) {
  float k[6];
  orc_gaborish_inverse_weights(mul, k);
  const float n_c = k[0], n_r = k[1], n_d = k[2], n_r2 = k[3], n_l = k[4], n_d2 = k[5];
  for (int c = 0; c < 3; c++) {
    const float* p = in + (size_t)c * w * h;
    float* o = out + (size_t)c * w * h;
    for (size_t y = 0; y < h; y++) {
      const float* r0 = p + y * w;
      const float* rm1 = p + gab_reflect((long)y - 1, (long)h) * w;
      const float* rp1 = p + gab_reflect((long)y + 1, (long)h) * w;
      const float* rm2 = p + gab_reflect((long)y - 2, (long)h) * w;
      const float* rp2 = p + gab_reflect((long)y + 2, (long)h) * w;
      for (size_t x = 0; x < w; x++) {
        const size_t xm1 = gab_reflect((long)x - 1, (long)w), xp1 = gab_reflect((long)x + 1, (long)w);
        const size_t xm2 = gab_reflect((long)x - 2, (long)w), xp2 = gab_reflect((long)x + 2, (long)w);
        const float s_r = rm1[x] + rp1[x] + r0[xm1] + r0[xp1];
        const float s_d = rm1[xm1] + rm1[xp1] + rp1[xm1] + rp1[xp1];
        const float s_r2 = rm2[x] + rp2[x] + r0[xm2] + r0[xp2];
        const float s_d2 = rm2[xm2] + rm2[xp2] + rp2[xm2] + rp2[xp2];
        const float s_l = rm2[xm1] + rm2[xp1] + rm1[xm2] + rm1[xp2] + rp1[xm2] + rp1[xp2] +
                          rp2[xm1] + rp2[xp1];
        float acc = n_c * r0[x];
        acc = fmla(n_r, s_r, acc);
        acc = fmla(n_d, s_d, acc);
        acc = fmla(n_r2, s_r2, acc);
        acc = fmla(n_d2, s_d2, acc);
        acc = fmla(n_l, s_l, acc);
        o[y * w + x] = acc;
      }
    }
  }
}

/* The decoder's Gaborish (src/epf_filter.rs:163-188, gaborish_pixel
 * src/epf_filter/kernels.rs:134-145): the 3x3 with clamped neighbours and
 * weights norm, W1 norm, W2 norm; products fused into the sums (the NEON
 * and AVX2+FMA backends). */
void orc_gaborish_weights(float* w3) {
  const float w1 = 1.1f * 0.10469957f, w2 = 1.1f * 0.05568054f;
  const float norm = 1.0f / (1.0f + 4.0f * (w1 + w2));
  w3[0] = norm;
  w3[1] = w1 * norm;
  w3[2] = w2 * norm;
}

void orc_gaborish(const float* in, float* out, size_t w, size_t h) {
  float k[3];
  orc_gaborish_weights(k);
  for (int c = 0; c < 3; c++) {
    const float* p = in + (size_t)c * w * h;
    float* o = out + (size_t)c * w * h;
    for (size_t y = 0; y < h; y++) {
      const float* t = p + (y > 0 ? y - 1 : 0) * w;
      const float* m = p + y * w;
      const float* b = p + (y + 1 < h ? y + 1 : h - 1) * w;
      for (size_t x = 0; x < w; x++) {
        const size_t l = x > 0 ? x - 1 : 0, r = x + 1 < w ? x + 1 : w - 1;
        const float side = (m[l] + m[r]) + (t[x] + b[x]);
        const float corner = (t[l] + t[r]) + (b[l] + b[r]);
        o[y * w + x] = fmla(corner, k[2], fmla(side, k[1], m[x] * k[0]));
      }
    }
  }
}

/* dct1d_16 / dct1d_32 of one vector in place (n = 8, 16 or 32). */
void orc_dct1d(float* b, int n) { dct1d_n(b, n); }

/* ------------------------------------------------------------------ */
/* Chroma-from-luma tiles (src/color_correlation.rs:333-512)            */
/* ------------------------------------------------------------------ */

#define K_INV_COLOR_FACTOR (1.0f / 84.0f)

/* src/color_correlation.rs:384-394 */
static float cfl_deadzone(float d) {
  if (d <= 1.0f) return 1.5f;
  if (d >= 2.0f) return 0.0f;
  const float s = 1.5f / (2.0f - 1.0f);
  return s * (2.0f - d);
}

/* src/color_correlation.rs:397-409 */
static int32_t solve_multiplier(float ca, float cb, size_t num, float dmul, float dz,
                                float units) {
  if (num == 0) return 0;
  float x = -cb / fmla((float)num * dmul, 0.5f, ca);
  if (fabsf(x) < dz) x = 0.0f;
  float r = clampf(roundf(x * units), -128.0f, 127.0f);
  return sat_i32(r);
}

/* compute_cmap_tile (src/color_correlation.rs:441-508) */
static void cmap_tile(const float* xyb, size_t w, size_t h, size_t bx0, size_t by0, size_t bxc,
                      size_t byc, float distance, const float* inv_x, const float* inv_b,
                      int8_t* ytox, int8_t* ytob) {
  size_t n = w * h;
  float ca_x = 0.0f, cb_x = 0.0f, ca_b = 0.0f, cb_b = 0.0f;
  size_t num = 0;
  float by_[64], bx_[64], bb_[64];
  for (size_t by = 0; by < byc; by++)
    for (size_t bx = 0; bx < bxc; bx++) {
      size_t px = (bx0 + bx) * 8, py = (by0 + by) * 8;
      if (px + 8 > w || py + 8 > h) continue;
      size_t off = py * w + px;
      dct8x8(xyb + n + off, w, by_);
      dct8x8(xyb + off, w, bx_);
      dct8x8(xyb + 2 * n + off, w, bb_);
      by_[0] = 0.0f;
      bx_[0] = 0.0f;
      bb_[0] = 0.0f;
      float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
      for (int i = 0; i < 64; i++) {
        float m_x = by_[i] * inv_x[i];
        float s_x = bx_[i] * inv_x[i];
        float a_x = K_INV_COLOR_FACTOR * m_x;
        float b_x = -s_x;
        s0 = fmla(a_x, a_x, s0);
        s1 = fmla(a_x, b_x, s1);
        float m_b = by_[i] * inv_b[i];
        float s_b = bb_[i] * inv_b[i];
        float a_b = K_INV_COLOR_FACTOR * m_b;
        float b_b = fmla(1.0f, m_b, -s_b);
        s2 = fmla(a_b, a_b, s2);
        s3 = fmla(a_b, b_b, s3);
      }
      ca_x += s0;
      cb_x += s1;
      ca_b += s2;
      cb_b += s3;
      num += 64;
    }
  float dz = cfl_deadzone(distance);
  *ytox = (int8_t)solve_multiplier(ca_x, cb_x, num, 1e-3f, dz, 84.0f / 84.0f);
  *ytob = (int8_t)solve_multiplier(ca_b, cb_b, num, 1e-3f, dz, 84.0f / 84.0f);
}

/* ------------------------------------------------------------------ */
/* Quantisation (src/group.rs)                                          */
/* ------------------------------------------------------------------ */

/* src/group.rs:406-455 for a single 8x8 block */
static void ac_thresholds(int c, float d, float qm_mul, float thr[4]) {
  float normal[4] = {0.58f, 0.635f, 0.66f, 0.7f};
  if (c == 0) {
    float up = clampf((d - 0.5f) / (0.75f - 0.5f), 0.0f, 1.0f);
    float down = clampf((2.0f - d) / (2.0f - 1.5f), 0.0f, 1.0f);
    float wv = rmin(up, down);
    normal[0] += wv * (0.5f - normal[0]);
    for (int i = 1; i < 4; i++) normal[i] += (1.0f - wv) * 0.08f;
  }
  if (c == 2) {
    float b_hf = qm_mul > 1.0f ? 0.65f : 0.75f;
    for (int i = 1; i < 4; i++) normal[i] = b_hf;
  }
  float hq[4];
  if (c == 1) { hq[0] = 0.50f; hq[1] = 0.51f; hq[2] = 0.52f; hq[3] = 0.54f; }
  else memcpy(hq, normal, sizeof(hq));
  float t = clampf((d - 0.1f) / 0.9f, 0.0f, 1.0f);
  for (int i = 0; i < 4; i++) thr[i] = hq[i] + t * (normal[i] - hq[i]);
}

/* quantize_block_ac_scalar (src/group.rs:560-612), 8x8 case */
static void quantize_ac(const float* in, int c, const float* qm, int32_t quant, float scale,
                        float qm_mul, float d, int32_t* out) {
  float thr[4];
  ac_thresholds(c, d, qm_mul, thr);
  float q_scaled = scale * (float)quant * qm_mul;
  for (int y = 0; y < 8; y++) {
    int yfix = y >= 4 ? 2 : 0;
    for (int x = 0; x < 8; x++) {
      float threshold = x >= 4 ? thr[yfix + 1] : thr[yfix];
      float q = qm[y * 8 + x] * q_scaled;
      float val = q * in[y * 8 + x];
      out[y * 8 + x] = fabsf(val) >= threshold ? sat_i32(roundf(val)) : 0;
    }
  }
}

static const float DEFAULT_BIAS_ONE[3] = {1.0f - 0.05465007330715401f,
                                          1.0f - 0.07005449891748593f,
                                          1.0f - 0.049935103337343655f};
#define BIAS_NUMERATOR 0.145f

/* DequantBias::level (src/group.rs:767-790) */
static inline float bias_level(int c, int32_t q) {
  uint32_t a = q < 0 ? (uint32_t)(-(int64_t)q) : (uint32_t)q;
  if (a <= 1) return q == 0 ? 0.0f : (q > 0 ? DEFAULT_BIAS_ONE[c] : -DEFAULT_BIAS_ONE[c]);
  float qf = (float)q;
  return qf - BIAS_NUMERATOR / qf;
}

/* ------------------------------------------------------------------ */
/* Contexts, scans and tokens                                          */
/* ------------------------------------------------------------------ */

/* libjxl CoeffOrderAndLut natural order as used by
 * src/coeff_order.rs:203-244 (cx = cy = 1). */
static void natural_scan_8x8(uint8_t* scan) {
  int cur = 1;
  for (int i = 0; i < 8; i++)
    for (int j = 0; j <= i; j++) {
      int x = j, y = i - j;
      if (i & 1) { int t = x; x = y; y = t; }
      int val = (x < 1 && y < 1) ? 0 : cur++;
      scan[val] = (uint8_t)(y * 8 + x);
    }
  for (int ip = 7; ip >= 1; ip--) {
    int i = ip - 1;
    for (int j = 0; j <= i; j++) {
      int x = 7 - (i - j), y = 7 - j;
      if (i & 1) { int t = x; x = y; y = t; }
      scan[cur++] = (uint8_t)(y * 8 + x);
    }
  }
}

void orc_natural_scan_8x8(uint8_t* scan) { natural_scan_8x8(scan); }

/* K_COEFF_FREQ_CONTEXT (src/ac_context.rs:40-44), written as its bands. */
static int freq_context(int k) {
  if (k < 16) return k - 1;
  if (k < 32) return 15 + (k - 16) / 2;
  return 23 + (k - 32) / 4;
}

/* K_COEFF_NUM_NONZERO_CONTEXT (src/ac_context.rs:47-53), as its bands. */
static int nonzero_context(int n) {
  if (n <= 1) return 0;
  if (n == 2) return 31;
  if (n <= 4) return 62;
  if (n <= 8) return 93;
  if (n <= 12) return 123;
  if (n <= 20) return 152;
  if (n <= 32) return 180;
  return 206;
}

int32_t orc_freq_context(int32_t k) { return freq_context(k); }
int32_t orc_nonzero_context(int32_t n) { return nonzero_context(n); }

/* src/ac_context.rs:96-105 */
static uint32_t non_zero_bucket(uint32_t n) {
  if (n < 8) return n;
  if (n >= 64) return 36;
  return 4 + n / 2;
}

/* block_context for the DCT8 order: Y -> 0, X -> 7, B -> 7
 * (K_COMPACT_BLOCK_CONTEXT_MAP / K_STRATEGY_ORDER / CHANNEL_ROW,
 * src/ac_context.rs:62-92). */
static uint32_t fine_block_context_dct8(int c, int qf_hi) {
  uint32_t bc = c == 1 ? 0u : 7u;
  return bc * 2u + (uint32_t)qf_hi;
}

/* src/group.rs:89-106 */
static uint8_t predict_top_left(const uint8_t* top, const uint8_t* row, size_t x) {
  if (x == 0) return top ? top[x] : 32;
  if (!top) return row[x - 1];
  return (uint8_t)(((uint32_t)top[x] + (uint32_t)row[x - 1] + 1u) / 2u);
}

/* src/entropy/token.rs:159-162 */
static inline uint32_t pack_signed(int32_t v) {
  int64_t x = v;
  return (uint32_t)((x << 1) ^ (x >> 63));
}

/* src/entropy/token.rs:115-127 */
static inline uint32_t hybrid_token(uint32_t value) {
  if (value < 16) return value;
  uint32_t n = 31u - (uint32_t)__builtin_clz(value);
  uint32_t m = value - (1u << n);
  return (n << 2) + (m >> (n - 2));
}

uint32_t orc_hybrid_token(uint32_t v) { return hybrid_token(v); }

/* src/frame/ac_groups.rs:92-113 */
static uint32_t qf_threshold_of(const uint8_t* qf, size_t n) {
  uint64_t hist[257];
  memset(hist, 0, sizeof(hist));
  for (size_t i = 0; i < n; i++) hist[qf[i]]++;
  uint64_t total = n, acc = 0;
  for (uint32_t v = 0; v < 257; v++) {
    acc += hist[v];
    if (acc * 2 >= total) return v;
  }
  return 1;
}

/* compute_cmap_tile on the tile at blocks (0, 0) of an XYB image (3 planes
 * of w*h), for known-answer tests. */
int orc_cmap_tile0(const float* xyb, size_t w, size_t h, float distance, int8_t* ytox,
                   int8_t* ytob) {
  float mat[192], inv[192];
  int st = orc_dct8_tables(distance, mat, inv);
  if (st) return st;
  size_t xb = (w + 7) / 8, yb = (h + 7) / 8;
  cmap_tile(xyb, w, h, 0, 0, minz(8, xb), minz(8, yb), distance, inv, inv + 128, ytox, ytob);
  return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* Alpha: fringe clearing, invisible fill, AQ factors                   */
/* ------------------------------------------------------------------ */

/* Fringe level of a sample for one sweep of alpha_fringe::sweep
 * (src/alpha_fringe.rs:121-124): its distance from one end of the range
 * (`invert` = from full opacity), kept when within REACH levels, else 0. */
static inline uint32_t fringe_level(uint32_t a, uint32_t maxv, int invert) {
  uint32_t reach = 4u * maxv / 255u;
  uint32_t level = invert ? maxv - (a < maxv ? a : maxv) : a;
  return level <= reach ? level : 0u;
}

/* alpha_fringe::sweep (src/alpha_fringe.rs:112-223): a sample with a
 * non-zero fringe level is replaced when the fringe levels over the 9x9
 * window around it (clipped to the plane, original samples) average at most
 * half a level: sum * 2 * 255 <= window_samples * max.  The reference slides
 * the window row by row and defers replacements until a row leaves it; here
 * the window sums come from a summed-area table of the original levels,
 * which gives the same sums.  Marks go to `mark` (1 = replace); returns the
 * number marked. */
static size_t fringe_marks(const uint16_t* alpha, size_t w, size_t h, uint32_t maxv, int invert,
                           uint8_t* mark) {
  uint64_t* sat = (uint64_t*)calloc((w + 1) * (h + 1), sizeof(uint64_t));
  for (size_t y = 0; y < h; y++) {
    uint64_t row = 0;
    for (size_t x = 0; x < w; x++) {
      row += fringe_level(alpha[y * w + x], maxv, invert);
      sat[(y + 1) * (w + 1) + x + 1] = sat[y * (w + 1) + x + 1] + row;
    }
  }
  size_t marked = 0;
  for (size_t y = 0; y < h; y++) {
    size_t y0 = y >= 4 ? y - 4 : 0, y1 = minz(y + 5, h);
    for (size_t x = 0; x < w; x++) {
      mark[y * w + x] = 0;
      if (fringe_level(alpha[y * w + x], maxv, invert) == 0) continue;
      size_t x0 = x >= 4 ? x - 4 : 0, x1 = minz(x + 5, w);
      uint64_t sum = sat[y1 * (w + 1) + x1] - sat[y0 * (w + 1) + x1] - sat[y1 * (w + 1) + x0] +
                     sat[y0 * (w + 1) + x0];
      if (sum * 2u * 255u <= (uint64_t)((y1 - y0) * (x1 - x0)) * maxv) {
        mark[y * w + x] = 1;
        marked++;
      }
    }
  }
  free(sat);
  return marked;
}

/* alpha_fringe::clear (src/alpha_fringe.rs:78-108), in place: clear the
 * near-transparent fringe to 0, then, when at least one sample in 12 sits
 * within REACH below full opacity and the second sweep would change at
 * least one in 12, fill those to full opacity. */
void orc_alpha_fringe_clear(uint16_t* alpha, size_t w, size_t h, uint32_t maxv) {
  if (w == 0 || h == 0) return;
  size_t n = w * h;
  uint8_t* mark = (uint8_t*)malloc(n);
  fringe_marks(alpha, w, h, maxv, 0, mark);
  for (size_t i = 0; i < n; i++)
    if (mark[i]) alpha[i] = 0;
  uint32_t reach = 4u * maxv / 255u;
  size_t near_opaque = 0;
  for (size_t i = 0; i < n; i++) {
    uint32_t d = maxv - (alpha[i] < maxv ? alpha[i] : maxv);
    if (d >= 1 && d <= reach) near_opaque++;
  }
  if (near_opaque * 12 >= n) {
    size_t changed = fringe_marks(alpha, w, h, maxv, 1, mark);
    if (changed * 12 >= n)
      for (size_t i = 0; i < n; i++)
        if (mark[i]) alpha[i] = (uint16_t)maxv;
  }
  free(mark);
}

/* invisible::fill_invisible (src/invisible.rs:34-149) on one plane: every
 * zero-alpha sample, in raster order and in place, becomes the weighted
 * mean of its left (weight 1, +1 when visible), upper-right (1, +2 when
 * visible), and visible right, up, down and lower-right (2 each) neighbours,
 * summed in that order. */
static void fill_invisible_plane(float* p, const uint16_t* alpha, size_t w, size_t h) {
  for (size_t y = 0; y < h; y++) {
    int up = y > 0, down = y + 1 < h;
    const float* pu = up ? p + (y - 1) * w : p + y * w;
    const float* pd = down ? p + (y + 1) * w : p + y * w;
    const uint16_t* au = up ? alpha + (y - 1) * w : alpha + y * w;
    const uint16_t* ad = down ? alpha + (y + 1) * w : alpha + y * w;
    float* row = p + y * w;
    const uint16_t* ar = alpha + y * w;
    for (size_t x = 0; x < w; x++) {
      if (ar[x] != 0) continue;
      float sum = 0.0f, weight = 0.0f;
      if (x > 0) {
        sum += row[x - 1];
        weight += 1.0f;
        if (ar[x - 1] != 0) {
          sum += row[x - 1];
          weight += 1.0f;
        }
      }
      if (x + 1 < w) {
        if (up) {
          sum += pu[x + 1];
          weight += 1.0f;
        }
        if (ar[x + 1] != 0) {
          sum += 2.0f * row[x + 1];
          weight += 2.0f;
        }
        if (up && au[x + 1] != 0) {
          sum += 2.0f * pu[x + 1];
          weight += 2.0f;
        }
        if (down && ad[x + 1] != 0) {
          sum += 2.0f * pd[x + 1];
          weight += 2.0f;
        }
      }
      if (up && au[x] != 0) {
        sum += 2.0f * pu[x];
        weight += 2.0f;
      }
      if (down && ad[x] != 0) {
        sum += 2.0f * pd[x];
        weight += 2.0f;
      }
      row[x] = weight > 1.0f ? sum / weight : sum;
    }
  }
}

void orc_fill_invisible(float* xyb, const uint16_t* alpha, size_t w, size_t h) {
  size_t n = w * h;
  int any = 0;
  for (size_t i = 0; i < n && !any; i++) any = alpha[i] == 0;
  if (!any) return; /* src/invisible.rs:45-47 */
  for (int c = 0; c < 3; c++) fill_invisible_plane(xyb + c * n, alpha, w, h);
}

/* alpha_block_factors (src/adaptive_quant.rs:953-1028): per 8x8 block, the
 * largest alpha over the block, normalised by the full-opacity value; 1 for
 * fully transparent or fully opaque blocks, else at least ALPHA_AQ_FLOOR
 * (0.1). */
void orc_alpha_block_factors(const uint16_t* alpha, size_t w, size_t h, uint32_t maxv,
                             float* factors) {
  size_t xb = (w + 7) / 8, yb = (h + 7) / 8;
  for (size_t by = 0; by < yb; by++)
    for (size_t bx = 0; bx < xb; bx++) {
      uint32_t peak = 0;
      for (size_t y = by * 8; y < minz(by * 8 + 8, h); y++)
        for (size_t x = bx * 8; x < minz(bx * 8 + 8, w); x++)
          if (alpha[y * w + x] > peak) peak = alpha[y * w + x];
      float a = (float)peak / (float)maxv;
      factors[by * xb + bx] = (a == 0.0f || a >= 1.0f) ? 1.0f : (a > 0.1f ? a : 0.1f);
    }
}

/* apply_alpha_factors (src/adaptive_quant.rs:1036-1070) for an all-DCT8
 * layout: each block's raw field value times its factor, rounded half away
 * and clamped to 1..255.  Skipped for a constant alpha plane
 * (src/frame/encoder.rs:60-70). */
void orc_apply_alpha_factors(uint8_t* qf, const uint16_t* alpha, size_t w, size_t h,
                             uint32_t maxv) {
  size_t n = w * h;
  int constant = 1;
  for (size_t i = 1; i < n && constant; i++) constant = alpha[i] == alpha[0];
  if (constant) return;
  size_t xb = (w + 7) / 8, yb = (h + 7) / 8;
  float* k = (float*)malloc(xb * yb * sizeof(float));
  orc_alpha_block_factors(alpha, w, h, maxv, k);
  for (size_t i = 0; i < xb * yb; i++) {
    int32_t q = sat_i32(roundf((float)qf[i] * k[i]));
    qf[i] = (uint8_t)(q < 1 ? 1 : (q > 255 ? 255 : q));
  }
  free(k);
}

/* ------------------------------------------------------------------ */
/* Whole front end                                                      */
/* ------------------------------------------------------------------ */

typedef struct {
  /* inputs */
  const void* pixels;
  int32_t bits;             /* 8, or 10 / 12 / 16 in 16-bit words */
  int32_t channels;         /* 3 or 4 (RGBA: lossy alpha, fill_invisible on) */
  int32_t transfer;         /* H.273 transfer code; 0 = sRGB (the default encoding) */
  int32_t speed;            /* 0 UltraFast, 1 Fastest */
  uint64_t width, height;
  float distance;
  int32_t num_threads;
  /* outputs (caller-allocated; NULL skips) */
  float* xyb;            /* 3 * w * h */
  uint8_t* quant_field;  /* xb * yb */
  int8_t* ytox;          /* tx * ty */
  int8_t* ytob;          /* tx * ty */
  int16_t* quant_dc;     /* 3 * xb * yb, planes X, Y, B */
  int32_t* coeffs;       /* xb * yb * 192, [block][X,Y,B][64] */
  uint8_t* nzeros;       /* 3 * xb * yb */
  uint32_t* tokens;      /* 2 * token_capacity: (context, value) pairs */
  uint64_t token_capacity;
  uint64_t* group_offsets; /* num_groups + 1 */
  uint32_t* histograms;    /* NUM_FINE_AC_CONTEXTS * 128 */
  uint16_t* alpha;         /* w * h: the alpha plane after fringe clearing (RGBA only) */
  uint8_t* ac_strategy;    /* xb * yb AcStrategyImage cells: raw << 1 | first */
  /* scalar outputs */
  orc_params params;
  uint32_t qf_threshold;
  uint64_t constant_blocks;
  int32_t screen_content;
  int32_t epf_sharpness;
  uint64_t num_tokens;
  double stage_seconds[5]; /* xyb+stats, AQ, CfL, AC groups, merge */
} orc_frame;

static double now_seconds(void) {
#ifdef _OPENMP
  return omp_get_wtime();
#else
  return 0.0;
#endif
}

uint64_t orc_sizeof_frame(void) { return sizeof(orc_frame); }
int32_t orc_num_fine_contexts(void) { return NUM_FINE_AC_CONTEXTS; }

/* One AC group (process_ac_group + write_ac_group for an all-DCT8 layout,
 * src/frame/ac_groups.rs:116-250, src/group.rs:1259-2426). */
typedef struct {
  uint32_t* tok; /* pairs */
  uint64_t count;
} group_tokens;

#include "jxg_oracle_search.inc"

static void encode_ac_group(const orc_frame* f, const float* xyb, const float* mat,
                            const float* inv, const uint8_t* qf, const int8_t* ytox,
                            const int8_t* ytob, int16_t* quant_dc, int32_t* coeffs_out,
                            uint8_t* nz_out, size_t gx, size_t gy, uint32_t qf_threshold,
                            const uint8_t* scan, group_tokens* gt, uint32_t* hist) {
  const orc_params* p = &f->params;
  size_t w = f->width, h = f->height, n = w * h;
  size_t xb = (w + 7) / 8, yb = (h + 7) / 8;
  size_t tx_count = (xb + 7) / 8;
  size_t bx0 = gx * GROUP_BLOCKS, by0 = gy * GROUP_BLOCKS;
  size_t gwb = minz(GROUP_BLOCKS, xb - bx0), ghb = minz(GROUP_BLOCKS, yb - by0);
  float inv_factor[3];
  static const float inv_dc_quant[3] = {4096.0f, 512.0f, 256.0f};
  static const float dc_quant[3] = {1.0f / 4096.0f, 1.0f / 512.0f, 1.0f / 256.0f};
  for (int c = 0; c < 3; c++) inv_factor[c] = inv_dc_quant[c] / p->dc_step[c] * p->scale_dc;
  float cfl_b = inv_dc_quant[2] / p->dc_step[2] * (dc_quant[1] * p->dc_step[1]) *
                (1.0f + 0.0f / 84.0f);
  float cfl_x = inv_dc_quant[0] / p->dc_step[0] * (dc_quant[1] * p->dc_step[1]) * 0.0f;
  uint8_t nzmap[3][GROUP_BLOCKS * GROUP_BLOCKS];
  memset(nzmap, 0, sizeof(nzmap));
  uint64_t cap = (uint64_t)gwb * ghb * 3 * 64;
  gt->tok = (uint32_t*)malloc(cap * 2 * sizeof(uint32_t));
  gt->count = 0;
  float src[3][64], coef[3][64];
  int32_t q[3][64];
  for (size_t by = 0; by < ghb; by++)
    for (size_t bx = 0; bx < gwb; bx++) {
      size_t ibx = bx0 + bx, iby = by0 + by, bi = iby * xb + ibx;
      int32_t quant = qf[bi];
      /* footprint with edge replication (src/ac_strategy.rs:451-478) */
      for (int c = 0; c < 3; c++)
        for (int yy = 0; yy < 8; yy++)
          for (int xx = 0; xx < 8; xx++) {
            size_t sx = minz(ibx * 8 + xx, w - 1), sy = minz(iby * 8 + yy, h - 1);
            src[c][yy * 8 + xx] = xyb[(size_t)c * n + sy * w + sx];
          }
      for (int c = 0; c < 3; c++) dct8x8(src[c], 8, coef[c]);
      /* Y DC + AC round trip */
      int16_t ydc = sat_i16(roundf(coef[1][0] * inv_factor[1]));
      quantize_ac(coef[1], 1, inv + 64, quant, p->scale, 1.0f, p->distance, q[1]);
      float inv_qac = 1.0f / (p->scale * (float)quant);
      for (int k = 0; k < 64; k++) coef[1][k] = bias_level(1, q[1][k]) * mat[64 + k] * inv_qac;
      /* CfL */
      size_t t = (iby / 8) * tx_count + ibx / 8;
      float xf = fmla((float)ytox[t], 1.0f / 84.0f, 0.0f);
      float bf = fmla((float)ytob[t], 1.0f / 84.0f, 1.0f);
      coef[1][0] = 0.0f;
      for (int k = 0; k < 64; k++) {
        coef[0][k] = fmla(-xf, coef[1][k], coef[0][k]);
        coef[2][k] = fmla(-bf, coef[1][k], coef[2][k]);
      }
      int16_t xdc;
      if (cfl_x != 0.0f) xdc = sat_i16(roundf(fmla(coef[0][0], inv_factor[0], -(float)ydc * cfl_x)));
      else xdc = sat_i16(roundf(coef[0][0] * inv_factor[0]));
      quantize_ac(coef[0], 0, inv, quant, p->scale, p->x_qm_mul, p->distance, q[0]);
      int16_t bdc = sat_i16(roundf(fmla(coef[2][0], inv_factor[2], -(float)ydc * cfl_b)));
      quantize_ac(coef[2], 2, inv + 128, quant, p->scale, p->b_qm_mul, p->distance, q[2]);
      size_t nb = xb * yb;
      quant_dc[0 * nb + bi] = xdc;
      quant_dc[1 * nb + bi] = ydc;
      quant_dc[2 * nb + bi] = bdc;
      if (coeffs_out)
        for (int c = 0; c < 3; c++) memcpy(coeffs_out + bi * 192 + c * 64, q[c], 64 * 4);
      /* tokens in channel order Y, X, B */
      static const int order[3] = {1, 0, 2};
      for (int oi = 0; oi < 3; oi++) {
        int c = order[oi];
        const int32_t* blk = q[c];
        int32_t nzeros = 0;
        for (int k = 1; k < 64; k++) nzeros += blk[k] != 0;
        nzmap[c][by * GROUP_BLOCKS + bx] = (uint8_t)nzeros;
        if (nz_out) nz_out[(size_t)c * nb + bi] = (uint8_t)nzeros;
        const uint8_t* top = by ? &nzmap[c][(by - 1) * GROUP_BLOCKS] : NULL;
        uint8_t predicted = predict_top_left(top, &nzmap[c][by * GROUP_BLOCKS], bx);
        uint32_t bctx = fine_block_context_dct8(c, (uint32_t)quant > qf_threshold);
        uint32_t nz_ctx = non_zero_bucket(predicted) * NUM_FINE_BLOCK_CTXS + bctx;
        uint32_t histo = NUM_FINE_BLOCK_CTXS * NON_ZERO_BUCKETS + ZERO_DENSITY_CONTEXTS * bctx;
        uint32_t* o = gt->tok + gt->count * 2;
        o[0] = nz_ctx;
        o[1] = (uint32_t)nzeros;
        gt->count++;
        hist[nz_ctx * ALPHABET + hybrid_token((uint32_t)nzeros)]++;
        int prev = nzeros > 64 / 16 ? 0 : 1;
        int32_t remaining = nzeros;
        for (int k = 1; k < 64 && remaining != 0; k++) {
          int32_t v = blk[scan[k]];
          uint32_t ctx = histo + (uint32_t)((nonzero_context(remaining) + freq_context(k)) * 2 + prev);
          uint32_t val = pack_signed(v);
          o = gt->tok + gt->count * 2;
          o[0] = ctx;
          o[1] = val;
          gt->count++;
          hist[ctx * ALPHABET + hybrid_token(val)]++;
          prev = v != 0;
          if (v != 0) remaining--;
        }
      }
    }
}

/* encode_frame_core_inner through pass one (src/frame/vardct_encoder.rs:798-1100)
 * for Speed::UltraFast: DC-group setup (AQ + CfL, all-DCT8 layout), the qf
 * threshold, then every AC group. */
int orc_frontend(orc_frame* f) {
  size_t w = f->width, h = f->height;
  if (w == 0 || h == 0) return ORC_ERR_EMPTY;
  if (!(f->bits == 8 || f->bits == 10 || f->bits == 12 || f->bits == 16)) return ORC_ERR_INPUT;
  if (f->channels < 1 || f->channels > 4) return ORC_ERR_INPUT;
  int st = orc_params_for(f->distance, &f->params);
  if (st) return st;
  /* Fastest searches transforms unless the distance takes the DCT8-only
   * shortcut (use_dct8_only, src/ac_strategy.rs:73-80); up to 1.709 the
   * reference also reranks merges in the reconstruction domain
   * (FAST_RERANK_MAX_DISTANCE, src/ac_strategy.rs:67), which is not
   * restated here */
  if (f->speed != 0 && f->speed != 1) return ORC_ERR_UNSUPPORTED;
  const int search = f->speed == 1 && !(f->params.distance <= 0.056713393f);
  if (search && f->params.distance <= 1.7090991223128462f) return ORC_ERR_UNSUPPORTED;
  float mat[192], inv[192];
  st = orc_dct8_tables(f->params.distance, mat, inv);
  if (st) return st;
  init_exp2_table();
#ifdef _OPENMP
  int threads = f->num_threads > 0 ? f->num_threads : omp_get_max_threads();
  omp_set_num_threads(threads);
#endif
  size_t n = w * h;
  size_t xb = (w + 7) / 8, yb = (h + 7) / 8, nb = xb * yb;
  size_t txn = (xb + 7) / 8, tyn = (yb + 7) / 8;
  size_t xg = (w + GROUP - 1) / GROUP, yg = (h + GROUP - 1) / GROUP;
  size_t xdc = (w + DC_GROUP - 1) / DC_GROUP, ydc = (h + DC_GROUP - 1) / DC_GROUP;
  float* xyb = f->xyb ? f->xyb : (float*)malloc(3 * n * sizeof(float));
  uint8_t* qf = f->quant_field ? f->quant_field : (uint8_t*)malloc(nb);
  int8_t* ytox = f->ytox ? f->ytox : (int8_t*)malloc(txn * tyn);
  int8_t* ytob = f->ytob ? f->ytob : (int8_t*)malloc(txn * tyn);
  int16_t* qdc = f->quant_dc ? f->quant_dc : (int16_t*)malloc(3 * nb * sizeof(int16_t));
  if (!xyb || !qf || !ytox || !ytob || !qdc) return ORC_ERR_ALLOC;
  double t0 = now_seconds();
  st = orc_to_xyb(f->pixels, f->bits, f->transfer, f->channels, w, h, xyb);
  if (st) return st;
  /* RGBA (encode_lossy_u8_alpha_arms, src/encode_image.rs:3639-3657, and
   * encode_high_depth_rgba :4290-4303): the alpha plane loses its fringe,
   * then the XYB planes their invisible colours (src/frame/encoder.rs:152) */
  uint16_t* alpha = NULL;
  /* the largest code value; high-depth alpha is capped to it
   * (encode_high_depth_rgba, src/encode_image.rs:4270-4290) */
  const uint32_t alpha_max = (1u << f->bits) - 1u;
  if (f->channels == 4 || f->channels == 2) { /* RGBA, or grey + alpha (encode_gray_impl) */
    alpha = f->alpha ? f->alpha : (uint16_t*)malloc(n * sizeof(uint16_t));
    if (!alpha) return ORC_ERR_ALLOC;
    for (size_t i = 0; i < n; i++) {
      const size_t at = i * (size_t)f->channels + (size_t)f->channels - 1;
      const uint32_t a = f->bits == 8 ? ((const uint8_t*)f->pixels)[at]
                                      : ((const uint16_t*)f->pixels)[at];
      alpha[i] = (uint16_t)(a < alpha_max ? a : alpha_max);
    }
    orc_alpha_fringe_clear(alpha, w, h, alpha_max);
    orc_fill_invisible(xyb, alpha, w, h);
  }
  /* grey input is encoded as achromatic (with_grayscale, src/encode_image.rs:3968):
   * snap_achromatic_xyb (src/frame/encoder.rs:155-157, :351-357) sets X to 0
   * and B to Y after the XYB conversion and the invisible fill */
  if (f->channels < 3) orc_snap_achromatic(xyb, n);
  f->constant_blocks = orc_constant_blocks(xyb, w, h);
  f->screen_content = orc_is_screen_content(f->constant_blocks, w, h);
  f->epf_sharpness = orc_epf_sharpness_id(f->params.distance, f->screen_content);
  float inv_scale = 1.0f / f->params.scale;
  double t1 = now_seconds();
  /* DC groups: AQ field, then CfL tiles (setup_dc_group, src/frame/dc_groups.rs:127-180) */
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic) num_threads(threads)
#endif
  for (long g = 0; g < (long)(xdc * ydc); g++) {
    size_t gx = (size_t)g % xdc, gy = (size_t)g / xdc;
    size_t x0 = gx * DC_GROUP, y0 = gy * DC_GROUP;
    size_t gxs = minz(DC_GROUP, w - x0), gys = minz(DC_GROUP, h - y0);
    size_t gxb = (gxs + 7) / 8, gyb = (gys + 7) / 8;
    fill_quant_field(xyb, w, h, x0, y0, gxb, gyb, f->params.distance, inv_scale, qf, xb);
  }
  /* the alpha factors come last in setup_dc_group (src/frame/dc_groups.rs:303-312):
   * for an all-DCT8 layout here, after the transform search otherwise */
  if (alpha && !search) orc_apply_alpha_factors(qf, alpha, w, h, alpha_max);
  double t2 = now_seconds();
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic) num_threads(threads)
#endif
  for (long t = 0; t < (long)(txn * tyn); t++) {
    size_t tx = (size_t)t % txn, ty = (size_t)t / txn;
    /* tiles never cross DC groups (2048 = 32 tiles); clip to the DC group */
    size_t bx0 = tx * 8, by0 = ty * 8;
    size_t dcbx_end = minz(((bx0 / 256) + 1) * 256, xb);
    size_t dcby_end = minz(((by0 / 256) + 1) * 256, yb);
    size_t bxc = minz(8, dcbx_end - bx0), byc = minz(8, dcby_end - by0);
    cmap_tile(xyb, w, h, bx0, by0, bxc, byc, f->params.distance, inv, inv + 128, &ytox[t],
              &ytob[t]);
  }
  uint8_t* map = f->ac_strategy ? f->ac_strategy : (uint8_t*)malloc(nb);
  if (!map) return ORC_ERR_ALLOC;
  for (size_t i = 0; i < nb; i++) map[i] = 1;
  orc_tables* tables = NULL;
  orc_orders* orders = NULL;
  if (search) {
    /* fill_ac_strategy per DC group, then the alpha factors over the layout,
     * then the frame's account_matrix_headers (src/frame/dc_groups.rs:183-312,
     * src/frame/vardct_encoder.rs:960-969) */
    tables = (orc_tables*)malloc(sizeof(orc_tables));
    orders = (orc_orders*)malloc(sizeof(orc_orders));
    uint8_t* block_qf = (uint8_t*)malloc(nb);
    if (!tables || !orders || !block_qf) return ORC_ERR_ALLOC;
    if ((st = orc_build_tables(f->params.distance, tables))) return st;
    build_orders(orders);
    init_rate_log2();
    memcpy(block_qf, qf, nb);
    search_ctx sc = {xyb, w, h, n, xb, yb, txn, tables, orders, f->params.distance, f->params.scale,
                     f->params.x_qm_mul, f->params.b_qm_mul, ytox, ytob};
    const float dampen = clampf(aq_schedule(AQ_STRENGTH, f->params.distance), 0.0f, 1.0f);
    fastest_search(&sc, qf, map, dampen);
    if (alpha) apply_alpha_factors_layout(qf, map, alpha, w, h, alpha_max);
    account_matrix_headers(&sc, qf, block_qf, map);
    free(block_qf);
  }
  double t3 = now_seconds();
  f->qf_threshold = qf_threshold_of(qf, nb);
  uint8_t scan[64];
  natural_scan_8x8(scan);
  size_t ng = xg * yg;
  group_tokens* gts = (group_tokens*)calloc(ng, sizeof(group_tokens));
  size_t hist_len = (size_t)NUM_FINE_AC_CONTEXTS * ALPHABET;
  if (f->histograms) memset(f->histograms, 0, hist_len * sizeof(uint32_t));
  uint32_t* hist = f->histograms ? f->histograms : (uint32_t*)calloc(hist_len, 4);
#ifdef _OPENMP
#pragma omp parallel num_threads(threads)
#endif
  {
    uint32_t* local = (uint32_t*)calloc(hist_len, 4);
#ifdef _OPENMP
#pragma omp for schedule(dynamic)
#endif
    for (long g = 0; g < (long)ng; g++) {
      size_t gx = (size_t)g % xg, gy = (size_t)g / xg;
      if (search)
        encode_ac_group_layout(f, xyb, tables, orders, map, qf, ytox, ytob, qdc, f->coeffs,
                               f->nzeros, gx, gy, f->qf_threshold, &gts[g], local);
      else
        encode_ac_group(f, xyb, mat, inv, qf, ytox, ytob, qdc, f->coeffs, f->nzeros, gx, gy,
                        f->qf_threshold, scan, &gts[g], local);
    }
#ifdef _OPENMP
#pragma omp critical
#endif
    for (size_t i = 0; i < hist_len; i++) hist[i] += local[i];
    free(local);
  }
  double t4 = now_seconds();
  uint64_t total = 0;
  uint64_t* starts = (uint64_t*)malloc((ng + 1) * sizeof(uint64_t));
  for (size_t g = 0; g < ng; g++) {
    starts[g] = total;
    total += gts[g].count;
  }
  starts[ng] = total;
  if (f->group_offsets) memcpy(f->group_offsets, starts, (ng + 1) * sizeof(uint64_t));
  int fits = f->tokens && total <= f->token_capacity;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic) num_threads(threads)
#endif
  for (long g = 0; g < (long)ng; g++) {
    if (fits) memcpy(f->tokens + starts[g] * 2, gts[g].tok, gts[g].count * 2 * sizeof(uint32_t));
    free(gts[g].tok);
  }
  free(starts);
  f->num_tokens = total;
  double t5 = now_seconds();
  f->stage_seconds[0] = t1 - t0;
  f->stage_seconds[1] = t2 - t1;
  f->stage_seconds[2] = t3 - t2;
  f->stage_seconds[3] = t4 - t3;
  f->stage_seconds[4] = t5 - t4;
  free(gts);
  free(tables);
  free(orders);
  if (!f->ac_strategy) free(map);
  if (!f->histograms) free(hist);
  if (!f->xyb) free(xyb);
  if (alpha && !f->alpha) free(alpha);
  if (!f->quant_field) free(qf);
  if (!f->ytox) free(ytox);
  if (!f->ytob) free(ytob);
  if (!f->quant_dc) free(qdc);
  if (f->tokens && total > f->token_capacity) return ORC_ERR_ALLOC;
  return ORC_OK;
}

/* fill_quant_field over every DC group of an XYB image (the oracle side of
 * the FillQuantFieldFn operator, src/adaptive_quant.rs:474). */
/* apply_chroma_hf_protection (src/adaptive_quant.rs:303-402) over a whole
 * frame's field, with chroma_hf_stats_scalar (:222-279): per 8x8 block (cut
 * at the image edge) the opponent magnitude and the chroma and luma gradient
 * sums in the reference's order, then the fitted boost of blocks whose edges
 * are mostly chromatic. */
void orc_chroma_hf_protection(const float* xyb, size_t w, size_t h, float distance, uint8_t* field) {
  const float fade_in_start = 0.35f, fade_in_width = 0.40f, fade_out_start = 1.0f;
  const float fade_out_width = 1.0f, strength = 0.40f, ceil_base = 0.35f, ceil_share = 1.4f;
  const size_t xb = (w + 7) / 8, yb = (h + 7) / 8, n = w * h;
  if (xb == 0 || yb == 0 || distance < fade_in_start) return;
  const float fade_in = clampf((distance - fade_in_start) / fade_in_width, 0.0f, 1.0f);
  const float fade_out = 1.0f - clampf((distance - fade_out_start) / fade_out_width, 0.0f, 1.0f);
  const float distance_strength = strength * fade_in * fade_out;
  if (distance_strength <= 0.0f) return;
  const float *X = xyb, *Y = xyb + n, *B = xyb + 2 * n;
  for (size_t by = 0; by < yb; by++)
    for (size_t bx = 0; bx < xb; bx++) {
      const size_t px = bx * 8, py = by * 8;
      const size_t bw = w - px < 8 ? w - px : 8, bh = h - py < 8 ? h - py : 8;
      float chroma_sum = 0.0f, chroma_grad = 0.0f, luma_grad = 0.0f;
      size_t edges = 0;
      for (size_t y = py; y < py + bh; y++)
        for (size_t x = px; x < px + bw; x++) {
          const size_t i = y * w + x;
          chroma_sum += fabsf(X[i]) + fabsf(B[i] - Y[i]);
        }
      if (bw > 1) {
        for (size_t y = py; y < py + bh; y++)
          for (size_t x = px; x + 1 < px + bw; x++) {
            const size_t i = y * w + x, j = i + 1;
            chroma_grad += fabsf(X[j] - X[i]) + fabsf((B[j] - Y[j]) - (B[i] - Y[i]));
            luma_grad += fabsf(Y[j] - Y[i]);
          }
        edges += (bw - 1) * bh;
      }
      if (bh > 1) {
        for (size_t y = py; y + 1 < py + bh; y++)
          for (size_t x = px; x < px + bw; x++) {
            const size_t i = y * w + x, j = i + w;
            chroma_grad += fabsf(X[j] - X[i]) + fabsf((B[j] - Y[j]) - (B[i] - Y[i]));
            luma_grad += fabsf(Y[j] - Y[i]);
          }
        edges += bw * (bh - 1);
      }
      if (edges == 0) continue;
      const float mean_chroma = chroma_sum / (float)(bw * bh);
      const float mean_gradient = chroma_grad / (float)edges;
      const float chroma_share = chroma_grad / (chroma_grad + luma_grad + 1e-4f);
      const float chroma_w = clampf((mean_chroma - 0.025f) / 0.075f, 0.0f, 1.0f);
      const float gradient_w = clampf((mean_gradient - 0.006f) / 0.030f, 0.0f, 1.0f);
      const float share_w = clampf((chroma_share - 0.25f) / 0.55f, 0.0f, 1.0f);
      const float risk = chroma_w * gradient_w * share_w;
      if (risk > 0.0f) {
        const float ceiling = fmla(ceil_share, share_w * share_w, ceil_base);
        const float gain = fmla(ceiling * distance_strength, risk, 1.0f);
        const float q = (float)field[by * xb + bx];
        field[by * xb + bx] = (uint8_t)clampf(roundf(q * gain), 1.0f, 255.0f);
      }
    }
}

void orc_fill_quant_field_image(const float* xyb, size_t w, size_t h, float distance,
                                float inv_scale, uint8_t* qf) {
  init_exp2_table();
  size_t xb = (w + 7) / 8;
  size_t xdc = (w + DC_GROUP - 1) / DC_GROUP, ydc = (h + DC_GROUP - 1) / DC_GROUP;
  for (size_t gy = 0; gy < ydc; gy++)
    for (size_t gx = 0; gx < xdc; gx++) {
      size_t x0 = gx * DC_GROUP, y0 = gy * DC_GROUP;
      size_t gxb = (minz(DC_GROUP, w - x0) + 7) / 8, gyb = (minz(DC_GROUP, h - y0) + 7) / 8;
      fill_quant_field(xyb, w, h, x0, y0, gxb, gyb, distance, inv_scale, qf, xb);
    }
}
