// Host-side per-frame constants.  Compiled with -ffp-contract=off: every
// fused multiply-add below is an explicit std::fma, as the reference's
// `fmla` (src/dct.rs:31-41) is on aarch64.
#include "frame_params.h"
#include "library_dct8.h"
#include "library_tables.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace jxg {
namespace {

inline float fmla(float a, float b, float c) { return std::fma(a, b, c); }

inline int32_t cast_i32(float v) {  // Rust `as i32`
  if (std::isnan(v)) return 0;
  if (v >= 2147483647.0f) return INT32_MAX;
  if (v <= -2147483648.0f) return INT32_MIN;
  return static_cast<int32_t>(v);
}

inline float clamp(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }

uint16_t to_half(float v) {  // IEEE binary16, round to nearest even
  uint32_t bits;
  std::memcpy(&bits, &v, 4);
  uint16_t sign = static_cast<uint16_t>((bits >> 16) & 0x8000u);
  int32_t e = static_cast<int32_t>((bits >> 23) & 0xFF) - 112;
  uint32_t mant = bits & 0x7FFFFFu;
  if (e >= 31) return sign | 0x7BFF;
  if (e <= 0) {
    if (e < -10) return sign;
    uint32_t m = mant | 0x800000u;
    uint32_t shift = static_cast<uint32_t>(14 - e);
    uint32_t r = (m + (1u << (shift - 1)) - 1 + ((m >> shift) & 1)) >> shift;
    return sign | static_cast<uint16_t>(r);
  }
  uint32_t m = (mant + 0xFFFu + ((mant >> 13) & 1)) >> 13;
  uint32_t ex = static_cast<uint32_t>(e);
  if (m == 0x400) {
    m = 0;
    if (++ex >= 31) return sign | 0x7BFF;
  }
  return sign | static_cast<uint16_t>(ex << 10) | static_cast<uint16_t>(m);
}

float from_half(uint16_t h) {
  uint32_t e = (h >> 10) & 0x1F, m = h & 0x3FF;
  float v;
  if (e == 0) {
    v = (1.0f / 16384.0f) * (static_cast<float>(m) * (1.0f / 1024.0f));
  } else if (e == 31) {
    v = m ? NAN : INFINITY;
  } else {
    uint32_t b = ((e + 112u) << 23) | (m << 13);
    std::memcpy(&v, &b, 4);
  }
  return (h >> 15) ? -v : v;
}

inline float half_round(float v) { return from_half(to_half(v)); }

// dcepf_vlq_t, src/frame/quantization.rs:72-75
inline float vlq_t(float d) { return clamp((d - 8.0f) / (15.0f - 8.0f), 0.0f, 1.0f); }

// quant_dc, src/frame/quantization.rs:56-86
float luma_dc_quant(float d) {
  float refine;
  if (d <= 3.0f) {
    refine = 1.35f;
  } else if (d >= 5.0f) {
    refine = 1.0f;
  } else {
    const float recip = 1.0f / (5.0f - 3.0f);
    refine = fmla(1.0f - 1.35f, (d - 3.0f) * recip, 1.35f);
  }
  float vlq = fmla(vlq_t(d), 0.7f - 1.0f, 1.0f);
  float eff = 2.9f * std::pow(d / 2.9f, 0.57f);
  eff = clamp(eff, 0.5f * d, d);
  return std::min(1.12f / eff, 50.0f) * refine * vlq;
}

// luma_dc_coarsening, src/frame/quantization.rs:163-178
float dc_coarsening(float d) {
  float t;
  if (d <= 1.25f || d >= 5.0f) t = 0.0f;
  else if (d < 1.75f) t = (d - 1.25f) / (1.75f - 1.25f);
  else if (d <= 4.25f) t = 1.0f;
  else t = (5.0f - d) / (5.0f - 4.25f);
  return fmla(t, 1.15f - 1.0f, 1.0f);
}

const float kDcQuant[3] = {1.0f / 4096.0f, 1.0f / 512.0f, 1.0f / 256.0f};
const float kInvDcQuant[3] = {4096.0f, 512.0f, 256.0f};

// signaled_dc_step, src/color_correlation.rs:1835-1838
float wire_dc_step(int c, float mul) {
  return half_round(kDcQuant[c] * 128.0f * mul) / (kDcQuant[c] * 128.0f);
}

// DCT8 band parameters (src/quant_weights.rs:123-131)
const float kDct8Bands[3][6] = {{3150.0f, 0.0f, -0.4f, -0.4f, -0.4f, -2.0f},
                                {560.0f, 0.0f, -0.3f, -0.3f, -0.3f, -0.3f},
                                {512.0f, -2.0f, -1.0f, 0.0f, -1.0f, -2.0f}};
const float kFlatB8Hq[6] = {512.0f, -0.5f, -0.25f, 0.0f, -0.25f, -0.5f};
const float kFlatB8Mid[6] = {512.0f, -0.13f, -0.235f, -0.276f, -0.609f, -0.339f};

inline float band_mult(float v) { return v > 0.0f ? 1.0f + v : 1.0f / (1.0f - v); }

void round_bands(float b[3][6]) {
  for (int c = 0; c < 3; ++c)
    for (int i = 0; i < 6; ++i)
      b[c][i] = i == 0 ? half_round(b[c][i] / 64.0f) * 64.0f : half_round(b[c][i]);
}

}  // namespace

float distance_from_quality(float quality) {
  float q = clamp(quality, 0.0f, 100.0f);
  float d;
  if (q >= 99.0f) d = 0.05f * std::pow(2.0f, 100.0f - q);
  else if (q >= 90.0f) d = std::pow(10.0f, (99.0f - q) / 9.0f - 1.0f);
  else if (q >= 30.0f) d = 0.1f + (100.0f - q) * 0.09f;
  else d = 6.24f + std::pow(2.5f, (30.0f - q) / 5.0f) / 6.25f;
  return std::min(d, 25.0f);
}

int compute_distance_params(float distance, DistanceParams* p) {
  if (!(distance > 0.0f) || std::isinf(distance)) return 1;
  const float d = std::max(distance, 0.05f);  // MIN_DISTANCE, src/encode_image.rs:95
  float fine = luma_dc_quant(d);
  float coarsen = dc_coarsening(d);
  float qdc = fine / coarsen;
  float scale = 65536.0f * 0.8f / (d * 10.0f);
  int32_t gs = std::clamp(cast_i32(std::round(scale)), 1, 1 << 15);
  float scale_f = static_cast<float>(gs) / 65536.0f;
  int32_t qd = std::clamp(cast_i32((qdc / scale_f) + 0.5f), 1, 1 << 16);
  p->distance = d;
  p->global_scale = gs;
  p->quant_dc = qd;
  p->scale = scale_f;
  p->scale_dc = static_cast<float>(qd) * scale_f;
  p->x_qm_scale = 2u + (d >= 1.25f) + (d > 9.0f) + (d < 0.299f);
  p->b_qm_scale = 2;
  uint32_t iters = (d >= 0.7f) + (d >= 1.5f);
  float t = vlq_t(d);
  bool pass0 = d >= 2.5f && t < 0.5f;  // epf_pass0_scale is Some
  if (pass0 || t >= 0.5f) iters = 3;
  p->epf_iters = iters;
  // chroma_dc_steps, src/frame/quantization.rs:188-194
  float growth = std::max(luma_dc_quant(3.5f) / fine, 1.0f);
  float x = 2.0f * std::pow(growth, 0.75f - 1.0f);
  float b = std::pow(growth, 0.5f - 1.0f);
  p->dc_step[0] = wire_dc_step(0, x / coarsen);
  p->dc_step[1] = wire_dc_step(1, 1.0f);
  p->dc_step[2] = wire_dc_step(2, b / coarsen);
  p->x_qm_mul = std::pow(1.25f, static_cast<float>(p->x_qm_scale) - 2.0f);
  static const float kBMul[6] = {1.0f, 1.25f, 1.5625f, 1.953125f, 2.4414062f, 3.0517578f};
  p->b_qm_mul = kBMul[p->b_qm_scale - 2];
  return 0;
}

int dct8_tables(float distance, float matrix[3][64], float inv[3][64]) {
  const float d = std::max(distance, 0.05f);
  if (d < 0.3f) {
    // DequantMatrices::new below the flat-B gate: the library table
    // (src/quant_weights.rs:2261-2291, :1986-1992)
    for (int c = 0; c < 3; ++c) {
      std::memcpy(matrix[c], kLibraryDct8Bits[c], sizeof(float) * 64);
      inv[c][0] = 0.0f;
      for (int k = 1; k < 64; ++k) inv[c][k] = 1.0f / matrix[c][k];
    }
    return 0;
  }
  const bool ss2 = d >= 2.25f;
  const bool coarse = ss2 && d >= 3.5f;
  const float* flat = d >= 1.25f ? kFlatB8Mid : kFlatB8Hq;
  float bands[3][6];
  std::memcpy(bands, kDct8Bands, sizeof(bands));
  if (coarse) {  // coarse_dct8_override, src/quant_weights.rs:170-200
    float step = std::pow(1.25f, 1.0f / 5.0f);
    for (int i = 1; i < 6; ++i) {
      float r = band_mult(kDct8Bands[1][i]) * step;
      bands[1][i] = r > 1.0f ? r - 1.0f : 1.0f - 1.0f / r;
    }
    round_bands(bands);
  }
  std::memcpy(bands[2], flat, sizeof(float) * 6);
  round_bands(bands);
  // compute_dct8x8_matrix, src/quant_weights.rs:1564-1586
  for (int c = 0; c < 3; ++c) {
    float acc[6];
    acc[0] = bands[c][0];
    for (int i = 1; i < 6; ++i) acc[i] = acc[i - 1] * band_mult(bands[c][i]);
    float sc = (6.0f - 1.0f) / (1.41421356237309505f + 1e-6f);
    float rcp = sc / 7.0f;
    for (int y = 0; y < 8; ++y) {
      float dy = static_cast<float>(y) * rcp;
      float dy2 = dy * dy;
      for (int x = 0; x < 8; ++x) {
        float dx = static_cast<float>(x) * rcp;
        float pos = std::sqrt(fmla(dx, dx, dy2));
        float fl = std::floor(pos);
        float frac = pos - fl;
        size_t idx = static_cast<size_t>(fl);
        float a = acc[idx], bb = acc[idx + 1];
        matrix[c][y * 8 + x] = 1.0f / (std::pow(bb / a, frac) * a);
      }
    }
    inv[c][0] = 0.0f;
    for (int k = 1; k < 64; ++k) inv[c][k] = 1.0f / matrix[c][k];
  }
  return 0;
}

void fill_kernel_args(const DistanceParams& p, KernelArgs* a) {
  const float d = p.distance;
  a->distance = d;
  a->scale = p.scale;
  a->inv_scale = 1.0f / p.scale;
  for (int c = 0; c < 3; ++c) a->inv_dc_factor[c] = kInvDcQuant[c] / p.dc_step[c] * p.scale_dc;
  // dc_cfl_factor_x / dc_cfl_factor, src/color_correlation.rs:1598-1611
  a->cfl_dc_factor_x = kInvDcQuant[0] / p.dc_step[0] * (kDcQuant[1] * p.dc_step[1]) * 0.0f;
  a->cfl_dc_factor_b =
      kInvDcQuant[2] / p.dc_step[2] * (kDcQuant[1] * p.dc_step[1]) * (1.0f + 0.0f / 84.0f);
  a->qm_mul[0] = p.x_qm_mul;
  a->qm_mul[1] = 1.0f;
  a->qm_mul[2] = p.b_qm_mul;
  // quantize_ac_thresholds_scaled, src/group.rs:420-455 (one 8x8 block)
  for (int c = 0; c < 3; ++c) {
    float normal[4] = {0.58f, 0.635f, 0.66f, 0.7f};
    if (c == 0) {
      float up = clamp((d - 0.5f) / (0.75f - 0.5f), 0.0f, 1.0f);
      float down = clamp((2.0f - d) / (2.0f - 1.5f), 0.0f, 1.0f);
      float w = std::min(up, down);
      normal[0] += w * (0.5f - normal[0]);
      for (int i = 1; i < 4; ++i) normal[i] += (1.0f - w) * 0.08f;
    } else if (c == 2) {
      float hf = a->qm_mul[2] > 1.0f ? 0.65f : 0.75f;
      for (int i = 1; i < 4; ++i) normal[i] = hf;
    }
    const float hq_y[4] = {0.50f, 0.51f, 0.52f, 0.54f};
    const float* hq = c == 1 ? hq_y : normal;
    float t = clamp((d - 0.1f) / 0.9f, 0.0f, 1.0f);
    for (int i = 0; i < 4; ++i) a->thresholds[c][i] = hq[i] + t * (normal[i] - hq[i]);
  }
  // fill_quant_field_scalar stage 3 and FuzzyErosion weights,
  // src/adaptive_quant.rs:658-700 and :103-120
  static const float knots[7] = {0.5f, 1.0f, 1.4f, 1.75f, 3.0f, 5.0f, 8.0f};
  static const float strength[7] = {0.26565f, 0.275459f, 0.058287f, 0.0f, 0.0f, 0.0f, 0.0f};
  static const float base[7] = {0.636493f, 0.648351f, 0.606759f, 0.48f, 0.48f, 0.48f, 0.48f};
  auto sched = [&](const float* v) {
    if (d <= knots[0]) return v[0];
    for (int i = 1; i < 7; ++i)
      if (d <= knots[i]) {
        float f = (d - knots[i - 1]) / (knots[i] - knots[i - 1]);
        return v[i - 1] + f * (v[i] - v[i - 1]);
      }
    return v[6];
  };
  float aq_scale = 0.8294f / d;
  float base_level = sched(base) * aq_scale;
  float dampen = clamp(sched(strength), 0.0f, 1.0f);
  a->aq_mul = aq_scale * dampen;
  a->aq_add = (1.0f - dampen) * base_level;
  a->aq_hf_strength = clamp(1.06836f * d, 0.1f, 0.890398f);
  float fe_mul = d < 2.0f ? (2.0f - d) * 0.5f : 0.0f;
  const float fe_base[4] = {0.125f, 0.1f, 0.09f, 0.06f};
  const float fe_add[4] = {0.0f, -0.1f, -0.09f, -0.06f};
  float norm = 0.0f;
  for (int i = 0; i < 4; ++i) {
    a->aq_fe_weights[i] = fe_base[i] + fe_mul * fe_add[i];
    norm += a->aq_fe_weights[i];
  }
  const float total = 0.29959705784054957f;
  for (int i = 0; i < 4; ++i) a->aq_fe_weights[i] *= total / norm;
  const float k_mul = 211.66567973503678f;
  const float mul_v = k_mul * 1e8f;
  a->aq_masking_sqrt_mul = std::sqrt(mul_v);
  // cfl_deadzone, src/color_correlation.rs:384-394
  if (d <= 1.0f) a->cfl_deadzone = 1.5f;
  else if (d >= 2.0f) a->cfl_deadzone = 0.0f;
  else a->cfl_deadzone = (1.5f / (2.0f - 1.0f)) * (2.0f - d);
}

int32_t epf_sharpness_id(float d, bool screen) {
  float t = vlq_t(d);
  if (t >= 0.75f) return 1;
  if (t >= 0.5f) return 2;
  if (t >= 0.25f) return 3;
  if (d < 1.4f || (screen && d < 5.0f)) return 7;
  if (d < 1.75f) return 6;
  if (d < 3.5f) return 5;
  return 4;
}

// LoopFilter::new at the encoder's defaults for XYB (src/epf_filter.rs:56-85)
// with compute_distance_params' pass-0 scale (src/frame/quantization.rs:
// 116-127, :200-216): a signalled bundle is read back through F16.
void loop_filter_params(float d, LoopFilterParams* out) {
  DistanceParams p{};
  compute_distance_params(d, &p);
  out->iters = p.epf_iters;
  const float t = vlq_t(d);
  out->channel_scale[0] = 40.0f;
  out->channel_scale[1] = 5.0f;
  out->channel_scale[2] = 3.5f;
  if (d >= 2.5f && t < 0.5f) {
    const float pass0 = fmla(2.0f * t, 0.9f - 3.6f, 3.6f);
    out->quant_mul = half_round(0.46f);
    out->pass0 = half_round(pass0);
    out->pass2 = half_round(6.5f);
    out->border = half_round(2.0f / 3.0f);
  } else {
    out->quant_mul = 0.46f;
    out->pass0 = 0.9f;
    out->pass2 = 6.5f;
    out->border = 2.0f / 3.0f;
  }
}

float f16_round(float v) { return half_round(v); }

bool is_screen_content(uint64_t constant_blocks, uint64_t w, uint64_t h) {
  uint64_t bw = w / 8, bh = h / 8;
  if (bw == 0 || bh == 0) return false;
  return static_cast<float>(constant_blocks) / static_cast<float>(bw * bh) >= 0.15f;
}

void srgb_to_linear_table(float out[256]) {
  // srgb_to_linear_u8_ref, src/color.rs:35-42: f64 math, f32 result
  for (int v = 0; v < 256; ++v) {
    double x = static_cast<double>(v) * (1.0 / 255.0);
    out[v] = static_cast<float>(x <= 0.04045 ? x / 12.92 : std::pow((x + 0.055) / 1.055, 2.4));
  }
}

namespace {

// The transfer functions of integer samples (src/color.rs:44-199), on the
// sample over the largest code value, in f32 with the C library's powf.
float unit_clamp(float v) { return v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v); }
float decode_srgb(float v) {  // srgb_to_linear_f32
  v = unit_clamp(v);
  return v <= 0.04045f ? v / 12.92f : ::powf((v + 0.055f) / 1.055f, 2.4f);
}
float decode_linear(float v) { return unit_clamp(v); }
float decode_bt709(float v) {
  v = unit_clamp(v);
  const float alpha = 1.0992968f, beta = 0.01805397f;
  return v < 4.5f * beta ? v / 4.5f : ::powf((v + alpha - 1.0f) / alpha, 1.0f / 0.45f);
}
float decode_bt470m(float v) { return ::powf(unit_clamp(v), 2.2f); }
float decode_bt470bg(float v) { return ::powf(unit_clamp(v), 2.8f); }
float decode_smpte240(float v) {
  v = unit_clamp(v);
  return v < 0.0912f ? v / 4.0f : ::powf((v + 0.1115f) / 1.1115f, 1.0f / 0.45f);
}
float decode_smpte428(float v) { return ::powf(unit_clamp(v), 2.6f); }

}  // namespace

namespace {

// select_transfer, src/color.rs:201-222
int select_decode(int transfer, float (**decode)(float)) {
  switch (transfer) {
    case 1: case 6: case 14: case 15: *decode = decode_bt709; return 0;
    case 4: *decode = decode_bt470m; return 0;
    case 5: *decode = decode_bt470bg; return 0;
    case 7: *decode = decode_smpte240; return 0;
    case 8: *decode = decode_linear; return 0;
    case 17: *decode = decode_smpte428; return 0;
    case 0: case 2: case 9: case 10: case 11: case 12: case 13: *decode = decode_srgb; return 0;
    case 16: case 18: return 1;  // PQ and HLG: display model not built
    default: return 2;
  }
}

}  // namespace

int transfer_status(int transfer) {
  float (*decode)(float) = nullptr;
  return select_decode(transfer, &decode);
}

int transfer_table(int bits, int transfer, float* out) {
  if (bits != 8 && bits != 10 && bits != 12 && bits != 16) return 2;
  float (*decode)(float) = nullptr;
  const int st = select_decode(transfer, &decode);
  if (st) return st;
  // 0 is the C ABI's "not set" (the default encoding, sRGB = 13), not H.273
  // Reserved; only 8-bit sRGB takes the f64 table (src/color.rs:315-318)
  if (bits == 8 && (transfer == 0 || transfer == 13)) {
    srgb_to_linear_table(out);
    return 0;
  }
  const int size = 1 << bits, domain = bits == 8 ? 256 : 65536;
  const float max = static_cast<float>(size - 1);
  for (int v = 0; v < domain; ++v) out[v] = v < size ? decode(static_cast<float>(v) / max) : 0.0f;
  return 0;
}

namespace {

// scaled_override (src/quant_weights.rs:202-222): the base band scaled,
// every parameter F16 round-tripped as signalled
void scaled_override(const float* defaults, int nb, float scale, float* out) {
  for (int c = 0; c < 3; ++c)
    for (int i = 0; i < nb; ++i) {
      const float v = i == 0 ? defaults[c * nb] * scale : defaults[c * nb + i];
      out[c * nb + i] = i == 0 ? half_round(v / 64.0f) * 64.0f : half_round(v);
    }
}

// compute_dct16x16_matrix / compute_dct32x32_matrix (src/quant_weights.rs:1588-1651)
// with fill_ac_reciprocals (:3136-3141)
void square_band_matrix(const float* src, int nb, int n, float* m, float* inv) {
  for (int c = 0; c < 3; ++c) {
    float bands[8];
    bands[0] = src[c * nb];
    for (int i = 1; i < nb; ++i) bands[i] = bands[i - 1] * band_mult(src[c * nb + i]);
    const float scale = (static_cast<float>(nb) - 1.0f) / (1.41421356237309505f + 1e-6f);
    const float rcp = scale / static_cast<float>(n - 1);
    for (int y = 0; y < n; ++y) {
      const float dy = static_cast<float>(y) * rcp;
      const float dy2 = dy * dy;
      for (int x = 0; x < n; ++x) {
        const float dx = static_cast<float>(x) * rcp;
        const float pos = std::sqrt(fmla(dx, dx, dy2));
        const float fl = std::floor(pos);
        const float frac = pos - fl;
        const size_t idx = static_cast<size_t>(fl);
        const float a = bands[idx], b = bands[idx + 1];
        m[c * n * n + y * n + x] = 1.0f / (std::pow(b / a, frac) * a);
      }
    }
    inv[c * n * n] = 0.0f;
    for (int k = 1; k < n * n; ++k) inv[c * n * n + k] = 1.0f / m[c * n * n + k];
  }
}

// natural_scan_generic (src/coeff_order.rs:203-244): scan position -> raw
// index of a cx >= cy block in its cy*8-row x cx*8-column layout
void natural_scan(int cx, int cy, uint16_t* scan, uint16_t* pos) {
  const int side = cx * 8, xs = cx / cy, xsm = xs - 1;
  int xss = 0;
  while ((1 << xss) < xs) ++xss;
  int cur = cx * cy;
  for (int i = 0; i < side; ++i)
    for (int j = 0; j <= i; ++j) {
      int x = j, y = i - j;
      if (i % 2) std::swap(x, y);
      if (y & xsm) continue;
      y >>= xss;
      const int val = (x < cx && y < cy) ? y * cx + x : cur++;
      scan[val] = static_cast<uint16_t>(y * side + x);
    }
  for (int ip = side - 1; ip >= 1; --ip) {
    const int i = ip - 1;
    for (int j = 0; j <= i; ++j) {
      int x = side - 1 - (i - j), y = side - 1 - j;
      if (i % 2) std::swap(x, y);
      if (y & xsm) continue;
      y >>= xss;
      scan[cur++] = static_cast<uint16_t>(y * side + x);
    }
  }
  for (int k = 0; k < cx * cy * 64; ++k) pos[scan[k]] = static_cast<uint16_t>(k);
}

// quantize_ac_thresholds_scaled (src/group.rs:420-455)
void ac_thresholds_scaled(int c, int xs, int ys, float d, float qm_mul, float thr[4]) {
  float normal[4] = {0.58f, 0.635f, 0.66f, 0.7f};
  if (c == 0) {
    const float up = clamp((d - 0.5f) / (0.75f - 0.5f), 0.0f, 1.0f);
    const float down = clamp((2.0f - d) / (2.0f - 1.5f), 0.0f, 1.0f);
    const float w = std::min(up, down);
    normal[0] += w * (0.5f - normal[0]);
    for (int i = 1; i < 4; ++i) normal[i] += (1.0f - w) * 0.08f;
  }
  if (c == 2) {
    const float hf = qm_mul > 1.0f ? 0.65f : 0.75f;
    for (int i = 1; i < 4; ++i) normal[i] = hf;
  }
  if (xs > 1 || ys > 1) {
    const float delta = clamp(0.003f * static_cast<float>(xs) * static_cast<float>(ys), 0.0f,
                              c > 0 ? 0.08f : 0.12f);
    for (int i = 0; i < 4; ++i) normal[i] -= delta;
  }
  const float hq_y[4] = {0.50f, 0.51f, 0.52f, 0.54f};
  const float* hq = c == 1 ? hq_y : normal;
  const float t = clamp((d - 0.1f) / 0.9f, 0.0f, 1.0f);
  for (int i = 0; i < 4; ++i) thr[i] = hq[i] + t * (normal[i] - hq[i]);
}

// Banded::at and merge_margin (src/ac_strategy.rs:103-113, :174-180)
float banded(float hq, float base, float d) {
  const float t = clamp((d - 0.5f) / (1.5f - 0.5f), 0.0f, 1.0f);
  return fmla(t, base - hq, hq);
}
float merge_margin(float d, float hq, float base) {
  const float fade = clamp((d - 1.0f) / (4.0f - 1.0f), 0.0f, 1.0f);
  return banded(hq, base, d) * (1.0f - fade * (1.0f - 0.82f));
}

// tokenize_permutation (src/coeff_order.rs:89-105) of `zigzag` (a
// permutation in natural-scan space), its first `skip` entries left alone:
// only the count of its tokens, the length of the Lehmer code (Fenwick tree,
// compute_lehmer_code, :54-71) without its trailing zeros, plus one.
size_t permutation_token_count(const std::vector<uint32_t>& zigzag, int skip) {
  const int n = static_cast<int>(zigzag.size());
  std::vector<uint32_t> tree(n + 1, 0), code(n);
  for (int idx = 0; idx < n; ++idx) {
    const uint32_t s = zigzag[idx];
    uint32_t penalty = 0;
    for (uint32_t i = s + 1; i != 0; i &= i - 1) penalty += tree[i];
    code[idx] = s - penalty;
    for (uint32_t i = s + 1; i < static_cast<uint32_t>(n + 1); i += i & (~i + 1)) ++tree[i];
  }
  int end = n;
  while (end > skip && code[end - 1] == 0) --end;
  return 1 + static_cast<size_t>(end - skip);
}

// OrderStats::expected_walk (src/coeff_order.rs:570-581): the expected
// tokens a block under `order` walks, in f64.
double expected_walk(const uint32_t* counts, uint32_t blocks, const std::vector<uint32_t>& order,
                     int llf) {
  const double inv = 1.0 / static_cast<double>(std::max(blocks, 1u));
  double none_at_or_after = 1.0, expected = 0.0;
  for (int k = static_cast<int>(order.size()) - 1; k >= llf; --k) {
    expected += 1.0 - none_at_or_after;
    const double p = std::clamp(static_cast<double>(counts[order[k]]) * inv, 0.0, 1.0);
    none_at_or_after *= 1.0 - p;
  }
  return expected;
}

// OrderStats::derive (src/coeff_order.rs:586-601): the LLF entries stay, the
// rest by descending count, ties by natural rank (unique keys).
std::vector<uint32_t> derive_order(const uint32_t* counts, const std::vector<uint32_t>& natural,
                                   int llf) {
  const int n = static_cast<int>(natural.size());
  std::vector<uint64_t> ranked;
  ranked.reserve(n - llf);
  for (int rank = llf; rank < n; ++rank)
    ranked.push_back((static_cast<uint64_t>(0xFFFFFFFFu - counts[natural[rank]]) << 32) |
                     static_cast<uint64_t>(rank));
  std::sort(ranked.begin(), ranked.end());
  std::vector<uint32_t> out(natural.begin(), natural.begin() + llf);
  for (uint64_t key : ranked) out.push_back(natural[static_cast<uint32_t>(key)]);
  return out;
}

}  // namespace

// ORDER_SPECS (src/coeff_order.rs:117-125)
const OrderSpec kOrderSpecs[kOrderSlots] = {{0, 1, 64},    {1, 1, 64},   {2, 4, 256}, {3, 16, 1024},
                                            {4, 2, 128},   {5, 4, 256},  {6, 8, 512}};

int order_slot_offset(int slot) {
  int off = 0;
  for (int k = 0; k < slot; ++k) off += 3 * kOrderSpecs[k].size;
  return off;
}

// derive_orders (src/coeff_order.rs:621-673).  The natural order of each
// slot is natural_scan_generic's (CoeffOrders::natural, :425-448): 8x8 for
// the DCT8 and 8x8-sized groups, then 16x16, 32x32, 16x8, 8x32 and 32x16.
double derive_orders(const uint32_t* counts, const uint32_t* blocks, uint16_t* used_mask,
                     uint32_t* orders) {
  constexpr uint32_t kMinBlocks = 64;           // MIN_BLOCKS_FOR_ORDER, :606
  constexpr double kBitsPerSavedToken = 0.2;    // :608
  constexpr double kGateMargin = 1.5;           // :611
  constexpr double kBitsPerPermutationToken = 5.0;  // :616
  static const int shape[kOrderSlots][2] = {{1, 1}, {1, 1}, {2, 2}, {4, 4}, {2, 1}, {4, 1}, {4, 2}};
  uint16_t used = 0;
  double natural_walk = 0.0, saved_walk = 0.0;
  for (int slot = 0; slot < kOrderSlots; ++slot) {
    const OrderSpec& spec = kOrderSpecs[slot];
    const int off = order_slot_offset(slot), size = spec.size, llf = spec.llf;
    std::vector<uint16_t> scan16(size), pos16(size);
    natural_scan(shape[slot][0], shape[slot][1], scan16.data(), pos16.data());
    const std::vector<uint32_t> natural(scan16.begin(), scan16.end());
    for (int c = 0; c < 3; ++c) std::copy(natural.begin(), natural.end(), orders + off + c * size);
    const uint32_t nb = blocks[slot];
    if (nb < kMinBlocks) continue;
    std::vector<uint32_t> derived[3];
    double saved_bits = 0.0, cost_bits = 0.0, slot_saved_walk = 0.0;
    bool any = false;
    for (int c = 0; c < 3; ++c) {
      const uint32_t* cnt = counts + off + c * size;
      std::vector<uint32_t> candidate = derive_order(cnt, natural, llf);
      const double walk = expected_walk(cnt, nb, natural, llf);
      const double gain = walk - expected_walk(cnt, nb, candidate, llf);
      natural_walk += walk * static_cast<double>(nb);
      std::vector<uint32_t> zigzag(size);
      for (int k = 0; k < size; ++k) zigzag[k] = pos16[candidate[k]];
      const size_t tokens = permutation_token_count(zigzag, llf);
      const double channel_saved = gain * static_cast<double>(nb) * kBitsPerSavedToken;
      const double channel_cost = static_cast<double>(tokens) * kBitsPerPermutationToken;
      if (gain > 0.0 && channel_saved > channel_cost * kGateMargin) {
        any = true;
        slot_saved_walk += gain * static_cast<double>(nb);
        saved_bits += channel_saved;
        cost_bits += channel_cost;
        derived[c] = std::move(candidate);
      } else {
        derived[c] = natural;
      }
    }
    if (any && saved_bits > cost_bits * kGateMargin) {
      used = static_cast<uint16_t>(used | (1u << spec.group));
      for (int c = 0; c < 3; ++c) std::copy(derived[c].begin(), derived[c].end(), orders + off + c * size);
      saved_walk += slot_saved_walk;
    }
  }
  *used_mask = used;
  return natural_walk > 0.0 ? saved_walk / natural_walk : 0.0;
}

void rate_log2_table(float* out) {
  for (int i = 0; i < kRateLog2Entries; ++i) out[i] = ::log2f(1.0f + static_cast<float>(i));
}

int fastest_search_mode(float distance) {
  const float d = std::max(distance, 0.05f);
  if (d <= 0.056713393f) return 0;            // DCT8_ONLY_MAX_DISTANCE
  if (d <= 1.7090991223128462f) return 2;     // FAST_RERANK_MAX_DISTANCE
  return 1;
}

int search_tables(const DistanceParams& p, SearchTables* t, SearchParams* sp) {
  const float d = p.distance;
  if (t && search_matrices(p, t)) return 1;
  search_params(d, sp);
  return 0;
}

int search_matrices(const DistanceParams& p, SearchTables* t) {
  const float d = p.distance;
  if (dct8_tables(d, t->mat8, t->inv8)) return 1;
  for (int c = 0; c < 3; ++c) {
    for (int k = 0; k < 128; ++k) t->mat16x8[c][k] = LIB_DCT16X8_MATRIX[c][k];
    t->inv16x8[c][0] = 0.0f;
    for (int k = 1; k < 128; ++k) t->inv16x8[c][k] = 1.0f / t->mat16x8[c][k];
  }
  // DequantMatrices::new_fast: the 16x16 / 32x32 tables are the library's
  // below the SS2 gate, their bases scaled by 0.78 / 0.89 from it
  // (dct16_override / dct32_override, src/quant_weights.rs:2068-2089)
  const bool ss2 = d >= 2.25f;
  float b16[21], b32[24];
  if (ss2) {
    scaled_override(&LIB_DCT16X16_BANDS[0][0], 7, 0.78f, b16);
    scaled_override(&LIB_DCT32X32_BANDS[0][0], 8, 0.89f, b32);
  } else {
    std::memcpy(b16, LIB_DCT16X16_BANDS, sizeof(b16));
    std::memcpy(b32, LIB_DCT32X32_BANDS, sizeof(b32));
  }
  square_band_matrix(b16, 7, 16, &t->mat16[0][0], &t->inv16[0][0]);
  square_band_matrix(b32, 8, 32, &t->mat32[0][0], &t->inv32[0][0]);
  natural_scan(1, 1, t->scan8, t->pos8);
  natural_scan(2, 1, t->scan16x8, t->pos16x8);
  natural_scan(2, 2, t->scan16, t->pos16);
  natural_scan(4, 4, t->scan32, t->pos32);
  const int dims[4][2] = {{1, 1}, {2, 1}, {2, 2}, {4, 4}};
  const float qm[3] = {p.x_qm_mul, 1.0f, p.b_qm_mul};
  for (int k = 0; k < 4; ++k)
    for (int c = 0; c < 3; ++c) ac_thresholds_scaled(c, dims[k][0], dims[k][1], d, qm[c], t->thr[k][c]);
  exp2_table(t->exp2);
  return 0;
}

void search_params(float d, SearchParams* sp) {
  // MergeTuning::new at Fastest (site_k = SITE_BIAS_K), arbiter SSIMULACRA2
  sp->site_k = 0.2f;
  sp->bias_16x16 = banded(1.2059275f, 1.05f, d);
  sp->bias_32x32 = banded(1.2059275f, 1.06f, d);
  sp->accept_16 = 1.0f - merge_margin(d, 0.19243888f, 0.048f);
  sp->accept_32 = 1.0f - merge_margin(d, 0.21398508f, 0.234f);
  // risk_k = MERGE_RISK_K while aq_dampen(d) > 0 (AQ_STRENGTH, src/adaptive_quant.rs:105-121)
  {
    static const float knots[7] = {0.5f, 1.0f, 1.4f, 1.75f, 3.0f, 5.0f, 8.0f};
    static const float strength[7] = {0.26565f, 0.275459f, 0.058287f, 0.0f, 0.0f, 0.0f, 0.0f};
    float v = strength[6];
    if (d <= knots[0]) {
      v = strength[0];
    } else {
      for (int i = 1; i < 7; ++i)
        if (d <= knots[i]) {
          const float fr = (d - knots[i - 1]) / (knots[i] - knots[i - 1]);
          v = strength[i - 1] + fr * (strength[i] - strength[i - 1]);
          break;
        }
    }
    sp->risk_k = clamp(v, 0.0f, 1.0f) > 0.0f ? 1.44269504088896340736f : 0.0f;
  }
  const float vlq_t = clamp((d - 4.0f) / (7.5f - 4.0f), 0.0f, 1.0f);
  if (vlq_t > 0.0f) {
    sp->bias_16x16 = fmla(vlq_t, 0.880f - sp->bias_16x16, sp->bias_16x16);
    sp->bias_32x32 = fmla(vlq_t, 0.867f - sp->bias_32x32, sp->bias_32x32);
    sp->accept_16 = fmla(vlq_t, (1.0f - 0.067f) - sp->accept_16, sp->accept_16);
    sp->accept_32 = fmla(vlq_t, (1.0f - 0.029250f) - sp->accept_32, sp->accept_32);
  }
  if (d >= 1.5f) sp->bias_32x32 *= 0.94f;
  sp->sel_scale = (d >= 1.0f && d <= 4.0f) ? 1 : 0;
  const bool ss2 = d >= 2.25f;
  // MatrixHeaderCost of new_fast's tables: the DCT8 override (6 bands), the
  // 4x8 refit (4 bands + 48), the 8x32 bands (8), and from the SS2 gate the
  // 16x16 (7), 32x32 (8) and 32x16 (8) overrides
  std::memset(sp->payload, 0, sizeof(sp->payload));
  sp->payload[0] = d >= 0.3f ? 4 + 48 * 6 : 0;
  sp->payload[5] = 4 + 48 * 4 + 48;
  sp->payload[12] = 4 + 48 * 8;
  if (ss2) {
    sp->payload[1] = 4 + 48 * 7;
    sp->payload[2] = 4 + 48 * 8;
    sp->payload[4] = 4 + 48 * 8;
  }
  sp->custom = 0;
  for (int i = 0; i < 13; ++i) sp->custom |= static_cast<uint32_t>(sp->payload[i] != 0) << i;
  sp->headers = ss2 ? 1 : 0;
}

void exp2_table(float out[64]) {
  // fast_exp2's table: 2^((i - 32) / 64) rounded to f32
  for (int i = 0; i < 64; ++i) out[i] = static_cast<float>(std::exp2((i - 32) / 64.0));
}

void natural_order_8x8(uint8_t scan[64], uint8_t position[64]) {
  // Zig-zag over anti-diagonals, odd diagonals walked with x and y swapped,
  // DC first (CoeffOrderAndLut with cx = cy = 1, src/coeff_order.rs:203-244).
  int k = 0;
  for (int s = 0; s < 15; ++s) {
    int lo = std::max(0, s - 7), hi = std::min(7, s);
    for (int j = lo; j <= hi; ++j) {
      int a = (s & 1) ? j : s - j;  // row in storage
      int b = s - a;
      // even diagonals run up-right from (row=s..), matching the scan table
      scan[k++] = static_cast<uint8_t>(a * 8 + b);
    }
  }
  for (int i = 0; i < 64; ++i) position[scan[i]] = static_cast<uint8_t>(i);
}

void gaborish_inverse_weights(float mul, float out[6]) {
  // K_GABORISH (src/gaborish.rs:32-38)
  static const float k[5] = {-0.09495815671340026f, -0.041031725066768575f, 0.013710004822696948f,
                             0.006510206083837737f, -0.0014789063378272242f};
  const float w_r = mul * k[0], w_d = mul * k[1], w_r2 = mul * k[2], w_l = mul * k[3];
  const float w_d2 = mul * k[4];
  float sum = 1.0f + mul * 4.0f * (k[0] + k[1] + k[2] + k[4] + 2.0f * k[3]);
  if (sum < 1e-5f) sum = 1e-5f;
  const float norm = 1.0f / sum;
  out[0] = norm;
  out[1] = norm * w_r;
  out[2] = norm * w_d;
  out[3] = norm * w_r2;
  out[4] = norm * w_l;
  out[5] = norm * w_d2;
}

void gaborish_weights(float out[3]) {
  const float w1 = 1.1f * 0.10469957f, w2 = 1.1f * 0.05568054f;
  const float norm = 1.0f / (1.0f + 4.0f * (w1 + w2));
  out[0] = norm;
  out[1] = w1 * norm;
  out[2] = w2 * norm;
}

}  // namespace jxg
