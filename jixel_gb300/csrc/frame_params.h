// Host-side per-frame constants of the VarDCT front end: distance parameters,
// quant tables, the sRGB transfer table and the kernel argument block.
#pragma once

#include <cstddef>
#include <cstdint>

namespace jxg {

constexpr int kBlockDim = 8;
constexpr int kTileDim = 64;
constexpr int kGroupDim = 256;
constexpr int kDcGroupDim = 2048;
constexpr int kGroupBlocks = 32;
constexpr int kTileBlocks = 8;
constexpr int kFineBlockCtxs = 30;
constexpr int kNonZeroBuckets = 37;
constexpr int kZeroDensityCtxs = 458;
constexpr int kNumFineAcContexts = kFineBlockCtxs * (kNonZeroBuckets + kZeroDensityCtxs);
constexpr int kAlphabet = 128;

// DistanceParams (src/frame/quantization.rs:35-48) resolved for an
// UltraFast XYB frame.
struct DistanceParams {
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
};

// Everything a kernel needs about one frame, passed by value (< 4 KB).
struct KernelArgs {
  float opsin[9];          // forward opsin matrix (XybMatrix::SPEC)
  int32_t width, height;
  int32_t xb, yb;          // blocks
  int32_t tiles_x, tiles_y;
  int32_t groups_x, groups_y;
  int32_t plane;           // float elements between XYB planes
  float distance;
  float scale;             // quantizer scale (global_scale / 2^16)
  float inv_scale;         // 1 / scale, the AQ field's divisor
  float inv_dc_factor[3];  // INV_DC_QUANT / dc_step * scale_dc
  float cfl_dc_factor_x;   // dc_cfl_factor_x (0 for XYB bases)
  float cfl_dc_factor_b;   // dc_cfl_factor with ytob_dc = 0
  float qm_mul[3];         // x_qm_mul, 1, b_qm_mul
  float thresholds[3][4];  // quantize_ac_thresholds_scaled per channel
  float aq_mul, aq_add, aq_hf_strength, aq_fe_weights[4];
  float aq_masking_sqrt_mul;  // sqrt(211.66567973503678 * 1e8) in f32
  float cfl_deadzone;
  float matrix[3][64];     // DCT8 dequant weights
  float inv_matrix[3][64]; // their reciprocals (index 0 = 0)
};

// Strategies of the Fastest search (AcStrategyImage raw codes,
// src/dc_group_data.rs:32-36).
constexpr int kStDct = 0, kSt16x8 = 1, kSt8x16 = 2, kSt16x16 = 3, kSt32x32 = 4;
constexpr int kRateLog2Entries = 1 << 18;

// Constant tables of the Fastest search and layout coding of one frame:
// DequantMatrices::new_fast's tables of the five transforms and their
// reciprocals (src/quant_weights.rs:1588-1652, :2294-2339, :2606-2730), the
// natural orders (src/coeff_order.rs:203-244) both ways, the AC thresholds
// per shape class (1x1, 2x1, 2x2, 4x4 blocks) and channel
// (quantize_ac_thresholds_scaled, src/group.rs:420-455) and fast_exp2's table.
struct SearchTables {
  float inv8[3][64], inv16x8[3][128], inv16[3][256], inv32[3][1024];
  float mat8[3][64], mat16x8[3][128], mat16[3][256], mat32[3][1024];
  uint16_t scan8[64], scan16x8[128], scan16[256], scan32[1024];  // scan position -> raw
  uint16_t pos8[64], pos16x8[128], pos16[256], pos32[1024];      // raw -> scan position
  float thr[4][3][4];
  float exp2[64];
};

// log2(1 + i) by the host's libm for i < kRateLog2Entries (rate_log2_lut,
// src/inflated_cost.rs:57-66, extended past its 1024 entries with the same
// function the reference calls beyond them).
void rate_log2_table(float* out);

// MergeTuning at the frame's distance (src/ac_strategy.rs:87-136, :270-343),
// the selection quantizer's gate and the matrix-header costs.
struct SearchParams {
  float bias_16x16, bias_32x32, accept_16, accept_32, risk_k, site_k;
  int32_t sel_scale;      // selection_quantizer::enabled at Fastest: 1 <= d <= 4
  int32_t headers;        // account_matrix_headers can change the layout (d >= 2.25)
  uint32_t payload[13];   // MatrixHeaderCost (src/quant_weights.rs:54-101)
  uint32_t custom;        // its custom mask
  // 1: every f64 running sum the reference keeps is taken serially in its
  // order, never settled from a parallel sum's error interval (the
  // environment variable JXG_SERIAL_SUMS=1 sets it; results are the same)
  int32_t serial_sums;
};

// Speed::Fastest's transform search runs (not the DCT8-only shortcut,
// src/ac_strategy.rs:73-80); 2 when the distance also asks for the
// reconstruction-domain rerank (FAST_RERANK_MAX_DISTANCE, :67), which this
// build does not have.
int fastest_search_mode(float distance);
// The tables (skipped when `t` is null) and the parameters at p's distance.
int search_tables(const DistanceParams& p, SearchTables* t, SearchParams* sp);
int search_matrices(const DistanceParams& p, SearchTables* t);
void search_params(float distance, SearchParams* sp);

// Gaborish weights: gaborish_inverse's normalised centre, r, d, R, L, D at
// `mul` (src/gaborish.rs:44-72), and the decoder's 3x3 norm, W1 norm, W2
// norm (src/epf_filter.rs:165-169).
void gaborish_inverse_weights(float mul, float out[6]);
void gaborish_weights(float out[3]);

int compute_distance_params(float distance, DistanceParams* out);
// DCT8 tables of DequantMatrices::new_fast (the library table below d = 0.3).
int dct8_tables(float distance, float matrix[3][64], float inv[3][64]);
void fill_kernel_args(const DistanceParams& p, KernelArgs* a);
float distance_from_quality(float quality);
int32_t epf_sharpness_id(float distance, bool screen_content);
// The decoder's loop-filter bundle for an XYB frame at `distance`.
struct LoopFilterParams {
  uint32_t iters;
  float quant_mul, pass0, pass2, border;
  float channel_scale[3];
};
void loop_filter_params(float distance, LoopFilterParams* out);
// A float read back through F16 (a signalled field's value).
float f16_round(float v);
bool is_screen_content(uint64_t constant_blocks, uint64_t width, uint64_t height);
void srgb_to_linear_table(float out[256]);
// TransferLut::build (src/color.rs:297-333) for integer samples of `bits`
// 8, 10, 12 or 16 and an H.273 transfer code (0 = sRGB, the default
// encoding): 256 entries for 8-bit samples, else 65536, codes above the
// largest decoding to 0.  Returns 0, 1 for a transfer the front end does
// not take (PQ, HLG), 2 for an invalid depth or code.
int transfer_table(int bits, int transfer, float* out);
// The same status for a transfer code alone, without building the table.
int transfer_status(int transfer);
void exp2_table(float out[64]);
// libjxl natural 8x8 order: scan position -> raw coefficient index.
void natural_order_8x8(uint8_t scan[64], uint8_t position[64]);

// Coefficient-order statistics (src/coeff_order.rs).  The order groups the
// reference signals, ORDER_SPECS (:117-125), as (order group, LLF entries,
// coefficients); statistics and orders are laid out [slot][channel][raw]
// (orders: [slot][channel][scan position]), slot s starting at
// order_slot_offset(s).
constexpr int kOrderSlots = 7;
constexpr int kOrderCounters = 3 * (64 + 64 + 256 + 1024 + 128 + 256 + 512);
struct OrderSpec {
  int group, llf, size;
};
extern const OrderSpec kOrderSpecs[kOrderSlots];
int order_slot_offset(int slot);
// derive_orders (src/coeff_order.rs:621-673) from the natural orders, over
// pass-one statistics (`counts`, `blocks` per slot): the used-order mask, the
// orders (natural where not adopted) and the share of the expected scan
// walk the adopted orders remove.
double derive_orders(const uint32_t* counts, const uint32_t* blocks, uint16_t* used_mask,
                     uint32_t* orders);

}  // namespace jxg
