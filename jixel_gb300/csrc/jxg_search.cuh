// Speed::Fastest on the device: the AC strategy search and the coding of the
// transforms it places (DCT8, DCT16X8, DCT8X16, DCT16X16, DCT32X32).
//
// Stages of one frame (each a launch over independent work units):
//   k_cost<S>          one warp per candidate transform S: gather, forward
//                      transform, chroma-from-luma, the coefficient-model
//                      rate/distortion cost (strategy_cost, src/ac_strategy.rs:724,
//                      :1295-1378; channel_rd / sse_and_rate / model_bits,
//                      src/inflated_cost.rs:435-547) at the quantizer each
//                      consumer prices it with;
//   k_site             one thread per 16x16 / 32x32 site: the merge bias
//                      (site_bias, src/ac_strategy.rs:210-268);
//   k_select           one thread per 4x4-block cell: select_band /
//                      select_super_block in the squares scope
//                      (src/ac_strategy/selection.rs:238-475, :1000-1245);
//   k_retile           one warp per 8x8-block tile: retile_coefficient's
//                      exact broken-profile DP (src/ac_strategy/selection/
//                      layout_dp.rs:1811-2198);
//   k_adjust           adjust_quant_field (selection.rs:503-527) and the
//                      alpha factors over the layout (src/adaptive_quant.rs:1036);
//   k_mh_incumbent, k_mh_sum, k_mh_choose, k_mh_apply   account_matrix_headers
//                      (src/ac_strategy/matrix_overhead.rs:117-268) where the
//                      16x16 / 32x32 tables are custom (d >= 2.25);
//   k_qf_median        ac_qf_threshold over the final field;
//   k_layout<S>        write_ac_group for every transform of shape S, one warp
//                      each (src/group.rs:1259-2426);
//   k_tokenize_layout  the tokens and histograms (src/group.rs:2428-2660).
// Every float operation keeps the reference's order: per-coefficient terms
// are computed in parallel, and each f32 running sum the reference keeps is
// summed by one lane in the reference's order.  An f64 running sum that is
// only compared or rounded to f32 (the selection quantizer's erased energy,
// the matrix-header sums) is summed in parallel and settled from an error
// interval that provably holds the serial sum, with the serial sum taken
// whenever the interval leaves the outcome open; the other f64 sums (site
// variance) run serially, one site per lane.
#pragma once

namespace jxg {

constexpr float kRdLambda = 0.08086717f;
constexpr float kMetaR = 4.0f;

// Launch geometry the autotuner chooses (warps, i.e. candidates, tiles or
// strips, per CTA) for the kernels whose warps work independently: the
// cost and layout kernels of DCT8 / 16x8 / 8x16 / 16x16, the re-tiling and
// the site variance.  Results do not depend on it.
constexpr int kMaxTuneWarps = 8;
enum TuneKernel {
  kTuneCostDct8, kTuneCost16x8, kTuneCost8x16, kTuneCost16x16,
  kTuneLayoutDct8, kTuneLayout16x8, kTuneLayout8x16, kTuneLayout16x16,
  kTuneRetile, kTuneSite, kTuneKernels
};

// Shapes: pixel footprint W x H, normalised coefficient block CX >= CY (in
// 8x8 blocks), and how the forward transform runs (src/dct.rs: dct8x8 rows
// then transposed columns; dct16x8 / dct16x16 / dct32x32 columns first;
// dct8x16 rows first).
template <int S> struct Shape;
template <> struct Shape<kStDct> {
  static constexpr int W = 8, H = 8, CX = 1, CY = 1, COVX = 1, COVY = 1, CLASS = 0;
};
template <> struct Shape<kSt16x8> {
  static constexpr int W = 8, H = 16, CX = 2, CY = 1, COVX = 1, COVY = 2, CLASS = 1;
};
template <> struct Shape<kSt8x16> {
  static constexpr int W = 16, H = 8, CX = 2, CY = 1, COVX = 2, COVY = 1, CLASS = 1;
};
template <> struct Shape<kSt16x16> {
  static constexpr int W = 16, H = 16, CX = 2, CY = 2, COVX = 2, COVY = 2, CLASS = 2;
};
template <> struct Shape<kSt32x32> {
  static constexpr int W = 32, H = 32, CX = 4, CY = 4, COVX = 4, COVY = 4, CLASS = 3;
};

__host__ __device__ constexpr int cov_x_of(int s) { return s == kSt8x16 || s == kSt16x16 ? 2 : s == kSt32x32 ? 4 : 1; }
__host__ __device__ constexpr int cov_y_of(int s) { return s == kSt16x8 || s == kSt16x16 ? 2 : s == kSt32x32 ? 4 : 1; }

// Per-frame search state (device memory): the host's SearchParams plus the
// pass buffers.
struct SearchFrame {
  const SearchTables* t;
  const float* rate_log2;  // kRateLog2Entries
  SearchParams p;
  float qm_mult[3];     // x_qm_mul, 1, b_qm_mul
  float distance, scale;
  // per block (xb * yb), at the candidate's first block
  float *c8, *c16s, *c16r, *cw, *ct, *c32, *m16, *m32, *mh_inc;
  uint8_t *map, *block_qf;
  uint8_t* dp_choices;  // 32 KB per 8x8-block tile
  uint32_t* sites;      // matrix-header sites in DC-group order (serial path)
  uint8_t* mh_kind;     // per block: the table slot of the site there, 0 for none
  double* mh_loss;      // per block at a site: the DCT and 16x16 alternatives' losses
  double* mh_part;      // k_mh_sum's partials, kMhQuantities per CTA
  uint32_t* mh_decision;  // {chosen table set, pinned families, used set}
};

// ---------------------------------------------------------------------------
// Cost of one candidate, by one warp
// ---------------------------------------------------------------------------

template <int S>
struct alignas(16) CostSmem {
  static constexpr int W = Shape<S>::W, H = Shape<S>::H, SIZE = W * H;
  float in[3][H][W + 1];  // gathered pixels; then the sse terms
  float co[3][SIZE];      // coefficients
  float mag[3][SIZE];     // magnitude-rate terms
  // the running sums read whole channels of terms four at a time
  static_assert(SIZE % 4 == 0 && (3 * H * (W + 1) + 3 * SIZE) % 4 == 0, "16-byte aligned terms");
};

// The block position of candidate `cand` of shape S: every block (DCT8),
// even bx (8x16), even by (16x8), even bx and by (16x16), 4-aligned (32x32);
// false past the last.
template <int S>
__device__ __forceinline__ bool candidate_position(int64_t cand, int xb, int yb, int* bx, int* by) {
  if (S == kStDct) {
    if (cand >= static_cast<int64_t>(xb) * yb) return false;
    *bx = static_cast<int>(cand % xb), *by = static_cast<int>(cand / xb);
  } else if (S == kSt8x16) {
    const int nx = xb / 2;
    if (nx == 0 || cand >= static_cast<int64_t>(nx) * yb) return false;
    *bx = 2 * static_cast<int>(cand % nx), *by = static_cast<int>(cand / nx);
  } else if (S == kSt16x8) {
    const int ny = yb / 2;
    if (ny == 0 || cand >= static_cast<int64_t>(xb) * ny) return false;
    *bx = static_cast<int>(cand % xb), *by = 2 * static_cast<int>(cand / xb);
  } else if (S == kSt16x16) {
    const int nx = xb / 2, ny = yb / 2;
    if (nx == 0 || cand >= static_cast<int64_t>(nx) * ny) return false;
    *bx = 2 * static_cast<int>(cand % nx), *by = 2 * static_cast<int>(cand / nx);
  } else {
    const int nx = xb / 4, ny = yb / 4;
    if (nx == 0 || cand >= static_cast<int64_t>(nx) * ny) return false;
    *bx = 4 * static_cast<int>(cand % nx), *by = 4 * static_cast<int>(cand / nx);
  }
  return true;
}


__device__ __forceinline__ const float* inv_of(const SearchTables* t, int s, int c) {
  switch (s) {
    case kStDct: return t->inv8[c];
    case kSt16x16: return t->inv16[c];
    case kSt32x32: return t->inv32[c];
    default: return t->inv16x8[c];
  }
}
__device__ __forceinline__ const float* mat_of(const SearchTables* t, int s, int c) {
  switch (s) {
    case kStDct: return t->mat8[c];
    case kSt16x16: return t->mat16[c];
    case kSt32x32: return t->mat32[c];
    default: return t->mat16x8[c];
  }
}
__device__ __forceinline__ const uint16_t* pos_of(const SearchTables* t, int s) {
  switch (s) {
    case kStDct: return t->pos8;
    case kSt16x16: return t->pos16;
    case kSt32x32: return t->pos32;
    default: return t->pos16x8;
  }
}
__device__ __forceinline__ const uint16_t* scan_of(const SearchTables* t, int s) {
  switch (s) {
    case kStDct: return t->scan8;
    case kSt16x16: return t->scan16;
    case kSt32x32: return t->scan32;
    default: return t->scan16x8;
  }
}

// rate_log2_with_lut (src/inflated_cost.rs:69-76); the table runs past the
// reference's 1024 entries with the same libm values
__device__ __forceinline__ float rate_log2(const float* table, float qabs) {
  const float k = truncf(qabs);
  if (k < static_cast<float>(kRateLog2Entries)) return table[static_cast<int>(k)];
  return static_cast<float>(log2(1.0 + static_cast<double>(qabs)));
}

// Gather a channel's footprint with edge replication (gather_pixels,
// src/ac_strategy.rs:451-478), then the forward transform into `out`.
template <int S>
__device__ __forceinline__ void warp_forward(const Frame& f, int c, int px, int py,
                                             float (*in)[Shape<S>::W + 1], float* out) {
  constexpr int W = Shape<S>::W, H = Shape<S>::H;
  const int lane = threadIdx.x & 31;
  const int w = f.a.width, h = f.a.height;
  const float* plane = f.xyb + static_cast<int64_t>(c) * f.a.plane;
#pragma unroll 8
  for (int k = lane; k < W * H; k += 32) {
    const int v = k / W, u = k % W;
    const int sy = imin(py + v, h - 1), sx = imin(px + u, w - 1);
    in[v][u] = __ldg(plane + static_cast<int64_t>(sy) * w + sx);
  }
  __syncwarp();
  if (S == kStDct) {
    // dct8x8: rows, then the columns stored transposed, scaled 1/64
    if (lane < 8) {
      float b[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) b[k] = in[lane][k];
      dct1d_8(b);
#pragma unroll
      for (int k = 0; k < 8; ++k) in[lane][k] = b[k];
    }
    __syncwarp();
    if (lane < 8) {
      float b[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) b[k] = in[k][lane];
      dct1d_8(b);
#pragma unroll
      for (int k = 0; k < 8; ++k) out[lane * 8 + k] = b[k] * (1.0f / 64.0f);
    }
  } else if (S == kSt8x16) {
    // rows first, stored out[v W + u]
    const float scale = 1.0f / static_cast<float>(W * H);
    for (int r = lane; r < H; r += 32) {
      float row[W];
#pragma unroll
      for (int u = 0; u < W; ++u) row[u] = in[r][u];
      dct1d_n<W>(row);
#pragma unroll
      for (int u = 0; u < W; ++u) in[r][u] = row[u];
    }
    __syncwarp();
    for (int u = lane; u < W; u += 32) {
      float col[H];
#pragma unroll
      for (int i = 0; i < H; ++i) col[i] = in[i][u];
      dct1d_n<H>(col);
#pragma unroll
      for (int v = 0; v < H; ++v) out[v * W + u] = col[v] * scale;
    }
  } else {
    // columns first, stored out[u H + v]
    const float scale = 1.0f / static_cast<float>(W * H);
    for (int u = lane; u < W; u += 32) {
      float col[H];
#pragma unroll
      for (int i = 0; i < H; ++i) col[i] = in[i][u];
      dct1d_n<H>(col);
#pragma unroll
      for (int v = 0; v < H; ++v) in[v][u] = col[v];
    }
    __syncwarp();
    for (int v = lane; v < H; v += 32) {
      float row[W];
#pragma unroll
      for (int u = 0; u < W; ++u) row[u] = in[v][u];
      dct1d_n<W>(row);
#pragma unroll
      for (int u = 0; u < W; ++u) out[u * H + v] = row[u] * scale;
    }
  }
  __syncwarp();
}

// warp_forward for the three channels at once: one gather, then each pass of
// 1-D transforms spread over the channels' rows or columns together, so a
// DCT8 takes two passes of 24 lanes instead of six of 8.  Every coefficient
// comes from the same operations in the same order.
template <int S>
__device__ __forceinline__ void warp_forward3(const Frame& f, int px, int py,
                                              float (*in)[Shape<S>::H][Shape<S>::W + 1],
                                              float (*out)[Shape<S>::W * Shape<S>::H]) {
  constexpr int W = Shape<S>::W, H = Shape<S>::H;
  const int lane = threadIdx.x & 31;
  const int w = f.a.width, h = f.a.height;
  const int64_t plane = f.a.plane;
#pragma unroll 4
  for (int k = lane; k < W * H; k += 32) {
    const int v = k / W, u = k % W;
    const int64_t at = static_cast<int64_t>(imin(py + v, h - 1)) * w + imin(px + u, w - 1);
#pragma unroll
    for (int c = 0; c < 3; ++c) in[c][v][u] = __ldg(f.xyb + c * plane + at);
  }
  __syncwarp();
  if (S == kStDct) {
    // dct8x8: rows, then the columns stored transposed, scaled 1/64
    const int c = lane >> 3, r = lane & 7;
    if (lane < 24) {
      float b[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) b[k] = in[c][r][k];
      dct1d_8(b);
#pragma unroll
      for (int k = 0; k < 8; ++k) in[c][r][k] = b[k];
    }
    __syncwarp();
    if (lane < 24) {
      float b[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) b[k] = in[c][k][r];
      dct1d_8(b);
#pragma unroll
      for (int k = 0; k < 8; ++k) out[c][r * 8 + k] = b[k] * (1.0f / 64.0f);
    }
  } else if (S == kSt8x16) {
    // rows first, stored out[v W + u]
    const float scale = 1.0f / static_cast<float>(W * H);
    for (int j = lane; j < 3 * H; j += 32) {
      const int c = j / H, r = j % H;
      float row[W];
#pragma unroll
      for (int u = 0; u < W; ++u) row[u] = in[c][r][u];
      dct1d_n<W>(row);
#pragma unroll
      for (int u = 0; u < W; ++u) in[c][r][u] = row[u];
    }
    __syncwarp();
    for (int j = lane; j < 3 * W; j += 32) {
      const int c = j / W, u = j % W;
      float col[H];
#pragma unroll
      for (int i = 0; i < H; ++i) col[i] = in[c][i][u];
      dct1d_n<H>(col);
#pragma unroll
      for (int v = 0; v < H; ++v) out[c][v * W + u] = col[v] * scale;
    }
  } else {
    // columns first, stored out[u H + v]
    const float scale = 1.0f / static_cast<float>(W * H);
    for (int j = lane; j < 3 * W; j += 32) {
      const int c = j / W, u = j % W;
      float col[H];
#pragma unroll
      for (int i = 0; i < H; ++i) col[i] = in[c][i][u];
      dct1d_n<H>(col);
#pragma unroll
      for (int v = 0; v < H; ++v) in[c][v][u] = col[v];
    }
    __syncwarp();
    for (int j = lane; j < 3 * H; j += 32) {
      const int c = j / H, v = j % H;
      float row[W];
#pragma unroll
      for (int u = 0; u < W; ++u) row[u] = in[c][v][u];
      dct1d_n<W>(row);
#pragma unroll
      for (int u = 0; u < W; ++u) out[c][u * H + v] = row[u] * scale;
    }
  }
  __syncwarp();
}

// The three channels' coefficients with chroma-from-luma applied
// (prepare_strategy_coeffs, src/ac_strategy.rs:1380-1407).
template <int S>
__device__ __forceinline__ void warp_coefficients(const Frame& f, int bx, int by, CostSmem<S>& sm) {
  constexpr int SIZE = Shape<S>::W * Shape<S>::H;
  const int lane = threadIdx.x & 31;
  warp_forward3<S>(f, bx * 8, by * 8, sm.in, sm.co);
  // cmap_factors (src/ac_strategy.rs:1841-1857): the tile of the first block
  const int t = (by >> 3) * f.a.tiles_x + (bx >> 3);
  const float xf = fmla(static_cast<float>(f.ytox[t]), 1.0f / 84.0f, 0.0f);
  const float bf = fmla(static_cast<float>(f.ytob[t]), 1.0f / 84.0f, 1.0f);
  for (int i = lane; i < SIZE; i += 32) {
    const float y = sm.co[1][i];
    sm.co[0][i] = fmla(-xf, y, sm.co[0][i]);
    sm.co[2][i] = fmla(-bf, y, sm.co[2][i]);
  }
  __syncwarp();
}

// selection_quantizer::scale (src/ac_strategy/selection_quantizer.rs:78-125):
// only DCT32X32 here; the erased energy is an f64 sum in raster order.
//
// The serial f64 sum R is only ever read as an f32.  The warp sums the same
// non-negative terms in parallel (P: four running sums of eight terms a
// lane, their pairwise sum, then a butterfly over the lanes, so no term goes
// through more than 14 additions); |R - P| <= (n + 36) u E for n <= 960
// terms (u = 2^-53, E the exact sum; error bounds of recursive and pairwise
// summation), below M = 2^-42 P.  Rounding to f32 is monotonic, so when
// P - M and P + M round to the same f32 that f32 is R's; otherwise lane 0
// takes the serial sum.
__device__ __forceinline__ float selection_scale_32(const SearchFrame& s, const float* co_y,
                                                   float qac) {
  if (!s.p.sel_scale) return 1.0f;
  const int lane = threadIdx.x & 31;
  const float* inv = s.t->inv32[1];
  auto erased_term = [&](int i) -> double {
    const int y = i >> 5, x = i & 31;
    if (x < 8 && y < 8) return 0.0;
    const float l = co_y[i];
    return fabsf(__fmul_rn(__fmul_rn(l, __ldg(inv + i)), qac)) < 0.5f
               ? __dmul_rn(static_cast<double>(l), static_cast<double>(l))
               : 0.0;
  };
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int i = lane; i < 1024; i += 32) acc[(i >> 5) & 3] = __dadd_rn(acc[(i >> 5) & 3], erased_term(i));
  double part = __dadd_rn(__dadd_rn(acc[0], acc[1]), __dadd_rn(acc[2], acc[3]));
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) part = __dadd_rn(part, __shfl_xor_sync(0xffffffffu, part, d));
  const double margin = __dmul_rn(part, 0x1p-42);
  float erased = static_cast<float>(__dsub_rn(part, margin));
  const bool settled = erased == static_cast<float>(__dadd_rn(part, margin)) && !s.p.serial_sums;
  if (!settled) {
    double energy = 0.0;
    if (lane == 0)
      for (int i = 0; i < 1024; ++i) energy = __dadd_rn(energy, erased_term(i));
    erased = __shfl_sync(0xffffffffu, static_cast<float>(energy), 0);
  }
  const float d = s.distance;
  const float r = __fsub_rn(__fdiv_rn(erased, __fmul_rn(__fmul_rn(2e-4f, d), d)), 1.0f);
  return __fadd_rn(1.0f, __fmul_rn(0.6f, fminf(fmaxf(r, 0.0f), 1.0f)));
}
template <int S>
__device__ __forceinline__ float warp_selection_scale(const SearchFrame& s, const CostSmem<S>& sm,
                                                      float qac) {
  return S == kSt32x32 ? selection_scale_32(s, sm.co[1], qac) : 1.0f;
}

// The coefficient-model terms of channel c at quantizer `q` (already scaled
// by the selection quantizer), by one warp: each coefficient's squared error
// into `sse` and magnitude rate into `mag` (0 for the LLF), and the channel's
// non-zero count and highest non-zero scan position (channel_rd /
// sse_and_rate, src/inflated_cost.rs:435-537).
template <int S>
__device__ __forceinline__ void rd_channel(const SearchFrame& s, const float* co, int c, float q,
                                           float* sse, float* mag, int* nz, uint32_t* max_scan) {
  constexpr int CX = Shape<S>::CX, CY = Shape<S>::CY, WIDTH = CX * 8, HEIGHT = CY * 8;
  constexpr int SIZE = WIDTH * HEIGHT;
  const int lane = threadIdx.x & 31;
  const SearchTables* t = s.t;
  const uint16_t* pos = pos_of(t, S);
  const float* inv = inv_of(t, S, c);
  const float* thr = t->thr[Shape<S>::CLASS][c];
  const float q_scaled = __fmul_rn(q, s.qm_mult[c]);
  int n = 0;
  uint32_t ms = 0;
#pragma unroll 4
  for (int i = lane; i < SIZE; i += 32) {
    const int y = i / WIDTH, x = i % WIDTH;
    float e2 = 0.0f, m = 0.0f;
    if (!(x < CX && y < CY)) {
      const int yfix = y >= HEIGHT / 2 ? 2 : 0;
      const float threshold = x >= WIDTH / 2 ? thr[yfix + 1] : thr[yfix];
      const float a = __fmul_rn(__fmul_rn(inv[i], q_scaled), co[i]);
      const float qv = fabsf(a) >= threshold ? roundf(a) : 0.0f;
      const float e = __fsub_rn(a, bias_level(c, cast_i32(qv)));
      e2 = __fmul_rn(e, e);
      if (qv != 0.0f) {
        ++n;
        m = rate_log2(s.rate_log2, fabsf(qv));
        ms = max(ms, static_cast<uint32_t>(pos[i]));
      }
    }
    sse[i] = e2;
    mag[i] = m;
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    n += __shfl_xor_sync(0xffffffffu, n, d);
    ms = max(ms, __shfl_xor_sync(0xffffffffu, ms, d));
  }
  *nz = n;
  *max_scan = ms;
}

// A running f32 sum in raster order by one thread (a skipped coefficient
// adds +0, which leaves a sum of non-negative terms as it is).
// `terms` is 16-byte aligned: four terms a shared load.
template <int SIZE>
__device__ __forceinline__ float serial_sum(const float* terms) {
  static_assert(SIZE % 4 == 0, "terms are read four at a time");
  const float4* quad = reinterpret_cast<const float4*>(terms);
  float sum = 0.0f;
#pragma unroll 4
  for (int i = 0; i < SIZE / 4; ++i) {
    const float4 v = quad[i];
    sum = __fadd_rn(sum, v.x);
    sum = __fadd_rn(sum, v.y);
    sum = __fadd_rn(sum, v.z);
    sum = __fadd_rn(sum, v.w);
  }
  return sum;
}

// model_bits over the channels, the weighted distortion and the visible
// fraction: the strategy cost (strategy_cost, src/ac_strategy.rs:1295-1378;
// model_bits, src/inflated_cost.rs:540-547; Footprint::visible_fraction,
// :650-659).
template <int S>
__device__ __forceinline__ float rd_finish(const Frame& f, const SearchFrame& s, int bx, int by,
                                           const int* nz, const uint32_t* max_scan,
                                           const float* sse, const float* mag, float meta_r) {
  constexpr int CX = Shape<S>::CX, CY = Shape<S>::CY;
  const float weights[3] = {0.30f, 1.0f, 0.28f};
  float d_total = 0.0f, r_total = 0.0f;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float header = __fmul_rn(0.4f, rate_log2(s.rate_log2, static_cast<float>(nz[c])));
    float visited = 0.0f;
    if (nz[c]) {
      const int v = static_cast<int>(max_scan[c]) + 1 - (CX * CY + nz[c]);
      visited = v > 0 ? static_cast<float>(v) : 0.0f;
    }
    const float bits = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(static_cast<float>(nz[c]), 1.6f),
                                                     __fmul_rn(1.0f, mag[c])), header),
                                 __fmul_rn(0.5f, visited));
    d_total = __fadd_rn(d_total, __fmul_rn(weights[c], sse[c]));
    r_total = __fadd_rn(r_total, bits);
  }
  const int px = bx * 8, py = by * 8;
  const int vw = imin(Shape<S>::W, imax(f.a.width - px, 0));
  const int vh = imin(Shape<S>::H, imax(f.a.height - py, 0));
  const float visible = (vw == Shape<S>::W && vh == Shape<S>::H)
                            ? 1.0f
                            : __fdiv_rn(static_cast<float>(vw * vh),
                                        static_cast<float>(Shape<S>::W * Shape<S>::H));
  return fmla(kRdLambda, __fadd_rn(r_total, meta_r), __fmul_rn(d_total, visible));
}

// The coefficient-model cost at quantizer `q` (already scaled by the
// selection quantizer) of the coefficients in `sm`, by one warp; every lane
// returns it.  The six running sums go to lanes 0-5.
template <int S>
__device__ __forceinline__ float warp_rd(const Frame& f, const SearchFrame& s, CostSmem<S>& sm,
                                         int bx, int by, float q, float meta_r) {
  constexpr int SIZE = Shape<S>::W * Shape<S>::H;
  const int lane = threadIdx.x & 31;
  float* sse_terms = &sm.in[0][0][0];  // the gather buffer is free again
  int nz[3];
  uint32_t max_scan[3];
#pragma unroll
  for (int c = 0; c < 3; ++c)
    rd_channel<S>(s, sm.co[c], c, q, sse_terms + c * SIZE, sm.mag[c], &nz[c], &max_scan[c]);
  __syncwarp();
  float sum = 0.0f;
  if (lane < 6) sum = serial_sum<SIZE>(lane < 3 ? sse_terms + lane * SIZE : sm.mag[lane - 3]);
  float sse[3], mag[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    sse[c] = __shfl_sync(0xffffffffu, sum, c);
    mag[c] = __shfl_sync(0xffffffffu, sum, 3 + c);
  }
  __syncwarp();
  return rd_finish<S>(f, s, bx, by, nz, max_scan, sse, mag, meta_r);
}

// region_quant (src/ac_strategy/selection.rs:910-927) over a w x h region
// of the field, and aggregate_quant (:484-493)
__device__ __forceinline__ float mean_max_mixer(float d) {
  return fmaxf(__fsub_rn(1.0f, __fmul_rn(fmaxf(__fsub_rn(d, 1.54138f), 0.0f), 0.56391f)), 0.0f);
}
__device__ __forceinline__ uint8_t aggregate_quant(uint32_t max_q, uint32_t sum, int covered, float d) {
  if (covered < 4) return static_cast<uint8_t>(max_q);
  const float mixer = mean_max_mixer(d);
  const float mean = __fdiv_rn(static_cast<float>(sum), static_cast<float>(covered));
  const float mixed = __fadd_rn(__fmul_rn(static_cast<float>(max_q), mixer),
                                __fmul_rn(mean, __fsub_rn(1.0f, mixer)));
  const float v = fminf(fmaxf(__fadd_rn(mixed, 0.5f), 1.0f), 255.0f);
  return static_cast<uint8_t>(cast_i32(v));
}
__device__ __forceinline__ uint8_t region_quant(const uint8_t* qf, int xb, int bx, int by, int w,
                                                int h, float d) {
  uint32_t max_q = 1, sum = 0;
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const uint32_t q = qf[(by + y) * xb + bx + x];
      max_q = max(max_q, q);
      sum += q;
    }
  return aggregate_quant(max_q, sum, w * h, d);
}

// site_variance_rect and site_bias (src/ac_strategy.rs:210-268): f64 sums in
// raster order by one lane; fast_exp (src/util.rs:342-356)
__device__ __forceinline__ float util_fast_exp(float x) {
  const int32_t exponent = cast_i32(roundf(__fmul_rn(x, 1.44269504088896340736f)));
  float r = fmla(static_cast<float>(exponent), -0.69314575f, x);
  r = fmla(static_cast<float>(exponent), -1.4286068e-6f, r);
  const float square = __fmul_rn(r, r);
  float p = fmla(-0.002775669f, square, 0.16666707f);
  p = fmla(p, square, 2.0f);
  const float scale = __uint_as_float(static_cast<uint32_t>(exponent + 127) << 23);
  return __fmul_rn(__fadd_rn(1.0f, __fdiv_rn(__fmul_rn(2.0f, r), __fsub_rn(p, r))), scale);
}
// site_variance_rect / site_bias (src/ac_strategy.rs:210-268) of the n x n
// sites, n = 16 (even block coordinates) or 32 (4-aligned): the variance of
// the site's luma, clipped to the image, from two f64 sums in raster order.
//
// The sums are serial, and GB300's f64 pipe retires a warp instruction in
// tens of cycles whether one lane or 32 are active, so they run one site per
// lane: a warp takes a strip of 32 adjacent sites along a row of sites, whose
// rows together are one contiguous run of luma.  Row by row, the warp loads
// the run coalesced (the next row's loads in flight while the lanes sum the
// current one) and stages each sample's two terms in shared memory; each lane
// then adds its site's terms, one f64 add a sample:
//   s2: v * v is exact in f64 (a 24-bit mantissa squared has at most 48
//       significant bits) and is built from v's bits with integer
//       instructions;
//   s1: when every sample of the site is a multiple of 2^-42 below 1 in
//       magnitude (every normal sample from 2^-19 up, and any whose low
//       mantissa bits are zero, such as black's 2^-26), every partial sum is
//       a multiple of 2^-42 below 2^10, so no add rounds and the serial f64
//       sum equals the int64 sum of v * 2^42.
// A site with any other sample takes s1 serially, and s2 too when a sample
// is subnormal or non-finite: its warp goes over the rows once more.
// Strips per CTA: tuned per device (default one: the long 32x32 strips
// spread over the SMs); the kernel reads it from blockDim.
constexpr int kSiteWarps = 1;
struct SiteSmem {
  double sq[32][33];
  long long q[32][33];
  uint32_t odd[32];
};

__device__ __forceinline__ float site_bias_of(const SearchFrame& s, double s1, double s2, int cnt) {
  float var = 0.0f;
  if (cnt) {
    const double mean = __ddiv_rn(s1, static_cast<double>(cnt));
    const double vv = __dsub_rn(__ddiv_rn(s2, static_cast<double>(cnt)), __dmul_rn(mean, mean));
    var = static_cast<float>(vv > 0.0 ? vv : 0.0);
  }
  var = fmaxf(var, 1e-9f);
  const float sv = fminf(fmaxf(__fdiv_rn(dirty_log2f(__fdiv_rn(var, 0.003f)), 8.0f), -1.0f), 1.0f);
  return util_fast_exp(__fmul_rn(s.p.site_k, sv));
}

// the warp's strips: 32x32 sites first (they take longer), then 16x16
template <int N>
__device__ __forceinline__ void site_strip(const Frame& f, const SearchFrame& s, SiteSmem& sm,
                                           int strip) {
  constexpr int STEP = N / 8;  // blocks between sites
  constexpr int PER_LANE = N;  // a row of 32 sites is 32 N samples
  const int lane = threadIdx.x & 31;
  const int xb = f.a.xb, w = f.a.width, h = f.a.height;
  const int nx = xb / STEP, per_row = (nx + 31) / 32;
  const int row = strip / per_row, first = (strip % per_row) * 32;
  const int sites = imin(32, nx - first);
  const int x0 = first * N, y0 = row * N;
  const int vh = imin(y0 + N, h) - y0;
  const int run = imin(sites * N, w - x0);  // samples of a row inside the image
  const float* yp = f.xyb + f.a.plane;
  sm.odd[lane] = 0u;
  __syncwarp();
  float v[PER_LANE];
  auto load = [&](int y) {
    const float* src = yp + static_cast<int64_t>(y0 + y) * w + x0;
#pragma unroll
    for (int m = 0; m < PER_LANE; ++m) {
      const int k = lane + 32 * m;
      v[m] = k < run ? __ldg(src + k) : 0.0f;
    }
  };
  const bool mine = lane < sites;
  const int my_x0 = x0 + lane * N;
  const int vw = mine ? imax(imin(my_x0 + N, w) - my_x0, 0) : 0;
  double s2 = 0.0;
  long long isum = 0;
  if (vh > 0) load(0);
  for (int y = 0; y < vh; ++y) {
#pragma unroll
    for (int m = 0; m < PER_LANE; ++m) {
      const int k = lane + 32 * m, i = k / N, x = k % N;
      const uint32_t u = __float_as_uint(v[m]);
      const uint32_t ex = (u >> 23) & 0xffu;
      const uint32_t mant = (u & 0x7fffffu) | 0x800000u;
      const bool zero = (u & 0x7fffffffu) == 0u;
      // |v| < 1 and v a multiple of 2^-42: its lowest set bit, 2^(ex - 150 +
      // ctz(mant)), at or above 2^-42
      const int lowest = static_cast<int>(ex) + __ffs(static_cast<int>(mant)) - 1;
      const bool in_range = ex >= 1u && ex <= 126u && lowest >= 108;
      // bit 0: s1 needs the serial sum; bit 1: s2 too (subnormal, non-finite)
      if (!zero && !in_range && k < run) atomicOr(&sm.odd[i], (ex == 0u || ex == 0xffu) ? 3u : 1u);
      // v * v = p * 2^(2 ex - 300), 2^46 <= p < 2^48: biased f64 exponent
      // 2 ex - 300 + 46 + top + 1023
      const uint64_t p = static_cast<uint64_t>(mant) * mant;
      const uint32_t top = static_cast<uint32_t>(p >> 47);
      const uint64_t frac = (p << (6u - top)) & ((1ull << 52) - 1ull);
      const uint64_t bits = (static_cast<uint64_t>(2u * ex + top + 769u) << 52) | frac;
      sm.sq[i][x] = zero ? 0.0 : __longlong_as_double(static_cast<long long>(bits));
      // v * 2^42 = mant * 2^(ex - 108), exact when in range (a right shift
      // drops only zero bits)
      const int sh = static_cast<int>(ex) - 108;
      const uint64_t mq = sh >= 0 ? static_cast<uint64_t>(mant) << (sh & 31)
                                  : static_cast<uint64_t>(mant >> ((-sh) & 31));
      const long long q = in_range ? static_cast<long long>(mq) : 0;
      sm.q[i][x] = (u >> 31) ? -q : q;
    }
    __syncwarp();
    if (y + 1 < vh) load(y + 1);
    for (int x = 0; x < vw; ++x) {
      s2 = __dadd_rn(s2, sm.sq[lane][x]);
      isum += sm.q[lane][x];
    }
    __syncwarp();
  }
  double s1 = __dmul_rn(static_cast<double>(isum), 0x1p-42);
  const uint32_t odd = mine ? (s.p.serial_sums ? 3u : sm.odd[lane]) : 0u;
  // the serial sums of the odd sites: the rows once more, coalesced, staged
  // as f64 for the lanes that need them
  if (__any_sync(0xffffffffu, odd != 0u)) {
    const bool both = (odd & 2u) != 0u;
    double t1 = 0.0, t2 = 0.0;
    if (vh > 0) load(0);
    for (int y = 0; y < vh; ++y) {
#pragma unroll
      for (int m = 0; m < PER_LANE; ++m) {
        const int k = lane + 32 * m;
        sm.sq[k / N][k % N] = static_cast<double>(v[m]);
      }
      __syncwarp();
      if (y + 1 < vh) load(y + 1);
      if (odd)
        for (int x = 0; x < vw; ++x) {
          const double d = sm.sq[lane][x];
          t1 = __dadd_rn(t1, d);
          if (both) t2 = __dadd_rn(t2, __dmul_rn(d, d));
        }
      __syncwarp();
    }
    if (odd) s1 = t1;
    if (both) s2 = t2;
  }
  if (!mine) return;
  float* out = N == 32 ? s.m32 : s.m16;
  out[static_cast<int64_t>(row * STEP) * xb + (first + lane) * STEP] =
      s.p.site_k == 0.0f ? 1.0f : site_bias_of(s, s1, s2, vw * vh);
}

__host__ __device__ inline int64_t site_strips(int xb, int yb, int n) {
  const int step = n / 8, nx = xb / step, ny = yb / step;
  return nx == 0 ? 0 : static_cast<int64_t>((nx + 31) / 32) * ny;
}

__global__ void __launch_bounds__(32 * kMaxTuneWarps) k_site(const __grid_constant__ Frame f) {
  extern __shared__ __align__(16) unsigned char site_smem_raw[];
  SiteSmem& sm = reinterpret_cast<SiteSmem*>(site_smem_raw)[threadIdx.x >> 5];
  const SearchFrame& s = *static_cast<const SearchFrame*>(f.search);
  const int64_t strip = static_cast<int64_t>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int64_t n32 = site_strips(f.a.xb, f.a.yb, 32), n16 = site_strips(f.a.xb, f.a.yb, 16);
  if (strip < n32) site_strip<32>(f, s, sm, static_cast<int>(strip));
  else if (strip < n32 + n16) site_strip<16>(f, s, sm, static_cast<int>(strip - n32));
}

// One warp per candidate of shape S: the costs every consumer of it reads.
//   DCT8     every block, at scale * q (select_super_block's c8, the DP's leaves)
//   16x16    even (bx, by): at aggregate_qac_2x2 (selection) and at region_qac
//            (the DP's squares, the matrix-header alternatives)
//   8x16     even bx (the DP's horizontal pairs), 16x8 even by (vertical pairs)
//   32x32    4-aligned: at region_qac with the selection quantizer
template <int S>
__global__ void __launch_bounds__(32 * kMaxTuneWarps) k_cost(const __grid_constant__ Frame f) {
  extern __shared__ __align__(16) unsigned char cost_smem_raw[];
  CostSmem<S>& sm = reinterpret_cast<CostSmem<S>*>(cost_smem_raw)[threadIdx.x >> 5];
  const SearchFrame& s = *static_cast<const SearchFrame*>(f.search);
  const int lane = threadIdx.x & 31;
  const int xb = f.a.xb, yb = f.a.yb;
  const int64_t cand = static_cast<int64_t>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5);
  int bx, by;
  if (!candidate_position<S>(cand, xb, yb, &bx, &by)) return;
  const int bi = by * xb + bx;
  const uint8_t* qf = f.qf;  // the pre-selection field
  warp_coefficients<S>(f, bx, by, sm);
  if (S == kStDct) {
    const float qac = __fmul_rn(s.scale, static_cast<float>(qf[bi]));
    const float c = warp_rd<S>(f, s, sm, bx, by, qac, kMetaR);
    if (lane == 0) s.c8[bi] = c;
  } else if (S == kSt16x16) {
    // aggregate_qac_2x2 (src/ac_strategy/selection.rs:495-501)
    const float q00 = __fmul_rn(s.scale, static_cast<float>(qf[bi]));
    const float q01 = __fmul_rn(s.scale, static_cast<float>(qf[bi + 1]));
    const float q10 = __fmul_rn(s.scale, static_cast<float>(qf[bi + xb]));
    const float q11 = __fmul_rn(s.scale, static_cast<float>(qf[bi + xb + 1]));
    const float max_q = fmaxf(fmaxf(fmaxf(q00, q01), q10), q11);
    const float mixer = mean_max_mixer(s.distance);
    const float mean = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(q00, q01), q10), q11), 0.25f);
    const float mixed_q = __fdiv_rn(__fadd_rn(__fmul_rn(max_q, mixer),
                                              __fmul_rn(mean, __fsub_rn(1.0f, mixer))),
                                    s.scale);
    const float qsel = __fmul_rn(s.scale, floorf(fminf(fmaxf(__fadd_rn(mixed_q, 0.5f), 1.0f), 255.0f)));
    const float qreg = __fmul_rn(s.scale,
                                 static_cast<float>(region_quant(qf, xb, bx, by, 2, 2, s.distance)));
    const float csel = warp_rd<S>(f, s, sm, bx, by, qsel, kMetaR);
    const float creg = qreg == qsel ? csel : warp_rd<S>(f, s, sm, bx, by, qreg, kMetaR);
    if (lane == 0) {
      s.c16s[bi] = csel;
      s.c16r[bi] = creg;
    }
  } else {
    constexpr int w = Shape<S>::COVX, h = Shape<S>::COVY;
    const float qac = __fmul_rn(s.scale,
                                static_cast<float>(region_quant(qf, xb, bx, by, w, h, s.distance)));
    const float c = warp_rd<S>(f, s, sm, bx, by, qac, kMetaR);
    if (lane == 0) (S == kSt8x16 ? s.cw : s.ct)[bi] = c;
  }
}

// The 32x32 candidates (4-aligned, at region_qac with the selection
// quantizer): a CTA of three warps each, one per channel, so that a
// candidate's 37 KB of shared memory keeps three warps busy: the gather and
// forward transform, then chroma-from-luma on X and B while the Y warp takes
// the selection quantizer, then each channel's terms and its two running
// sums (lanes 0 and 1), then the cost.
constexpr int kCost32Threads = 96;
struct alignas(16) Cost32Smem {
  float in[3][32][33];  // gathered pixels; then the channel's sse terms (16-byte aligned)
  float co[3][1024];    // coefficients; then the channel's magnitude-rate terms
};
__global__ void __launch_bounds__(kCost32Threads) k_cost32(const __grid_constant__ Frame f) {
  extern __shared__ __align__(16) unsigned char cost_smem_raw[];
  Cost32Smem& sm = *reinterpret_cast<Cost32Smem*>(cost_smem_raw);
  __shared__ float s_scale, s_sum[6];
  __shared__ int s_nz[3];
  __shared__ uint32_t s_ms[3];
  const SearchFrame& s = *static_cast<const SearchFrame*>(f.search);
  const int c = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int xb = f.a.xb, yb = f.a.yb;
  int bx, by;
  if (!candidate_position<kSt32x32>(blockIdx.x, xb, yb, &bx, &by)) return;
  const int bi = by * xb + bx;
  warp_forward<kSt32x32>(f, c, bx * 8, by * 8, sm.in[c], sm.co[c]);
  __syncthreads();
  const float qac = __fmul_rn(s.scale, static_cast<float>(region_quant(f.qf, xb, bx, by, 4, 4, s.distance)));
  if (c == 1) {
    const float scale = selection_scale_32(s, sm.co[1], qac);
    if (lane == 0) s_scale = scale;
  } else {
    // cmap_factors (src/ac_strategy.rs:1841-1857): the tile of the first block
    const int t = (by >> 3) * f.a.tiles_x + (bx >> 3);
    const float factor = c == 0 ? fmla(static_cast<float>(f.ytox[t]), 1.0f / 84.0f, 0.0f)
                                : fmla(static_cast<float>(f.ytob[t]), 1.0f / 84.0f, 1.0f);
    for (int i = lane; i < 1024; i += 32) sm.co[c][i] = fmla(-factor, sm.co[1][i], sm.co[c][i]);
  }
  __syncthreads();
  const float q = __fmul_rn(qac, s_scale);
  float* sse = &sm.in[c][0][0];  // this channel's gather buffer is free again
  int n;
  uint32_t ms;
  // each lane writes the magnitude term over the coefficient it reads
  rd_channel<kSt32x32>(s, sm.co[c], c, q, sse, sm.co[c], &n, &ms);
  if (lane == 0) {
    s_nz[c] = n;
    s_ms[c] = ms;
  }
  __syncthreads();
  // the six running sums (sse, then magnitude, per channel) on lanes 0-5 of
  // one warp: the same chains, a third of the instructions
  if (c != 0) return;
  if (lane < 6) {
    const int ch = lane % 3;
    s_sum[lane] = serial_sum<1024>(lane < 3 ? &sm.in[ch][0][0] : sm.co[ch]);
  }
  __syncwarp();
  if (lane == 0) s.c32[bi] = rd_finish<kSt32x32>(f, s, bx, by, s_nz, s_ms, s_sum, s_sum + 3, kMetaR);
}


// ---------------------------------------------------------------------------
// Selection (squares scope) and re-tiling
// ---------------------------------------------------------------------------

__device__ __forceinline__ void map_set_first(uint8_t* map, int xb, int x, int y, int st) {
  const int cx = cov_x_of(st), cy = cov_y_of(st);
  for (int iy = 0; iy < cy; ++iy)
    for (int ix = 0; ix < cx; ++ix)
      map[(y + iy) * xb + x + ix] = static_cast<uint8_t>((st << 1) | (iy == 0 && ix == 0 ? 1 : 0));
}

// can_place_strategy (src/dc_group_data.rs:171-201) on absolute blocks (DC
// groups start at multiples of 256 blocks)
__device__ __forceinline__ bool can_place(int xb, int yb, int x, int y, int st) {
  const int cx = cov_x_of(st), cy = cov_y_of(st);
  if (x + cx > xb || y + cy > yb) return false;
  if (x / 32 != (x + cx - 1) / 32 || y / 32 != (y + cy - 1) / 32) return false;
  return x / 8 == (x + cx - 1) / 8 && y / 8 == (y + cy - 1) / 8;
}

// risk_gated (src/ac_strategy.rs:1860-1866)
__device__ __forceinline__ float risk_gated(const SearchFrame& s, float accept, float q_min,
                                            float q_max, float area) {
  if (q_min <= 0.0f || s.p.risk_k <= 0.0f) return accept;
  const float spread = __fsub_rn(__fdiv_rn(q_max, q_min), 1.0f);
  return __fmul_rn(accept, fast_exp2(__fmul_rn(__fmul_rn(-s.p.risk_k, area), spread), s.t->exp2));
}

struct SuperCost {
  float chosen, dct8;
};

// select_super_block (src/ac_strategy/selection.rs:238-475), squares scope
__device__ __forceinline__ SuperCost select_super(const Frame& f, const SearchFrame& s, int bx0,
                                                  int by0) {
  const int xb = f.a.xb;
  float qac[2][2], c8[2][2];
  for (int dy = 0; dy < 2; ++dy)
    for (int dx = 0; dx < 2; ++dx) {
      const int b = (by0 + dy) * xb + bx0 + dx;
      qac[dy][dx] = __fmul_rn(s.scale, static_cast<float>(f.qf[b]));
      c8[dy][dx] = s.c8[b];
    }
  const float left = __fadd_rn(c8[0][0], c8[1][0]), right = __fadd_rn(c8[0][1], c8[1][1]);
  const float top = __fadd_rn(c8[0][0], c8[0][1]), bottom = __fadd_rn(c8[1][0], c8[1][1]);
  const float total = __fadd_rn(left, right);
  const int b0 = by0 * xb + bx0;
  const float c16 = __fmul_rn(__fmul_rn(s.p.bias_16x16, s.m16[b0]), s.c16s[b0]);
  const float cost_16x8 = __fadd_rn(left, right), cost_8x16 = __fadd_rn(top, bottom);
  const float best_rect = fminf(cost_16x8, cost_8x16);
  float q_min = INFINITY, q_max = 0.0f;
  for (int dy = 0; dy < 2; ++dy)
    for (int dx = 0; dx < 2; ++dx) {
      q_min = fminf(q_min, qac[dy][dx]);
      q_max = fmaxf(q_max, qac[dy][dx]);
    }
  const bool pick = can_place(xb, f.a.yb, bx0, by0, kSt16x16) && c16 < best_rect &&
                    c16 < __fmul_rn(total, risk_gated(s, s.p.accept_16, q_min, q_max, 1.0f));
  SuperCost out;
  out.dct8 = total;
  if (pick) {
    map_set_first(s.map, xb, bx0, by0, kSt16x16);
    out.chosen = c16;
  } else {
    out.chosen = cost_16x8 <= cost_8x16 ? cost_16x8 : cost_8x16;
  }
  return out;
}

// One thread per 4x4-block cell: the cells the reference's band loop visits
// at this cell's rows and columns (select_band, src/ac_strategy/selection.rs:
// 1000-1200; rows advance by 4 while four fit, then by 2).
__global__ void __launch_bounds__(128) k_select(const __grid_constant__ Frame f) {
  const SearchFrame& s = *static_cast<const SearchFrame*>(f.search);
  const int xb = f.a.xb, yb = f.a.yb;
  const int ncx = (xb + 3) / 4, ncy = (yb + 3) / 4;
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= ncx * ncy) return;
  const int bx0 = 4 * (cell % ncx), by0 = 4 * (cell / ncx);
  if (by0 + 1 >= yb) return;
  const bool four_row = by0 + 4 <= yb;
  if (four_row && bx0 + 4 <= xb) {
    float ch[2][2], base[2][2];
    for (int sy = 0; sy < 2; ++sy)
      for (int sx = 0; sx < 2; ++sx) {
        const SuperCost c = select_super(f, s, bx0 + 2 * sx, by0 + 2 * sy);
        ch[sy][sx] = c.chosen;
        base[sy][sx] = c.dct8;
      }
    const int b0 = by0 * xb + bx0;
    const float merge32 = __fmul_rn(__fmul_rn(s.p.bias_32x32, s.m32[b0]), s.c32[b0]);
    uint32_t qmin = 255, qmax = 0;
    for (int iy = 0; iy < 4; ++iy)
      for (int ix = 0; ix < 4; ++ix) {
        const uint32_t q = f.qf[b0 + iy * xb + ix];
        qmin = min(qmin, q);
        qmax = max(qmax, q);
      }
    const float accept = risk_gated(s, s.p.accept_32, static_cast<float>(qmin),
                                    static_cast<float>(qmax), 2.0f);
    // choose_merge_partition (src/ac_strategy/selection.rs:115-152) with the
    // rectangles priced infinite: only the square merge can pass its gate
    const float child = __fadd_rn(__fadd_rn(__fadd_rn(ch[0][0], ch[0][1]), ch[1][0]), ch[1][1]);
    const float bsum = __fadd_rn(__fadd_rn(__fadd_rn(base[0][0], base[0][1]), base[1][0]), base[1][1]);
    if (merge32 < child && merge32 < __fmul_rn(bsum, accept)) map_set_first(s.map, xb, bx0, by0, kSt32x32);
    return;
  }
  for (int sbx = bx0; sbx < bx0 + 4; sbx += 2) {
    if (sbx + 1 >= xb) break;
    select_super(f, s, sbx, by0);
    if (four_row) select_super(f, s, sbx, by0 + 2);
  }
}

// plan_small and search_tile_coefficient (src/ac_strategy/selection/
// layout_dp.rs:1864-2198), one warp per tile.
constexpr int kSmallLeaf = 1, kSmallWide = 2, kSmallTall = 3, kSmallSquare = 4;
__device__ __forceinline__ int small_strategy(int choice) {
  return choice == kSmallLeaf ? kStDct : choice == kSmallWide ? kSt8x16
         : choice == kSmallTall ? kSt16x8 : kSt16x16;
}

// One warp's DP state.  The reference walks a layer's active profiles in
// order and relaxes each successor with a strict `<`, so a successor keeps
// the cheapest relaxation and, among equal costs, the earliest; the next
// layer lists the successors in the order they were first reached.  The
// warp relaxes every profile at once: a successor's 64-bit key (a
// generation, the cost mapped to an order-preserving integer, then the
// relaxation's rank a * 4 + k) takes an atomicMin, so it ends at the same
// winner; `first` takes the smallest (generation, rank) that reached it, and
// ballots lay the next layer out in that order.  The generation, 64 - cell,
// makes every entry a later cell writes smaller than the ones earlier cells
// left behind, so no entry is ever reset.
struct RetileSmem {
  unsigned long long key_a[512], key_b[512];
  uint32_t first[512];
  uint16_t act_a[512], act_b[512];
  float leaf[64], wide[64], tall[64], square[64];
  uint8_t live[64];
  int8_t current[64];  // the map's strategy at each first block of the tile, -1 elsewhere
  int8_t plan[64];     // the winning plan's strategy at each first block it places, -1 elsewhere
};
constexpr int kRetileWarps = 4;  // tiles per CTA by default (tuned per device)
constexpr unsigned long long kNoKey = ~0ull;

__device__ __forceinline__ uint32_t ordered_bits(float v) {
  const uint32_t u = __float_as_uint(__fadd_rn(v, 0.0f));  // -0 -> +0
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
// key: bits 43-49 generation, 11-42 ordered cost, 0-10 rank
__device__ __forceinline__ unsigned long long dp_key(uint32_t gen, float cv, uint32_t rank) {
  return (static_cast<unsigned long long>(gen) << 43) |
         (static_cast<unsigned long long>(ordered_bits(cv)) << 11) | rank;
}
__device__ __forceinline__ float dp_cost(unsigned long long key) {
  const uint32_t k = static_cast<uint32_t>(key >> 11);
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// The relaxations of active profile `state` at one cell, in the reference's
// order: k = 0 keep (a filled cell) or leaf, 1 wide, 2 tall, 3 square; an
// absent one has an infinite cost.
struct Relax {
  int to[4];
  float cv[4];
  uint8_t ch[4];
};
__device__ __forceinline__ void relaxations(int state, float here, int corner, int mask, int w,
                                            int shapes, float lf, float wd, float tl, float sq,
                                            Relax* r) {
  const int below_bit = 1 << w;
  auto set = [&](int k, int filled, float cv, int ch) {
    r->to[k] = ((filled >> 1) | corner) & mask;
    r->cv[k] = cv;
    r->ch[k] = static_cast<uint8_t>(ch);
  };
  if (state & 1) {
    set(0, state, here, 0);
    set(1, 0, INFINITY, 0);
    set(2, 0, INFINITY, 0);
    set(3, 0, INFINITY, 0);
    return;
  }
  set(0, state, __fadd_rn(here, lf), kSmallLeaf);
  const bool right = (state & 2) == 0, below = (state & below_bit) == 0;
  if (right && (shapes & 1)) set(1, state | 2, __fadd_rn(here, wd), kSmallWide);
  else set(1, 0, INFINITY, 0);
  if (below && (shapes & 2)) set(2, state | below_bit, __fadd_rn(here, tl), kSmallTall);
  else set(2, 0, INFINITY, 0);
  if (right && below && corner == 0 && (shapes & 4))
    set(3, state | 2 | below_bit | (2 << w), __fadd_rn(here, sq), kSmallSquare);
  else set(3, 0, INFINITY, 0);
}

// The relaxations of one round's profile (a < len) into the next layer.
__device__ __forceinline__ void relax_push(const Relax& r, int a, uint32_t gen,
                                           unsigned long long* nxt, uint32_t* first) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (!(r.cv[k] < INFINITY)) continue;
    const uint32_t rank = static_cast<uint32_t>(a * 4 + k);
    atomicMin(&nxt[r.to[k]], dp_key(gen, r.cv[k], rank));
    atomicMin(&first[r.to[k]], (gen << 11) | rank);
  }
}

// After the round's atomics: the relaxations that won their successor write
// its choice; those that reached it first place it in the next layer (ranks
// ascend with the lane, then with k: one ballot per k).  Returns the
// round's count of placed successors.
__device__ __forceinline__ int relax_place(const Relax& r, bool valid, int a, uint32_t gen,
                                           const unsigned long long* nxt, const uint32_t* first,
                                           uint8_t* from, uint16_t* nact, int nlen) {
  const int lane = threadIdx.x & 31;
  uint32_t own = 0;
  if (valid) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (!(r.cv[k] < INFINITY)) continue;
      const uint32_t rank = static_cast<uint32_t>(a * 4 + k);
      if (first[r.to[k]] == ((gen << 11) | rank)) own |= 1u << k;
      if ((static_cast<uint32_t>(nxt[r.to[k]]) & 0x7ffu) == rank) from[r.to[k]] = r.ch[k];
    }
  }
  const unsigned below = (1u << lane) - 1u;
  int pos = nlen, total = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const unsigned b = __ballot_sync(0xffffffffu, (own >> k) & 1u);
    pos += __popc(b & below);
    total += __popc(b);
  }
#pragma unroll
  for (int k = 0; k < 4; ++k)
    if (own & (1u << k)) nact[pos++] = static_cast<uint16_t>(r.to[k]);
  return total;
}

// The whole warp calls it with the same arguments.  When its total is finite
// and below `replace_below`, its plan replaces `sm.plan`.
__device__ float plan_small(RetileSmem& sm, uint64_t fixed, int w, int h, uint8_t* choices,
                            float replace_below) {
  const int lane = threadIdx.x & 31;
  const int cells = w * h, states = 1 << (w + 1), mask = states - 1;
  const int below_bit = 1 << w;
  unsigned long long* cur = sm.key_a;
  unsigned long long* nxt = sm.key_b;
  uint16_t* act = sm.act_a;
  uint16_t* nact = sm.act_b;
  for (int i = lane; i < states; i += 32) {
    cur[i] = nxt[i] = kNoKey;
    sm.first[i] = ~0u;
  }
  __syncwarp();
  const int start = static_cast<int>(fixed & static_cast<uint64_t>(mask));
  if (lane == 0) {
    cur[start] = dp_key(65u, 0.0f, 0u);  // the layer before cell 0
    act[0] = static_cast<uint16_t>(start);
  }
  int len = 1;
  uint64_t incoming = fixed >> (w + 1);
  __syncwarp();
  for (int i = 0; i < cells; ++i) {
    const uint32_t gen = static_cast<uint32_t>(64 - i);
    uint8_t* from = choices + i * states;
    const int corner = static_cast<int>(incoming & 1u) << w;
    incoming >>= 1;
    const int shapes = sm.live[i];
    const float lf = sm.leaf[i], wd = sm.wide[i], tl = sm.tall[i], sq = sm.square[i];
    int nlen = 0;
    if (len <= 32) {
      // one round: the relaxations stay in registers between the two steps
      const bool valid = lane < len;
      Relax r;
      if (valid) {
        const int state = act[lane];
        relaxations(state, dp_cost(cur[state]), corner, mask, w, shapes, lf, wd, tl, sq, &r);
        relax_push(r, lane, gen, nxt, sm.first);
      }
      __syncwarp();
      nlen = relax_place(r, valid, lane, gen, nxt, sm.first, from, nact, 0);
    } else {
#pragma unroll 2
      for (int a0 = 0; a0 < len; a0 += 32) {
        const int a = a0 + lane;
        if (a < len) {
          const int state = act[a];
          Relax r;
          relaxations(state, dp_cost(cur[state]), corner, mask, w, shapes, lf, wd, tl, sq, &r);
          relax_push(r, a, gen, nxt, sm.first);
        }
      }
      __syncwarp();
      for (int a0 = 0; a0 < len; a0 += 32) {
        const int a = a0 + lane;
        const bool valid = a < len;
        Relax r;
        if (valid) {
          const int state = act[a];
          relaxations(state, dp_cost(cur[state]), corner, mask, w, shapes, lf, wd, tl, sq, &r);
        }
        nlen += relax_place(r, valid, a, gen, nxt, sm.first, from, nact, nlen);
      }
    }
    __syncwarp();
    unsigned long long* tk = cur;
    cur = nxt;
    nxt = tk;
    uint16_t* ta = act;
    act = nact;
    nact = ta;
    len = nlen;
  }
  // state 0 of the last layer, if the last cell reached it
  const unsigned long long k0 = cur[0];
  const float total = (k0 >> 43) == static_cast<unsigned long long>(65 - cells) ? dp_cost(k0) : INFINITY;
  __syncwarp();
  if (!(isfinite(total) && total < replace_below)) return total;
  for (int i = lane; i < 64; i += 32) sm.plan[i] = -1;
  __syncwarp();
  // The backtrack from state 0 of the last layer: the profile before cell i
  // follows from the profile after it and the cell's choice.  Each round
  // loads, at once, the choice of cell i, the five choices cell i - 1 could
  // be asked for (one per choice at i) and the 25 of cell i - 2, then
  // follows the three the walk takes: three cells a memory round trip, the
  // same walk as one cell at a time.
  auto before = [&](int state, int choice) {
    const int added = choice == 2 ? 2 : choice == 3 ? below_bit : choice == 4 ? 2 | below_bit | (2 << w) : 0;
    return (((state << 1) ^ added) & mask) | (choice == 0 ? 1 : 0);
  };
  const int c1 = lane >= 6 ? (lane - 6) / 5 : lane - 1, c2 = (lane - 6) % 5;
  const int depth = lane == 0 ? 0 : lane <= 5 ? 1 : lane <= 30 ? 2 : -1;
  int state = 0;
  for (int i = cells - 1; i >= 0; i -= 3) {
    int mine = 0;
    const int cell = i - depth;
    if (depth >= 0 && cell >= 0) {
      const int st = depth == 0 ? state : depth == 1 ? before(state, c1) : before(before(state, c1), c2);
      mine = choices[cell * states + st];
    }
    const int a = __shfl_sync(0xffffffffu, mine, 0);
    const int a_in = a <= 4 ? a : 0;
    const int b = __shfl_sync(0xffffffffu, mine, 1 + a_in);
    const int b_in = b <= 4 ? b : 0;
    const int c = __shfl_sync(0xffffffffu, mine, 6 + 5 * a_in + b_in);
    if (lane == 0) {
      if (a != 0) sm.plan[i] = static_cast<int8_t>(small_strategy(a));
      if (i >= 1 && b != 0) sm.plan[i - 1] = static_cast<int8_t>(small_strategy(b));
      if (i >= 2 && c != 0) sm.plan[i - 2] = static_cast<int8_t>(small_strategy(c));
    }
    state = before(before(before(state, a), b), c);
  }
  __syncwarp();
  return total;
}

struct Piece {
  int8_t x, y, s;
};

__global__ void __launch_bounds__(32 * kMaxTuneWarps) k_retile(const __grid_constant__ Frame f) {
  extern __shared__ __align__(16) unsigned char retile_smem_raw[];
  RetileSmem& sm = reinterpret_cast<RetileSmem*>(retile_smem_raw)[threadIdx.x >> 5];
  const SearchFrame& s = *static_cast<const SearchFrame*>(f.search);
  const int lane = threadIdx.x & 31;
  const int xb = f.a.xb, yb = f.a.yb;
  const int tx = (xb + 7) / 8, ty = (yb + 7) / 8;
  const int tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (tile >= tx * ty) return;
  const int bx = 8 * (tile % tx), by = 8 * (tile / tx);
  const int w = imin(8, xb - bx), h = imin(8, yb - by);
  if (w * h < 2) return;
  uint8_t* map = s.map;
  // the piece score of a candidate at tile cell (x, y): its unbiased cost
  auto score = [&](Piece p) -> float {
    const int b = (by + p.y) * xb + bx + p.x;
    switch (p.s) {
      case kStDct: return s.c8[b];
      case kSt8x16: return s.cw[b];
      case kSt16x8: return s.ct[b];
      case kSt16x16: return s.c16r[b];
      default: return s.c32[b];
    }
  };
  for (int i = lane; i < 64; i += 32) {
    sm.leaf[i] = sm.wide[i] = sm.tall[i] = sm.square[i] = INFINITY;
    sm.live[i] = 0;
  }
  __syncwarp();
  for (int i = lane; i < w * h; i += 32) {
    const int x = i % w, y = i / w, gx = bx + x, gy = by + y;
    const int8_t px = static_cast<int8_t>(x), py = static_cast<int8_t>(y);
    sm.leaf[i] = score(Piece{px, py, kStDct});
    if (x + 2 <= w && gx % 2 == 0 && can_place(xb, yb, gx, gy, kSt8x16))
      sm.wide[i] = score(Piece{px, py, kSt8x16});
    if (y + 2 <= h && gy % 2 == 0 && can_place(xb, yb, gx, gy, kSt16x8))
      sm.tall[i] = score(Piece{px, py, kSt16x8});
    if (x + 2 <= w && y + 2 <= h && gx % 2 == 0 && gy % 2 == 0 && can_place(xb, yb, gx, gy, kSt16x16))
      sm.square[i] = score(Piece{px, py, kSt16x16});
  }
  __syncwarp();
  // SmallCosts::live_masks
  for (int i = lane; i < w * h; i += 32) {
    const int x = i % w, y = i / w, st = y * w;
    const float* leaf = sm.leaf;
    uint8_t m = 0;
    if (y + 1 == h) {
      if (x + 1 < w) m = sm.wide[st + x] < __fadd_rn(leaf[st + x], leaf[st + x + 1]);
    } else if (x + 1 < w) {
      const int bl = st + w;
      const float tl = leaf[st + x], tr = leaf[st + x + 1], bll = leaf[bl + x], brr = leaf[bl + x + 1];
      const float top_leaves = __fadd_rn(tl, tr);
      const float leaves = __fadd_rn(__fadd_rn(top_leaves, bll), brr);
      const float wides = __fadd_rn(sm.wide[st + x], sm.wide[bl + x]);
      const float talls = __fadd_rn(sm.tall[st + x], sm.tall[st + x + 1]);
      m = static_cast<uint8_t>((sm.wide[st + x] < top_leaves ? 1 : 0) |
                               (sm.tall[st + x] < __fadd_rn(tl, bll) ? 2 : 0) |
                               (sm.square[st + x] < fminf(fminf(leaves, wides), talls) ? 4 : 0));
    } else {
      m = sm.tall[st + x] < __fadd_rn(leaf[st + x], leaf[st + w + x]) ? 2 : 0;
    }
    sm.live[i] = m;
  }
  // The tile's current pieces (the map's strategy at each first block) and
  // the fixed ones (larger than 16x16): their cells and their cost, summed in
  // raster order of first blocks.
  uint32_t fixed_half[2] = {0u, 0u};
  float fixed_term[2] = {0.0f, 0.0f};
  unsigned fixed_first[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int i = lane + 32 * r;
    int cs = -1;
    if (i < w * h) {
      const uint8_t cell = map[(by + i / w) * xb + bx + i % w];
      if (cell & 1) cs = cell >> 1;
    }
    sm.current[i] = static_cast<int8_t>(cs);
    const bool big = cs > kSt16x16;
    if (big) {
      const int x = i % w, y = i / w;
      const uint64_t row = (1ull << cov_x_of(cs)) - 1ull;
      uint64_t cover = 0;
      for (int yy = 0; yy < cov_y_of(cs); ++yy) cover |= row << (y * w + x + yy * w);
      fixed_half[0] |= static_cast<uint32_t>(cover);
      fixed_half[1] |= static_cast<uint32_t>(cover >> 32);
      fixed_term[r] = score(Piece{static_cast<int8_t>(x), static_cast<int8_t>(y), static_cast<int8_t>(cs)});
    }
    fixed_first[r] = __ballot_sync(0xffffffffu, big);
  }
  const uint64_t fixed = static_cast<uint64_t>(__reduce_or_sync(0xffffffffu, fixed_half[0])) |
                         (static_cast<uint64_t>(__reduce_or_sync(0xffffffffu, fixed_half[1])) << 32);
  float fixed_cost = 0.0f;
#pragma unroll
  for (int r = 0; r < 2; ++r)
    for (unsigned m = fixed_first[r]; m != 0u; m &= m - 1u)
      fixed_cost = __fadd_rn(fixed_cost, __shfl_sync(0xffffffffu, fixed_term[r], __ffs(m) - 1));
  __syncwarp();
  uint8_t* choices = s.dp_choices + static_cast<int64_t>(tile) * 64 * 512;
  const float around = __fadd_rn(plan_small(sm, fixed, w, h, choices, INFINITY), fixed_cost);
  bool keep_fixed = true;
  float winner = around;
  if (fixed != 0) {
    const float over = plan_small(sm, 0, w, h, choices, around);
    if (over < around) {
      winner = over;
      keep_fixed = false;
    }
  }
  if (!isfinite(winner)) return;
  // The new layout at each first block: the winning plan, with the fixed
  // pieces when they stay.  A piece is in both layouts when the same
  // strategy starts at the same block, so the pieces that change are the
  // blocks where the two strategies differ.  Their costs, summed in raster
  // order of first blocks, decide.  The DP's cost arrays are free again and
  // hold the terms: the old layout's in `leaf`, the new one's in `wide`.
  int ns_of[2];
  unsigned gone[2], added[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int i = lane + 32 * r;
    const int cs = sm.current[i];
    int ns = sm.plan[i];
    if (keep_fixed && cs > kSt16x16) ns = cs;
    ns_of[r] = ns;
    const int8_t x = static_cast<int8_t>(i % w), y = static_cast<int8_t>(i / w);
    const bool g = cs >= 0 && ns != cs, a = ns >= 0 && ns != cs;
    if (g) sm.leaf[i] = score(Piece{x, y, static_cast<int8_t>(cs)});
    if (a) sm.wide[i] = score(Piece{x, y, static_cast<int8_t>(ns)});
    gone[r] = __ballot_sync(0xffffffffu, g);
    added[r] = __ballot_sync(0xffffffffu, a);
  }
  __syncwarp();
  float old_cost = 0.0f, new_cost = 0.0f;
  if (lane == 0) {
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        if (gone[r] & (1u << j)) old_cost = __fadd_rn(old_cost, sm.leaf[32 * r + j]);
        if (added[r] & (1u << j)) new_cost = __fadd_rn(new_cost, sm.wide[32 * r + j]);
      }
  }
  old_cost = __shfl_sync(0xffffffffu, old_cost, 0);
  new_cost = __shfl_sync(0xffffffffu, new_cost, 0);
  if (!(new_cost < old_cost)) return;
  // the new pieces cover exactly the blocks the changed old ones did
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int i = lane + 32 * r;
    if (added[r] & (1u << lane)) map_set_first(map, xb, bx + i % w, by + i / w, ns_of[r]);
  }
}

// adjust_quant_field (src/ac_strategy/selection.rs:503-527), then the alpha
// factors over the layout (apply_alpha_factors, src/adaptive_quant.rs:1036-1070):
// one thread per first block.
__global__ void __launch_bounds__(256) k_adjust(const __grid_constant__ Frame f) {
  const SearchFrame& s = *static_cast<const SearchFrame*>(f.search);
  const int xb = f.a.xb, yb = f.a.yb;
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= xb * yb) return;
  const uint8_t cell = s.map[b];
  if (!(cell & 1)) return;
  const int st = cell >> 1, cx = cov_x_of(st), cy = cov_y_of(st);
  const int x = b % xb, y = b / xb;
  uint8_t* qf = f.qf;
  uint32_t q = qf[b];
  if (cx * cy > 1) {
    uint32_t max_q = 0, sum = 0;
    for (int iy = 0; iy < cy; ++iy)
      for (int ix = 0; ix < cx; ++ix) {
        const uint32_t v = qf[(y + iy) * xb + x + ix];
        max_q = max(max_q, v);
        sum += v;
      }
    q = aggregate_quant(max_q, sum, cx * cy, s.distance);
  }
  const DeviceStats* stats = f.stats;
  if (f.alpha != nullptr && stats->alpha_max != 0xFFFFu - stats->alpha_min_inv) {
    float k = 0.0f;
    for (int iy = 0; iy < cy && k != 1.0f; ++iy)
      for (int ix = 0; ix < cx; ++ix) {
        const float af = __fdiv_rn(static_cast<float>(f.alpha_peak[(y + iy) * xb + x + ix]),
                                   static_cast<float>(f.alpha_full));
        const float kb = (af == 0.0f || af >= 1.0f) ? 1.0f : fmaxf(af, 0.1f);
        k = fmaxf(k, kb);
      }
    int32_t qi = cast_i32(roundf(__fmul_rn(static_cast<float>(q), k)));
    q = static_cast<uint32_t>(qi < 1 ? 1 : (qi > 255 ? 255 : qi));
  }
  for (int iy = 0; iy < cy; ++iy)
    for (int ix = 0; ix < cx; ++ix) qf[(y + iy) * xb + x + ix] = static_cast<uint8_t>(q);
}

// ---------------------------------------------------------------------------
// account_matrix_headers (src/ac_strategy/matrix_overhead.rs:117-268)
// ---------------------------------------------------------------------------

// The incumbent's score at its own (adjusted) quantizer, one warp per site.
template <int S>
__device__ __forceinline__ void mh_incumbent_warp(const Frame& f, const SearchFrame& s, int bx,
                                                  int by, unsigned char* raw) {
  CostSmem<S>& sm = reinterpret_cast<CostSmem<S>*>(raw)[threadIdx.x >> 5];
  const int b = by * f.a.xb + bx;
  // the search priced this transform at the aggregate of the pre-selection
  // field (region_qac), the value adjust_quant_field gives it unless the
  // alpha factors moved it: the same cost, no need to recompute
  const uint8_t agg = region_quant(s.block_qf, f.a.xb, bx, by, Shape<S>::COVX, Shape<S>::COVY, s.distance);
  if (f.qf[b] == agg) {
    if ((threadIdx.x & 31) == 0) s.mh_inc[b] = S == kSt16x16 ? s.c16r[b] : s.c32[b];
    return;
  }
  warp_coefficients<S>(f, bx, by, sm);
  const float qac = __fmul_rn(s.scale, static_cast<float>(f.qf[b]));
  const float q = __fmul_rn(qac, warp_selection_scale<S>(s, sm, qac));
  const float c = warp_rd<S>(f, s, sm, bx, by, q, kMetaR);
  if ((threadIdx.x & 31) == 0) s.mh_inc[b] = c;
}

__global__ void __launch_bounds__(128) k_mh_incumbent(const __grid_constant__ Frame f) {
  extern __shared__ __align__(16) unsigned char mh_smem_raw[];
  const SearchFrame& s = *static_cast<const SearchFrame*>(f.search);
  const int xb = f.a.xb, yb = f.a.yb;
  // sites sit at even block coordinates
  const int nx = (xb + 1) / 2;
  const int64_t e = static_cast<int64_t>(blockIdx.x) * 4 + (threadIdx.x >> 5);
  if (e >= static_cast<int64_t>(nx) * ((yb + 1) / 2)) return;
  const int bx = 2 * static_cast<int>(e % nx), by = 2 * static_cast<int>(e / nx);
  const int64_t b = static_cast<int64_t>(by) * xb + bx;
  const uint8_t cell = s.map[b];
  if (!(cell & 1)) return;
  const int st = cell >> 1;
  if (st == kSt16x16 && (s.p.custom & 2u)) mh_incumbent_warp<kSt16x16>(f, s, bx, by, mh_smem_raw);
  else if (st == kSt32x32 && (s.p.custom & 4u)) mh_incumbent_warp<kSt32x32>(f, s, bx, by, mh_smem_raw);
}

// The reference sums each family's unavoidable loss and every table
// subset's cost serially in f64, in DC-group order, and only compares those
// sums.  The device sums the same non-negative terms in parallel (P) and
// settles each comparison from an interval that holds the serial result: for
// n terms both |serial - exact| and |P - exact| stay below n u E (u = 2^-53,
// error bounds of recursive and pairwise summation; an addition of zero is
// exact), so the serial sum lies within M = (n + 64) 2^-51 P of P.  A
// comparison the interval leaves open (in practice an exact tie of different
// sums) is settled by the serial sums in the reference's order.

// k_mh_sum's per-CTA partials: [0] [1] the 16x16 / 32x32 families'
// unavoidable losses; [2 + a] / [10 + a] the families' cheapest alternatives
// under allowed & 7 == a (best_alternative reads only slots 0-2); [18] [19]
// the families' site counts; [20] the custom slots the layout uses.
constexpr int kMhQuantities = 21;
constexpr int kMhSumThreads = 256;
constexpr int kMhThreads = 1024;

// best_alternative (matrix_overhead.rs:50-63) of a site of table slot `slot`
// under `allowed`: incumbent (requires its own slot), DCT (slot 0 when
// custom), 16x16 (slot 1 when custom); strict `<` keeps the earlier one on a
// tie; `which` is 0, 1, 2 for them, -1 for none.
__device__ __forceinline__ double mh_best(uint32_t slot, double ld, double l16, uint32_t allowed,
                                          uint32_t custom, int* which) {
  double best = INFINITY;
  *which = -1;
  if (((1u << slot) & ~allowed) == 0u) { best = 0.0; *which = 0; }
  if (ld >= 0.0 && ((1u & custom) & ~allowed) == 0u && (*which < 0 || ld < best)) { best = ld; *which = 1; }
  if (l16 >= 0.0 && ((2u & custom) & ~allowed) == 0u && (*which < 0 || l16 < best)) { best = l16; *which = 2; }
  return best;
}

__device__ __forceinline__ uint32_t mh_slot(uint8_t cell) {
  const int st = cell >> 1;
  return st == kStDct ? 0u : st == kSt16x16 ? 1u : st == kSt32x32 ? 2u : 3u;
}

// One thread per 2x2-block cell (its first block at even coordinates): the
// custom slots its first blocks use, and for a site (a 16x16 / 32x32 whose
// table is custom) the alternatives' losses (mh_score, matrix_overhead.rs:
// 65-91, an f64 sum in raster order) and its terms of every sum; then the
// CTA's partials in a fixed order.
__global__ void __launch_bounds__(kMhSumThreads) k_mh_sum(const __grid_constant__ Frame f) {
  const SearchFrame& s = *static_cast<const SearchFrame*>(f.search);
  const int xb = f.a.xb, yb = f.a.yb;
  const int nx = (xb + 1) / 2;
  const int64_t e = static_cast<int64_t>(blockIdx.x) * kMhSumThreads + threadIdx.x;
  const uint32_t custom = s.p.custom;
  double q[kMhQuantities];
#pragma unroll
  for (int i = 0; i < kMhQuantities; ++i) q[i] = 0.0;
  if (e < static_cast<int64_t>(nx) * ((yb + 1) / 2)) {
    const int bx = 2 * static_cast<int>(e % nx), by = 2 * static_cast<int>(e / nx);
    const int64_t b = static_cast<int64_t>(by) * xb + bx;
    uint32_t used = 0;
    for (int iy = 0; iy < 2 && by + iy < yb; ++iy)
      for (int ix = 0; ix < 2 && bx + ix < xb; ++ix) {
        const uint8_t cell = s.map[b + iy * xb + ix];
        if ((cell & 1) && (custom & (1u << mh_slot(cell)))) used |= 1u << mh_slot(cell);
      }
    q[20] = static_cast<double>(used);
    const uint8_t cell = s.map[b];
    const uint32_t slot = mh_slot(cell);
    uint8_t kind = 0;
    if ((cell & 1) && (slot == 1u || slot == 2u) && (custom & (1u << slot))) {
      kind = static_cast<uint8_t>(slot);
      const int st = cell >> 1, cx = cov_x_of(st), cy = cov_y_of(st);
      const double lambda = static_cast<double>(kRdLambda);
      const double inc = static_cast<double>(s.mh_inc[b]) / lambda;
      double c = 0.0;
      for (int iy = 0; iy < cy; ++iy)
        for (int ix = 0; ix < cx; ++ix)
          c = __dadd_rn(c, static_cast<double>(s.c8[b + iy * xb + ix]) / lambda);
      double loss = __dsub_rn(c, inc);
      const double ld = (isfinite(c) && isfinite(inc)) ? (loss > 0.0 ? loss : 0.0) : -1.0;
      double l16 = -1.0;
      if (st == kSt32x32) {
        double c2 = 0.0;
        for (int iy = 0; iy < 4; iy += 2)
          for (int ix = 0; ix < 4; ix += 2)
            c2 = __dadd_rn(c2, static_cast<double>(s.c16r[b + iy * xb + ix]) / lambda);
        loss = __dsub_rn(c2, inc);
        l16 = (isfinite(c2) && isfinite(inc)) ? (loss > 0.0 ? loss : 0.0) : -1.0;
      }
      s.mh_loss[2 * b] = ld;
      s.mh_loss[2 * b + 1] = l16;
      double mn = INFINITY;
      if (ld >= 0.0) mn = fmin(mn, ld);
      if (l16 >= 0.0) mn = fmin(mn, l16);
      double best[8];
#pragma unroll
      for (uint32_t a = 0; a < 8; ++a) {
        int which;
        best[a] = mh_best(slot, ld, l16, a, custom, &which);
      }
      if (slot == 1u) {
        q[0] = mn;
        q[18] = 1.0;
#pragma unroll
        for (int a = 0; a < 8; ++a) q[2 + a] = best[a];
      } else {
        q[1] = mn;
        q[19] = 1.0;
#pragma unroll
        for (int a = 0; a < 8; ++a) q[10 + a] = best[a];
      }
    }
    s.mh_kind[b] = kind;
  }
  // the CTA's partials: warp butterflies, then one thread per quantity over the warps
  __shared__ double part[kMhSumThreads / 32][kMhQuantities];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < kMhQuantities; ++i) {
    double v = q[i];
    if (i == 20) {
      uint32_t u = static_cast<uint32_t>(v);
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) u |= __shfl_xor_sync(0xffffffffu, u, d);
      v = static_cast<double>(u);
    } else {
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) v = __dadd_rn(v, __shfl_xor_sync(0xffffffffu, v, d));
    }
    if (lane == 0) part[warp][i] = v;
  }
  __syncthreads();
  if (threadIdx.x < kMhQuantities) {
    const int i = threadIdx.x;
    double v = 0.0;
    uint32_t u = 0;
    for (int w = 0; w < kMhSumThreads / 32; ++w) {
      v = __dadd_rn(v, part[w][i]);
      u |= static_cast<uint32_t>(part[w][i]);
    }
    s.mh_part[static_cast<int64_t>(blockIdx.x) * kMhQuantities + i] = i == 20 ? static_cast<double>(u) : v;
  }
}

__device__ __forceinline__ uint32_t header_bits(const SearchFrame& s, uint32_t used) {
  uint32_t payload = 0;
  for (int i = 0; i < 13; ++i)
    if (used & (1u << i)) payload += s.p.payload[i];
  return 1u + payload + (payload != 0u ? 17u * 3u : 0u);
}

// An interval [lo, hi] that holds the serial sum of `n` non-negative terms
// whose parallel sum is p; `terms` is the parallel sum of the terms after the
// first (the header bits).  Zero there means every later term is zero, and
// adding zero is exact: the serial sum is p itself.
struct SumRange {
  double lo, hi;
};
__device__ __forceinline__ SumRange sum_range(double p, double n, double terms) {
  if (!isfinite(p) || terms == 0.0) return SumRange{p, p};
  const double m = __dmul_rn(__dmul_rn(p, __dadd_rn(n, 64.0)), 0x1p-51);
  return SumRange{__dsub_rn(p, m), __dadd_rn(p, m)};
}

// One CTA: the partials' totals, the pinned families, the cheapest table set
// (every subset of the custom slots in the reference's order: custom, then
// (prev - 1) & custom down to 0; losses are non-negative, so the reference's
// early exits never change which set wins or which family is pinned),
// written to mh_decision as {best, pinned, used}.  The serial path builds
// the site lists in DC-group order (16x16 sites, then 32x32 sites: the order
// in which the reference sums its regions).
__global__ void __launch_bounds__(kMhThreads) k_mh_choose(const __grid_constant__ Frame f,
                                                          int parts) {
  const SearchFrame& s = *static_cast<const SearchFrame*>(f.search);
  const int xb = f.a.xb, yb = f.a.yb;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  __shared__ double tot[kMhQuantities];
  __shared__ uint32_t s_n[2], s_warp[2][32], s_flags, s_pinned, s_best;
  __shared__ double s_unavoidable[2], s_subset_cost[64];
  if (warp < kMhQuantities) {
    double v = 0.0;
    uint32_t u = 0;
    for (int k = lane; k < parts; k += 32) {
      const double x = s.mh_part[static_cast<int64_t>(k) * kMhQuantities + warp];
      v = __dadd_rn(v, x);
      u |= static_cast<uint32_t>(x);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      v = __dadd_rn(v, __shfl_xor_sync(0xffffffffu, v, d));
      u |= __shfl_xor_sync(0xffffffffu, u, d);
    }
    if (lane == 0) tot[warp] = warp == 20 ? static_cast<double>(u) : v;
  }
  __syncthreads();
  const uint32_t used = static_cast<uint32_t>(tot[20]), custom = s.p.custom;
  if ((used & ~1u) == 0u) {
    if (tid == 0) {
      s.mh_decision[0] = used;
      s.mh_decision[1] = 0;
      s.mh_decision[2] = used;
    }
    return;
  }
  const double cnt[2] = {tot[18], tot[19]};
  // 1: the pinned families (matrix_overhead.rs:180-215)
  if (tid == 0) {
    uint32_t pinned = used & 1u, open = 0;
    for (int slot = 1; slot <= 2; ++slot) {
      if (!(used & (1u << slot))) continue;
      const double thr = static_cast<double>(s.p.payload[slot] + 17u * 3u);
      const SumRange r = sum_range(tot[slot - 1], cnt[slot - 1], tot[slot - 1]);
      if (r.lo > thr) pinned |= 1u << slot;
      else if (!(r.hi <= thr)) open = 1;
    }
    s_pinned = pinned;
    s_flags = open || s.p.serial_sums;
  }
  __syncthreads();
  const bool serial = s_flags != 0;
  const int xdc = (xb + 255) / 256, ydc = (yb + 255) / 256;
  const int64_t nb = static_cast<int64_t>(xb) * yb;
  uint32_t* list16 = s.sites;
  uint32_t* list32 = s.sites + nb / 2;
  auto build_lists = [&]() {
    if (tid == 0) s_n[0] = s_n[1] = 0;
    __syncthreads();
    for (int64_t base = 0; base < nb; base += kMhThreads) {
      const int64_t k = base + tid;
      int fam = -1, b = -1;
      if (k < nb) {
        int64_t rem = k;
        int gx0 = 0, gy0 = 0, gw = 0, gh = 0;
        for (int g = 0; g < xdc * ydc; ++g) {
          gx0 = (g % xdc) * 256;
          gy0 = (g / xdc) * 256;
          gw = imin(256, xb - gx0);
          gh = imin(256, yb - gy0);
          if (rem < static_cast<int64_t>(gw) * gh) break;
          rem -= static_cast<int64_t>(gw) * gh;
        }
        b = (gy0 + static_cast<int>(rem / gw)) * xb + gx0 + static_cast<int>(rem % gw);
        const uint8_t cell = s.map[b];
        const uint32_t slot = mh_slot(cell);
        if ((cell & 1) && (slot == 1u || slot == 2u) && (custom & (1u << slot))) fam = static_cast<int>(slot) - 1;
      }
      const unsigned b0 = __ballot_sync(0xffffffffu, fam == 0), b1 = __ballot_sync(0xffffffffu, fam == 1);
      if (lane == 0) {
        s_warp[0][warp] = __popc(b0);
        s_warp[1][warp] = __popc(b1);
      }
      __syncthreads();
      if (fam >= 0) {
        uint32_t before = 0;
        for (int w = 0; w < warp; ++w) before += s_warp[fam][w];
        const unsigned bal = fam == 0 ? b0 : b1;
        (fam == 0 ? list16 : list32)[s_n[fam] + before + __popc(bal & ((1u << lane) - 1u))] =
            static_cast<uint32_t>(b);
      }
      __syncthreads();
      if (tid < 2) {
        uint32_t total = 0;
        for (int w = 0; w < 32; ++w) total += s_warp[tid][w];
        s_n[tid] += total;
      }
      __syncthreads();
    }
  };
  if (serial) {
    build_lists();
    // the unavoidable losses in site order (thread 0: 16x16, 32: 32x32)
    if (tid == 0 || tid == 32) {
      const uint32_t* list = tid == 0 ? list16 : list32;
      const uint32_t n = s_n[tid == 0 ? 0 : 1];
      double u = 0.0;
      for (uint32_t k = 0; k < n; ++k) {
        const double ld = s.mh_loss[2 * list[k]], l16 = s.mh_loss[2 * list[k] + 1];
        double mn = INFINITY;
        if (ld >= 0.0) mn = fmin(mn, ld);
        if (l16 >= 0.0) mn = fmin(mn, l16);
        u = __dadd_rn(u, mn);
      }
      s_unavoidable[tid == 0 ? 0 : 1] = u;
    }
    __syncthreads();
    if (tid == 0) {
      uint32_t pinned = used & 1u;
      for (int slot = 1; slot <= 2; ++slot)
        if ((used & (1u << slot)) &&
            s_unavoidable[slot - 1] > static_cast<double>(s.p.payload[slot] + 17u * 3u))
          pinned |= 1u << slot;
      s_pinned = pinned;
    }
    __syncthreads();
  }
  const uint32_t pinned = s_pinned;
  const int nsub = 1 << __popc(custom);
  // 2: the subsets' costs, as intervals; settle the reference's running
  // choice (strict `<` against the best so far, starting from `used`)
  if (tid == 0) {
    uint32_t best = used, allowed = custom;
    const double hb_used = static_cast<double>(header_bits(s, used));
    SumRange best_r{hb_used, hb_used};
    bool open = serial;
    for (int j = 0; j < nsub && !open; ++j) {
      if ((pinned & ~allowed) == 0u) {
        const uint32_t a = allowed & 7u;
        double p = static_cast<double>(header_bits(s, allowed)), n = 1.0, terms = 0.0;
        if (!(pinned & 2u)) { terms = tot[2 + a]; n = __dadd_rn(n, cnt[0]); }
        if (!(pinned & 4u)) { terms = __dadd_rn(terms, tot[10 + a]); n = __dadd_rn(n, cnt[1]); }
        p = __dadd_rn(p, terms);
        const SumRange r = sum_range(p, n, terms);
        if (r.hi < best_r.lo) {
          best = allowed;
          best_r = r;
        } else if (!(r.lo >= best_r.hi)) {
          open = true;
        }
      }
      allowed = (allowed - 1u) & custom;
    }
    s_best = best;
    s_flags = open;
  }
  __syncthreads();
  if (s_flags) {
    if (!serial) build_lists();
    const uint32_t n16 = s_n[0], count = s_n[0] + s_n[1];
    if (tid < nsub) {
      uint32_t allowed = custom;
      for (int j = 0; j < tid; ++j) allowed = (allowed - 1u) & custom;
      double cost = INFINITY;
      if ((pinned & ~allowed) == 0u) {
        cost = static_cast<double>(header_bits(s, allowed));
        // a pinned family's regions were dropped
        const uint32_t lo = (pinned & 2u) ? n16 : 0u;
        const uint32_t hi = (pinned & 4u) ? n16 : count;
        for (uint32_t k = lo; k < hi; ++k) {
          const uint32_t b = k < n16 ? list16[k] : list32[k - n16];
          int which;
          cost = __dadd_rn(cost, mh_best(k < n16 ? 1u : 2u, s.mh_loss[2 * b], s.mh_loss[2 * b + 1],
                                         allowed, custom, &which));
        }
      }
      s_subset_cost[tid] = cost;
    }
    __syncthreads();
    if (tid == 0) {
      uint32_t best = used;
      double best_cost = static_cast<double>(header_bits(s, used));
      uint32_t allowed = custom;
      for (int j = 0; j < nsub; ++j) {
        if ((pinned & ~allowed) == 0u && s_subset_cost[j] < best_cost) {
          best_cost = s_subset_cost[j];
          best = allowed;
        }
        allowed = (allowed - 1u) & custom;
      }
      s_best = best;
    }
    __syncthreads();
  }
  if (tid == 0) {
    s.mh_decision[0] = s_best;
    s.mh_decision[1] = pinned;
    s.mh_decision[2] = used;
  }
}

// One thread per 2x2-block cell: a site of a family not pinned takes its
// cheapest alternative under the chosen set (matrix_overhead.rs:240-268).
__global__ void __launch_bounds__(256) k_mh_apply(const __grid_constant__ Frame f) {
  const SearchFrame& s = *static_cast<const SearchFrame*>(f.search);
  const int xb = f.a.xb, yb = f.a.yb;
  const int nx = (xb + 1) / 2;
  const int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= static_cast<int64_t>(nx) * ((yb + 1) / 2)) return;
  const uint32_t best = s.mh_decision[0], pinned = s.mh_decision[1], used = s.mh_decision[2];
  if (best == used) return;
  const int bx = 2 * static_cast<int>(e % nx), by = 2 * static_cast<int>(e / nx);
  const int64_t b = static_cast<int64_t>(by) * xb + bx;
  const uint32_t slot = s.mh_kind[b];
  if (slot == 0u || (pinned & (1u << slot))) return;
  int which;
  mh_best(slot, s.mh_loss[2 * b], s.mh_loss[2 * b + 1], best, s.p.custom, &which);
  if (which <= 0) return;
  const int chosen = which == 1 ? kStDct : kSt16x16;
  const int st = slot == 2u ? kSt32x32 : kSt16x16;
  const int w = cov_x_of(st), h = cov_y_of(st), cx = cov_x_of(chosen), cy = cov_y_of(chosen);
  for (int yy = 0; yy < h; yy += cy)
    for (int xx = 0; xx < w; xx += cx) {
      map_set_first(s.map, xb, bx + xx, by + yy, chosen);
      // merged_quant (matrix_overhead.rs:93-113) from the pre-selection field
      uint8_t q;
      if (cx * cy == 1) {
        q = s.block_qf[(by + yy) * xb + bx + xx];
      } else {
        uint32_t max_q = 0, sum = 0;
        for (int iy = 0; iy < cy; ++iy)
          for (int ix = 0; ix < cx; ++ix) {
            const uint32_t v = s.block_qf[(by + yy + iy) * xb + bx + xx + ix];
            max_q = max(max_q, v);
            sum += v;
          }
        q = aggregate_quant(max_q, sum, cx * cy, s.distance);
      }
      for (int iy = 0; iy < cy; ++iy)
        for (int ix = 0; ix < cx; ++ix) f.qf[(by + yy + iy) * xb + bx + xx + ix] = q;
    }
}


// ac_qf_threshold over the final field (src/frame/ac_groups.rs:92-113), one CTA.
__global__ void __launch_bounds__(256) k_qf_median(const __grid_constant__ Frame f) {
  __shared__ uint32_t hist[256];
  hist[threadIdx.x] = 0;
  __syncthreads();
  const int64_t nb = static_cast<int64_t>(f.a.xb) * f.a.yb;
  for (int64_t i = threadIdx.x; i < nb; i += 256) atomicAdd(&hist[f.qf[i]], 1u);
  __syncthreads();
  f.stats->qf_hist[threadIdx.x] = hist[threadIdx.x];
  __syncthreads();
  __threadfence_block();
  qf_threshold_from_histogram(f.stats, hist);
}

// ---------------------------------------------------------------------------
// write_ac_group over the layout (src/group.rs:1259-2426)
// ---------------------------------------------------------------------------

// One warp's buffers for a transform of shape S: one channel's gathered
// pixels, the parked Y levels and the three channels' coefficients.
template <int S>
struct LayoutSmem {
  static constexpr int W = Shape<S>::W, H = Shape<S>::H, SIZE = W * H;
  float in[H][W + 1];
  int32_t ylev[SIZE];
  float co[3][SIZE];
};

__device__ __forceinline__ int dct_kind_of(int st) {
  switch (st) {
    case kSt16x8: return kDct16x8;
    case kSt8x16: return kDct8x16;
    case kSt16x16: return kDct16x16;
    case kSt32x32: return kDct32x32;
    default: return kDct8x8;
  }
}

// dc_from_coefficients (src/group.rs:183-261): a DCT8 carries its DC in
// coefficient 0
__device__ __forceinline__ void piece_dc(int kind, const float* c, float* dc) {
  if (kind == kDct8x8) dc[0] = c[0];
  else dc_from_coefficients(kind, c, dc);
}

// quantize_block_ac's threshold of coefficient i of a CX x CY block
__device__ __forceinline__ float layout_threshold(const float* thr, int i, int cx, int cy) {
  const int width = cx * 8, y = i / width, x = i % width;
  const int yfix = y >= cy * 4 ? 2 : 0;
  return x >= width / 2 ? thr[yfix + 1] : thr[yfix];
}

// The steps of write_ac_group for one transform of shape S at (bx, by); a
// warp runs a channel's loops, one thread the DC steps.
template <int S>
struct LayoutShape {
  static constexpr int CX = Shape<S>::CX, CY = Shape<S>::CY, COVX = Shape<S>::COVX;
  static constexpr int COVY = Shape<S>::COVY, SIZE = CX * CY * 64, COVERED = CX * CY;
  static constexpr int LOG2C = COVERED == 1 ? 0 : COVERED == 2 ? 1 : COVERED == 4 ? 2 : 4;
};

// Y DC levels of the covered blocks (quantize_dc_scalar, src/group.rs:286-292)
template <int S>
__device__ __forceinline__ void layout_y_dc(const KernelArgs& a, const float* co_y, int16_t* ydq) {
  float dcv[16];
  piece_dc(dct_kind_of(S), co_y, dcv);
  for (int k = 0; k < LayoutShape<S>::COVERED; ++k)
    ydq[k] = cast_i16(roundf(__fmul_rn(dcv[k], a.inv_dc_factor[1])));
}

// Y AC round trip (quantize_roundtrip_y_block, src/group.rs:795-820): the
// levels parked in ylev, co_y's AC replaced by the dequantised AC.  The
// round trip's LLF is zero; co_y keeps its LLF coefficients (the Y DC reads
// them) and the chroma-from-luma step reads zero there.
template <int S>
__device__ __forceinline__ void layout_y_roundtrip(const SearchFrame& s, int32_t quant, float* co_y,
                                                   int32_t* ylev) {
  using L = LayoutShape<S>;
  const int lane = threadIdx.x & 31;
  const SearchTables* t = s.t;
  const float* inv_y = inv_of(t, S, 1);
  const float* mat_y = mat_of(t, S, 1);
  const float* thr_y = t->thr[Shape<S>::CLASS][1];
  const float qs_y = __fmul_rn(__fmul_rn(s.scale, static_cast<float>(quant)), 1.0f);
  const float inv_qac = __fdiv_rn(1.0f, __fmul_rn(s.scale, static_cast<float>(quant)));
  for (int i = lane; i < L::SIZE; i += 32) {
    const float val = __fmul_rn(__fmul_rn(inv_y[i], qs_y), co_y[i]);
    const int32_t q = quantize_level(val, layout_threshold(thr_y, i, L::CX, L::CY));
    ylev[i] = q;
    const int width = L::CX * 8, r = i / width, u = i % width;
    if (!(r < L::CY && u < L::CX)) co_y[i] = __fmul_rn(__fmul_rn(bias_level(1, q), mat_y[i]), inv_qac);
  }
}

// chroma from luma on the whole block (src/group.rs:1831-1858), channel c (0 or 2)
template <int S>
__device__ __forceinline__ void layout_cfl(const Frame& f, int bx, int by, int c, float* co_c,
                                           const float* co_y) {
  const int lane = threadIdx.x & 31;
  const int tt = (by >> 3) * f.a.tiles_x + (bx >> 3);
  const float factor = c == 0 ? fmla(static_cast<float>(f.ytox[tt]), 1.0f / 84.0f, 0.0f)
                              : fmla(static_cast<float>(f.ytob[tt]), 1.0f / 84.0f, 1.0f);
  constexpr int CX = LayoutShape<S>::CX, CY = LayoutShape<S>::CY, WIDTH = CX * 8;
  for (int i = lane; i < LayoutShape<S>::SIZE; i += 32) {
    const bool llf = i / WIDTH < CY && i % WIDTH < CX;  // the round trip's zeros
    co_c[i] = fmla(-factor, llf ? 0.0f : co_y[i], co_c[i]);
  }
}

// one covered block's X and B DC levels with the DC chroma-from-luma, and
// its three channels' DC stores
__device__ __forceinline__ void layout_dc_block(const Frame& f, int64_t b, int64_t nb, float xdp,
                                                float bdp, int16_t ydq) {
  const KernelArgs& a = f.a;
  int16_t xq;
  if (a.cfl_dc_factor_x != 0.0f)
    xq = cast_i16(roundf(fmla(xdp, a.inv_dc_factor[0], __fmul_rn(-static_cast<float>(ydq), a.cfl_dc_factor_x))));
  else
    xq = cast_i16(roundf(__fmul_rn(xdp, a.inv_dc_factor[0])));
  const int16_t bq = cast_i16(roundf(fmla(bdp, a.inv_dc_factor[2],
                                          __fmul_rn(-static_cast<float>(ydq), a.cfl_dc_factor_b))));
  f.quant_dc[b] = xq;
  f.quant_dc[nb + b] = ydq;
  f.quant_dc[2 * nb + b] = bq;
}

// X and B DC levels with the DC chroma-from-luma, and the three channels' DC stores
template <int S>
__device__ __forceinline__ void layout_xb_dc(const Frame& f, int bx, int by, const float* co_x,
                                             const float* co_b, const int16_t* ydq) {
  using L = LayoutShape<S>;
  const KernelArgs& a = f.a;
  const int xb = a.xb;
  const int64_t nb = static_cast<int64_t>(xb) * a.yb;
  float xdp[16], bdp[16];
  piece_dc(dct_kind_of(S), co_x, xdp);
  piece_dc(dct_kind_of(S), co_b, bdp);
  for (int iy = 0; iy < L::COVY; ++iy)
    for (int ix = 0; ix < L::COVX; ++ix) {
      const int k = iy * L::COVX + ix;
      layout_dc_block(f, static_cast<int64_t>(by + iy) * xb + bx + ix, nb, xdp[k], bdp[k], ydq[k]);
    }
}

// channel c's levels (Y's from ylev) stored per covered block, its non-zero
// count outside the LLF and its highest non-zero scan position
template <int S>
__device__ __forceinline__ void layout_levels(const Frame& f, const SearchFrame& s, int bx, int by,
                                              int32_t quant, int c, const float* co_c,
                                              const int32_t* ylev, int* nz, uint32_t* last) {
  using L = LayoutShape<S>;
  const int lane = threadIdx.x & 31;
  const int xb = f.a.xb;
  const SearchTables* t = s.t;
  const uint16_t* pos = pos_of(t, S);
  const float* inv = inv_of(t, S, c);
  const float* thr = t->thr[Shape<S>::CLASS][c];
  const float qs = __fmul_rn(__fmul_rn(s.scale, static_cast<float>(quant)), f.a.qm_mul[c]);
  int n = 0;
  uint32_t lst = 0;
  for (int i = lane; i < L::SIZE; i += 32) {
    int32_t q;
    if (c == 1) {
      q = ylev[i];
    } else {
      const float val = __fmul_rn(__fmul_rn(inv[i], qs), co_c[i]);
      q = quantize_level(val, layout_threshold(thr, i, L::CX, L::CY));
    }
    const int chunk = i >> 6;
    const int64_t b = static_cast<int64_t>(by + chunk / L::COVX) * xb + bx + chunk % L::COVX;
    const int64_t at = b * 192 + c * 64 + (i & 63);
    if (q < -32767 || q > 32767) {
      f.levels[at] = kLevelEscape;
      f.wide_levels[at] = q;
    } else {
      f.levels[at] = static_cast<int16_t>(q);
    }
    const int width = L::CX * 8, r = i / width, u = i % width;
    if (q != 0 && !(r < L::CY && u < L::CX)) {
      ++n;
      lst = max(lst, static_cast<uint32_t>(pos[i]));
    }
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    n += __shfl_xor_sync(0xffffffffu, n, d);
    lst = max(lst, __shfl_xor_sync(0xffffffffu, lst, d));
  }
  *nz = n;
  *last = lst;
}

// the shifted non-zero counts of the covered blocks and the token counts at
// the first block ([Y, X, B, 0] per group-local block), by lanes < COVERED
template <int S>
__device__ __forceinline__ void layout_counts(const Frame& f, int bx, int by, const int* nz,
                                              const uint32_t* last) {
  using L = LayoutShape<S>;
  const int lane = threadIdx.x & 31;
  if (lane >= L::COVERED) return;
  const KernelArgs& a = f.a;
  const int xb = a.xb;
  const int64_t nb = static_cast<int64_t>(xb) * a.yb;
  const int ix = lane % L::COVX, iy = lane / L::COVX;
  const int64_t b = static_cast<int64_t>(by + iy) * xb + bx + ix;
  uint32_t packed = 0;
  for (int c = 0; c < 3; ++c) {
    const uint32_t sh = (static_cast<uint32_t>(nz[c]) + L::COVERED - 1u) >> L::LOG2C;
    f.nzeros[c * nb + b] = static_cast<uint8_t>(sh);
    packed |= (sh & 0xffu) << (8 * c);
  }
  f.nz_packed[b] = packed;
  const int gx = (bx + ix) / kGroupBlocks, gy = (by + iy) / kGroupBlocks;
  const int g = gy * a.groups_x + gx;
  const int lb = ((by + iy) % kGroupBlocks) * kGroupBlocks + (bx + ix) % kGroupBlocks;
  uint4 cnt = make_uint4(0u, 0u, 0u, 0u);
  if (lane == 0) {
    auto walk = [&](int c) { return 1u + (nz[c] ? last[c] - L::COVERED + 1u : 0u); };
    cnt = make_uint4(walk(1), walk(0), walk(2), 0u);
  }
  reinterpret_cast<uint4*>(f.counts)[static_cast<int64_t>(g) * 1024 + lb] = cnt;
}

// write_ac_group for one transform, by one warp
template <int S>
__device__ __forceinline__ void layout_piece(const Frame& f, const SearchFrame& s, int bx, int by,
                                             LayoutSmem<S>& sm) {
  const int lane = threadIdx.x & 31;
  for (int c = 0; c < 3; ++c) warp_forward<S>(f, c, bx * 8, by * 8, sm.in, sm.co[c]);
  const int32_t quant = f.qf[by * f.a.xb + bx];
  int16_t ydq[16];
  if (lane == 0) layout_y_dc<S>(f.a, sm.co[1], ydq);
  __syncwarp();
  layout_y_roundtrip<S>(s, quant, sm.co[1], sm.ylev);
  __syncwarp();
  layout_cfl<S>(f, bx, by, 0, sm.co[0], sm.co[1]);
  layout_cfl<S>(f, bx, by, 2, sm.co[2], sm.co[1]);
  __syncwarp();
  if (lane == 0) layout_xb_dc<S>(f, bx, by, sm.co[0], sm.co[2], ydq);
  int nz[3];
  uint32_t last[3];
  for (int c = 0; c < 3; ++c) layout_levels<S>(f, s, bx, by, quant, c, sm.co[c], sm.ylev, &nz[c], &last[c]);
  layout_counts<S>(f, bx, by, nz, last);
  __syncwarp();
}

// The 32x32 transforms: a CTA of three warps each, one per channel: the
// three forward transforms; then the Y round trip beside the Y DC (one
// thread of the X warp: it reads the LLF, which the round trip leaves
// alone); then on each warp its channel's levels, the X and B warps first
// taking chroma-from-luma and their DC (one thread each); then the counts
// beside the 16 blocks' DC stores.
constexpr int kLayout32Threads = 96;
struct Layout32Smem {
  float in[3][32][33];
  int32_t ylev[1024];
  float co[3][1024];
};
__global__ void __launch_bounds__(kLayout32Threads) k_layout32(const __grid_constant__ Frame f) {
  extern __shared__ __align__(16) unsigned char layout_smem_raw[];
  Layout32Smem& sm = *reinterpret_cast<Layout32Smem*>(layout_smem_raw);
  __shared__ int16_t s_ydq[16];
  __shared__ float s_dc[2][16];  // X and B DC of the covered blocks
  __shared__ int s_nz[3];
  __shared__ uint32_t s_last[3];
  constexpr int S = kSt32x32;
  const SearchFrame& s = *static_cast<const SearchFrame*>(f.search);
  const int c = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int bx, by;
  if (!candidate_position<S>(blockIdx.x, f.a.xb, f.a.yb, &bx, &by)) return;
  if (s.map[static_cast<int64_t>(by) * f.a.xb + bx] != static_cast<uint8_t>((S << 1) | 1)) return;
  warp_forward<S>(f, c, bx * 8, by * 8, sm.in[c], sm.co[c]);
  const int32_t quant = f.qf[by * f.a.xb + bx];
  __syncthreads();
  if (c == 1) layout_y_roundtrip<S>(s, quant, sm.co[1], sm.ylev);
  else if (c == 0 && lane == 0) layout_y_dc<S>(f.a, sm.co[1], s_ydq);
  __syncthreads();
  if (c != 1) {
    layout_cfl<S>(f, bx, by, c, sm.co[c], sm.co[1]);
    __syncwarp();
    if (lane == 0) piece_dc(dct_kind_of(S), sm.co[c], s_dc[c >> 1]);
  }
  int n;
  uint32_t lst;
  layout_levels<S>(f, s, bx, by, quant, c, sm.co[c], sm.ylev, &n, &lst);
  if (lane == 0) {
    s_nz[c] = n;
    s_last[c] = lst;
  }
  __syncthreads();
  if (c == 0) {
    layout_counts<S>(f, bx, by, s_nz, s_last);
  } else if (c == 1 && lane < 16) {
    const int64_t b = static_cast<int64_t>(by + lane / 4) * f.a.xb + bx + lane % 4;
    layout_dc_block(f, b, static_cast<int64_t>(f.a.xb) * f.a.yb, s_dc[0][lane], s_dc[1][lane], s_ydq[lane]);
  }
}

// One warp per position a transform of shape S can start at; the warp codes
// the transform placed there, if any.  Every placement the search makes
// starts at such a position (squares at even, 32x32 at 4-aligned blocks,
// pairs at even coordinates along their long side).
template <int S>
__global__ void __launch_bounds__(32 * kMaxTuneWarps) k_layout(const __grid_constant__ Frame f) {
  extern __shared__ __align__(16) unsigned char layout_smem_raw[];
  LayoutSmem<S>& sm = reinterpret_cast<LayoutSmem<S>*>(layout_smem_raw)[threadIdx.x >> 5];
  const SearchFrame& s = *static_cast<const SearchFrame*>(f.search);
  const int64_t cand = static_cast<int64_t>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5);
  int bx, by;
  if (!candidate_position<S>(cand, f.a.xb, f.a.yb, &bx, &by)) return;
  if (s.map[static_cast<int64_t>(by) * f.a.xb + bx] != static_cast<uint8_t>((S << 1) | 1)) return;
  layout_piece<S>(f, s, bx, by, sm);
}

// ---------------------------------------------------------------------------
// Tokens of the layout (src/group.rs:2428-2660)
// ---------------------------------------------------------------------------

// fine_block_context (src/ac_context.rs:62-124) by strategy code
__device__ __forceinline__ uint32_t fine_block_ctx(int c, int st, bool qf_hi) {
  // K_STRATEGY_ORDER of the codes DCT8 0, 16x8 6, 8x16 7, 16x16 4, 32x32 5
  // and K_COMPACT_BLOCK_CONTEXT_MAP's rows (Y, then X / B)
  const int order = st == kStDct ? 0 : st == kSt16x16 ? 2 : st == kSt32x32 ? 3 : 4;
  const int y_row[5] = {0, 1, 2, 2, 3};
  const int xb_row[5] = {7, 8, 9, 9, 10};
  const uint32_t bc = static_cast<uint32_t>(c == 1 ? y_row[order] : xb_row[order]);
  return bc * 2u + (qf_hi ? 1u : 0u);
}

constexpr int kLayoutTokThreads = 256;
// One CTA per chunk of 64 blocks in token order: the chunk's first token by
// the tokenizer's decoupled look-back, then each (transform, channel) walk
// by a warp: the lanes take 32 scan positions at a time; the remaining
// count and the previous flag of every position follow from a ballot of the
// non-zero levels.  Histogram counts go to the frame's table by atomics.
__global__ void __launch_bounds__(kLayoutTokThreads) k_tokenize_layout(
    const __grid_constant__ Frame f, uint2* __restrict__ tokens, const __grid_constant__ TokenScan scan) {
  const int64_t idx = take_chunk(scan);
  const int lc = static_cast<int>(idx);
  const SearchFrame& s = *static_cast<const SearchFrame*>(f.search);
  const KernelArgs& a = f.a;
  const int xb = a.xb;
  const int64_t nb = static_cast<int64_t>(xb) * a.yb;
  const ChunkPlace pl = chunk_place(a, lc);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  __shared__ uint32_t s_off[kTokenChunk + 1];  // each block's first token within the chunk
  __shared__ uint4 s_cnt[kTokenChunk];
  __shared__ unsigned long long s_prefix;
  if (tid < kTokenChunk) {
    uint4 n = make_uint4(0u, 0u, 0u, 0u);
    if (tid < pl.count) {
      const int l = pl.first + tid;
      const int lx = l % pl.gw, ly = l / pl.gw;
      n = reinterpret_cast<const uint4*>(f.counts)[static_cast<int64_t>(pl.g) * 1024 + ly * kGroupBlocks + lx];
    }
    s_cnt[tid] = n;
  }
  __syncthreads();
  if (tid < 32) {
    const uint32_t t0 = s_cnt[2 * tid].x + s_cnt[2 * tid].y + s_cnt[2 * tid].z;
    const uint32_t t1 = s_cnt[2 * tid + 1].x + s_cnt[2 * tid + 1].y + s_cnt[2 * tid + 1].z;
    uint32_t inc = t0 + t1;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t up = __shfl_up_sync(0xffffffffu, inc, d);
      if (tid >= d) inc += up;
    }
    s_off[2 * tid] = inc - t0 - t1;
    s_off[2 * tid + 1] = inc - t1;
    const unsigned long long chunk_total = __shfl_sync(0xffffffffu, inc, 31);
    if (tid == 31) s_off[kTokenChunk] = inc;
    if (tid == 0)
      atomicExch(scan.status + 1 + idx, (idx == 0 ? kLookPrefix : kLookAggregate) | chunk_total);
    const unsigned long long before = idx == 0 ? 0ull : look_back(scan.status, idx, &f.stats->flags);
    if (tid == 0) {
      if (idx != 0) atomicExch(scan.status + 1 + idx, kLookPrefix | (before + chunk_total));
      s_prefix = before;
      if (pl.first == 0) f.group_offsets[pl.g] = before;
      if (idx == scan.chunks - 1) *scan.pass_end = before + chunk_total;
    }
  }
  __syncthreads();
  const uint64_t base = s_prefix;
  uint32_t* __restrict__ hist = f.histograms;
  const uint32_t qf_threshold = f.stats->qf_threshold;
  // work items: (block of the chunk, channel in emission order Y, X, B)
  for (int item = warp; item < 3 * pl.count; item += kLayoutTokThreads / 32) {
    const int blk = item / 3, order = item % 3;
    const int c = order == 0 ? 1 : order == 1 ? 0 : 2;
    const uint4 cnt = s_cnt[blk];
    if (cnt.x == 0u) continue;  // not a first block
    const int l = pl.first + blk;
    const int lx = l % pl.gw, ly = l / pl.gw;
    const int bx = pl.gx * kGroupBlocks + lx, by = pl.gy * kGroupBlocks + ly;
    const int64_t bi = static_cast<int64_t>(by) * xb + bx;
    const int st = s.map[bi] >> 1;
    const int cx = cov_x_of(st), cy = cov_y_of(st);
    const int covered = cx * cy, size = covered * 64;
    const int log2c = covered == 1 ? 0 : covered == 2 ? 1 : covered == 4 ? 2 : 4;
    const uint32_t walk = c == 1 ? cnt.x : c == 0 ? cnt.y : cnt.z;
    uint64_t at = base + s_off[blk] + (c == 1 ? 0u : c == 0 ? cnt.x : cnt.x + cnt.y);
    // the non-zero count and its context from the top and left neighbours
    // (predict_from_top_and_left, src/group.rs:89-106, within the group)
    const uint8_t* nzp = f.nzeros + c * nb;
    uint32_t nzeros = 0;
    const int wcx = st == kStDct ? 1 : 2;  // normalised width in blocks: 8x16 / 16x8 both 2
    const int ncx = st == kSt32x32 ? 4 : wcx, ncy = st == kSt32x32 ? 4 : st == kSt16x16 ? 2 : 1;
    // recount the non-zeros (outside the LLF) from the stored levels
    {
      uint32_t n = 0;
      for (int i = lane; i < size; i += 32) {
        const int chunk = i >> 6;
        const int64_t b = static_cast<int64_t>(by + chunk / cx) * xb + bx + chunk % cx;
        const int16_t v = f.levels[b * 192 + c * 64 + (i & 63)];
        const int width = ncx * 8, r = i / width, u = i % width;
        if (v != 0 && !(r < ncy && u < ncx)) ++n;
      }
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) n += __shfl_xor_sync(0xffffffffu, n, d);
      nzeros = n;
    }
    uint32_t predicted;
    {
      const bool top = ly > 0, left = lx > 0;
      const uint32_t t = top ? nzp[bi - xb] : 0u, lf = left ? nzp[bi - 1] : 0u;
      predicted = !left ? (top ? t : 32u) : !top ? lf : (t + lf + 1u) / 2u;
    }
    const bool qf_hi = static_cast<uint32_t>(f.qf[bi]) > qf_threshold;
    const uint32_t bctx = fine_block_ctx(c, st, qf_hi);
    const uint32_t nzb = predicted < 8u ? predicted : predicted >= 64u ? 36u : 4u + predicted / 2u;
    const uint32_t nz_ctx = nzb * kFineBlockCtxs + bctx;
    const uint32_t histo = kFineBlockCtxs * kNonZeroBuckets + kZeroDensityCtxs * bctx;
    if (lane == 0) {
      tokens[at] = make_uint2(nz_ctx, nzeros);
      atomicAdd(&hist[nz_ctx * kAlphabet + hybrid_token(nzeros)], 1u);
    }
    ++at;
    const uint16_t* scan_t = scan_of(s.t, st);
    const uint32_t npos = walk - 1u;  // walk tokens after the count
    uint32_t before_nz = 0;           // non-zeros at scan positions before this window
    int prev_last = nzeros > static_cast<uint32_t>(size / 16) ? 0 : 1;
    for (uint32_t j0 = 0; j0 < npos; j0 += 32) {
      const uint32_t j = j0 + lane;
      int32_t v = 0;
      if (j < npos) {
        const int k = covered + static_cast<int>(j);
        const int raw = scan_t[k];
        const int chunk = raw >> 6;
        const int64_t b = static_cast<int64_t>(by + chunk / cx) * xb + bx + chunk % cx;
        const int64_t atl = b * 192 + c * 64 + (raw & 63);
        const int16_t lv = f.levels[atl];
        v = lv == kLevelEscape ? f.wide_levels[atl] : lv;
      }
      const unsigned ballot = __ballot_sync(0xffffffffu, v != 0);
      if (j < npos) {
        const int k = covered + static_cast<int>(j);
        const uint32_t left = nzeros - before_nz - __popc(ballot & ((1u << lane) - 1u));
        const int prev = lane == 0 ? prev_last : ((ballot >> (lane - 1)) & 1u);
        uint32_t ctx;
        if (covered == 1) {
          ctx = histo + static_cast<uint32_t>((nonzero_context(static_cast<int>(left)) + freq_context(k)) * 2 + prev);
        } else {
          const int nzq = (static_cast<int>(left) + covered - 1) >> log2c;
          const int kk = k >> log2c;
          ctx = histo + static_cast<uint32_t>((nonzero_context(nzq) + freq_context(kk)) * 2 + prev);
        }
        const uint32_t val = pack_signed(v);
        if (val > kPackedMaxValue) {  // the group keeps the wide token form
          atomicOr(f.group_wide + pl.g, 1u);
          atomicOr(&f.stats->any_wide, 1u);
        }
        tokens[at + j] = make_uint2(ctx, val);
        atomicAdd(&hist[ctx * kAlphabet + hybrid_token(val)], 1u);
      }
      before_nz += __popc(ballot);
      prev_last = (ballot >> 31) & 1u;
    }
    (void)wcx;
  }
}

// OrderStats::tally / tally_block (src/coeff_order.rs:511-540) over a
// frame's pass-one levels, as the tokeniser calls them (src/group.rs:
// 2555-2574): per order slot the transforms (first blocks) it holds, and per
// slot, channel and raw coefficient index the transforms whose level there is
// non-zero, over the whole transform.  `map` is the strategy map of a
// searched frame (null: every block a DCT8); `position_g` maps a raw index to
// its place in a block's stored levels.  A warp takes one block at a time;
// the CTA's counts gather in shared memory, then one global add per non-zero
// counter (integer counts: the order of the adds does not matter).
constexpr int kOrderStatsThreads = 256;
__device__ __forceinline__ int order_slot_of_strategy(int st) {
  // STRATEGY_CODE_LUT (src/dc_group_data.rs:79-81), K_STRATEGY_ORDER
  // (src/ac_context.rs:80-83) and ORDER_SPECS (src/coeff_order.rs:117-125)
  // for the strategies a frame of this build holds
  switch (st) {
    case kStDct: return 0;
    case kSt16x16: return 2;
    case kSt32x32: return 3;
    case kSt16x8:
    case kSt8x16: return 4;
    default: return -1;
  }
}
__device__ __forceinline__ int order_counter_offset(int slot) {
  // 3 x (64, 64, 256, 1024, 128, 256, 512), accumulated
  constexpr int kOffsets[kOrderSlots] = {0, 192, 384, 1152, 4224, 4608, 5376};
  return kOffsets[slot];
}
__global__ void __launch_bounds__(kOrderStatsThreads)
    k_order_stats(const int16_t* __restrict__ levels, const uint8_t* __restrict__ map,
                  const uint8_t* __restrict__ position_g, int xb, int yb,
                  uint32_t* __restrict__ counts, uint32_t* __restrict__ blocks) {
  __shared__ uint32_t s_counts[kOrderCounters];
  __shared__ uint32_t s_blocks[kOrderSlots];
  __shared__ uint8_t position[64];
  for (int i = threadIdx.x; i < kOrderCounters; i += blockDim.x) s_counts[i] = 0u;
  if (threadIdx.x < kOrderSlots) s_blocks[threadIdx.x] = 0u;
  if (threadIdx.x < 64) position[threadIdx.x] = position_g[threadIdx.x];
  __syncthreads();
  const int lane = threadIdx.x & 31, warps = blockDim.x >> 5;
  const int64_t nb = static_cast<int64_t>(xb) * yb;
  for (int64_t b = static_cast<int64_t>(blockIdx.x) * warps + (threadIdx.x >> 5); b < nb;
       b += static_cast<int64_t>(gridDim.x) * warps) {
    const uint8_t cell = map ? map[b] : static_cast<uint8_t>(1);
    if (!(cell & 1)) continue;
    const int st = cell >> 1, slot = order_slot_of_strategy(st);
    if (slot < 0) continue;
    const int bx = static_cast<int>(b % xb), by = static_cast<int>(b / xb);
    const int cx = cov_x_of(st), size = cx * cov_y_of(st) * 64;
    if (lane == 0) atomicAdd(&s_blocks[slot], 1u);
    uint32_t* sc = s_counts + order_counter_offset(slot);
    for (int c = 0; c < 3; ++c)
      for (int i = lane; i < size; i += 32) {
        const int chunk = i >> 6;
        const int64_t blk = static_cast<int64_t>(by + chunk / cx) * xb + bx + chunk % cx;
        if (levels[blk * 192 + c * 64 + position[i & 63]] != 0) atomicAdd(&sc[c * size + i], 1u);
      }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kOrderCounters; i += blockDim.x)
    if (s_counts[i]) atomicAdd(&counts[i], s_counts[i]);
  if (threadIdx.x < kOrderSlots && s_blocks[threadIdx.x]) atomicAdd(&blocks[threadIdx.x], s_blocks[threadIdx.x]);
}

// pixel_chromacity_steps (src/frame/chroma.rs:89-165), its counts: over
// every pixel with a left and an upper neighbour, the X steps reaching
// 0.015 / 0.022 / 0.026, the B - Y steps above 0.28 / 0.33 / 0.38 and the
// strongly exposed blue.  A thread per pixel; each test is counted with a
// ballot, a CTA's counts gather in shared memory, then one global add each
// (integer counts: the order of the adds does not matter).  The steps
// follow from the counts on the host.
constexpr int kChromacityThreads = 256;
__global__ void __launch_bounds__(kChromacityThreads)
    k_pixel_chromacity(const float* __restrict__ xyb, int w, int h, int64_t plane,
                       uint32_t* __restrict__ counts) {
  __shared__ uint32_t s_counts[7];
  if (threadIdx.x < 7) s_counts[threadIdx.x] = 0u;
  __syncthreads();
  const float* X = xyb;
  const float* Y = xyb + plane;
  const float* B = xyb + 2 * plane;
  const int64_t cols = w - 1, total = cols * (h - 1);
  uint32_t mine[7] = {0u, 0u, 0u, 0u, 0u, 0u, 0u};
  // the trip count is the CTA's, so every ballot has the whole warp
  for (int64_t i0 = static_cast<int64_t>(blockIdx.x) * blockDim.x; i0 < total;
       i0 += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t i = i0 + threadIdx.x;
    bool t[7] = {false, false, false, false, false, false, false};
    if (i < total) {
      const int64_t at = (1 + i / cols) * w + 1 + i % cols, left = at - 1, up = at - w;
      const float xv = X[at], yv = Y[at], bv = B[at];
      const float step_x = fmaxf(fabsf(__fsub_rn(xv, X[left])), fabsf(__fsub_rn(xv, X[up])));
      const float diff_b = __fsub_rn(bv, yv);
      const float left_diff = __fsub_rn(B[left], Y[left]), up_diff = __fsub_rn(B[up], Y[up]);
      const float step_b = fmaxf(fabsf(__fsub_rn(diff_b, left_diff)), fabsf(__fsub_rn(diff_b, up_diff)));
      t[0] = step_x >= 0.015f;
      t[1] = step_x >= 0.022f;
      t[2] = step_x >= 0.026f;
      t[3] = step_b > 0.28f;
      t[4] = step_b > 0.33f;
      t[5] = step_b > 0.38f;
      const float step = __fadd_rn(fabsf(__fsub_rn(bv, B[left])), fabsf(__fsub_rn(bv, B[up])));
      t[6] = __fmul_rn(__fsub_rn(bv, __fmul_rn(yv, 1.2f)), step) >= 0.13f;
    }
#pragma unroll
    for (int k = 0; k < 7; ++k) mine[k] += __popc(__ballot_sync(0xffffffffu, t[k]));
  }
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int k = 0; k < 7; ++k)
      if (mine[k]) atomicAdd(&s_counts[k], mine[k]);
  __syncthreads();
  if (threadIdx.x < 7 && s_counts[threadIdx.x]) atomicAdd(&counts[threadIdx.x], s_counts[threadIdx.x]);
}

// apply_chroma_hf_protection (src/adaptive_quant.rs:303-402) with
// chroma_hf_stats_scalar (:222-279): a thread per 8x8 block (cut at the
// image edge) sums the opponent magnitude, then the chroma and luma
// gradients of the horizontal and the vertical neighbour pairs, in the
// reference's order; a block whose edges are mostly chromatic has its field
// value raised by the fitted gain.  `strength` is the distance's fade
// (positive; the host skips the launch otherwise).
__global__ void __launch_bounds__(128)
    k_chroma_hf_protection(const float* __restrict__ xyb, int w, int h, int64_t plane, int xb, int yb,
                           float strength, uint8_t* __restrict__ field) {
  const int64_t blk = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (blk >= static_cast<int64_t>(xb) * yb) return;
  const int bx = static_cast<int>(blk % xb), by = static_cast<int>(blk / xb);
  const int px = bx * 8, py = by * 8, bw = imin(8, w - px), bh = imin(8, h - py);
  const float* X = xyb;
  const float* Y = xyb + plane;
  const float* B = xyb + 2 * plane;
  float chroma_sum = 0.0f, chroma_grad = 0.0f, luma_grad = 0.0f;
  int edges = 0;
  for (int y = py; y < py + bh; ++y)
    for (int x = px; x < px + bw; ++x) {
      const int64_t i = static_cast<int64_t>(y) * w + x;
      chroma_sum = __fadd_rn(chroma_sum, __fadd_rn(fabsf(X[i]), fabsf(__fsub_rn(B[i], Y[i]))));
    }
  auto pair = [&](int64_t i, int64_t j) {
    const float dx = fabsf(__fsub_rn(X[j], X[i]));
    const float db = fabsf(__fsub_rn(__fsub_rn(B[j], Y[j]), __fsub_rn(B[i], Y[i])));
    chroma_grad = __fadd_rn(chroma_grad, __fadd_rn(dx, db));
    luma_grad = __fadd_rn(luma_grad, fabsf(__fsub_rn(Y[j], Y[i])));
  };
  if (bw > 1) {
    for (int y = py; y < py + bh; ++y)
      for (int x = px; x + 1 < px + bw; ++x) {
        const int64_t i = static_cast<int64_t>(y) * w + x;
        pair(i, i + 1);
      }
    edges += (bw - 1) * bh;
  }
  if (bh > 1) {
    for (int y = py; y + 1 < py + bh; ++y)
      for (int x = px; x < px + bw; ++x) {
        const int64_t i = static_cast<int64_t>(y) * w + x;
        pair(i, i + w);
      }
    edges += bw * (bh - 1);
  }
  if (edges == 0) return;
  auto unit = [](float v) { return v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v); };
  const float mean_chroma = __fdiv_rn(chroma_sum, static_cast<float>(bw * bh));
  const float mean_gradient = __fdiv_rn(chroma_grad, static_cast<float>(edges));
  const float chroma_share = __fdiv_rn(chroma_grad, __fadd_rn(__fadd_rn(chroma_grad, luma_grad), 1e-4f));
  const float chroma_w = unit(__fdiv_rn(__fsub_rn(mean_chroma, 0.025f), 0.075f));
  const float gradient_w = unit(__fdiv_rn(__fsub_rn(mean_gradient, 0.006f), 0.030f));
  const float share_w = unit(__fdiv_rn(__fsub_rn(chroma_share, 0.25f), 0.55f));
  const float risk = __fmul_rn(__fmul_rn(chroma_w, gradient_w), share_w);
  if (!(risk > 0.0f)) return;
  const float ceiling = fmla(1.4f, __fmul_rn(share_w, share_w), 0.35f);
  const float gain = fmla(__fmul_rn(ceiling, strength), risk, 1.0f);
  const float q = static_cast<float>(field[blk]);
  const float r = roundf(__fmul_rn(q, gain));
  field[blk] = static_cast<uint8_t>(r < 1.0f ? 1.0f : (r > 255.0f ? 255.0f : r));
}

// Dynamic shared memory above the 48 KB default for the search kernels.
inline cudaError_t set_search_attributes() {
  cudaError_t e = cudaSuccess;
  auto set = [&](const void* fn, size_t bytes) {
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
  };
  set(reinterpret_cast<const void*>(k_cost<kStDct>), kMaxTuneWarps * sizeof(CostSmem<kStDct>));
  set(reinterpret_cast<const void*>(k_cost<kSt16x8>), kMaxTuneWarps * sizeof(CostSmem<kSt16x8>));
  set(reinterpret_cast<const void*>(k_cost<kSt8x16>), kMaxTuneWarps * sizeof(CostSmem<kSt8x16>));
  set(reinterpret_cast<const void*>(k_cost<kSt16x16>), kMaxTuneWarps * sizeof(CostSmem<kSt16x16>));
  set(reinterpret_cast<const void*>(k_cost32), sizeof(Cost32Smem));
  set(reinterpret_cast<const void*>(k_mh_incumbent), 4 * sizeof(CostSmem<kSt32x32>));
  set(reinterpret_cast<const void*>(k_layout<kStDct>), kMaxTuneWarps * sizeof(LayoutSmem<kStDct>));
  set(reinterpret_cast<const void*>(k_layout<kSt16x8>), kMaxTuneWarps * sizeof(LayoutSmem<kSt16x8>));
  set(reinterpret_cast<const void*>(k_layout<kSt8x16>), kMaxTuneWarps * sizeof(LayoutSmem<kSt8x16>));
  set(reinterpret_cast<const void*>(k_layout<kSt16x16>), kMaxTuneWarps * sizeof(LayoutSmem<kSt16x16>));
  set(reinterpret_cast<const void*>(k_layout32), sizeof(Layout32Smem));
  set(reinterpret_cast<const void*>(k_retile), kMaxTuneWarps * sizeof(RetileSmem));
  set(reinterpret_cast<const void*>(k_site), kMaxTuneWarps * sizeof(SiteSmem));
  return e;
}

}  // namespace jxg
