// Speed::Fastest on the device: the AC strategy search and the coding of the
// transforms it places (DCT8, DCT16X8, DCT8X16, DCT16X16, DCT32X32).
//
// Stages of one frame (each a launch over independent work units):
//   k_cost<S>          one warp per candidate transform S: gather, forward
//                      transform, chroma-from-luma, the coefficient-model
//                      rate/distortion cost (strategy_cost, src/ac_strategy.rs:724,
//                      :1295-1378; channel_rd / sse_and_rate / model_bits,
//                      src/inflated_cost.rs:435-547) at the quantizer each
//                      consumer prices it with, plus the per-site merge bias
//                      (site_bias, src/ac_strategy.rs:210-268);
//   k_select           one thread per 4x4-block cell: select_band /
//                      select_super_block in the squares scope
//                      (src/ac_strategy/selection.rs:238-475, :1000-1245);
//   k_retile           one thread per 8x8-block tile: retile_coefficient's
//                      exact broken-profile DP (src/ac_strategy/selection/
//                      layout_dp.rs:1811-2198);
//   k_adjust           adjust_quant_field (selection.rs:503-527) and the
//                      alpha factors over the layout (src/adaptive_quant.rs:1036);
//   k_mh_incumbent / k_mh_choose   account_matrix_headers
//                      (src/ac_strategy/matrix_overhead.rs:117-268) where the
//                      16x16 / 32x32 tables are custom (d >= 2.25);
//   k_qf_median        ac_qf_threshold over the final field;
//   k_layout_tile      write_ac_group for every transform (src/group.rs:1259-2426);
//   k_tokenize_layout  the tokens and histograms (src/group.rs:2428-2660).
// Every float operation keeps the reference's order: per-coefficient terms
// are computed in parallel, and each running sum the reference keeps is
// summed by one lane in the reference's order.
#pragma once

namespace jxg {

constexpr float kRdLambda = 0.08086717f;
constexpr float kMetaR = 4.0f;

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
  uint32_t* sites;      // matrix-header sites in DC-group order
  double* mh_loss;      // per site: the DCT and 16x16 alternatives' losses
};

// ---------------------------------------------------------------------------
// Cost of one candidate, by one warp
// ---------------------------------------------------------------------------

template <int S>
struct CostSmem {
  static constexpr int W = Shape<S>::W, H = Shape<S>::H, SIZE = W * H;
  float in[3][H][W + 1];  // gathered pixels; then the sse terms
  float co[3][SIZE];      // coefficients
  float mag[3][SIZE];     // magnitude-rate terms
};

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

// The three channels' coefficients with chroma-from-luma applied
// (prepare_strategy_coeffs, src/ac_strategy.rs:1380-1407).
template <int S>
__device__ __forceinline__ void warp_coefficients(const Frame& f, int bx, int by, CostSmem<S>& sm) {
  constexpr int SIZE = Shape<S>::W * Shape<S>::H;
  const int lane = threadIdx.x & 31;
  for (int c = 0; c < 3; ++c) warp_forward<S>(f, c, bx * 8, by * 8, sm.in[c], sm.co[c]);
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
template <int S>
__device__ __forceinline__ float warp_selection_scale(const SearchFrame& s, const CostSmem<S>& sm,
                                                      float qac) {
  if (S != kSt32x32 || !s.p.sel_scale) return 1.0f;
  const int lane = threadIdx.x & 31;
  float out = 1.0f;
  if (lane == 0) {
    const float* inv = s.t->inv32[1];
    double energy = 0.0;
    for (int y = 0; y < 32; ++y)
      for (int x = 0; x < 32; ++x) {
        if (x < 8 && y < 8) continue;
        const int i = y * 32 + x;
        const float l = sm.co[1][i];
        if (fabsf(__fmul_rn(__fmul_rn(l, inv[i]), qac)) < 0.5f)
          energy = __dadd_rn(energy, __dmul_rn(static_cast<double>(l), static_cast<double>(l)));
      }
    const float erased = static_cast<float>(energy);
    const float d = s.distance;
    const float r = __fsub_rn(__fdiv_rn(erased, __fmul_rn(__fmul_rn(2e-4f, d), d)), 1.0f);
    out = __fadd_rn(1.0f, __fmul_rn(0.6f, fminf(fmaxf(r, 0.0f), 1.0f)));
  }
  return __shfl_sync(0xffffffffu, out, 0);
}

// The coefficient-model cost at quantizer `q` (already scaled by the
// selection quantizer) of the coefficients in `sm`; every lane returns it.
template <int S>
__device__ __forceinline__ float warp_rd(const Frame& f, const SearchFrame& s, CostSmem<S>& sm,
                                         int bx, int by, float q, float meta_r) {
  constexpr int CX = Shape<S>::CX, CY = Shape<S>::CY, WIDTH = CX * 8, HEIGHT = CY * 8;
  constexpr int SIZE = WIDTH * HEIGHT;
  const int lane = threadIdx.x & 31;
  const SearchTables* t = s.t;
  const uint16_t* pos = pos_of(t, S);
  float* sse_terms = &sm.in[0][0][0];  // the gather buffer is free again
  int nz[3];
  uint32_t max_scan[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float* inv = inv_of(t, S, c);
    const float* thr = t->thr[Shape<S>::CLASS][c];
    const float q_scaled = __fmul_rn(q, s.qm_mult[c]);
    int n = 0;
    uint32_t ms = 0;
    for (int i = lane; i < SIZE; i += 32) {
      const int y = i / WIDTH, x = i % WIDTH;
      float e2 = 0.0f, mag = 0.0f;
      if (!(x < CX && y < CY)) {
        const int yfix = y >= HEIGHT / 2 ? 2 : 0;
        const float threshold = x >= WIDTH / 2 ? thr[yfix + 1] : thr[yfix];
        const float a = __fmul_rn(__fmul_rn(inv[i], q_scaled), sm.co[c][i]);
        const float qv = fabsf(a) >= threshold ? roundf(a) : 0.0f;
        const float e = __fsub_rn(a, bias_level(c, cast_i32(qv)));
        e2 = __fmul_rn(e, e);
        if (qv != 0.0f) {
          ++n;
          mag = rate_log2(s.rate_log2, fabsf(qv));
          ms = max(ms, static_cast<uint32_t>(pos[i]));
        }
      }
      sse_terms[c * SIZE + i] = e2;
      sm.mag[c][i] = mag;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      n += __shfl_xor_sync(0xffffffffu, n, d);
      ms = max(ms, __shfl_xor_sync(0xffffffffu, ms, d));
    }
    nz[c] = n;
    max_scan[c] = ms;
  }
  __syncwarp();
  // the reference's running sums, each in raster order by one lane (a
  // skipped coefficient adds +0, which leaves a sum of non-negative terms as it is)
  float sum = 0.0f;
  if (lane < 6) {
    const float* terms = lane < 3 ? sse_terms + lane * SIZE : sm.mag[lane - 3];
    for (int i = 0; i < SIZE; ++i) sum = __fadd_rn(sum, terms[i]);
  }
  float sse[3], mag[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    sse[c] = __shfl_sync(0xffffffffu, sum, c);
    mag[c] = __shfl_sync(0xffffffffu, sum, 3 + c);
  }
  __syncwarp();
  const float weights[3] = {0.30f, 1.0f, 0.28f};
  float d_total = 0.0f, r_total = 0.0f;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    // model_bits (src/inflated_cost.rs:540-547)
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
  // Footprint::visible_fraction (src/inflated_cost.rs:650-659)
  const int px = bx * 8, py = by * 8;
  const int vw = imin(Shape<S>::W, imax(f.a.width - px, 0));
  const int vh = imin(Shape<S>::H, imax(f.a.height - py, 0));
  const float visible = (vw == Shape<S>::W && vh == Shape<S>::H)
                            ? 1.0f
                            : __fdiv_rn(static_cast<float>(vw * vh),
                                        static_cast<float>(Shape<S>::W * Shape<S>::H));
  return fmla(kRdLambda, __fadd_rn(r_total, meta_r), __fmul_rn(d_total, visible));
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
// The warp stages the site's luma (clipped to the image) in `stage` (n * n
// floats); lane 0 then takes the f64 sums in raster order.
__device__ __forceinline__ float site_bias(const Frame& f, const SearchFrame& s, int x0, int y0,
                                           int n, float* stage) {
  if (s.p.site_k == 0.0f) return 1.0f;
  const int lane = threadIdx.x & 31;
  const float* yp = f.xyb + f.a.plane;
  const int w = f.a.width, h = f.a.height;
  const int y1 = imin(y0 + n, h), x1 = imin(x0 + n, w);
  const int vw = x1 - x0, vh = y1 - y0;
  for (int k = lane; k < vw * vh; k += 32)
    stage[k] = __ldg(yp + static_cast<int64_t>(y0 + k / vw) * w + x0 + k % vw);
  __syncwarp();
  float out = 1.0f;
  if (lane == 0) {
    double s1 = 0.0, s2 = 0.0;
    const int cnt = vw * vh;
#pragma unroll 8
    for (int k = 0; k < cnt; ++k) {
      const double v = static_cast<double>(stage[k]);
      s1 = __dadd_rn(s1, v);
      s2 = __dadd_rn(s2, __dmul_rn(v, v));
    }
    float var = 0.0f;
    if (cnt) {
      const double mean = __ddiv_rn(s1, static_cast<double>(cnt));
      const double vv = __dsub_rn(__ddiv_rn(s2, static_cast<double>(cnt)), __dmul_rn(mean, mean));
      var = static_cast<float>(vv > 0.0 ? vv : 0.0);
    }
    var = fmaxf(var, 1e-9f);
    const float sv = fminf(fmaxf(__fdiv_rn(dirty_log2f(__fdiv_rn(var, 0.003f)), 8.0f), -1.0f), 1.0f);
    out = util_fast_exp(__fmul_rn(s.p.site_k, sv));
  }
  __syncwarp();
  return __shfl_sync(0xffffffffu, out, 0);
}

// One warp per candidate of shape S: the costs every consumer of it reads.
//   DCT8     every block, at scale * q (select_super_block's c8, the DP's leaves)
//   16x16    even (bx, by): at aggregate_qac_2x2 (selection) and at region_qac
//            (the DP's squares, the matrix-header alternatives), the site bias
//   8x16     even bx (the DP's horizontal pairs), 16x8 even by (vertical pairs)
//   32x32    4-aligned: at region_qac with the selection quantizer, site bias
template <int S>
__global__ void __launch_bounds__(128) k_cost(const __grid_constant__ Frame f) {
  extern __shared__ __align__(16) unsigned char cost_smem_raw[];
  CostSmem<S>& sm = reinterpret_cast<CostSmem<S>*>(cost_smem_raw)[threadIdx.x >> 5];
  const SearchFrame& s = *static_cast<const SearchFrame*>(f.search);
  const int lane = threadIdx.x & 31;
  const int xb = f.a.xb, yb = f.a.yb;
  const int64_t cand = static_cast<int64_t>(blockIdx.x) * 4 + (threadIdx.x >> 5);
  int bx, by;
  if (S == kStDct) {
    if (cand >= static_cast<int64_t>(xb) * yb) return;
    bx = static_cast<int>(cand % xb), by = static_cast<int>(cand / xb);
  } else if (S == kSt8x16) {
    const int nx = xb / 2;
    if (nx == 0 || cand >= static_cast<int64_t>(nx) * yb) return;
    bx = 2 * static_cast<int>(cand % nx), by = static_cast<int>(cand / nx);
  } else if (S == kSt16x8) {
    const int ny = yb / 2;
    if (ny == 0 || cand >= static_cast<int64_t>(xb) * ny) return;
    bx = static_cast<int>(cand % xb), by = 2 * static_cast<int>(cand / xb);
  } else if (S == kSt16x16) {
    const int nx = xb / 2, ny = yb / 2;
    if (nx == 0 || cand >= static_cast<int64_t>(nx) * ny) return;
    bx = 2 * static_cast<int>(cand % nx), by = 2 * static_cast<int>(cand / nx);
  } else {
    const int nx = xb / 4, ny = yb / 4;
    if (nx == 0 || cand >= static_cast<int64_t>(nx) * ny) return;
    bx = 4 * static_cast<int>(cand % nx), by = 4 * static_cast<int>(cand / nx);
  }
  const int bi = by * xb + bx;
  const uint8_t* qf = f.qf;  // the pre-selection field
  float m_site = 1.0f;
  if (S == kSt16x16 || S == kSt32x32) m_site = site_bias(f, s, bx * 8, by * 8, Shape<S>::W, sm.mag[0]);
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
      s.m16[bi] = m_site;
    }
  } else if (S == kSt32x32) {
    const float qac = __fmul_rn(s.scale,
                                static_cast<float>(region_quant(qf, xb, bx, by, 4, 4, s.distance)));
    const float q = __fmul_rn(qac, warp_selection_scale<S>(s, sm, qac));
    const float c = warp_rd<S>(f, s, sm, bx, by, q, kMetaR);
    if (lane == 0) {
      s.c32[bi] = c;
      s.m32[bi] = m_site;
    }
  } else {
    constexpr int w = Shape<S>::COVX, h = Shape<S>::COVY;
    const float qac = __fmul_rn(s.scale,
                                static_cast<float>(region_quant(qf, xb, bx, by, w, h, s.distance)));
    const float c = warp_rd<S>(f, s, sm, bx, by, qac, kMetaR);
    if (lane == 0) (S == kSt8x16 ? s.cw : s.ct)[bi] = c;
  }
}

template <int S>
constexpr size_t cost_smem_bytes() { return 4 * sizeof(CostSmem<S>); }

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
// layout_dp.rs:1864-2198), one thread per tile.
constexpr int kSmallLeaf = 1, kSmallWide = 2, kSmallTall = 3, kSmallSquare = 4;
__device__ __forceinline__ int small_strategy(int choice) {
  return choice == kSmallLeaf ? kStDct : choice == kSmallWide ? kSt8x16
         : choice == kSmallTall ? kSt16x8 : kSt16x16;
}

struct SmallPlan {
  int n;
  uint8_t cell[64], choice[64];
};

// The DP's state of one thread: two layers of costs and active lists, in
// shared memory.
struct SmallState {
  float cost_a[512], cost_b[512];
  uint16_t act_a[512], act_b[512];
};
constexpr int kRetileThreads = 16;
constexpr size_t kRetileSmemBytes = kRetileThreads * sizeof(SmallState);

__device__ float plan_small(const float* leaf, const float* wide, const float* tall,
                            const float* square, const uint8_t* live, uint64_t fixed, int w,
                            int h, uint8_t* choices, float replace_below, SmallPlan* plan,
                            SmallState& st) {
  const int cells = w * h, states = 1 << (w + 1), mask = states - 1;
  const int below_bit = 1 << w;
  const int added[5] = {0, 0, 2, below_bit, 2 | below_bit | (2 << w)};
  float* cost_a = st.cost_a;
  float* cost_b = st.cost_b;
  uint16_t* act_a = st.act_a;
  uint16_t* act_b = st.act_b;
  for (int i = 0; i < states; ++i) cost_a[i] = cost_b[i] = INFINITY;
  float* cost = cost_a;
  float* next = cost_b;
  uint16_t* active = act_a;
  uint16_t* next_active = act_b;
  const int start = static_cast<int>(fixed & static_cast<uint64_t>(mask));
  cost[start] = 0.0f;
  active[0] = static_cast<uint16_t>(start);
  int active_len = 1;
  uint64_t incoming = fixed >> (w + 1);
  for (int i = 0; i < cells; ++i) {
    uint8_t* from = choices + i * states;
    const int corner = static_cast<int>(incoming & 1u) << w;
    incoming >>= 1;
    const int shapes = live[i];
    int next_len = 0;
    for (int a = 0; a < active_len; ++a) {
      const int state = active[a];
      const float here = cost[state];
      cost[state] = INFINITY;
      auto relax = [&](int filled, float cv, int ch) {
        const int to = ((filled >> 1) | corner) & mask;
        if (cv < next[to]) {
          if (next[to] == INFINITY) next_active[next_len++] = static_cast<uint16_t>(to);
          next[to] = cv;
          from[to] = static_cast<uint8_t>(ch);
        }
      };
      if (state & 1) {
        relax(state, here, 0);
        continue;
      }
      relax(state, __fadd_rn(here, leaf[i]), kSmallLeaf);
      const bool right = (state & 2) == 0, below = (state & below_bit) == 0;
      if (right && (shapes & 1)) relax(state | 2, __fadd_rn(here, wide[i]), kSmallWide);
      if (below && (shapes & 2)) relax(state | below_bit, __fadd_rn(here, tall[i]), kSmallTall);
      if (right && below && corner == 0 && (shapes & 4))
        relax(state | added[kSmallSquare], __fadd_rn(here, square[i]), kSmallSquare);
    }
    float* tc = cost;
    cost = next;
    next = tc;
    uint16_t* ta = active;
    active = next_active;
    next_active = ta;
    active_len = next_len;
  }
  const float total = cost[0];
  if (!(isfinite(total) && total < replace_below)) return total;
  plan->n = 0;
  int state = 0;
  for (int i = cells - 1; i >= 0; --i) {
    const int choice = choices[i * states + state];
    if (choice != 0) {
      plan->cell[plan->n] = static_cast<uint8_t>(i);
      plan->choice[plan->n] = static_cast<uint8_t>(choice);
      ++plan->n;
    }
    state = (((state << 1) ^ added[choice]) & mask) | (choice == 0 ? 1 : 0);
  }
  return total;
}

struct Piece {
  int8_t x, y, s;
};

__device__ __forceinline__ bool piece_in(const Piece* set, int n, Piece p) {
  for (int i = 0; i < n; ++i)
    if (set[i].x == p.x && set[i].y == p.y && set[i].s == p.s) return true;
  return false;
}

__global__ void __launch_bounds__(kRetileThreads) k_retile(const __grid_constant__ Frame f) {
  extern __shared__ __align__(16) unsigned char retile_smem_raw[];
  SmallState& dp = reinterpret_cast<SmallState*>(retile_smem_raw)[threadIdx.x];
  const SearchFrame& s = *static_cast<const SearchFrame*>(f.search);
  const int xb = f.a.xb, yb = f.a.yb;
  const int tx = (xb + 7) / 8, ty = (yb + 7) / 8;
  const int tile = blockIdx.x * blockDim.x + threadIdx.x;
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
  Piece current[64];
  int ncur = 0;
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const uint8_t cell = map[(by + y) * xb + bx + x];
      if (cell & 1) current[ncur++] = Piece{static_cast<int8_t>(x), static_cast<int8_t>(y), static_cast<int8_t>(cell >> 1)};
    }
  float leaf[64], wide[64], tall[64], square[64];
  for (int i = 0; i < 64; ++i) leaf[i] = wide[i] = tall[i] = square[i] = INFINITY;
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const int i = y * w + x;
      const int gx = bx + x, gy = by + y;
      leaf[i] = score(Piece{static_cast<int8_t>(x), static_cast<int8_t>(y), kStDct});
      if (x + 2 <= w && gx % 2 == 0 && can_place(xb, yb, gx, gy, kSt8x16))
        wide[i] = score(Piece{static_cast<int8_t>(x), static_cast<int8_t>(y), kSt8x16});
      if (y + 2 <= h && gy % 2 == 0 && can_place(xb, yb, gx, gy, kSt16x8))
        tall[i] = score(Piece{static_cast<int8_t>(x), static_cast<int8_t>(y), kSt16x8});
      if (x + 2 <= w && y + 2 <= h && gx % 2 == 0 && gy % 2 == 0 && can_place(xb, yb, gx, gy, kSt16x16))
        square[i] = score(Piece{static_cast<int8_t>(x), static_cast<int8_t>(y), kSt16x16});
    }
  uint64_t fixed = 0;
  float fixed_cost = 0.0f;
  for (int k = 0; k < ncur; ++k) {
    if (current[k].s <= kSt16x16) continue;
    const Piece p = current[k];
    const uint64_t row = (1ull << cov_x_of(p.s)) - 1ull;
    for (int yy = 0; yy < cov_y_of(p.s); ++yy) fixed |= row << (p.y * w + p.x + yy * w);
    fixed_cost = __fadd_rn(fixed_cost, score(p));
  }
  // SmallCosts::live_masks
  uint8_t live[64];
  for (int i = 0; i < 64; ++i) live[i] = 0;
  for (int y = 0; y < h; ++y) {
    const int st = y * w;
    if (y + 1 == h) {
      for (int x = 0; x + 1 < w; ++x) live[st + x] = wide[st + x] < __fadd_rn(leaf[st + x], leaf[st + x + 1]);
      continue;
    }
    const int bl = st + w;
    for (int x = 0; x + 1 < w; ++x) {
      const float tl = leaf[st + x], tr = leaf[st + x + 1], bll = leaf[bl + x], brr = leaf[bl + x + 1];
      const float top_leaves = __fadd_rn(tl, tr);
      const float leaves = __fadd_rn(__fadd_rn(top_leaves, bll), brr);
      const float wides = __fadd_rn(wide[st + x], wide[bl + x]);
      const float talls = __fadd_rn(tall[st + x], tall[st + x + 1]);
      live[st + x] = static_cast<uint8_t>((wide[st + x] < top_leaves ? 1 : 0) |
                                          (tall[st + x] < __fadd_rn(tl, bll) ? 2 : 0) |
                                          (square[st + x] < fminf(fminf(leaves, wides), talls) ? 4 : 0));
    }
    live[st + w - 1] = tall[st + w - 1] < __fadd_rn(leaf[st + w - 1], leaf[bl + w - 1]) ? 2 : 0;
  }
  uint8_t* choices = s.dp_choices + static_cast<int64_t>(tile) * 64 * 512;
  SmallPlan plan;
  plan.n = 0;
  const float around = __fadd_rn(plan_small(leaf, wide, tall, square, live, fixed, w, h, choices,
                                            INFINITY, &plan, dp),
                                 fixed_cost);
  bool keep_fixed = true;
  float winner = around;
  if (fixed != 0) {
    const float over = plan_small(leaf, wide, tall, square, live, 0, w, h, choices, around, &plan, dp);
    if (over < around) {
      winner = over;
      keep_fixed = false;
    }
  }
  if (!isfinite(winner)) return;
  Piece layout[64];
  int nl = 0;
  for (int k = 0; k < plan.n; ++k) {
    const int i = plan.cell[k];
    layout[nl++] = Piece{static_cast<int8_t>(i % w), static_cast<int8_t>(i / w),
                         static_cast<int8_t>(small_strategy(plan.choice[k]))};
  }
  if (keep_fixed)
    for (int k = 0; k < ncur; ++k)
      if (current[k].s > kSt16x16) layout[nl++] = current[k];
  // sort by (y, x, strategy): insertion sort over at most 64 pieces
  for (int i = 1; i < nl; ++i) {
    const Piece p = layout[i];
    int j = i - 1;
    while (j >= 0 && (layout[j].y > p.y || (layout[j].y == p.y && (layout[j].x > p.x ||
                                             (layout[j].x == p.x && layout[j].s > p.s))))) {
      layout[j + 1] = layout[j];
      --j;
    }
    layout[j + 1] = p;
  }
  float old_cost = 0.0f, new_cost = 0.0f;
  for (int k = 0; k < ncur; ++k)
    if (!piece_in(layout, nl, current[k])) old_cost = __fadd_rn(old_cost, score(current[k]));
  for (int k = 0; k < nl; ++k)
    if (!piece_in(current, ncur, layout[k])) new_cost = __fadd_rn(new_cost, score(layout[k]));
  if (new_cost < old_cost)
    for (int k = 0; k < nl; ++k)
      if (!piece_in(current, ncur, layout[k]))
        map_set_first(map, xb, bx + layout[k].x, by + layout[k].y, layout[k].s);
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

__device__ __forceinline__ uint32_t header_bits(const SearchFrame& s, uint32_t used) {
  uint32_t payload = 0;
  for (int i = 0; i < 13; ++i)
    if (used & (1u << i)) payload += s.p.payload[i];
  return 1u + payload + (payload != 0u ? 17u * 3u : 0u);
}

constexpr int kMhThreads = 1024;
// One CTA: the sites in DC-group order, as two lists (16x16 sites, then
// 32x32 sites: the order in which the reference sums its regions), each
// site's alternatives, the families a lower bound pins, the cheapest table
// set (every subset's sum over the sites in order; losses are non-negative,
// so the reference's early exit never changes which set wins), and the
// chosen alternatives.
__global__ void __launch_bounds__(kMhThreads) k_mh_choose(const __grid_constant__ Frame f) {
  const SearchFrame& s = *static_cast<const SearchFrame*>(f.search);
  const int xb = f.a.xb, yb = f.a.yb;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  __shared__ uint32_t s_used, s_n[2], s_warp[2][32];
  __shared__ double s_unavoidable[2];
  __shared__ uint32_t s_pinned, s_best;
  __shared__ double s_subset_cost[64];
  if (tid == 0) {
    s_used = 0;
    s_n[0] = s_n[1] = 0;
  }
  __syncthreads();
  const int xdc = (xb + 255) / 256, ydc = (yb + 255) / 256;
  uint32_t used_local = 0;
  const int64_t nb = static_cast<int64_t>(xb) * yb;
  uint32_t* list16 = s.sites;
  uint32_t* list32 = s.sites + nb / 2;
  // enumerate blocks in DC-group order, raster within each DC group
  for (int64_t base = 0; base < nb; base += kMhThreads) {
    const int64_t k = base + tid;
    int fam = -1;
    int b = -1;
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
      if (cell & 1) {
        const int st = cell >> 1;
        const uint32_t slot = st == kStDct ? 0u : st == kSt16x16 ? 1u : st == kSt32x32 ? 2u : 3u;
        if (s.p.custom & (1u << slot)) {
          used_local |= 1u << slot;
          if (slot == 1u || slot == 2u) fam = static_cast<int>(slot) - 1;
        }
      }
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
  atomicOr(&s_used, used_local);
  __syncthreads();
  const uint32_t used = s_used, n16 = s_n[0], n32 = s_n[1], count = n16 + n32;
  if ((used & ~1u) == 0u) return;
  const double lambda = static_cast<double>(kRdLambda);
  // every site's losses, family-major: the DCT alternative's and (32x32)
  // the 16x16 alternative's, -1 where the alternative is absent
  double* loss = s.mh_loss;
  for (uint32_t k = tid; k < count; k += kMhThreads) {
    const uint32_t b = k < n16 ? list16[k] : list32[k - n16];
    const int st = k < n16 ? kSt16x16 : kSt32x32, cx = cov_x_of(st), cy = cov_y_of(st);
    const double inc = static_cast<double>(s.mh_inc[b]) / lambda;
    double c = 0.0;
    for (int iy = 0; iy < cy; ++iy)
      for (int ix = 0; ix < cx; ++ix)
        c = __dadd_rn(c, static_cast<double>(s.c8[b + iy * xb + ix]) / lambda);
    loss[2 * k] = (isfinite(c) && isfinite(inc)) ? fmax(c - inc, 0.0) : -1.0;
    double l16 = -1.0;
    if (st == kSt32x32) {
      double c2 = 0.0;
      for (int iy = 0; iy < 4; iy += 2)
        for (int ix = 0; ix < 4; ix += 2)
          c2 = __dadd_rn(c2, static_cast<double>(s.c16r[b + iy * xb + ix]) / lambda);
      l16 = (isfinite(c2) && isfinite(inc)) ? fmax(c2 - inc, 0.0) : -1.0;
    }
    loss[2 * k + 1] = l16;
  }
  __syncthreads();
  // the families' unavoidable losses in site order (thread 0: 16x16, 32: 32x32)
  if (tid == 0 || tid == 32) {
    const uint32_t lo = tid == 0 ? 0u : n16, hi = tid == 0 ? n16 : count;
    double u = 0.0;
#pragma unroll 8
    for (uint32_t k = lo; k < hi; ++k) {
      const double ld = loss[2 * k], l16 = loss[2 * k + 1];
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
  const uint32_t pinned = s_pinned, custom = s.p.custom;
  // best_alternative (matrix_overhead.rs:50-63) of site k under `allowed`:
  // incumbent (requires its own slot), DCT (slot 0 when custom), 16x16
  // (slot 1 when custom); strict `<` keeps the earlier one on a tie
  auto best_of = [&](uint32_t k, uint32_t allowed, int* which) -> double {
    const uint32_t slot = k < n16 ? 1u : 2u;
    const double ld = loss[2 * k], l16 = loss[2 * k + 1];
    double best = INFINITY;
    bool any = false;
    *which = 0;
    if (((1u << slot) & ~allowed) == 0u) { best = 0.0; any = true; }
    if (ld >= 0.0 && ((1u & custom) & ~allowed) == 0u && (!any || ld < best)) { best = ld; any = true; *which = 1; }
    if (l16 >= 0.0 && ((2u & custom) & ~allowed) == 0u && (!any || l16 < best)) { best = l16; any = true; *which = 2; }
    return any ? best : INFINITY;
  };
  // subsets of `custom` in the reference's order: custom, then
  // (prev - 1) & custom down to 0; thread j takes the j-th
  const int nsub = 1 << __popc(custom);
  if (tid < nsub) {
    uint32_t allowed = custom;
    for (int j = 0; j < tid; ++j) allowed = (allowed - 1u) & custom;
    double cost = INFINITY;
    if ((pinned & ~allowed) == 0u) {
      cost = static_cast<double>(header_bits(s, allowed));
      // a pinned family's regions were dropped
      const uint32_t lo = (pinned & 2u) ? n16 : 0u;
      const uint32_t hi = (pinned & 4u) ? n16 : count;
#pragma unroll 8
      for (uint32_t k = lo; k < hi; ++k) {
        int which;
        cost = __dadd_rn(cost, best_of(k, allowed, &which));
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
  const uint32_t best = s_best;
  if (best == used) return;
  for (uint32_t k = tid; k < count; k += kMhThreads) {
    const uint32_t slot = k < n16 ? 1u : 2u;
    if (pinned & (1u << slot)) continue;
    int which;
    best_of(k, best, &which);
    if (which == 0) continue;
    const int chosen = which == 1 ? kStDct : kSt16x16;
    const uint32_t b = k < n16 ? list16[k] : list32[k - n16];
    const int st = slot == 2u ? kSt32x32 : kSt16x16;
    const int bx = static_cast<int>(b % xb), by = static_cast<int>(b / xb);
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

constexpr int kLayoutWarps = 4;
struct LayoutSmem {
  float in[3][32][33];
  float co[3][1024];
};
constexpr size_t kLayoutSmemBytes = kLayoutWarps * sizeof(LayoutSmem);

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

template <int S>
__device__ __forceinline__ void layout_piece(const Frame& f, const SearchFrame& s, int bx, int by,
                                             LayoutSmem& sm) {
  constexpr int CX = Shape<S>::CX, CY = Shape<S>::CY, COVX = Shape<S>::COVX;
  constexpr int COVY = Shape<S>::COVY, SIZE = CX * CY * 64, COVERED = CX * CY;
  constexpr int LOG2C = COVERED == 1 ? 0 : COVERED == 2 ? 1 : COVERED == 4 ? 2 : 4;
  const int lane = threadIdx.x & 31;
  const KernelArgs& a = f.a;
  const int xb = a.xb, yb = a.yb;
  const int64_t nb = static_cast<int64_t>(xb) * yb;
  const int bi = by * xb + bx;
  const SearchTables* t = s.t;
  const int kind = dct_kind_of(S);
  for (int c = 0; c < 3; ++c)
    warp_forward<S>(f, c, bx * 8, by * 8, reinterpret_cast<float (*)[Shape<S>::W + 1]>(sm.in[0][0]),
                    sm.co[c]);
  const int32_t quant = f.qf[bi];
  // Y DC levels of the covered blocks (quantize_dc_scalar, src/group.rs:286-292)
  int16_t ydq[16];
  if (lane == 0) {
    float dcv[16];
    piece_dc(kind, sm.co[1], dcv);
    for (int k = 0; k < COVERED; ++k) ydq[k] = cast_i16(roundf(__fmul_rn(dcv[k], a.inv_dc_factor[1])));
  }
  __syncwarp();
  // Y AC round trip (quantize_roundtrip_y_block, src/group.rs:795-820); the
  // levels stay in registers until the store
  const float* inv_y = inv_of(t, S, 1);
  const float* mat_y = mat_of(t, S, 1);
  const float* thr_y = t->thr[Shape<S>::CLASS][1];
  const float qs_y = __fmul_rn(__fmul_rn(s.scale, static_cast<float>(quant)), 1.0f);
  const float inv_qac = __fdiv_rn(1.0f, __fmul_rn(s.scale, static_cast<float>(quant)));
  for (int i = lane; i < SIZE; i += 32) {
    const float val = __fmul_rn(__fmul_rn(inv_y[i], qs_y), sm.co[1][i]);
    const int32_t q = quantize_level(val, layout_threshold(thr_y, i, CX, CY));
    sm.in[1][0][i] = __int_as_float(q);  // park the Y level
    const int width = CX * 8, r = i / width, u = i % width;
    sm.co[1][i] = (r < CY && u < CX) ? 0.0f
                                     : __fmul_rn(__fmul_rn(bias_level(1, q), mat_y[i]), inv_qac);
  }
  __syncwarp();
  // chroma from luma on the whole block (src/group.rs:1831-1858)
  const int tt = (by >> 3) * a.tiles_x + (bx >> 3);
  const float xf = fmla(static_cast<float>(f.ytox[tt]), 1.0f / 84.0f, 0.0f);
  const float bf = fmla(static_cast<float>(f.ytob[tt]), 1.0f / 84.0f, 1.0f);
  for (int i = lane; i < SIZE; i += 32) {
    const float y = sm.co[1][i];
    sm.co[0][i] = fmla(-xf, y, sm.co[0][i]);
    sm.co[2][i] = fmla(-bf, y, sm.co[2][i]);
  }
  __syncwarp();
  if (lane == 0) {
    float xdp[16], bdp[16];
    piece_dc(kind, sm.co[0], xdp);
    piece_dc(kind, sm.co[2], bdp);
    for (int iy = 0; iy < COVY; ++iy)
      for (int ix = 0; ix < COVX; ++ix) {
        const int k = iy * COVX + ix;
        const int64_t b = static_cast<int64_t>(by + iy) * xb + bx + ix;
        int16_t xq;
        if (a.cfl_dc_factor_x != 0.0f)
          xq = cast_i16(roundf(fmla(xdp[k], a.inv_dc_factor[0], __fmul_rn(-static_cast<float>(ydq[k]), a.cfl_dc_factor_x))));
        else
          xq = cast_i16(roundf(__fmul_rn(xdp[k], a.inv_dc_factor[0])));
        const int16_t bq = cast_i16(roundf(fmla(bdp[k], a.inv_dc_factor[2],
                                                __fmul_rn(-static_cast<float>(ydq[k]), a.cfl_dc_factor_b))));
        f.quant_dc[b] = xq;
        f.quant_dc[nb + b] = ydq[k];
        f.quant_dc[2 * nb + b] = bq;
      }
  }
  // X and B levels, then every channel's store, non-zero count and walk end
  const uint16_t* pos = pos_of(t, S);
  int nz[3];
  uint32_t last[3];
  for (int c = 0; c < 3; ++c) {
    int n = 0;
    uint32_t lst = 0;
    const float* inv = inv_of(t, S, c);
    const float* thr = t->thr[Shape<S>::CLASS][c];
    const float qs = __fmul_rn(__fmul_rn(s.scale, static_cast<float>(quant)), a.qm_mul[c]);
    for (int i = lane; i < SIZE; i += 32) {
      int32_t q;
      if (c == 1) {
        q = __float_as_int(sm.in[1][0][i]);
      } else {
        const float val = __fmul_rn(__fmul_rn(inv[i], qs), sm.co[c][i]);
        q = quantize_level(val, layout_threshold(thr, i, CX, CY));
      }
      const int chunk = i >> 6;
      const int64_t b = static_cast<int64_t>(by + chunk / COVX) * xb + bx + chunk % COVX;
      const int64_t at = b * 192 + c * 64 + (i & 63);
      if (q < -32767 || q > 32767) {
        f.levels[at] = kLevelEscape;
        f.wide_levels[at] = q;
      } else {
        f.levels[at] = static_cast<int16_t>(q);
      }
      const int width = CX * 8, r = i / width, u = i % width;
      if (q != 0 && !(r < CY && u < CX)) {
        ++n;
        lst = max(lst, static_cast<uint32_t>(pos[i]));
      }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      n += __shfl_xor_sync(0xffffffffu, n, d);
      lst = max(lst, __shfl_xor_sync(0xffffffffu, lst, d));
    }
    nz[c] = n;
    last[c] = lst;
  }
  if (lane < COVERED) {
    const int ix = lane % COVX, iy = lane / COVX;
    const int64_t b = static_cast<int64_t>(by + iy) * xb + bx + ix;
    uint32_t packed = 0;
    for (int c = 0; c < 3; ++c) {
      const uint32_t sh = (static_cast<uint32_t>(nz[c]) + COVERED - 1u) >> LOG2C;
      f.nzeros[c * nb + b] = static_cast<uint8_t>(sh);
      packed |= (sh & 0xffu) << (8 * c);
    }
    f.nz_packed[b] = packed;
    // token counts at the first block ([Y, X, B, 0] per group-local block)
    const int gx = (bx + ix) / kGroupBlocks, gy = (by + iy) / kGroupBlocks;
    const int g = gy * a.groups_x + gx;
    const int lb = ((by + iy) % kGroupBlocks) * kGroupBlocks + (bx + ix) % kGroupBlocks;
    uint4 cnt = make_uint4(0u, 0u, 0u, 0u);
    if (lane == 0) {
      auto walk = [&](int c) { return 1u + (nz[c] ? last[c] - COVERED + 1u : 0u); };
      cnt = make_uint4(walk(1), walk(0), walk(2), 0u);
    }
    reinterpret_cast<uint4*>(f.counts)[static_cast<int64_t>(g) * 1024 + lb] = cnt;
  }
  __syncwarp();
}

// One CTA per 64x64 tile; its transforms (first blocks in raster order)
// taken by the warps in turn.
__global__ void __launch_bounds__(32 * kLayoutWarps) k_layout_tile(const __grid_constant__ Frame f) {
  extern __shared__ __align__(16) unsigned char layout_smem_raw[];
  LayoutSmem& sm = reinterpret_cast<LayoutSmem*>(layout_smem_raw)[threadIdx.x >> 5];
  const SearchFrame& s = *static_cast<const SearchFrame*>(f.search);
  const int xb = f.a.xb, yb = f.a.yb;
  const int tx = blockIdx.x % f.a.tiles_x, ty = blockIdx.x / f.a.tiles_x;
  const int bx0 = tx * 8, by0 = ty * 8;
  const int w = imin(8, xb - bx0), h = imin(8, yb - by0);
  const int warp = threadIdx.x >> 5;
  int k = 0;
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const uint8_t cell = s.map[(by0 + y) * xb + bx0 + x];
      if (!(cell & 1)) continue;
      if ((k++ % kLayoutWarps) != warp) continue;
      switch (cell >> 1) {
        case kStDct: layout_piece<kStDct>(f, s, bx0 + x, by0 + y, sm); break;
        case kSt16x8: layout_piece<kSt16x8>(f, s, bx0 + x, by0 + y, sm); break;
        case kSt8x16: layout_piece<kSt8x16>(f, s, bx0 + x, by0 + y, sm); break;
        case kSt16x16: layout_piece<kSt16x16>(f, s, bx0 + x, by0 + y, sm); break;
        default: layout_piece<kSt32x32>(f, s, bx0 + x, by0 + y, sm); break;
      }
    }
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

// Dynamic shared memory above the 48 KB default for the search kernels.
inline cudaError_t set_search_attributes() {
  cudaError_t e = cudaSuccess;
  auto set = [&](const void* fn, size_t bytes) {
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
  };
  set(reinterpret_cast<const void*>(k_cost<kStDct>), cost_smem_bytes<kStDct>());
  set(reinterpret_cast<const void*>(k_cost<kSt16x8>), cost_smem_bytes<kSt16x8>());
  set(reinterpret_cast<const void*>(k_cost<kSt8x16>), cost_smem_bytes<kSt8x16>());
  set(reinterpret_cast<const void*>(k_cost<kSt16x16>), cost_smem_bytes<kSt16x16>());
  set(reinterpret_cast<const void*>(k_cost<kSt32x32>), cost_smem_bytes<kSt32x32>());
  set(reinterpret_cast<const void*>(k_mh_incumbent), cost_smem_bytes<kSt32x32>());
  set(reinterpret_cast<const void*>(k_layout_tile), kLayoutSmemBytes);
  set(reinterpret_cast<const void*>(k_retile), kRetileSmemBytes);
  return e;
}

}  // namespace jxg
