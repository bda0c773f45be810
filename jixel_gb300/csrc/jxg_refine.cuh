// Differentiable quant-field refinement of an all-DCT8 frame (the frame the
// last UltraFast pass of a context coded).  Not in the reference, which has no
// gradients anywhere; it refines what adaptive_quant.rs gives it.
//
// Parameters: theta, one log quant scale per 8x8 block; block b's quantiser is
// s_b = scale * qf_b * exp(theta_b), qf the pass's adaptive field.
//
// Forward model (FP32), per block, as the front end quantises (k_tile_quantize
// and write_ac_group, src/group.rs:560-612, :767-818, :1831-1858):
//   Y AC levels at s, their dequantised values with the decoder's bias
//   (DequantBias, src/group.rs:767); CfL on X and B from the dequantised Y; X
//   and B levels at s; the decoder's coefficients X^ = deq(X) + xf Y^,
//   B^ = deq(B) + bf Y^.  The DC slot holds the decoded DC: the pass's DC
//   levels dequantised (quantize_dc / quantize_dc_cfl inverted,
//   src/group.rs:286-306); theta does not move it, and the decoder's
//   adaptive DC smoothing (src/frame/dc_smoothing.rs) is not modelled;
//   the 8x8 inverse transform as a 64 x 64 matrix M taken from the library's
//   own IDCT (src/dct.rs:1500-1620), so its adjoint is exactly M^T;
//   XYB to linear RGB (xyb_to_rgb_pixel_f32, src/xyb.rs:265-283);
//   the distortion proxy: 1 - SSIM of the linear planes against the source's,
//   at three scales (2x2 box average between them), with a 5-tap binomial blur
//   (zero outside the image), averaged over channels, pixels and scales;
//   the rate model: per non-zero AC level 1.6 + log2(1 + |level|) bits (the
//   coefficient model's per-level terms, src/inflated_cost.rs:540-547); a
//   level that rounds to zero costs 2.6 (|v| / z)^4 bits, v its quantiser
//   input and z = max(threshold, 0.5) the edge of its zero region, so that
//   finer quantisation sees the levels it is about to create;
//   loss = distortion + lambda * bits / pixels.
// Rounding is straight-through: the backward pass treats each non-zero level
// as its unrounded value, keeps zero levels' decoded values at zero, and
// differentiates the bias for |level| >= 2 (1 + 0.145 / level^2; 0 at
// |level| = 1).
// The decoder's edge-preserving filter is modelled (Epf::apply,
// src/epf_filter.rs:268-350: the frame's stages, per-block sigma from the
// field at theta, patch SADs over mirrored borders); its adjoint holds the
// weights fixed at the forward's values, the same straight-through stance
// as the rounding.  Gaborish (off in the reference's encoder) and DC
// smoothing are not modelled.
#pragma once

namespace jxg {

struct RefineArgs {
  int32_t w, h, xb, yb, pw;  // image, blocks, padded plane width (xb * 8)
  int64_t plane;             // floats between the source XYB planes
  const float* xyb;          // source XYB
  float* coef;               // [block][X, Y, B][64] source DCT8 coefficients
  const uint8_t* qf;         // the pass's quant field
  const int8_t* ytox;
  const int8_t* ytob;
  int32_t tiles_x;
  float scale, qm_mul[3];
  float matrix[3][64], inv_matrix[3][64], thresholds[3][4];
  float* dc;                 // [block][X, Y, B] decoded DC (the pass's DC levels dequantised)
  // the decoder's edge-preserving filter (EPF): its stages in order (ids 0-2)
  int32_t epf_stages, epf_stage[3];
  float epf_sm[3];           // SAD multiplier of each stage (SAD_MUL x its sigma scale)
  float epf_border;          // border_sad_mul
  float epf_channel[3];      // channel_scale
  float epf_quant_mul, epf_lut, epf_quant_scale;
  float* sigma;              // per block: the inverse sigma at the current theta
  float* m;                  // [64 pixels][64 coefficients] inverse DCT8
  float* mt;                 // the same, [coefficient][pixel]
  float* recon;              // 3 padded planes (pw x yb * 8) of decoded XYB
};

// f64 partial sums: kRefineSlots per quantity (the three scales' 1 - SSIM,
// then the rate), CTAs spread over them; the host adds each quantity's slots.
constexpr int kRefineSlots = 32;

constexpr float kOpsinBias = 0.0037930734f, kNegBiasCbrt = -0.1559542f;
// OPSIN_INVERSE_MATRIX (src/xyb.rs:49-59)
__constant__ const float kOpsinInverse[9] = {11.031567f,   -9.866944f,  -0.16462299f,
                                             -3.2541473f,  4.4187703f,  -0.16462299f,
                                             -3.6588514f,  2.712923f,   1.9459282f};
constexpr float kLn2 = 0.6931471805599453f;
constexpr float kZeroBits = 2.6f;  // 1.6 + log2(1 + 1): a level of one

__device__ __forceinline__ float refine_bias(int c, int32_t q) { return bias_level(c, q); }
__device__ __forceinline__ float refine_bias_slope(int32_t q) {
  if (q == 1 || q == -1 || q == 0) return 0.0f;
  const float qf = static_cast<float>(q);
  return 1.0f + 0.145f / (qf * qf);
}

// One coefficient's decoded values and, for the backward pass, their
// derivatives by s.
struct CoefState {
  int32_t q[3];
  float hat[3];   // X^, Y^, B^
  float dhat[3];  // dX^/ds, dY^/ds, dB^/ds
  float dbits;    // d bits / ds
  float bits;
};

__device__ __forceinline__ void refine_coef(const RefineArgs& r, int i, float s, float xf, float bf,
                                            float cx, float cy, float cb, bool grad, CoefState* o) {
  const float inv_s = __fdiv_rn(1.0f, s);
  const int row = i >> 3, col = i & 7, yfix = row >= 4 ? 2 : 0;
  auto thr = [&](int c) { return col >= 4 ? r.thresholds[c][yfix + 1] : r.thresholds[c][yfix]; };
  // Y, as k_tile_quantize: (inv * (s * qm)) * c, then (bias * w) * (1 / s)
  const float vy = __fmul_rn(__fmul_rn(r.inv_matrix[1][i], __fmul_rn(s, r.qm_mul[1])), cy);
  const int32_t qy = quantize_level(vy, thr(1));
  const float yh = __fmul_rn(__fmul_rn(refine_bias(1, qy), r.matrix[1][i]), inv_s);
  float dyh = 0.0f;
  if (grad && qy != 0)
    dyh = __fmul_rn(__fdiv_rn(r.matrix[1][i], __fmul_rn(s, s)),
                    __fsub_rn(__fmul_rn(refine_bias_slope(qy), vy), refine_bias(1, qy)));
  float bits = 0.0f, dbits = 0.0f;
  // a level q from the quantiser input v (dv = dv/ds); a level that rounds
  // to zero costs kZeroBits (|v| / z)^4, z = max(threshold, 0.5) the edge of
  // its zero region, rising smoothly to the cost of a level of one
  auto rate = [&](int32_t q, float v, float dv, float t) {
    if (q == 0) {
      const float z = fmaxf(t, 0.5f), a = __fdiv_rn(fabsf(v), z), a2 = __fmul_rn(a, a);
      bits = __fmaf_rn(kZeroBits, __fmul_rn(a2, a2), bits);
      if (grad)
        dbits = __fmaf_rn(__fmul_rn(4.0f * kZeroBits, __fmul_rn(a2, a)), __fdiv_rn(copysignf(1.0f, v) * dv, z), dbits);
      return;
    }
    const float a = fabsf(static_cast<float>(q));
    bits = __fadd_rn(bits, __fadd_rn(1.6f, __log2f(1.0f + a)));
    if (grad) dbits = __fadd_rn(dbits, __fdiv_rn(copysignf(1.0f, static_cast<float>(q)) * dv,
                                                 __fmul_rn(1.0f + a, kLn2)));
  };
  rate(qy, vy, __fdiv_rn(vy, s), thr(1));
  // X and B after CfL from the dequantised Y
  const float cc[2] = {cx, cb}, ff[2] = {xf, bf};
  const int ch[2] = {0, 2};
  float hat[2], dhat[2];
  int32_t qq[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int c = ch[k];
    const float qm = r.qm_mul[c];
    const float v = __fmaf_rn(-ff[k], yh, cc[k]);
    const float u = __fmul_rn(__fmul_rn(r.inv_matrix[c][i], __fmul_rn(s, qm)), v);
    const int32_t q = quantize_level(u, thr(c));
    qq[k] = q;
    const float sq = __fmul_rn(s, qm);
    const float deq = q == 0 ? 0.0f : __fdiv_rn(__fmul_rn(refine_bias(c, q), r.matrix[c][i]), sq);
    hat[k] = __fmaf_rn(ff[k], yh, deq);
    dhat[k] = 0.0f;
    if (grad) {
      // du/ds = u / s - inv * s * qm * xf * dY^/ds
      const float du = __fsub_rn(__fdiv_rn(u, s),
                                 __fmul_rn(__fmul_rn(r.inv_matrix[c][i], sq), __fmul_rn(ff[k], dyh)));
      float dd = 0.0f;
      if (q != 0)
        dd = __fmul_rn(__fdiv_rn(r.matrix[c][i], sq),
                       __fsub_rn(__fmul_rn(refine_bias_slope(q), du), __fdiv_rn(refine_bias(c, q), s)));
      dhat[k] = __fmaf_rn(ff[k], dyh, dd);
      rate(q, u, du, thr(c));
    } else {
      rate(q, u, 0.0f, thr(c));
    }
  }
  o->q[0] = qq[0];
  o->q[1] = qy;
  o->q[2] = qq[1];
  o->hat[0] = hat[0];
  o->hat[1] = yh;
  o->hat[2] = hat[1];
  o->dhat[0] = dhat[0];
  o->dhat[1] = dyh;
  o->dhat[2] = dhat[1];
  o->bits = bits;
  o->dbits = dbits;
}

__device__ __forceinline__ float refine_s(const RefineArgs& r, int64_t b, float theta) {
  return __fmul_rn(__fmul_rn(r.scale, static_cast<float>(r.qf[b])), expf(theta));
}
__device__ __forceinline__ void refine_cfl(const RefineArgs& r, int bx, int by, float* xf, float* bf) {
  const int t = (by >> 3) * r.tiles_x + (bx >> 3);
  *xf = fmla(static_cast<float>(r.ytox[t]), 1.0f / 84.0f, 0.0f);
  *bf = fmla(static_cast<float>(r.ytob[t]), 1.0f / 84.0f, 1.0f);
}

// Source coefficients: one warp per block, the tile kernel's gather with edge
// replication, rows then columns, stored transposed and scaled by 1/64.
__global__ void __launch_bounds__(256) k_refine_dct(const RefineArgs r) {
  __shared__ float buf[8][3][8][9];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t b = static_cast<int64_t>(blockIdx.x) * 8 + warp;
  if (b >= static_cast<int64_t>(r.xb) * r.yb) return;
  const int bx = static_cast<int>(b % r.xb), by = static_cast<int>(b / r.xb);
  if (lane < 24) {
    const int c = lane >> 3, row = lane & 7;
    const float* p = r.xyb + c * r.plane;
    const int y = imin(by * 8 + row, r.h - 1);
    float v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = p[static_cast<int64_t>(y) * r.w + imin(bx * 8 + k, r.w - 1)];
    dct1d_8(v);
#pragma unroll
    for (int k = 0; k < 8; ++k) buf[warp][c][row][k] = v[k];
  }
  __syncwarp();
  if (lane < 24) {
    const int c = lane >> 3, cc = lane & 7;
    float v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = buf[warp][c][k][cc];
    dct1d_8(v);
#pragma unroll
    for (int k = 0; k < 8; ++k) r.coef[(b * 3 + c) * 64 + cc * 8 + k] = v[k] * (1.0f / 64.0f);
  }
}

// XYB -> linear RGB of one pixel (xyb_to_rgb_pixel_f32, src/xyb.rs:265-283);
// with `dcube`, the cube's derivatives 3 (t - bias)^2 for the adjoint.
__device__ __forceinline__ void xyb_to_linear(float x, float y, float b, float* out, float* dcube) {
  const float t[3] = {__fadd_rn(y, x), __fsub_rn(y, x), b};
  float m[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float c = __fsub_rn(t[k], kNegBiasCbrt);
    m[k] = __fsub_rn(__fmul_rn(__fmul_rn(c, c), c), kOpsinBias);
    if (dcube) dcube[k] = __fmul_rn(3.0f, __fmul_rn(c, c));
  }
#pragma unroll
  for (int j = 0; j < 3; ++j)
    out[j] = __fmaf_rn(kOpsinInverse[j * 3], m[0],
                       __fmaf_rn(kOpsinInverse[j * 3 + 1], m[1], __fmul_rn(kOpsinInverse[j * 3 + 2], m[2])));
}

// A CTA's sum of one quantity into its slot: each thread's partial (a few
// terms) and the warp's tree in FP32, the warps' sums and the slot in FP64
// (GB300's FP64 pipe is narrow: no per-term FP64 work).
// Every thread of the CTA calls it; calls may follow one another (the
// barrier first keeps a call's writes of `part` after the previous call's
// read).
__device__ __forceinline__ void refine_add_slot(float v, double* sums) {
  __shared__ double part[8];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
  const int nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = static_cast<double>(v);
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < nw; ++k) t += part[k];
    const unsigned cta = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    atomicAdd(sums + cta % kRefineSlots, t);
  }
}

// Forward: one warp per block, two coefficients per lane; the levels (when
// asked) and the rate, then the block's decoded XYB pixels M * c^ into the
// padded planes and, inside the image and without the EPF, their linear RGB
// into `lin` (3 planes of w x h; NULL when the EPF comes first).  The rate's
// CTA sum goes to `bit_sums`.
__global__ void __launch_bounds__(256) k_refine_forward(const RefineArgs r, const float* __restrict__ theta,
                                                        int32_t* __restrict__ levels, float* __restrict__ lin,
                                                        double* __restrict__ bit_sums) {
  __shared__ float cs[8][3][64];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t b = static_cast<int64_t>(blockIdx.x) * 8 + warp;
  const bool active = b < static_cast<int64_t>(r.xb) * r.yb;
  float bits = 0.0f;
  if (active) {
    const int bx = static_cast<int>(b % r.xb), by = static_cast<int>(b / r.xb);
    const float s = refine_s(r, b, theta[b]);
    float xf, bf;
    refine_cfl(r, bx, by, &xf, &bf);
#pragma unroll
    for (int h2 = 0; h2 < 2; ++h2) {
      const int i = lane + 32 * h2;
      const float* c = r.coef + b * 192;
      CoefState st;
      refine_coef(r, i, s, xf, bf, c[i], c[64 + i], c[128 + i], false, &st);
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) {
        cs[warp][ch][i] = i == 0 ? r.dc[b * 3 + ch] : st.hat[ch];
        if (levels) levels[b * 192 + ch * 64 + i] = i == 0 ? 0 : st.q[ch];
      }
      if (i != 0) bits = __fadd_rn(bits, st.bits);
    }
    __syncwarp();
    const int64_t pp = static_cast<int64_t>(r.pw) * r.yb * 8, n = static_cast<int64_t>(r.w) * r.h;
#pragma unroll
    for (int h2 = 0; h2 < 2; ++h2) {
      const int p = lane + 32 * h2;
      float acc[3] = {0.0f, 0.0f, 0.0f};
      for (int i = 0; i < 64; ++i) {
        const float m = r.mt[i * 64 + p];
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) acc[ch] = __fmaf_rn(m, cs[warp][ch][i], acc[ch]);
      }
      const int y = by * 8 + (p >> 3), x = bx * 8 + (p & 7);
      const int64_t at = static_cast<int64_t>(y) * r.pw + x;
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) r.recon[ch * pp + at] = acc[ch];
      if (lin && x < r.w && y < r.h) {
        float o[3];
        xyb_to_linear(acc[0], acc[1], acc[2], o, nullptr);
        const int64_t q = static_cast<int64_t>(y) * r.w + x;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) lin[ch * n + q] = o[ch];
      }
    }
  }
  refine_add_slot(bits, bit_sums);
}

// The decoded DC of every block from the pass's DC levels (3 planes of
// xb*yb): Y = q_Y / f_Y, X = (q_X + q_Y c_X) / f_X, B = (q_B + q_Y c_B) / f_B,
// f the inverse DC steps and c the DC chroma-from-luma factors the levels
// were taken with.
__global__ void __launch_bounds__(256) k_refine_dc(const int16_t* __restrict__ quant_dc, int64_t nb,
                                                   float fx, float fy, float fb, float cx, float cb,
                                                   float* __restrict__ dc) {
  const int64_t b = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const float qx = quant_dc[b], qy = quant_dc[nb + b], qb = quant_dc[2 * nb + b];
  dc[b * 3 + 0] = __fdiv_rn(__fmaf_rn(qy, cx, qx), fx);
  dc[b * 3 + 1] = __fdiv_rn(qy, fy);
  dc[b * 3 + 2] = __fdiv_rn(__fmaf_rn(qy, cb, qb), fb);
}

// ---------------------------------------------------------------------------
// The decoder's EPF (src/epf_filter.rs:213-263, :320-350, epf_filter/
// kernels.rs:88-132, epf_filter/stream.rs:157-265)
// ---------------------------------------------------------------------------

constexpr float kEpfInvSigmaNum = -1.1715729f, kEpfMinSigma = -3.905243f;
constexpr int kEpfMaxNeighbors = 12;
// The three stages: difference directions (dx, dy) and neighbours as
// (direction, along), in the decoder's order.
struct EpfStageTable {
  int dirs, neighbors, patch;
  int8_t dx[6], dy[6];
  int8_t dir[kEpfMaxNeighbors];
  int8_t along[kEpfMaxNeighbors];
};
__constant__ const EpfStageTable kEpfStages[3] = {
    {6, 12, 1, {1, 2, 0, 0, 1, -1}, {0, 0, 1, 2, 1, 1},
     {3, 4, 2, 5, 1, 0, 0, 1, 5, 2, 4, 3}, {0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1}},
    {2, 4, 1, {1, 0}, {0, 1}, {1, 0, 0, 1}, {0, 0, 1, 1}},
    {2, 4, 0, {1, 0}, {0, 1}, {1, 0, 0, 1}, {0, 0, 1, 1}},
};

__device__ __forceinline__ int epf_mirror(int i, int n) {
  while (i < 0 || i >= n) i = i < 0 ? -i - 1 : 2 * n - 1 - i;
  return i;
}

// The inverse sigma of every block at theta: the field qf * exp(theta) in
// place of the decoder's integer field (FrameBlocks::new and the sigma
// kernel, src/epf_filter.rs:118-146, epf_filter/kernels.rs:151-155).
__global__ void __launch_bounds__(256) k_refine_sigma(const RefineArgs r, const float* __restrict__ theta) {
  const int64_t b = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (b >= static_cast<int64_t>(r.xb) * r.yb) return;
  const float q = __fmul_rn(static_cast<float>(r.qf[b]), expf(theta[b]));
  const float sq = __fmul_rn(__fmul_rn(r.epf_quant_scale, q), kEpfInvSigmaNum);
  r.sigma[b] = __fdiv_rn(1.0f, fminf(__fmul_rn(__fdiv_rn(r.epf_quant_mul, sq), r.epf_lut), -1e-4f));
}

// The inverse sigma of every block from FrameBlocks' sigma_quant (the EPF
// operator): 1 / min(quant_mul / sigma_quant * lut, -1e-4).
__global__ void __launch_bounds__(256) k_epf_sigma(const float* __restrict__ sigma_quant, int64_t nb,
                                                   float quant_mul, float lut, float* __restrict__ out) {
  const int64_t b = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  out[b] = __fdiv_rn(1.0f, fminf(__fmul_rn(__fdiv_rn(quant_mul, sigma_quant[b]), lut), -1e-4f));
}

struct EpfPlanes {
  const float* p;
  int64_t plane;
  int stride, w, h;
  __device__ __forceinline__ float at(int c, int x, int y) const {
    return p[c * plane + static_cast<int64_t>(epf_mirror(y, h)) * stride + epf_mirror(x, w)];
  }
};

// One EPF stage over the w x h image: `in` (planes of stride `in_stride`,
// `in_plane` apart), `out` (3 planes of w x h); for the adjoint the
// normalised neighbour weights (`nw`, one plane of w x h per neighbour) and
// the centre's (`cw`).  A CTA takes a 32 x 8 tile: the pixels with a 4-pixel
// mirrored ring into shared memory, then each direction's channel-weighted
// differences once per position, then per pixel the patch SADs, weights and
// the weighted mean.
constexpr int kEpfTW = 32, kEpfTH = 8, kEpfHalo = 4;
constexpr int kEpfInW = kEpfTW + 2 * kEpfHalo, kEpfInH = kEpfTH + 2 * kEpfHalo;  // 40 x 16
// differences at x0-3 .. x0+33 and y0-3 .. y0+8: a SAD's centre lies within
// (-2, -2) .. (+1, 0) of its pixel (the neighbour offsets), its patch one more
constexpr int kEpfDW = kEpfTW + 5, kEpfDH = kEpfTH + 4;
__global__ void __launch_bounds__(256) k_refine_epf(const RefineArgs r, int stage, float sm,
                                                    const float* __restrict__ in, int64_t in_plane, int in_stride,
                                                    float* __restrict__ out, float* __restrict__ nw,
                                                    float* __restrict__ cw) {
  __shared__ float pix[3][kEpfInH][kEpfInW + 1];
  __shared__ float dif[6][kEpfDH][kEpfDW + 1];
  const int tid = threadIdx.x;
  const int x0 = blockIdx.x * kEpfTW, y0 = blockIdx.y * kEpfTH;
  const int w = r.w, h = r.h;
  const int64_t n = static_cast<int64_t>(w) * h;
  const EpfPlanes src{in, in_plane, in_stride, w, h};
  const EpfStageTable& t = kEpfStages[stage];
  for (int u = tid; u < kEpfInH * kEpfInW; u += 256) {
    const int ry = u / kEpfInW, rx = u % kEpfInW;
    const int X = x0 - kEpfHalo + rx, Y = y0 - kEpfHalo + ry;
#pragma unroll
    for (int c = 0; c < 3; ++c) pix[c][ry][rx] = src.at(c, X, Y);
  }
  __syncthreads();
  // d(P) = sum_c scale_c |p_c(P) - p_c(P + dir)|, P at x0 - 3 + i, y0 - 3 + j
  for (int u = tid; u < t.dirs * kEpfDH * kEpfDW; u += 256) {
    const int d = u / (kEpfDH * kEpfDW), rem = u % (kEpfDH * kEpfDW);
    const int j = rem / kEpfDW, i = rem % kEpfDW;
    const int px = i + 1, py = j + 1;  // P in the pixel tile (its ring starts at -4)
    const int qx = px + t.dx[d], qy = py + t.dy[d];
    float v = __fmul_rn(fabsf(__fsub_rn(pix[0][py][px], pix[0][qy][qx])), r.epf_channel[0]);
    v = __fadd_rn(__fmul_rn(fabsf(__fsub_rn(pix[1][py][px], pix[1][qy][qx])), r.epf_channel[1]), v);
    dif[d][j][i] = __fadd_rn(__fmul_rn(fabsf(__fsub_rn(pix[2][py][px], pix[2][qy][qx])), r.epf_channel[2]), v);
  }
  __syncthreads();
  const int lx = tid % kEpfTW, ly = tid / kEpfTW;
  const int x = x0 + lx, y = y0 + ly;
  if (x >= w || y >= h) return;
  const int64_t q = static_cast<int64_t>(y) * w + x;
  const int cx = lx + kEpfHalo, cy = ly + kEpfHalo;  // the pixel in `pix`
  float acc[3] = {pix[0][cy][cx], pix[1][cy][cx], pix[2][cy][cx]};
  const float s = r.sigma[static_cast<int64_t>(y >> 3) * r.xb + (x >> 3)];
  if (s < kEpfMinSigma) {  // unfiltered block: the centre, exactly
#pragma unroll
    for (int c = 0; c < 3; ++c) out[c * n + q] = acc[c];
    for (int k = 0; k < t.neighbors; ++k) nw[k * n + q] = 0.0f;
    cw[q] = 1.0f;
    return;
  }
  const bool border = (y & 7) == 0 || (y & 7) == 7 || (x & 7) == 0 || (x & 7) == 7;
  const float inv = __fmul_rn(s, border ? __fmul_rn(sm, r.epf_border) : sm);
  float sum = 1.0f, wk[kEpfMaxNeighbors];
  for (int k = 0; k < t.neighbors; ++k) {
    const int d = t.dir[k], dx = t.dx[d], dy = t.dy[d];
    const bool along = t.along[k] != 0;
    // the SAD's centre P = (sx, sy), as an index into `dif` (offset 3)
    const int di = (along ? lx : lx - dx) + 3, dj = (along ? ly : ly - dy) + 3;
    float sad;
    if (t.patch)
      sad = __fadd_rn(__fadd_rn(dif[d][dj][di], __fadd_rn(dif[d][dj][di - 1], dif[d][dj][di + 1])),
                      __fadd_rn(dif[d][dj - 1][di], dif[d][dj + 1][di]));
    else
      sad = dif[d][dj][di];
    const float wt = fmaxf(__fadd_rn(__fmul_rn(sad, inv), 1.0f), 0.0f);
    wk[k] = wt;
    sum = __fadd_rn(sum, wt);
    const int nx = cx + (along ? dx : -dx), ny = cy + (along ? dy : -dy);
#pragma unroll
    for (int c = 0; c < 3; ++c) acc[c] = __fadd_rn(__fmul_rn(wt, pix[c][ny][nx]), acc[c]);
  }
  const float inv_sum = __fdiv_rn(1.0f, sum);
#pragma unroll
  for (int c = 0; c < 3; ++c) out[c * n + q] = __fmul_rn(acc[c], inv_sum);
  for (int k = 0; k < t.neighbors; ++k) nw[k * n + q] = __fmul_rn(wk[k], inv_sum);
  cw[q] = inv_sum;
}

// Its adjoint with the weights held: g_in(q) = cw(q) g_out(q) plus, for every
// output pixel p whose neighbour k is q (through the mirrored borders),
// nw_k(p) g_out(p).  A gather: the candidates for p are q's mirror images
// less the neighbour's offset.
__global__ void __launch_bounds__(256) k_refine_epf_adjoint(const RefineArgs r, int stage,
                                                            const float* __restrict__ gout,
                                                            const float* __restrict__ nw,
                                                            const float* __restrict__ cw,
                                                            float* __restrict__ gin) {
  const int w = r.w, h = r.h;
  const int64_t n = static_cast<int64_t>(w) * h;
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int qx = static_cast<int>(q % w), qy = static_cast<int>(q / w);
  const EpfStageTable& t = kEpfStages[stage];
  float g[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) g[c] = __fmul_rn(cw[q], gout[c * n + q]);
  const bool interior = qx >= 3 && qx < w - 3 && qy >= 3 && qy < h - 3;
  const int cxs[3] = {qx, -1 - qx, 2 * w - 1 - qx}, cys[3] = {qy, -1 - qy, 2 * h - 1 - qy};
  for (int k = 0; k < t.neighbors; ++k) {
    const int d = t.dir[k];
    const int ox = t.along[k] ? t.dx[d] : -t.dx[d], oy = t.along[k] ? t.dy[d] : -t.dy[d];
    for (int iy = 0; iy < (interior ? 1 : 3); ++iy)
      for (int ix = 0; ix < (interior ? 1 : 3); ++ix) {
        const int px = cxs[ix] - ox, py = cys[iy] - oy;
        if (px < 0 || px >= w || py < 0 || py >= h) continue;
        if (!interior && (epf_mirror(px + ox, w) != qx || epf_mirror(py + oy, h) != qy)) continue;
        if (ix > 0 && cxs[ix] == cxs[0]) continue;  // the same mirror image twice
        if (iy > 0 && cys[iy] == cys[0]) continue;
        const int64_t p = static_cast<int64_t>(py) * w + px;
        const float wv = nw[k * n + p];
#pragma unroll
        for (int c = 0; c < 3; ++c) g[c] = __fadd_rn(g[c], __fmul_rn(wv, gout[c * n + p]));
      }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) gin[c * n + q] = g[c];
}

// The gradient by the decoded XYB planes (w x h): scale 0's linear-plane
// gradient plus a quarter of scale 1's, back through XYB -> linear at the
// decoded values (`xyb`: planes `xyb_plane` apart, rows `xyb_stride`).
__global__ void __launch_bounds__(256) k_refine_linear_adjoint(const float* __restrict__ xyb, int64_t xyb_plane,
                                                               int xyb_stride, const float* __restrict__ glin0,
                                                               const float* __restrict__ glin1, int w, int h,
                                                               int w1, int h1, float* __restrict__ gxyb) {
  const int64_t n = static_cast<int64_t>(w) * h, n1 = static_cast<int64_t>(w1) * h1;
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int x = static_cast<int>(q % w), y = static_cast<int>(q / w);
  float gl[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) gl[k] = glin0[k * n + q];
  if ((y >> 1) < h1 && (x >> 1) < w1) {
    const int64_t q1 = static_cast<int64_t>(y >> 1) * w1 + (x >> 1);
#pragma unroll
    for (int k = 0; k < 3; ++k) gl[k] = __fmaf_rn(0.25f, glin1[k * n1 + q1], gl[k]);
  }
  float o[3], dc[3];
  const int64_t at = static_cast<int64_t>(y) * xyb_stride + x;
  xyb_to_linear(xyb[at], xyb[xyb_plane + at], xyb[2 * xyb_plane + at], o, dc);
  float gm[3];
#pragma unroll
  for (int k = 0; k < 3; ++k)
    gm[k] = __fmul_rn(dc[k], __fmaf_rn(kOpsinInverse[k], gl[0],
                                       __fmaf_rn(kOpsinInverse[3 + k], gl[1], __fmul_rn(kOpsinInverse[6 + k], gl[2]))));
  gxyb[q] = __fsub_rn(gm[0], gm[1]);
  gxyb[n + q] = __fadd_rn(gm[0], gm[1]);
  gxyb[2 * n + q] = gm[2];
}

// Linear RGB of the w x h region of XYB planes with row stride `in_stride`.
__global__ void __launch_bounds__(256) k_refine_linear(const float* __restrict__ xyb, int64_t in_plane,
                                                       int in_stride, float* __restrict__ lin, int w,
                                                       int h) {
  const int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= static_cast<int64_t>(w) * h) return;
  const int y = static_cast<int>(p / w), x = static_cast<int>(p % w);
  const int64_t at = static_cast<int64_t>(y) * in_stride + x;
  float o[3];
  xyb_to_linear(xyb[at], xyb[in_plane + at], xyb[2 * in_plane + at], o, nullptr);
  const int64_t n = static_cast<int64_t>(w) * h;
#pragma unroll
  for (int c = 0; c < 3; ++c) lin[c * n + p] = o[c];
}

// 2x2 box average to the next scale (3 planes of w x h -> (w/2) x (h/2)).
__global__ void __launch_bounds__(256) k_refine_down(const float* __restrict__ in, float* __restrict__ out,
                                                     int w, int h) {
  const int w2 = w / 2, h2 = h / 2;
  const int64_t n2 = static_cast<int64_t>(w2) * h2;
  const int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= 3 * n2) return;
  const int c = static_cast<int>(p / n2);
  const int64_t q = p % n2;
  const int y = static_cast<int>(q / w2), x = static_cast<int>(q % w2);
  const float* src = in + c * static_cast<int64_t>(w) * h;
  const int64_t a = static_cast<int64_t>(2 * y) * w + 2 * x;
  out[p] = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(src[a], src[a + 1]), __fadd_rn(src[a + w], src[a + w + 1])));
}

// The adjoint: each fine pixel takes a quarter of its coarse pixel's gradient.
__global__ void __launch_bounds__(256) k_refine_up_add(const float* __restrict__ g2, float* __restrict__ g,
                                                       int w, int h) {
  const int w2 = w / 2, h2 = h / 2;
  const int64_t n = static_cast<int64_t>(w) * h;
  const int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= 3 * n) return;
  const int c = static_cast<int>(p / n);
  const int64_t q = p % n;
  const int y = static_cast<int>(q / w), x = static_cast<int>(q % w);
  if (y / 2 >= h2 || x / 2 >= w2) return;
  g[p] = __fadd_rn(g[p], __fmul_rn(0.25f, g2[c * static_cast<int64_t>(w2) * h2 + (y / 2) * w2 + x / 2]));
}

constexpr float kSsimC1 = 1e-4f, kSsimC2 = 9e-4f;
// SSIM tile of the fused kernel: 32 x 16 pixels of one channel, 256 threads
constexpr int kSsimTW = 32, kSsimTH = 16;
constexpr int kSsimInW = kSsimTW + 8, kSsimInH = kSsimTH + 8;     // inputs with a 4-pixel ring
constexpr int kSsimRingW = kSsimTW + 4, kSsimRingH = kSsimTH + 4; // SSIM with a 2-pixel ring

__device__ __forceinline__ float blur_tap(int d) {
  return d == 0 ? 6.0f / 16 : (d == 1 || d == -1 ? 4.0f / 16 : 1.0f / 16);
}

// 1 - SSIM of one scale and its gradient by the decoded plane, one channel
// per grid z, fused: the moments a, b, a a, b b, a b of the source a and the
// decoded b under the 5-tap binomial blur [1 4 6 4 1] / 16 (zero outside
// the plane, rows then columns), SSIM (C1 1e-4, C2 9e-4) and its partial
// derivatives by the blurred b, b b and a b on the tile and a 2-pixel ring,
// their blur (the blur is its own adjoint under zero padding), and
//   d L / d b = G(g_b) + 2 b G(g_bb) + a G(g_ab)
// into `grad` (3 planes of w x h).  L = weight * sum(1 - SSIM); the tile's
// sum goes to `sums`.
__global__ void __launch_bounds__(256) k_refine_ssim(const float* __restrict__ a_planes,
                                                     const float* __restrict__ b_planes, int w, int h,
                                                     float weight, float* __restrict__ grad,
                                                     double* __restrict__ sums) {
  __shared__ float in[2][kSsimInH][kSsimInW + 1];
  __shared__ float xm[5][kSsimInH][kSsimRingW];       // row-blurred moments; later the row-blurred grads
  __shared__ float g[3][kSsimRingH][kSsimRingW + 1];
  const int tid = threadIdx.x;
  const int x0 = blockIdx.x * kSsimTW, y0 = blockIdx.y * kSsimTH, ch = blockIdx.z;
  const int64_t n = static_cast<int64_t>(w) * h;
  const float* A = a_planes + ch * n;
  const float* B = b_planes + ch * n;
  // 0. inputs over the tile and a 4-pixel ring, zero outside the plane
  for (int u = tid; u < kSsimInH * kSsimInW; u += 256) {
    const int r = u / kSsimInW, c = u % kSsimInW;
    const int y = y0 - 4 + r, x = x0 - 4 + c;
    const bool inside = x >= 0 && x < w && y >= 0 && y < h;
    const int64_t at = static_cast<int64_t>(y) * w + x;
    in[0][r][c] = inside ? A[at] : 0.0f;
    in[1][r][c] = inside ? B[at] : 0.0f;
  }
  __syncthreads();
  // Each blur below gives a thread a run of neighbouring outputs along the
  // blur's direction, so one window of loads in registers serves the run.
  // 1. row blur of the five moments at columns -2 .. kSsimTW + 2: runs of 3
  //    columns (12 runs a row)
  constexpr int kRun1 = 3, kRuns1 = kSsimRingW / kRun1;
  static_assert(kSsimRingW % kRun1 == 0, "row runs tile the ring");
  for (int u = tid; u < kSsimInH * kRuns1; u += 256) {
    const int r = u / kRuns1, c0 = (u % kRuns1) * kRun1;
    float va[kRun1 + 4], vb[kRun1 + 4];
#pragma unroll
    for (int k = 0; k < kRun1 + 4; ++k) {
      va[k] = in[0][r][c0 + k];
      vb[k] = in[1][r][c0 + k];
    }
#pragma unroll
    for (int j = 0; j < kRun1; ++j) {
      float m[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int d = -2; d <= 2; ++d) {
        const float k = blur_tap(d), a = va[j + 2 + d], b = vb[j + 2 + d];
        m[0] = __fmaf_rn(k, a, m[0]);
        m[1] = __fmaf_rn(k, b, m[1]);
        m[2] = __fmaf_rn(k, __fmul_rn(a, a), m[2]);
        m[3] = __fmaf_rn(k, __fmul_rn(b, b), m[3]);
        m[4] = __fmaf_rn(k, __fmul_rn(a, b), m[4]);
      }
#pragma unroll
      for (int q = 0; q < 5; ++q) xm[q][r][c0 + j] = m[q];
    }
  }
  __syncthreads();
  // 2. column blur, SSIM and its derivatives on the tile and a 2-pixel ring:
  //    runs of 3 rows (7 runs a column, the last one short)
  constexpr int kRun2 = 3, kRuns2 = (kSsimRingH + kRun2 - 1) / kRun2;
  static_assert(kRuns2 * kSsimRingW <= 256, "one run per thread");
  float loss = 0.0f;
  if (tid < kRuns2 * kSsimRingW) {
    const int c = tid % kSsimRingW, r0 = (tid / kSsimRingW) * kRun2;
    float win[5][kRun2 + 4];
#pragma unroll
    for (int k = 0; k < kRun2 + 4; ++k)
#pragma unroll
      for (int q = 0; q < 5; ++q) win[q][k] = r0 + k < kSsimInH ? xm[q][r0 + k][c] : 0.0f;
#pragma unroll
    for (int j = 0; j < kRun2; ++j) {
      const int r = r0 + j;
      if (r >= kSsimRingH) break;
      const int y = y0 - 2 + r, x = x0 - 2 + c;
      float m[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int d = -2; d <= 2; ++d) {
        const float k = blur_tap(d);
#pragma unroll
        for (int q = 0; q < 5; ++q) m[q] = __fmaf_rn(k, win[q][j + 2 + d], m[q]);
      }
      float gm2 = 0.0f, gs22 = 0.0f, gs12 = 0.0f;
      if (x >= 0 && x < w && y >= 0 && y < h) {
        const float m1 = m[0], m2 = m[1];
        const float v1 = __fsub_rn(m[2], __fmul_rn(m1, m1)), v2 = __fsub_rn(m[3], __fmul_rn(m2, m2));
        const float c12 = __fsub_rn(m[4], __fmul_rn(m1, m2));
        const float n1 = __fadd_rn(__fmul_rn(2.0f, __fmul_rn(m1, m2)), kSsimC1);
        const float n2 = __fadd_rn(__fmul_rn(2.0f, c12), kSsimC2);
        const float d1 = __fadd_rn(__fadd_rn(__fmul_rn(m1, m1), __fmul_rn(m2, m2)), kSsimC1);
        const float d2 = __fadd_rn(__fadd_rn(v1, v2), kSsimC2);
        // one division: 1 / (d1 d2), and 1 / d2 = d1 / (d1 d2)
        const float inv_dd = __fdiv_rn(1.0f, __fmul_rn(d1, d2));
        const float ssim = __fmul_rn(__fmul_rn(n1, n2), inv_dd);
        if (r >= 2 && r < 2 + kSsimTH && c >= 2 && c < 2 + kSsimTW) loss += 1.0f - ssim;
        // d ssim / d m2, d s22, d s12 (the source's moments fixed)
        const float dm2 = __fmul_rn(__fsub_rn(__fmul_rn(__fmul_rn(2.0f, m1), __fsub_rn(n2, n1)),
                                              __fmul_rn(ssim, __fmul_rn(__fmul_rn(2.0f, m2), __fsub_rn(d2, d1)))),
                                    inv_dd);
        gm2 = -weight * dm2;
        gs22 = weight * __fmul_rn(ssim, __fmul_rn(d1, inv_dd));
        gs12 = -weight * __fmul_rn(__fmul_rn(2.0f, n1), inv_dd);
      }
      g[0][r][c] = gm2;
      g[1][r][c] = gs22;
      g[2][r][c] = gs12;
    }
  }
  __syncthreads();
  // 3. row blur of the derivatives (into xm, free now) at the tile's
  //    columns: runs of 4 columns
  constexpr int kRun3 = 4, kRuns3 = kSsimTW / kRun3;
  for (int u = tid; u < kSsimRingH * kRuns3; u += 256) {
    const int r = u / kRuns3, c0 = (u % kRuns3) * kRun3;
    float win[3][kRun3 + 4];
#pragma unroll
    for (int k = 0; k < kRun3 + 4; ++k)
#pragma unroll
      for (int q = 0; q < 3; ++q) win[q][k] = g[q][r][c0 + k];
#pragma unroll
    for (int j = 0; j < kRun3; ++j) {
      float v[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int d = -2; d <= 2; ++d) {
        const float k = blur_tap(d);
#pragma unroll
        for (int q = 0; q < 3; ++q) v[q] = __fmaf_rn(k, win[q][j + 2 + d], v[q]);
      }
#pragma unroll
      for (int q = 0; q < 3; ++q) xm[q][r][c0 + j] = v[q];
    }
  }
  __syncthreads();
  // 4. column blur and the gradient by the decoded plane: runs of 2 rows
  constexpr int kRun4 = 2;
  static_assert((kSsimTH / kRun4) * kSsimTW == 256, "one run per thread");
  {
    const int c = tid % kSsimTW, r0 = (tid / kSsimTW) * kRun4;
    float win[3][kRun4 + 4];
#pragma unroll
    for (int k = 0; k < kRun4 + 4; ++k)
#pragma unroll
      for (int q = 0; q < 3; ++q) win[q][k] = xm[q][r0 + k][c];
#pragma unroll
    for (int j = 0; j < kRun4; ++j) {
      const int r = r0 + j, y = y0 + r, x = x0 + c;
      if (x >= w || y >= h) continue;
      float v[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int d = -2; d <= 2; ++d) {
        const float k = blur_tap(d);
#pragma unroll
        for (int q = 0; q < 3; ++q) v[q] = __fmaf_rn(k, win[q][j + 2 + d], v[q]);
      }
      const float va = in[0][r + 4][c + 4], vb = in[1][r + 4][c + 4];
      grad[ch * n + static_cast<int64_t>(y) * w + x] =
          __fmaf_rn(va, v[2], __fmaf_rn(__fmul_rn(2.0f, vb), v[1], v[0]));
    }
  }
  refine_add_slot(loss, sums);
}

// Backward per block: the gradient by the decoded XYB (given, when the EPF
// is modelled; else from the linear planes: scale 0 plus a quarter of scale
// 1's at the covering coarse pixel, scale 1 already holding scale 2's, back
// through XYB -> linear), M^T to the coefficients, then d L / d theta.
__global__ void __launch_bounds__(256) k_refine_backward(const RefineArgs r, const float* __restrict__ theta,
                                                         const float* __restrict__ glin0,
                                                         const float* __restrict__ glin1, int w1, int h1,
                                                         const float* __restrict__ gxyb_in,
                                                         float rate_weight, float* __restrict__ gtheta) {
  __shared__ float gs[8][3][64];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t b = static_cast<int64_t>(blockIdx.x) * 8 + warp;
  if (b >= static_cast<int64_t>(r.xb) * r.yb) return;
  const int bx = static_cast<int>(b % r.xb), by = static_cast<int>(b / r.xb);
  const int64_t pp = static_cast<int64_t>(r.pw) * r.yb * 8, n = static_cast<int64_t>(r.w) * r.h;
  const int64_t n1 = static_cast<int64_t>(w1) * h1;
#pragma unroll
  for (int h2 = 0; h2 < 2; ++h2) {
    const int p = lane + 32 * h2;
    const int y = by * 8 + (p >> 3), x = bx * 8 + (p & 7);
    float gx[3] = {0.0f, 0.0f, 0.0f};
    if (x < r.w && y < r.h && gxyb_in) {  // through the EPF's adjoint already
      const int64_t q = static_cast<int64_t>(y) * r.w + x;
#pragma unroll
      for (int k = 0; k < 3; ++k) gx[k] = gxyb_in[k * n + q];
    } else if (x < r.w && y < r.h) {
      const int64_t q = static_cast<int64_t>(y) * r.w + x;
      float gl[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) gl[k] = glin0[k * n + q];
      if ((y >> 1) < h1 && (x >> 1) < w1) {
        const int64_t q1 = static_cast<int64_t>(y >> 1) * w1 + (x >> 1);
#pragma unroll
        for (int k = 0; k < 3; ++k) gl[k] = __fmaf_rn(0.25f, glin1[k * n1 + q1], gl[k]);
      }
      const int64_t at = static_cast<int64_t>(y) * r.pw + x;
      float o[3], dc[3];
      xyb_to_linear(r.recon[at], r.recon[pp + at], r.recon[2 * pp + at], o, dc);
      float gm[3];
#pragma unroll
      for (int k = 0; k < 3; ++k)
        gm[k] = __fmul_rn(dc[k], __fmaf_rn(kOpsinInverse[k], gl[0],
                                           __fmaf_rn(kOpsinInverse[3 + k], gl[1],
                                                     __fmul_rn(kOpsinInverse[6 + k], gl[2]))));
      // t0 = y + x, t1 = y - x, t2 = b
      gx[0] = __fsub_rn(gm[0], gm[1]);
      gx[1] = __fadd_rn(gm[0], gm[1]);
      gx[2] = gm[2];
    }
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) gs[warp][ch][p] = gx[ch];
  }
  __syncwarp();
  const float s = refine_s(r, b, theta[b]);
  float xf, bf;
  refine_cfl(r, bx, by, &xf, &bf);
  float acc = 0.0f;
#pragma unroll
  for (int h2 = 0; h2 < 2; ++h2) {
    const int i = lane + 32 * h2;
    if (i == 0) continue;  // the DC slot keeps the source value
    float gc[3] = {0.0f, 0.0f, 0.0f};
    for (int p = 0; p < 64; ++p) {
      const float m = r.m[p * 64 + i];
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) gc[ch] = __fmaf_rn(m, gs[warp][ch][p], gc[ch]);
    }
    const float* c = r.coef + b * 192;
    CoefState st;
    refine_coef(r, i, s, xf, bf, c[i], c[64 + i], c[128 + i], true, &st);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) acc = __fmaf_rn(gc[ch], st.dhat[ch], acc);
    acc = __fmaf_rn(rate_weight, st.dbits, acc);
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, d);
  if (lane == 0) gtheta[b] = __fmul_rn(acc, s);  // ds / dtheta = s
}

// ---------------------------------------------------------------------------
// The reference's six-term luma proxy as a distortion term (LumaProxy,
// src/epf_proxy.rs:132-214; box moments src/epf_proxy/box_filter.rs:84-240;
// pool and gradients src/epf_proxy/row_kernels.rs:60-115), on the decoded
// XYB Y plane against the source's, with its adjoint.  The box moments use
// the reference's running sums in its order (the moments' variances cancel,
// so their rounding shows in the score); the pools are parallel sums.
// ---------------------------------------------------------------------------

// src/epf_proxy.rs:186-193
__constant__ const float kProxyWeights[6] = {109.4163228369586f, 4.685925102200196f, 2.491781270704224f,
                                             2.167275675983448f, 4.55227651921194f,  2.847714678987977f};
constexpr int kProxySums = 7;  // half s, half s^4, quarter s, quarter s^4, error, excess, loss^4

__device__ __forceinline__ int proxy_mirror(int i, int n) {  // src/epf_proxy.rs:17-28
  if (i >= 0 && i < n) return i;
  i %= 2 * n;
  if (i < 0) i += 2 * n;
  return i < n ? i : 2 * n - i - 1;
}

// 2x2 means (half / half_y, row_kernels.rs:60-71), +0.01 a tap with `bias`.
__global__ void __launch_bounds__(256) k_proxy_half(const float* __restrict__ in, int in_stride, int w, int h,
                                                    int bias, float* __restrict__ out) {
  const int w2 = w / 2, h2 = h / 2;
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= static_cast<int64_t>(w2) * h2) return;
  const int x = static_cast<int>(q % w2), y = static_cast<int>(q / w2);
  const float* r0 = in + static_cast<int64_t>(2 * y) * in_stride + 2 * x;
  const float* r1 = r0 + in_stride;
  const float b = bias ? 0.01f : 0.0f;
  float t00 = r0[0], t01 = r0[1], t10 = r1[0], t11 = r1[1];
  if (bias) {
    t00 = __fadd_rn(t00, b);
    t01 = __fadd_rn(t01, b);
    t10 = __fadd_rn(t10, b);
    t11 = __fadd_rn(t11, b);
  }
  out[q] = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(__fadd_rn(t00, t10), t01), t11));
}

// Vertical pass of the reflected 5x5 box (x 0.2) of t, t^2 and, with `ref`,
// ref * t (2 or 3 planes of w x h into `out`), one thread per column walking
// down it with the reference's running sums (Scratch::run, accumulate and
// step, src/epf_proxy/box_filter.rs:84-226): the sums start at -0 over rows
// -2..2, each output row is sum x 0.2, then the entering row minus the
// leaving one is added (a a - b b for the squares, ra a - rb b for the cross).
__global__ void __launch_bounds__(128) k_proxy_box_v(const float* __restrict__ t, const float* __restrict__ ref,
                                                     int w, int h, float* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= w) return;
  const int64_t n = static_cast<int64_t>(w) * h;
  auto at = [&](int y) { return static_cast<int64_t>(proxy_mirror(y, h)) * w + x; };
  float m = -0.0f, sq = -0.0f, cr = -0.0f;
  for (int d = -2; d <= 2; ++d) {
    const float v = t[at(d)];
    m = __fadd_rn(m, v);
    sq = __fadd_rn(sq, __fmul_rn(v, v));
    if (ref) cr = __fadd_rn(cr, __fmul_rn(ref[at(d)], v));
  }
  for (int y = 0; y < h; ++y) {
    const int64_t q = static_cast<int64_t>(y) * w + x;
    out[q] = __fmul_rn(m, 0.2f);
    out[n + q] = __fmul_rn(sq, 0.2f);
    if (ref) out[2 * n + q] = __fmul_rn(cr, 0.2f);
    if (y + 1 < h) {
      const int64_t ea = at(y + 3), lb = at(y - 2);
      const float a = t[ea], b = t[lb];
      m = __fadd_rn(m, __fsub_rn(a, b));
      sq = __fadd_rn(sq, __fsub_rn(__fmul_rn(a, a), __fmul_rn(b, b)));
      if (ref) cr = __fadd_rn(cr, __fsub_rn(__fmul_rn(ref[ea], a), __fmul_rn(ref[lb], b)));
    }
  }
}

// Horizontal pass (x 0.2) of `count` planes, one thread per row with the
// running sum of `horizontal_scalar` (box_filter.rs:228-240).
__global__ void __launch_bounds__(128) k_proxy_box_h(const float* __restrict__ in, int count, int w, int h,
                                                     float* __restrict__ out) {
  const int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= static_cast<int64_t>(count) * h) return;
  const float* row = in + r * w;
  float* dst = out + r * w;
  float sum = 0.0f;
  for (int d = -2; d <= 2; ++d) sum = __fadd_rn(sum, row[proxy_mirror(d, w)]);
  for (int x = 0; x < w; ++x) {
    dst[x] = __fmul_rn(sum, 0.2f);
    if (x + 1 < w) sum = __fadd_rn(sum, __fsub_rn(row[proxy_mirror(x + 3, w)], row[proxy_mirror(x - 2, w)]));
  }
}

// The same two passes as direct 5-tap sums, one thread per output: the
// refinement's model (the box's values to rounding, fully parallel; the
// running sums above keep the reference's rounding for the operators).
__global__ void __launch_bounds__(256) k_proxy_box_v_par(const float* __restrict__ t, const float* __restrict__ ref,
                                                         int w, int h, float* __restrict__ out) {
  const int64_t n = static_cast<int64_t>(w) * h;
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int x = static_cast<int>(q % w), y = static_cast<int>(q / w);
  float m = 0.0f, sq = 0.0f, cr = 0.0f;
#pragma unroll
  for (int d = -2; d <= 2; ++d) {
    const int64_t at = static_cast<int64_t>(proxy_mirror(y + d, h)) * w + x;
    const float v = t[at];
    m = __fadd_rn(m, v);
    sq = __fadd_rn(sq, __fmul_rn(v, v));
    if (ref) cr = __fadd_rn(cr, __fmul_rn(ref[at], v));
  }
  out[q] = __fmul_rn(m, 0.2f);
  out[n + q] = __fmul_rn(sq, 0.2f);
  if (ref) out[2 * n + q] = __fmul_rn(cr, 0.2f);
}
__global__ void __launch_bounds__(256) k_proxy_box_h_par(const float* __restrict__ in, int count, int w, int h,
                                                         float* __restrict__ out) {
  const int64_t n = static_cast<int64_t>(w) * h;
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= n * count) return;
  const int64_t c = q / n, p = q % n;
  const int x = static_cast<int>(p % w), y = static_cast<int>(p / w);
  const float* row = in + c * n + static_cast<int64_t>(y) * w;
  float s = 0.0f;
#pragma unroll
  for (int d = -2; d <= 2; ++d) s = __fadd_rn(s, row[proxy_mirror(x + d, w)]);
  out[q] = __fmul_rn(s, 0.2f);
}

// The source level's variance max(E[t^2] - mean^2, 0) (variance,
// row_kernels.rs:81-85), in place of the box's second plane.
__global__ void __launch_bounds__(256) k_proxy_variance(float* __restrict__ moments, int64_t n) {
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float m = moments[q];
  moments[n + q] = fmaxf(__fsub_rn(moments[n + q], __fmul_rn(m, m)), 0.0f);
}

// The per-pixel structure loss s (pool, row_kernels.rs:86-103) of the test
// moments against the source's mean and variance; s and s^4 summed into two
// slot sets; the partial derivatives of s by the test mean, E[t^2] and
// E[ref t] into `parts` (3 planes).
__global__ void __launch_bounds__(256) k_proxy_pool(const float* __restrict__ ref_mv, const float* __restrict__ box,
                                                    int64_t n, float* __restrict__ s_out, float* __restrict__ parts,
                                                    double* __restrict__ sums) {
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  float sv = 0.0f, s4 = 0.0f;
  if (q < n) {
    const float a = ref_mv[q], vr = ref_mv[n + q];
    const float b = box[q], sq = box[n + q], cross = box[2 * n + q];
    const float vraw = __fsub_rn(sq, __fmul_rn(b, b));
    const float var = fmaxf(vraw, 0.0f);
    const bool cov_on = !(vr == 0.0f || var == 0.0f);
    const float cov = cov_on ? __fsub_rn(cross, __fmul_rn(a, b)) : 0.0f;
    const float dab = __fsub_rn(a, b);
    const float e1 = __fsub_rn(1.0f, __fmul_rn(dab, dab));
    const float num = __fadd_rn(__fmul_rn(2.0f, cov), 0.0009f);
    const float den = __fadd_rn(__fadd_rn(vr, var), 0.0009f);
    const float raw = __fsub_rn(1.0f, __fdiv_rn(__fmul_rn(e1, num), den));
    sv = fmaxf(raw, 0.0f);
    float pb = 0.0f, psq = 0.0f, pc = 0.0f;
    if (raw > 0.0f) {
      // s = 1 - e1 N / D: ds = -(de1 N / D + e1 dN / D - e1 N dD / D^2)
      const float inv_d = __fdiv_rn(1.0f, den);
      const float ratio = __fmul_rn(__fmul_rn(e1, num), __fmul_rn(inv_d, inv_d));  // e1 N / D^2
      const float dvar_on = vraw > 0.0f ? 1.0f : 0.0f;
      // d/db: de1 = 2 (a - b), dN = -2a (cov on), dD = -2b (var on)
      pb = -(__fmul_rn(__fmul_rn(2.0f, dab), __fmul_rn(num, inv_d)) +
             (cov_on ? __fmul_rn(e1, __fmul_rn(-2.0f * a, inv_d)) : 0.0f) -
             __fmul_rn(ratio, __fmul_rn(-2.0f * b, dvar_on)));
      psq = __fmul_rn(ratio, dvar_on);                                  // dD/dsq = 1
      pc = cov_on ? -__fmul_rn(e1, __fmul_rn(2.0f, inv_d)) : 0.0f;     // dN/dcross = 2
    }
    s_out[q] = sv;
    parts[q] = pb;
    parts[n + q] = psq;
    parts[2 * n + q] = pc;
    const float s2 = __fmul_rn(sv, sv);
    s4 = __fmul_rn(__fmul_rn(s2, sv), sv);
  }
  refine_add_slot(sv, sums);
  refine_add_slot(s4, sums + kRefineSlots);
}

// The full-resolution gradient terms (src/epf_proxy.rs:216-247): each pixel
// takes its pairs with the right and the lower neighbour.
__device__ __forceinline__ float proxy_pair(float a, float b, float* err, float* exc) {
  *err = fabsf(__fsub_rn(b, a));
  *exc = fmaxf(__fsub_rn(fabsf(b), fabsf(a)), 0.0f);
  const float l = fmaxf(__fsub_rn(fabsf(a), fabsf(b)), 0.0f);
  const float l2 = __fmul_rn(l, l);
  return __fmul_rn(__fmul_rn(l2, l), l);
}
__global__ void __launch_bounds__(256) k_proxy_gradients(const float* __restrict__ src, const float* __restrict__ test,
                                                         int test_stride, int w, int h, double* __restrict__ sums) {
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  float err = 0.0f, exc = 0.0f, l4 = 0.0f;
  if (q < static_cast<int64_t>(w) * h) {
    const int x = static_cast<int>(q % w), y = static_cast<int>(q / w);
    const float s0 = src[q], t0 = test[static_cast<int64_t>(y) * test_stride + x];
    float e, x2;
    if (x + 1 < w) {
      l4 = __fadd_rn(l4, proxy_pair(__fsub_rn(src[q + 1], s0),
                                    __fsub_rn(test[static_cast<int64_t>(y) * test_stride + x + 1], t0), &e, &x2));
      err = __fadd_rn(err, e);
      exc = __fadd_rn(exc, x2);
    }
    if (y + 1 < h) {
      l4 = __fadd_rn(l4, proxy_pair(__fsub_rn(src[q + w], s0),
                                    __fsub_rn(test[static_cast<int64_t>(y + 1) * test_stride + x], t0), &e, &x2));
      err = __fadd_rn(err, e);
      exc = __fadd_rn(exc, x2);
    }
  }
  refine_add_slot(err, sums);
  refine_add_slot(exc, sums + kRefineSlots);
  refine_add_slot(l4, sums + 2 * kRefineSlots);
}

// The scalars the adjoint needs, from the slot sums: per level the weight of
// a pixel's s and of its s^3 (the 4th-root pool), and the gradient terms'.
struct ProxyScalars {
  float g_s[2], g_s3[2];   // half, quarter
  float g_err, g_exc, g_l3;
};
__global__ void k_proxy_finalize(const double* __restrict__ sums, double n2, double n4, double npairs,
                                 float weight, ProxyScalars* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double t[kProxySums];
  for (int k = 0; k < kProxySums; ++k) {
    t[k] = 0.0;
    for (int j = 0; j < kRefineSlots; ++j) t[k] += sums[k * kRefineSlots + j];
  }
  // terms: qs0 = S_q / n4 (w 0), hs0 = S_h / n2 (w 1), hs1 = (S4_h / n2)^(1/4) (w 2),
  // error / np (w 3), excess / np (w 4), (L4 / np)^(1/4) (w 5)
  const double f_h = t[1] / n2;
  out->g_s[0] = static_cast<float>(weight * kProxyWeights[1] / n2);
  out->g_s3[0] = f_h > 0.0 ? static_cast<float>(weight * kProxyWeights[2] / (n2 * pow(f_h, 0.75))) : 0.0f;
  out->g_s[1] = static_cast<float>(weight * kProxyWeights[0] / n4);
  out->g_s3[1] = 0.0f;
  out->g_err = static_cast<float>(weight * kProxyWeights[3] / npairs);
  out->g_exc = static_cast<float>(weight * kProxyWeights[4] / npairs);
  const double f_l = t[6] / npairs;
  out->g_l3 = f_l > 0.0 ? static_cast<float>(weight * kProxyWeights[5] / (npairs * pow(f_l, 0.75))) : 0.0f;
}

// d L / d (test mean, E[t^2], E[ref t]) of one level: gs times the parts.
__global__ void __launch_bounds__(256) k_proxy_pool_grad(const float* __restrict__ s_map, const float* __restrict__ parts,
                                                         int64_t n, const ProxyScalars* __restrict__ k, int level,
                                                         float* __restrict__ g) {
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float sv = s_map[q];
  const float gs = __fadd_rn(k->g_s[level], __fmul_rn(k->g_s3[level], __fmul_rn(__fmul_rn(sv, sv), sv)));
#pragma unroll
  for (int c = 0; c < 3; ++c) g[c * n + q] = __fmul_rn(gs, parts[c * n + q]);
}

// The adjoint of one reflected 5-tap pass (x 0.2) along x (dir 0) or y (1):
// g_in(j) = 0.2 sum over outputs o and taps d with mirror(o + d) = j.
__device__ __forceinline__ float proxy_box_adjoint_1d(const float* __restrict__ g, int j, int n, int64_t step) {
  float acc = 0.0f;
  if (j >= 2 && j < n - 2) {
#pragma unroll
    for (int d = -2; d <= 2; ++d) acc = __fadd_rn(acc, g[static_cast<int64_t>(j - d) * step]);
    return __fmul_rn(acc, 0.2f);
  }
  // near an edge: every output within 4 whose taps reflect onto j
  for (int o = j - 4 < 0 ? 0 : j - 4; o <= j + 4 && o < n; ++o)
#pragma unroll
    for (int d = -2; d <= 2; ++d)
      if (proxy_mirror(o + d, n) == j) acc = __fadd_rn(acc, g[static_cast<int64_t>(o) * step]);
  return __fmul_rn(acc, 0.2f);
}
__global__ void __launch_bounds__(256) k_proxy_box_adjoint_h(const float* __restrict__ g, int w, int h,
                                                             float* __restrict__ out) {
  const int64_t n = static_cast<int64_t>(w) * h;
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= 3 * n) return;
  const int64_t c = q / n, p = q % n;
  const int x = static_cast<int>(p % w), y = static_cast<int>(p / w);
  out[q] = proxy_box_adjoint_1d(g + c * n + static_cast<int64_t>(y) * w, x, w, 1);
}
// ... then the vertical adjoint, and the test plane's gradient:
// g_t = A(g_mean) + 2 t A(g_sq) + ref A(g_cross), added to `gt`.
__global__ void __launch_bounds__(256) k_proxy_box_adjoint_v(const float* __restrict__ g, const float* __restrict__ t,
                                                             const float* __restrict__ ref, int w, int h,
                                                             float* __restrict__ gt) {
  const int64_t n = static_cast<int64_t>(w) * h;
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int x = static_cast<int>(q % w), y = static_cast<int>(q / w);
  const float am = proxy_box_adjoint_1d(g + x, y, h, w);
  const float asq = proxy_box_adjoint_1d(g + n + x, y, h, w);
  const float acr = proxy_box_adjoint_1d(g + 2 * n + x, y, h, w);
  gt[q] = __fadd_rn(gt[q], __fmaf_rn(ref[q], acr, __fmaf_rn(__fmul_rn(2.0f, t[q]), asq, am)));
}

// A level's gradient into the finer level: each of the four pixels under a
// coarse pixel takes a quarter (the +0.01 bias is a constant).
__global__ void __launch_bounds__(256) k_proxy_up(const float* __restrict__ gc, int wc, int hc,
                                                  float* __restrict__ gf, int wf, int hf, int f_stride) {
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= static_cast<int64_t>(wf) * hf) return;
  const int x = static_cast<int>(q % wf), y = static_cast<int>(q / wf);
  if ((x >> 1) >= wc || (y >> 1) >= hc) return;
  float* at = gf + static_cast<int64_t>(y) * f_stride + x;
  *at = __fadd_rn(*at, __fmul_rn(0.25f, gc[static_cast<int64_t>(y >> 1) * wc + (x >> 1)]));
}

// The gradient terms' adjoint at each test pixel (the pairs it belongs to),
// added to `gt` (row stride `g_stride`).
__device__ __forceinline__ float proxy_pair_grad(float a, float b, const ProxyScalars& k) {
  // d/db of g_err |b - a| + g_exc max(|b| - |a|, 0) + (L4 pool) max(|a| - |b|, 0)^4
  float g = __fmul_rn(k.g_err, b > a ? 1.0f : (b < a ? -1.0f : 0.0f));
  const float sb = b > 0.0f ? 1.0f : (b < 0.0f ? -1.0f : 0.0f);
  if (fabsf(b) > fabsf(a)) g = __fadd_rn(g, __fmul_rn(k.g_exc, sb));
  const float l = __fsub_rn(fabsf(a), fabsf(b));
  if (l > 0.0f) g = __fsub_rn(g, __fmul_rn(k.g_l3, __fmul_rn(__fmul_rn(l, l), __fmul_rn(l, sb))));
  return g;
}
__global__ void __launch_bounds__(256) k_proxy_gradients_adjoint(const float* __restrict__ src,
                                                                 const float* __restrict__ test, int test_stride,
                                                                 int w, int h, const ProxyScalars* __restrict__ ks,
                                                                 float* __restrict__ gt, int g_stride) {
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= static_cast<int64_t>(w) * h) return;
  const ProxyScalars k = *ks;
  const int x = static_cast<int>(q % w), y = static_cast<int>(q / w);
  auto T = [&](int xx, int yy) { return test[static_cast<int64_t>(yy) * test_stride + xx]; };
  auto S = [&](int xx, int yy) { return src[static_cast<int64_t>(yy) * w + xx]; };
  float g = 0.0f;
  // b = t(right) - t(here): d b / d t(here) = -1, as the right member +1
  if (x + 1 < w) g = __fsub_rn(g, proxy_pair_grad(__fsub_rn(S(x + 1, y), S(x, y)), __fsub_rn(T(x + 1, y), T(x, y)), k));
  if (x > 0) g = __fadd_rn(g, proxy_pair_grad(__fsub_rn(S(x, y), S(x - 1, y)), __fsub_rn(T(x, y), T(x - 1, y)), k));
  if (y + 1 < h) g = __fsub_rn(g, proxy_pair_grad(__fsub_rn(S(x, y + 1), S(x, y)), __fsub_rn(T(x, y + 1), T(x, y)), k));
  if (y > 0) g = __fadd_rn(g, proxy_pair_grad(__fsub_rn(S(x, y), S(x, y - 1)), __fsub_rn(T(x, y), T(x, y - 1)), k));
  float* at = gt + static_cast<int64_t>(y) * g_stride + x;
  *at = __fadd_rn(*at, g);
}

// The refined field: qf * exp(theta), rounded, 1..255.
__global__ void __launch_bounds__(256) k_refine_field(const uint8_t* __restrict__ qf, const float* __restrict__ theta,
                                                      int64_t nb, uint8_t* __restrict__ out) {
  const int64_t b = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const float v = __fmul_rn(static_cast<float>(qf[b]), expf(theta[b]));
  out[b] = static_cast<uint8_t>(fminf(fmaxf(rintf(v), 1.0f), 255.0f));
}

// One Adam step on theta (beta 0.9 / 0.999, eps 1e-8; c1, c2 the bias
// corrections), clamped so that qf * exp(theta) stays within 1..255.
constexpr double kAdamBeta1 = 0.9, kAdamBeta2 = 0.999;
__global__ void __launch_bounds__(256) k_refine_adam(const uint8_t* __restrict__ qf, const float* __restrict__ g,
                                                     int64_t nb, float lr, float c1, float c2,
                                                     float* __restrict__ mv, float* __restrict__ theta) {
  const int64_t b = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const float gv = g[b];
  const float m = __fmaf_rn(0.9f, mv[b], 0.1f * gv);
  const float v = __fmaf_rn(0.999f, mv[nb + b], 0.001f * gv * gv);
  mv[b] = m;
  mv[nb + b] = v;
  const float q = static_cast<float>(qf[b]);
  const float t = theta[b] - lr * (m * c1) / (sqrtf(v * c2) + 1e-8f);
  theta[b] = fminf(fmaxf(t, logf(1.0f / q)), logf(255.0f / q));
}

}  // namespace jxg
