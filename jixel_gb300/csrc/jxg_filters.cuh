// Gaborish over the three XYB planes:
//   k_gaborish_inverse  the encoder's pre-inversion (gaborish_inverse,
//                       src/gaborish.rs:44-258): a symmetric 5x5 with
//                       mirror-reflected neighbours, every output from the
//                       source pixels;
//   k_gaborish          the decoder's forward 3x3 (src/epf_filter.rs:163-188,
//                       gaborish_pixel src/epf_filter/kernels.rs:134-145) with
//                       clamped neighbours.
// A CTA stages a 32x8 tile of one channel with its ring of neighbours (each
// staged sample at its own reflected or clamped coordinate, so a pixel's
// neighbour is the one the reference reads), then one thread per pixel sums
// in the reference's order.
#pragma once

namespace jxg {

struct GaborishWeights {
  float w[6];  // inverse: centre, r, d, R, L, D; forward: norm, W1 norm, W2 norm
};

__device__ __forceinline__ int gab_reflect(int i, int len) {
  while (i < 0 || i >= len) i = i < 0 ? -i - 1 : 2 * len - i - 1;
  return i;
}

constexpr int kGabTileX = 32, kGabTileY = 8, kGabThreads = kGabTileX * kGabTileY;

__global__ void __launch_bounds__(kGabThreads) k_gaborish_inverse(const float* __restrict__ in,
                                                                  float* __restrict__ out, int w, int h,
                                                                  GaborishWeights k) {
  __shared__ float t[kGabTileY + 4][kGabTileX + 5];
  const int64_t plane = static_cast<int64_t>(w) * h;
  const float* p = in + blockIdx.z * plane;
  const int x0 = blockIdx.x * kGabTileX, y0 = blockIdx.y * kGabTileY;
  for (int i = threadIdx.x; i < (kGabTileY + 4) * (kGabTileX + 4); i += kGabThreads) {
    const int ty = i / (kGabTileX + 4), tx = i % (kGabTileX + 4);
    const int y = gab_reflect(y0 + ty - 2, h), x = gab_reflect(x0 + tx - 2, w);
    t[ty][tx] = __ldg(p + static_cast<int64_t>(y) * w + x);
  }
  __syncthreads();
  const int tx = threadIdx.x % kGabTileX + 2, ty = threadIdx.x / kGabTileX + 2;
  const int x = x0 + tx - 2, y = y0 + ty - 2;
  if (x >= w || y >= h) return;
  const float* rm2 = t[ty - 2];
  const float* rm1 = t[ty - 1];
  const float* r0 = t[ty];
  const float* rp1 = t[ty + 1];
  const float* rp2 = t[ty + 2];
  const float s_r = __fadd_rn(__fadd_rn(__fadd_rn(rm1[tx], rp1[tx]), r0[tx - 1]), r0[tx + 1]);
  const float s_d = __fadd_rn(__fadd_rn(__fadd_rn(rm1[tx - 1], rm1[tx + 1]), rp1[tx - 1]), rp1[tx + 1]);
  const float s_r2 = __fadd_rn(__fadd_rn(__fadd_rn(rm2[tx], rp2[tx]), r0[tx - 2]), r0[tx + 2]);
  const float s_d2 = __fadd_rn(__fadd_rn(__fadd_rn(rm2[tx - 2], rm2[tx + 2]), rp2[tx - 2]), rp2[tx + 2]);
  float s_l = __fadd_rn(rm2[tx - 1], rm2[tx + 1]);
  s_l = __fadd_rn(s_l, rm1[tx - 2]);
  s_l = __fadd_rn(s_l, rm1[tx + 2]);
  s_l = __fadd_rn(s_l, rp1[tx - 2]);
  s_l = __fadd_rn(s_l, rp1[tx + 2]);
  s_l = __fadd_rn(s_l, rp2[tx - 1]);
  s_l = __fadd_rn(s_l, rp2[tx + 1]);
  float acc = __fmul_rn(k.w[0], r0[tx]);
  acc = __fmaf_rn(k.w[1], s_r, acc);
  acc = __fmaf_rn(k.w[2], s_d, acc);
  acc = __fmaf_rn(k.w[3], s_r2, acc);
  acc = __fmaf_rn(k.w[5], s_d2, acc);
  acc = __fmaf_rn(k.w[4], s_l, acc);
  out[blockIdx.z * plane + static_cast<int64_t>(y) * w + x] = acc;
}

__global__ void __launch_bounds__(kGabThreads) k_gaborish(const float* __restrict__ in,
                                                          float* __restrict__ out, int w, int h,
                                                          GaborishWeights k) {
  __shared__ float t[kGabTileY + 2][kGabTileX + 3];
  const int64_t plane = static_cast<int64_t>(w) * h;
  const float* p = in + blockIdx.z * plane;
  const int x0 = blockIdx.x * kGabTileX, y0 = blockIdx.y * kGabTileY;
  for (int i = threadIdx.x; i < (kGabTileY + 2) * (kGabTileX + 2); i += kGabThreads) {
    const int ty = i / (kGabTileX + 2), tx = i % (kGabTileX + 2);
    const int y = min(max(y0 + ty - 1, 0), h - 1), x = min(max(x0 + tx - 1, 0), w - 1);
    t[ty][tx] = __ldg(p + static_cast<int64_t>(y) * w + x);
  }
  __syncthreads();
  const int tx = threadIdx.x % kGabTileX + 1, ty = threadIdx.x / kGabTileX + 1;
  const int x = x0 + tx - 1, y = y0 + ty - 1;
  if (x >= w || y >= h) return;
  const float* tr = t[ty - 1];
  const float* m = t[ty];
  const float* b = t[ty + 1];
  const float side = __fadd_rn(__fadd_rn(m[tx - 1], m[tx + 1]), __fadd_rn(tr[tx], b[tx]));
  const float corner = __fadd_rn(__fadd_rn(tr[tx - 1], tr[tx + 1]), __fadd_rn(b[tx - 1], b[tx + 1]));
  out[blockIdx.z * plane + static_cast<int64_t>(y) * w + x] =
      __fmaf_rn(corner, k.w[2], __fmaf_rn(side, k.w[1], __fmul_rn(m[tx], k.w[0])));
}

}  // namespace jxg
