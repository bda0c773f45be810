// C ABI of the GB300 VarDCT front end: contexts, passes (one frame or a
// batch of frames), launches and result fetch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/jxg.h"
#include "frame_params.h"
#include "jxg_kernels.cuh"
#include "jxg_search.cuh"
#include "jxg_filters.cuh"
#include "jxg_refine.cuh"

namespace jxg {
namespace {

constexpr uint64_t kMaxDimension = 0x3FFFFFFFull;  // MAX_DIMENSION, src/encode_image.rs:99
constexpr size_t kHistBytes = static_cast<size_t>(kNumFineAcContexts) * kAlphabet * 4;

struct DevBuf {
  void* ptr = nullptr;
  size_t cap = 0;
};

struct HostBuf {  // pinned host staging
  void* ptr = nullptr;
  size_t cap = 0;
};

struct TimedKernel {
  double total_ms = 0.0;
  uint64_t launches = 0;
};

struct PendingEvent {
  const char* name;
  cudaEvent_t start, stop;
};

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Work prefixes in a plan: XYB chunks, tiles, token chunks, RGBA tiles,
// invisible-fill tiles.
constexpr int kPlanPrefixes = 5;

// Invisible-fill tiles of a w x h frame (32-row bands of sheared 32-column
// tiles, as the fill kernel walks them).
inline int64_t fill_tiles(uint64_t w, uint64_t h) {
  return static_cast<int64_t>((h + kFillBand - 1) / kFillBand) *
         static_cast<int64_t>((w + kFillBand - 1 + kFillCols - 1) / kFillCols);
}

}  // namespace

// Bytes of one sample: 8-bit samples, or 10/12/16-bit ones in 16-bit words.
inline size_t sample_bytes(int32_t bits) { return bits > 8 ? 2 : 1; }

// One image of a pass as the caller describes it.
struct PassImage {
  const void* pixels;
  uint64_t width, height;
  int32_t channels, bits;
  jxg_config config;
};

// Token chunks of one frame: runs of up to kTokenChunk blocks in token order
// (each group's blocks in raster order), as the tokenizer's chunk_place
// enumerates them.
int64_t token_chunks_of(const jxg_frame_info& fi) {
  auto per_group = [](uint64_t w, uint64_t h) {
    return static_cast<int64_t>((w * h + kTokenChunk - 1) / kTokenChunk);
  };
  const uint64_t gxn = fi.xsize_groups, gyn = fi.ysize_groups;
  const uint64_t gw_last = fi.xsize_blocks - (gxn - 1) * kGroupBlocks;
  const uint64_t gh_last = fi.ysize_blocks - (gyn - 1) * kGroupBlocks;
  const int64_t full_row = static_cast<int64_t>(gxn - 1) * per_group(kGroupBlocks, kGroupBlocks) +
                           per_group(gw_last, kGroupBlocks);
  const int64_t last_row = static_cast<int64_t>(gxn - 1) * per_group(kGroupBlocks, gh_last) +
                           per_group(gw_last, gh_last);
  return static_cast<int64_t>(gyn - 1) * full_row + last_row;
}

// Where one frame of the last pass lives, for fetching its results.
struct FrameLayout {
  uint64_t width = 0, height = 0;
  DistanceParams dp{};
  jxg_frame_info info{};
  int64_t plane = 0;
  size_t pix_off = 0, xyb_off = 0, block_off = 0, tile_off = 0, group_off = 0, count_off = 0;
  bool has_alpha = false;
  size_t alpha_off = 0, alpha_block_off = 0;  // RGBA frames only
  bool searched = false;  // Speed::Fastest's transform search ran on this frame
};

struct Context {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::string last_error;
  // constant tables
  // transfer tables on the device, one per (bits, transfer) in use:
  // 256 floats for 8-bit samples, 65536 otherwise
  std::map<int, float*> luts;
  float* d_exp2 = nullptr;      // fast_exp2 table, 64
  uint8_t* d_pos = nullptr;     // natural 8x8 order, raw index -> scan position
  uint8_t* d_pos_identity = nullptr;  // raw index -> itself (layout levels are in raw order)
  float* d_rate_log2 = nullptr;       // log2(1 + i), kRateLog2Entries
  // Speed::Fastest: search tables per distance, the frame's SearchFrame and
  // the search's pass buffers
  std::map<uint32_t, SearchTables*> search_tables;
  SearchFrame search_host{};
  DevBuf search_frame, search_costs, search_map, search_bqf, search_dp, search_sites, search_loss;
  // pass buffers (grown, never shrunk)
  DevBuf pixels, xyb, qf, ytox, ytob, quant_dc, levels, wide_levels, coeffs, nzeros, nz_packed,
      counts, tokens, hist, stats, group_offsets, plan, total, op_in, op_out,
      alpha, alpha_peak, alpha_zero, fill_flags, fill_deps, fill_queue, fill_masks, group_wide,
      packed, packed_offs, tok_status;
  HostBuf plan_host, pixels_host;
  // The plan (frame descriptors + chunk prefixes) lives in a ring of slots,
  // pinned on the host and mirrored on the device, so a pass can be planned
  // while earlier passes that were only enqueued still wait for their upload.
  static constexpr int kPlanSlots = 4;
  size_t plan_slot_cap = 0;
  int plan_slot = 0;
  cudaEvent_t plan_uploaded[kPlanSlots] = {};
  // last pass
  std::vector<FrameLayout> layouts;
  int64_t total_tiles = 0, xyb_chunks = 0, token_chunks = 0, total_counts = 0, total_groups = 0;
  int64_t alpha_tiles = 0;  // 64x64 tiles of the pass's RGBA frames
  int64_t fill_tiles = 0;   // invisible-fill tiles of the pass's RGBA frames
  int num_sms = 0;
  size_t frames_bytes = 0, pixel_bytes = 0;
  bool have_frame = false;
  uint64_t epoch = 0;  // bumped by every plan: batches recorded earlier re-plan
  // a caller's quant field for the next single-frame UltraFast pass (device
  // memory), replacing the adaptive field after its stage
  const uint8_t* qf_override = nullptr;
  // quant-field refinement of the last UltraFast frame (jxg_refine_*)
  bool refine_ready = false;
  jxg::RefineArgs refine{};
  int64_t refine_n[3] = {0, 0, 0};  // pixels per scale
  int refine_w[3] = {0, 0, 0}, refine_h[3] = {0, 0, 0};
  DevBuf refine_buf;
  float* refine_lin[2][3] = {};  // source / decoded linear RGB per scale
  float* refine_glin[3] = {};     // the loss's gradient by the decoded planes per scale
  double* refine_sums = nullptr;  // 4 x kRefineSlots partial sums
  DevBuf refine_levels;           // levels, when a caller asks for them
  // the EPF model: each stage's output and weights, the adjoint's ping-pong
  float* refine_epf_out[3] = {};
  float* refine_epf_nw[3] = {};
  float* refine_epf_cw[3] = {};
  float* refine_epf_g[2] = {};   // the decoded-XYB gradient (EPF or proxy), ping-pong
  // the distortion's mix: weight of 1 - SSIM and of the luma proxy
  float refine_w_ssim = 1.0f, refine_w_proxy = 0.1f;
  bool refine_proxy = false;  // the frame is large enough for the proxy (4 x 4)
  struct ProxyLevel {
    int w = 0, h = 0;
    float *ref_vals = nullptr, *ref_mv = nullptr;               // the source's level, mean and variance
    float *vals = nullptr, *tmp = nullptr, *box = nullptr, *s = nullptr, *parts = nullptr, *g = nullptr,
          *gtmp = nullptr, *gv = nullptr;
  } refine_pl[2];
  float* refine_src_y = nullptr;
  double* refine_proxy_sums = nullptr;
  jxg::ProxyScalars* refine_proxy_k = nullptr;
  // the context's own parameters, their gradient and Adam moments
  float *refine_theta = nullptr, *refine_grad = nullptr, *refine_adam = nullptr;
  int32_t refine_steps = 0;
  DevBuf field_buf;  // a caller's field, staged for jxg_frontend_run_with_field
  DevBuf order_buf;  // the order statistics' counters and per-slot block counts
  DevBuf chroma_buf;  // the pixel-chromacity counts
  // launch geometry of the tunable search and layout kernels (warps per CTA)
  uint8_t tune[jxg::kTuneKernels] = {4, 4, 4, 4, 4, 4, 4, 4, jxg::kRetileWarps, jxg::kSiteWarps};
  // timing
  bool timing = false;
  std::vector<PendingEvent> pending;
  std::vector<cudaEvent_t> spare_events;
  std::map<std::string, TimedKernel> times;
  std::vector<std::string> time_names;
  // asynchronous front end (jxg_frontend_enqueue / jxg_frontend_wait)
  struct AsyncSlot {
    DeviceStats stats;
    uint64_t token_count;
    uint64_t packed_count;  // words of the group storage form
  };
  HostBuf async_slot;                  // pinned AsyncSlot the pass's scalars land in
  bool async_pending = false;
  jxg_frame_params* async_params = nullptr;
  jxg_frontend_output async_out{};
};

struct Batch {
  Context* ctx = nullptr;
  bool on_device = false;
  std::vector<PassImage> images;
  bool planned = false;       // buffers sized and layout fixed for `images`
  uint64_t epoch = 0;         // context epoch of that plan
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
};

namespace {

int fail(Context* c, int code, const std::string& msg) {
  if (c) c->last_error = msg;
  return code;
}

// The device transfer table of (bits, transfer), built and uploaded on
// first use and kept for the context's life; null when it cannot be made.
float* transfer_lut(Context* c, int bits, int transfer) {
  const int key = (bits << 8) | (transfer & 0xff);
  const auto it = c->luts.find(key);
  if (it != c->luts.end()) return it->second;
  std::vector<float> host(65536);
  if (transfer_table(bits, transfer, host.data()) != 0) return nullptr;
  const size_t bytes = (bits == 8 ? 256 : 65536) * sizeof(float);
  float* d = nullptr;
  if (cudaMalloc(&d, bytes) != cudaSuccess) return nullptr;
  if (cudaMemcpy(d, host.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(d);
    return nullptr;
  }
  c->luts[key] = d;
  return d;
}

#define JXG_CUDA(ctx, call)                                                                    \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess)                                                                     \
      return ::jxg::fail(ctx, JXG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

int ensure(Context* c, DevBuf& b, size_t bytes) {
  if (bytes <= b.cap) return JXG_OK;
  if (b.ptr) cudaFree(b.ptr);
  b.ptr = nullptr;
  b.cap = 0;
  size_t want = std::max<size_t>(bytes, 256);
  cudaError_t e = cudaMalloc(&b.ptr, want);
  if (e != cudaSuccess) {
    b.ptr = nullptr;
    return fail(c, JXG_ERR_ALLOCATION_FAILED,
                "cudaMalloc(" + std::to_string(want) + "): " + cudaGetErrorString(e));
  }
  b.cap = want;
  return JXG_OK;
}

int ensure_host(Context* c, HostBuf& b, size_t bytes) {
  if (bytes <= b.cap) return JXG_OK;
  if (b.ptr) cudaFreeHost(b.ptr);
  b.ptr = nullptr;
  b.cap = 0;
  size_t want = std::max<size_t>(bytes, 4096);
  cudaError_t e = cudaMallocHost(&b.ptr, want);
  if (e != cudaSuccess) {
    b.ptr = nullptr;
    return fail(c, JXG_ERR_ALLOCATION_FAILED,
                "cudaMallocHost(" + std::to_string(want) + "): " + cudaGetErrorString(e));
  }
  b.cap = want;
  return JXG_OK;
}

cudaEvent_t take_event(Context* c) {
  if (!c->spare_events.empty()) {
    cudaEvent_t e = c->spare_events.back();
    c->spare_events.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

// Launch wrapper: records start/stop events around the launch when timing.
template <typename Launch>
int launch(Context* c, const char* name, bool timed, Launch&& fn) {
  cudaEvent_t s = nullptr, e = nullptr;
  if (timed) {
    s = take_event(c);
    e = take_event(c);
    cudaEventRecord(s, c->stream);
  }
  fn();
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return fail(c, JXG_ERR_CUDA, std::string(name) + ": " + cudaGetErrorString(err));
  if (timed) {
    cudaEventRecord(e, c->stream);
    c->pending.push_back({name, s, e});
  }
  return JXG_OK;
}

void collect_times(Context* c) {
  for (auto& p : c->pending) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, p.start, p.stop) == cudaSuccess) {
      auto& t = c->times[p.name];
      t.total_ms += ms;
      t.launches += 1;
    }
    c->spare_events.push_back(p.start);
    c->spare_events.push_back(p.stop);
  }
  c->pending.clear();
}

void frame_info(uint64_t w, uint64_t h, jxg_frame_info* o) {
  o->width = w;
  o->height = h;
  o->xsize_blocks = (w + 7) / 8;
  o->ysize_blocks = (h + 7) / 8;
  o->xsize_tiles = (o->xsize_blocks + 7) / 8;
  o->ysize_tiles = (o->ysize_blocks + 7) / 8;
  o->xsize_groups = (w + kGroupDim - 1) / kGroupDim;
  o->ysize_groups = (h + kGroupDim - 1) / kGroupDim;
  o->num_groups = o->xsize_groups * o->ysize_groups;
  o->num_dc_groups = ((w + kDcGroupDim - 1) / kDcGroupDim) * ((h + kDcGroupDim - 1) / kDcGroupDim);
  o->max_tokens = o->xsize_blocks * o->ysize_blocks * 3 * 64;
}

void opsin_matrix(float m[9]) {
  // XybMatrix::SPEC (src/xyb.rs:35-48), evaluated in f32 like the constants
  const float m00 = 0.30f, m02 = 0.078f, m10 = 0.23f, m12 = 0.078f;
  const float b_bias = 0.55180986f;
  const float ratio = 0.24342269f / (0.24342269f + 0.20476745f);
  m[0] = m00;
  m[1] = 1.0f - m02 - m00;
  m[2] = m02;
  m[3] = m10;
  m[4] = 1.0f - m12 - m10;
  m[5] = m12;
  m[6] = ratio * (1.0f - b_bias);
  m[7] = (1.0f - ratio) * (1.0f - b_bias);
  m[8] = 1.0f - m[6] - m[7];
}

int validate(Context* c, const void* pixels, uint64_t w, uint64_t h, int32_t channels,
             int32_t bits, const jxg_config* cfg) {
  if (!c || !pixels || !cfg) return fail(c, JXG_ERR_INVALID_ARGUMENT, "null argument");
  if (w == 0 || h == 0) return fail(c, JXG_ERR_EMPTY_IMAGE, "empty image");
  if (w > kMaxDimension || h > kMaxDimension)
    return fail(c, JXG_ERR_DIMENSION_TOO_LARGE, "dimension too large");
  if (channels < 1 || channels > 4) return fail(c, JXG_ERR_BAD_CHANNEL_COUNT, "channels");
  if (bits != 8 && bits != 10 && bits != 12 && bits != 16)
    return fail(c, JXG_ERR_BAD_BIT_DEPTH, "bits");
  const int tf = transfer_status(cfg->transfer);
  if (tf == 1) return fail(c, JXG_ERR_UNSUPPORTED, "PQ and HLG transfers are not built");
  if (tf != 0) return fail(c, JXG_ERR_INVALID_ARGUMENT, "transfer");
  if (!std::isfinite(cfg->distance) || cfg->distance <= 0.0f)
    return fail(c, JXG_ERR_INVALID_DISTANCE, "distance must be positive and finite");
  if (cfg->speed != JXG_SPEED_ULTRAFAST && cfg->speed != JXG_SPEED_FASTEST)
    return fail(c, JXG_ERR_UNSUPPORTED, "only the Speed::UltraFast and Speed::Fastest gates are built");
  if (cfg->speed == JXG_SPEED_FASTEST && fastest_search_mode(cfg->distance) == 2)
    return fail(c, JXG_ERR_UNSUPPORTED,
                "Speed::Fastest up to distance 1.709 reranks merges in the reconstruction "
                "domain, which this build does not have");
  if (w * h > (1ull << 31))
    return fail(c, JXG_ERR_DIMENSION_TOO_LARGE, "frames above 2^31 pixels are not supported");
  return JXG_OK;
}

// Device buffers of 16-bit samples must be 2-byte aligned.
int check_device_pixels(Context* c, const void* pixels, int32_t bits) {
  if (bits > 8 && (reinterpret_cast<uintptr_t>(pixels) & 1))
    return fail(c, JXG_ERR_INVALID_ARGUMENT, "16-bit device pixels must be 2-byte aligned");
  return JXG_OK;
}

// Device copy of the Fastest search tables at `dp`'s distance, built and
// uploaded on first use and kept for the context's life.
SearchTables* search_tables_for(Context* c, const DistanceParams& dp) {
  uint32_t key;
  std::memcpy(&key, &dp.distance, 4);
  const auto it = c->search_tables.find(key);
  if (it != c->search_tables.end()) return it->second;
  if (c->search_tables.size() >= 64) {  // bound the cache
    cudaStreamSynchronize(c->stream);
    for (auto& kv : c->search_tables) cudaFree(kv.second);
    c->search_tables.clear();
  }
  std::vector<char> host(sizeof(SearchTables));
  SearchTables* t = reinterpret_cast<SearchTables*>(host.data());
  SearchParams unused;
  if (search_tables(dp, t, &unused)) return nullptr;
  SearchTables* d = nullptr;
  if (cudaMalloc(&d, sizeof(SearchTables)) != cudaSuccess) return nullptr;
  if (cudaMemcpy(d, t, sizeof(SearchTables), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(d);
    return nullptr;
  }
  c->search_tables[key] = d;
  return d;
}

constexpr size_t kSearchFrameBytes = (sizeof(SearchFrame) + 255) / 256 * 256;
// k_mh_sum's CTAs: one thread per 2x2-block cell
size_t mh_sum_ctas(const FrameLayout& L) {
  const size_t cells = ((L.info.xsize_blocks + 1) / 2) * ((L.info.ysize_blocks + 1) / 2);
  return (cells + kMhSumThreads - 1) / kMhSumThreads;
}

// Lays out a pass of `n` frames in the context's buffers, sizes them, and
// fills the pinned plan (frame descriptors + chunk prefixes).  No launch.
// `stage`: host pixels go through the context's pinned staging buffer (what
// a recorded graph replays) instead of one copy per image from the caller.
int plan_pass(Context* c, const PassImage* imgs, int n, bool pixels_on_device, bool stage) {
  if (n <= 0) return fail(c, JXG_ERR_INVALID_ARGUMENT, "empty pass");
  int st;
  for (int i = 0; i < n; ++i)
    if ((st = validate(c, imgs[i].pixels, imgs[i].width, imgs[i].height, imgs[i].channels,
                       imgs[i].bits, &imgs[i].config)))
      return st;
  // Speed::Fastest searches one frame per pass
  bool any_search = false;
  for (int i = 0; i < n; ++i)
    any_search = any_search || (imgs[i].config.speed == JXG_SPEED_FASTEST &&
                                fastest_search_mode(imgs[i].config.distance) == 1);
  if (any_search && n > 1)
    return fail(c, JXG_ERR_UNSUPPORTED, "Speed::Fastest runs one frame per pass");
  c->have_frame = false;
  c->layouts.assign(n, FrameLayout{});
  size_t pix = 0, xyb = 0, blocks = 0, tiles = 0, groups = 0, counts = 0, tokens = 0;
  size_t alpha_px = 0, alpha_blocks = 0;
  int64_t xyb_chunks = 0, token_chunks = 0, alpha_tiles = 0, fill_total = 0;
  for (int i = 0; i < n; ++i) {
    FrameLayout& L = c->layouts[i];
    const PassImage& im = imgs[i];
    L.width = im.width;
    L.height = im.height;
    if (compute_distance_params(im.config.distance, &L.dp))
      return fail(c, JXG_ERR_INVALID_DISTANCE, "distance");
    frame_info(im.width, im.height, &L.info);
    const int64_t px = static_cast<int64_t>(im.width * im.height);
    L.plane = (px + 63) / 64 * 64;
    L.pix_off = pix;
    pix += align_up(static_cast<size_t>(px) * im.channels * sample_bytes(im.bits), 256);
    L.xyb_off = xyb;
    xyb += 3 * static_cast<size_t>(L.plane);
    L.block_off = blocks;
    blocks += L.info.xsize_blocks * L.info.ysize_blocks;
    L.tile_off = tiles;
    tiles += L.info.xsize_tiles * L.info.ysize_tiles;
    L.group_off = groups;
    groups += L.info.num_groups;
    L.count_off = counts;
    counts += L.info.num_groups * 4096;
    L.has_alpha = im.channels == 2 || im.channels == 4;
    if (L.has_alpha) {
      L.alpha_off = alpha_px;
      alpha_px += align_up(static_cast<size_t>(px), 128);
      L.alpha_block_off = alpha_blocks;
      alpha_blocks += align_up(L.info.xsize_blocks * L.info.ysize_blocks, 128);
      alpha_tiles += static_cast<int64_t>(L.info.xsize_tiles * L.info.ysize_tiles);
      fill_total += fill_tiles(L.width, L.height);
    }
    tokens += L.info.max_tokens;
    if (tokens > 0xFFFFFFFFull)  // token offsets are 32-bit
      return fail(c, JXG_ERR_DIMENSION_TOO_LARGE,
                  "pass holds more than 2^32 possible tokens: split the batch");
    xyb_chunks += (px + kXybChunk - 1) / kXybChunk;
    token_chunks += token_chunks_of(L.info);
  }
  c->total_tiles = static_cast<int64_t>(tiles);
  c->xyb_chunks = xyb_chunks;
  c->token_chunks = token_chunks;
  c->total_counts = static_cast<int64_t>(counts);
  c->total_groups = static_cast<int64_t>(groups);
  c->alpha_tiles = alpha_tiles;
  c->fill_tiles = fill_total;
  c->epoch += 1;
  {
    const FrameLayout& last = c->layouts.back();
    c->pixel_bytes = last.pix_off + static_cast<size_t>(last.width * last.height) *
                                        imgs[n - 1].channels * sample_bytes(imgs[n - 1].bits);
  }
  c->frames_bytes = align_up(sizeof(Frame) * n, 256);
  const size_t prefix_bytes = align_up(sizeof(int64_t) * (n + 1), 256);
  const size_t plan_bytes =
      align_up(c->frames_bytes + kPlanPrefixes * prefix_bytes, 256) + kSearchFrameBytes;
  if (plan_bytes > c->plan_slot_cap) {
    // grow every slot; the stream drains first, so no queued upload reads them
    JXG_CUDA(c, cudaStreamSynchronize(c->stream));
    const size_t cap = std::max<size_t>(plan_bytes, 64 << 10);
    if ((st = ensure(c, c->plan, cap * Context::kPlanSlots)) ||
        (st = ensure_host(c, c->plan_host, cap * Context::kPlanSlots)))
      return st;
    c->plan_slot_cap = cap;
  }
  c->plan_slot = (c->plan_slot + 1) % Context::kPlanSlots;
  // the slot's last upload must have left the host buffer before it is rewritten
  JXG_CUDA(c, cudaEventSynchronize(c->plan_uploaded[c->plan_slot]));
  char* plan_h = static_cast<char*>(c->plan_host.ptr) + c->plan_slot * c->plan_slot_cap;
  if ((!pixels_on_device && (st = ensure(c, c->pixels, pix))) ||
      (st = ensure(c, c->xyb, xyb * 4)) || (st = ensure(c, c->qf, blocks)) ||
      (st = ensure(c, c->ytox, tiles)) || (st = ensure(c, c->ytob, tiles)) ||
      (st = ensure(c, c->quant_dc, 3 * blocks * 2)) ||
      (st = ensure(c, c->levels, blocks * 192 * 2)) ||
      (st = ensure(c, c->wide_levels, blocks * 192 * 4)) ||
      (st = ensure(c, c->nzeros, 3 * blocks)) || (st = ensure(c, c->nz_packed, 4 * blocks)) ||
      (st = ensure(c, c->counts, counts * 4)) ||
      (st = ensure(c, c->tok_status, (token_chunks + 1) * 8)) ||
      (st = ensure(c, c->tokens, tokens * sizeof(uint2))) ||
      (st = ensure(c, c->hist, n * kHistBytes)) ||
      (st = ensure(c, c->stats, n * sizeof(DeviceStats))) ||
      (st = ensure(c, c->group_offsets, (groups + 1) * 8)) || (st = ensure(c, c->total, 256)) ||
      (st = ensure(c, c->group_wide, (groups + 1) * 4)) ||
      (alpha_px && (st = ensure(c, c->alpha, alpha_px * 2))) ||
      (alpha_blocks && (st = ensure(c, c->alpha_peak, alpha_blocks * 2))) ||
      (alpha_blocks && (st = ensure(c, c->alpha_zero, alpha_blocks))) ||
      (fill_total && (st = ensure(c, c->fill_flags, fill_total))) ||
      (fill_total && (st = ensure(c, c->fill_deps, fill_total * 4))) ||
      (fill_total && (st = ensure(c, c->fill_queue, fill_total * 4))) ||
      (fill_total && (st = ensure(c, c->fill_masks, fill_total * jxg::kFillMaskWords * 8))) ||
      (!pixels_on_device && stage && (st = ensure_host(c, c->pixels_host, pix))))
    return st;
  // frame descriptors
  Frame* frames = reinterpret_cast<Frame*>(plan_h);
  std::memset(frames, 0, sizeof(Frame) * n);
  float opsin[9];
  opsin_matrix(opsin);
  int64_t* pre_xyb = reinterpret_cast<int64_t*>(plan_h + c->frames_bytes);
  int64_t* pre_tile = reinterpret_cast<int64_t*>(reinterpret_cast<char*>(pre_xyb) + prefix_bytes);
  int64_t* pre_tok = reinterpret_cast<int64_t*>(reinterpret_cast<char*>(pre_tile) + prefix_bytes);
  int64_t* pre_alpha = reinterpret_cast<int64_t*>(reinterpret_cast<char*>(pre_tok) + prefix_bytes);
  int64_t* pre_fill = reinterpret_cast<int64_t*>(reinterpret_cast<char*>(pre_alpha) + prefix_bytes);
  int64_t ax = 0, at = 0, ak = 0, aa = 0, af = 0;
  for (int i = 0; i < n; ++i) {
    const FrameLayout& L = c->layouts[i];
    const PassImage& im = imgs[i];
    Frame& f = frames[i];
    KernelArgs& a = f.a;
    dct8_tables(L.dp.distance, a.matrix, a.inv_matrix);
    fill_kernel_args(L.dp, &a);
    std::memcpy(a.opsin, opsin, sizeof(opsin));
    a.width = static_cast<int32_t>(L.width);
    a.height = static_cast<int32_t>(L.height);
    a.xb = static_cast<int32_t>(L.info.xsize_blocks);
    a.yb = static_cast<int32_t>(L.info.ysize_blocks);
    a.tiles_x = static_cast<int32_t>(L.info.xsize_tiles);
    a.tiles_y = static_cast<int32_t>(L.info.ysize_tiles);
    a.groups_x = static_cast<int32_t>(L.info.xsize_groups);
    a.groups_y = static_cast<int32_t>(L.info.ysize_groups);
    a.plane = static_cast<int32_t>(L.plane);
    f.pixels = pixels_on_device ? im.pixels : static_cast<const char*>(c->pixels.ptr) + L.pix_off;
    f.channels = im.channels;
    f.bits = im.bits;
    f.transfer = im.config.transfer;
    f.lut = transfer_lut(c, im.bits, im.config.transfer);
    if (!f.lut) return fail(c, JXG_ERR_ALLOCATION_FAILED, "transfer table");
    f.xyb = static_cast<float*>(c->xyb.ptr) + L.xyb_off;
    f.qf = static_cast<uint8_t*>(c->qf.ptr) + L.block_off;
    f.ytox = static_cast<int8_t*>(c->ytox.ptr) + L.tile_off;
    f.ytob = static_cast<int8_t*>(c->ytob.ptr) + L.tile_off;
    f.quant_dc = static_cast<int16_t*>(c->quant_dc.ptr) + 3 * L.block_off;
    f.levels = static_cast<int16_t*>(c->levels.ptr) + 192 * L.block_off;
    f.wide_levels = static_cast<int32_t*>(c->wide_levels.ptr) + 192 * L.block_off;
    f.nzeros = static_cast<uint8_t*>(c->nzeros.ptr) + 3 * L.block_off;
    f.nz_packed = static_cast<uint32_t*>(c->nz_packed.ptr) + L.block_off;
    f.counts = static_cast<uint32_t*>(c->counts.ptr) + L.count_off;
    f.group_offsets = static_cast<uint64_t*>(c->group_offsets.ptr) + L.group_off;
    f.histograms = reinterpret_cast<uint32_t*>(static_cast<char*>(c->hist.ptr) + i * kHistBytes);
    f.stats = static_cast<DeviceStats*>(c->stats.ptr) + i;
    f.group_wide = static_cast<uint32_t*>(c->group_wide.ptr) + L.group_off;
    if (L.has_alpha) {
      f.alpha = static_cast<uint16_t*>(c->alpha.ptr) + L.alpha_off;
      f.alpha_peak = static_cast<uint16_t*>(c->alpha_peak.ptr) + L.alpha_block_off;
      f.alpha_zero = static_cast<uint8_t*>(c->alpha_zero.ptr) + L.alpha_block_off;
      f.alpha_full = (1 << im.bits) - 1;
    }
    const int64_t px = static_cast<int64_t>(L.width * L.height);
    pre_xyb[i] = ax;
    pre_tile[i] = at;
    pre_tok[i] = ak;
    pre_alpha[i] = aa;
    pre_fill[i] = af;
    if (L.has_alpha) {
      aa += static_cast<int64_t>(L.info.xsize_tiles * L.info.ysize_tiles);
      af += fill_tiles(L.width, L.height);
    }
    ax += (px + kXybChunk - 1) / kXybChunk;
    at += static_cast<int64_t>(L.info.xsize_tiles * L.info.ysize_tiles);
    ak += token_chunks_of(L.info);
  }
  pre_xyb[n] = ax;
  pre_tile[n] = at;
  pre_tok[n] = ak;
  pre_alpha[n] = aa;
  pre_fill[n] = af;
  if (any_search) {
    FrameLayout& L = c->layouts[0];
    L.searched = true;
    const size_t nb = L.info.xsize_blocks * L.info.ysize_blocks;
    const size_t tiles8 = L.info.xsize_tiles * L.info.ysize_tiles;
    if ((st = ensure(c, c->search_costs, 9 * nb * 4)) || (st = ensure(c, c->search_map, nb)) ||
        (st = ensure(c, c->search_bqf, nb)) || (st = ensure(c, c->search_dp, tiles8 * 64 * 512)) ||
        (st = ensure(c, c->search_sites, nb * 5)) ||
        (st = ensure(c, c->search_loss, nb * 16 + mh_sum_ctas(L) * kMhQuantities * 8 + 64)))
      return st;
    SearchFrame& sf = c->search_host;
    sf = SearchFrame{};
    sf.t = search_tables_for(c, L.dp);
    if (!sf.t) return fail(c, JXG_ERR_ALLOCATION_FAILED, "search tables");
    sf.rate_log2 = c->d_rate_log2;
    search_tables(L.dp, nullptr, &sf.p);
    sf.qm_mult[0] = L.dp.x_qm_mul;
    sf.qm_mult[1] = 1.0f;
    sf.qm_mult[2] = L.dp.b_qm_mul;
    sf.distance = L.dp.distance;
    sf.scale = L.dp.scale;
    float* costs = static_cast<float*>(c->search_costs.ptr);
    float** arrays[9] = {&sf.c8, &sf.c16s, &sf.c16r, &sf.cw, &sf.ct, &sf.c32, &sf.m16, &sf.m32, &sf.mh_inc};
    for (int k = 0; k < 9; ++k) *arrays[k] = costs + k * nb;
    sf.map = static_cast<uint8_t*>(c->search_map.ptr);
    sf.block_qf = static_cast<uint8_t*>(c->search_bqf.ptr);
    sf.dp_choices = static_cast<uint8_t*>(c->search_dp.ptr);
    sf.sites = static_cast<uint32_t*>(c->search_sites.ptr);
    sf.mh_kind = reinterpret_cast<uint8_t*>(sf.sites + nb);
    sf.mh_loss = static_cast<double*>(c->search_loss.ptr);
    sf.mh_part = sf.mh_loss + 2 * nb;
    sf.mh_decision = reinterpret_cast<uint32_t*>(sf.mh_part + mh_sum_ctas(L) * kMhQuantities);
    const char* serial = std::getenv("JXG_SERIAL_SUMS");
    sf.p.serial_sums = serial && serial[0] == '1' ? 1 : 0;
    const size_t search_off = plan_bytes - kSearchFrameBytes;
    std::memcpy(plan_h + search_off, &sf, sizeof(SearchFrame));
    frames[0].search = static_cast<char*>(c->plan.ptr) + c->plan_slot * c->plan_slot_cap + search_off;
  }
  return JXG_OK;
}

// Speed::Fastest's transform search and layout coding of the single frame
// `f` (see jxg_search.cuh), after the tile kernel has made the CfL maps.
int enqueue_search(Context* c, const Frame& f, bool timed) {
  cudaStream_t s = c->stream;
  const FrameLayout& L = c->layouts[0];
  const SearchFrame& sf = c->search_host;
  const int64_t xb = static_cast<int64_t>(L.info.xsize_blocks), yb = static_cast<int64_t>(L.info.ysize_blocks);
  const int64_t nb = xb * yb;
  const int64_t tiles = static_cast<int64_t>(L.info.xsize_tiles * L.info.ysize_tiles);
  JXG_CUDA(c, cudaMemcpyAsync(sf.block_qf, f.qf, nb, cudaMemcpyDeviceToDevice, s));
  JXG_CUDA(c, cudaMemsetAsync(sf.map, 1, nb, s));
  auto grid4 = [](int64_t n) { return static_cast<unsigned>((n + 3) / 4); };
  // the tuned warps per CTA of kernel k, its grid over n warps' work
  auto warps = [&](int k) { return static_cast<int>(c->tune[k]); };
  auto grid_of = [&](int64_t n, int k) { return static_cast<unsigned>((n + warps(k) - 1) / warps(k)); };
  int st;
  const int64_t n16 = (xb / 2) * (yb / 2), n8x16 = (xb / 2) * yb, n16x8 = xb * (yb / 2);
  const int64_t n32 = (xb / 4) * (yb / 4);
  if ((st = launch(c, "k_cost_dct8", timed, [&] {
         k_cost<kStDct><<<grid_of(nb, kTuneCostDct8), 32 * warps(kTuneCostDct8),
                          warps(kTuneCostDct8) * sizeof(CostSmem<kStDct>), s>>>(f);
       })))
    return st;
  if (n16 && (st = launch(c, "k_cost_16x16", timed, [&] {
                k_cost<kSt16x16><<<grid_of(n16, kTuneCost16x16), 32 * warps(kTuneCost16x16),
                                   warps(kTuneCost16x16) * sizeof(CostSmem<kSt16x16>), s>>>(f);
              })))
    return st;
  if (n8x16 && (st = launch(c, "k_cost_8x16", timed, [&] {
                  k_cost<kSt8x16><<<grid_of(n8x16, kTuneCost8x16), 32 * warps(kTuneCost8x16),
                                    warps(kTuneCost8x16) * sizeof(CostSmem<kSt8x16>), s>>>(f);
                })))
    return st;
  if (n16x8 && (st = launch(c, "k_cost_16x8", timed, [&] {
                  k_cost<kSt16x8><<<grid_of(n16x8, kTuneCost16x8), 32 * warps(kTuneCost16x8),
                                    warps(kTuneCost16x8) * sizeof(CostSmem<kSt16x8>), s>>>(f);
                })))
    return st;
  if (n32 && (st = launch(c, "k_cost_32x32", timed, [&] {
                k_cost32<<<static_cast<unsigned>(n32), kCost32Threads, sizeof(Cost32Smem), s>>>(f);
              })))
    return st;
  const int64_t strips = site_strips(static_cast<int>(xb), static_cast<int>(yb), 32) +
                         site_strips(static_cast<int>(xb), static_cast<int>(yb), 16);
  if (strips && (st = launch(c, "k_site", timed, [&] {
                   k_site<<<grid_of(strips, kTuneSite), 32 * warps(kTuneSite),
                            warps(kTuneSite) * sizeof(SiteSmem), s>>>(f);
                 })))
    return st;
  const int64_t cells = ((xb + 3) / 4) * ((yb + 3) / 4);
  if ((st = launch(c, "k_select", timed, [&] {
         k_select<<<static_cast<unsigned>((cells + 127) / 128), 128, 0, s>>>(f);
       })) ||
      (st = launch(c, "k_retile", timed, [&] {
         k_retile<<<grid_of(tiles, kTuneRetile), 32 * warps(kTuneRetile),
                    warps(kTuneRetile) * sizeof(RetileSmem), s>>>(f);
       })) ||
      (st = launch(c, "k_adjust", timed, [&] {
         k_adjust<<<static_cast<unsigned>((nb + 255) / 256), 256, 0, s>>>(f);
       })))
    return st;
  const int64_t cells2 = ((xb + 1) / 2) * ((yb + 1) / 2);
  const int parts = static_cast<int>(mh_sum_ctas(L));
  if (sf.p.headers &&
      ((st = launch(c, "k_mh_incumbent", timed, [&] {
          k_mh_incumbent<<<grid4(cells2), 128, 4 * sizeof(CostSmem<kSt32x32>), s>>>(f);
        })) ||
       (st = launch(c, "k_mh_sum", timed, [&] {
          k_mh_sum<<<static_cast<unsigned>(parts), kMhSumThreads, 0, s>>>(f);
        })) ||
       (st = launch(c, "k_mh_choose", timed, [&] { k_mh_choose<<<1, kMhThreads, 0, s>>>(f, parts); })) ||
       (st = launch(c, "k_mh_apply", timed, [&] {
          k_mh_apply<<<static_cast<unsigned>((cells2 + 255) / 256), 256, 0, s>>>(f);
        }))))
    return st;
  if ((st = launch(c, "k_qf_median", timed, [&] { k_qf_median<<<1, 256, 0, s>>>(f); })))
    return st;
  // the coding of the layout: a launch per transform shape
  if ((st = launch(c, "k_layout_dct8", timed, [&] {
         k_layout<kStDct><<<grid_of(nb, kTuneLayoutDct8), 32 * warps(kTuneLayoutDct8),
                            warps(kTuneLayoutDct8) * sizeof(LayoutSmem<kStDct>), s>>>(f);
       })))
    return st;
  if (n16 && (st = launch(c, "k_layout_16x16", timed, [&] {
                k_layout<kSt16x16><<<grid_of(n16, kTuneLayout16x16), 32 * warps(kTuneLayout16x16),
                                     warps(kTuneLayout16x16) * sizeof(LayoutSmem<kSt16x16>), s>>>(f);
              })))
    return st;
  if (n8x16 && (st = launch(c, "k_layout_8x16", timed, [&] {
                  k_layout<kSt8x16><<<grid_of(n8x16, kTuneLayout8x16), 32 * warps(kTuneLayout8x16),
                                      warps(kTuneLayout8x16) * sizeof(LayoutSmem<kSt8x16>), s>>>(f);
                })))
    return st;
  if (n16x8 && (st = launch(c, "k_layout_16x8", timed, [&] {
                  k_layout<kSt16x8><<<grid_of(n16x8, kTuneLayout16x8), 32 * warps(kTuneLayout16x8),
                                      warps(kTuneLayout16x8) * sizeof(LayoutSmem<kSt16x8>), s>>>(f);
                })))
    return st;
  if (n32 && (st = launch(c, "k_layout_32x32", timed, [&] {
                k_layout32<<<static_cast<unsigned>(n32), kLayout32Threads, sizeof(Layout32Smem), s>>>(f);
              })))
    return st;
  return JXG_OK;
}

// Enqueues a planned pass: uploads, clears, launches.  With `capturing` the
// launches are recorded into a graph, so no per-kernel timing events.
enum class PixelSource { kDevice, kStaged, kCaller };

int enqueue_pass(Context* c, const PassImage* imgs, int n, PixelSource src, bool capturing) {
  cudaStream_t s = c->stream;
  const size_t prefix_bytes = align_up(sizeof(int64_t) * (n + 1), 256);
  const size_t plan_bytes = c->frames_bytes + kPlanPrefixes * prefix_bytes;
  const size_t slot_off = c->plan_slot * c->plan_slot_cap;
  char* plan_d = static_cast<char*>(c->plan.ptr) + slot_off;
  const char* plan_h = static_cast<const char*>(c->plan_host.ptr) + slot_off;
  // one frame: its descriptor travels as a kernel parameter; a batch reads
  // the uploaded descriptor table
  const bool single = n == 1;
  if (!single) {
    JXG_CUDA(c, cudaMemcpyAsync(plan_d, plan_h, plan_bytes, cudaMemcpyHostToDevice, s));
    // a recorded graph replays the upload itself; every batch run waits for it
    if (!capturing) JXG_CUDA(c, cudaEventRecord(c->plan_uploaded[c->plan_slot], s));
  }
  const Frame& f0 = *reinterpret_cast<const Frame*>(plan_h);
  const bool searched = single && c->layouts[0].searched;
  if (searched) {
    // the SearchFrame the search kernels read, from the pinned plan slot
    const size_t off = align_up(c->frames_bytes + kPlanPrefixes * prefix_bytes, 256);
    JXG_CUDA(c, cudaMemcpyAsync(plan_d + off, plan_h + off, sizeof(SearchFrame), cudaMemcpyHostToDevice, s));
    if (!capturing) JXG_CUDA(c, cudaEventRecord(c->plan_uploaded[c->plan_slot], s));
  }
  if (src == PixelSource::kStaged)
    JXG_CUDA(c, cudaMemcpyAsync(c->pixels.ptr, c->pixels_host.ptr, c->pixel_bytes,
                                cudaMemcpyHostToDevice, s));
  if (src == PixelSource::kCaller)
    for (int i = 0; i < n; ++i) {
      const FrameLayout& L = c->layouts[i];
      const size_t bytes =
          static_cast<size_t>(L.width * L.height) * imgs[i].channels * sample_bytes(imgs[i].bits);
      JXG_CUDA(c, cudaMemcpyAsync(static_cast<char*>(c->pixels.ptr) + L.pix_off, imgs[i].pixels,
                                  bytes, cudaMemcpyHostToDevice, s));
    }
  JXG_CUDA(c, cudaMemsetAsync(c->stats.ptr, 0, n * sizeof(DeviceStats), s));
  JXG_CUDA(c, cudaMemsetAsync(c->hist.ptr, 0, n * kHistBytes, s));
  JXG_CUDA(c, cudaMemsetAsync(c->tok_status.ptr, 0, (c->token_chunks + 1) * 8, s));
  const Frame* frames = reinterpret_cast<const Frame*>(plan_d);
  const int64_t* pre_xyb = reinterpret_cast<const int64_t*>(plan_d + c->frames_bytes);
  const int64_t* pre_tile = reinterpret_cast<const int64_t*>(reinterpret_cast<const char*>(pre_xyb) + prefix_bytes);
  const int64_t* pre_tok = reinterpret_cast<const int64_t*>(reinterpret_cast<const char*>(pre_tile) + prefix_bytes);
  const int64_t* pre_alpha = reinterpret_cast<const int64_t*>(reinterpret_cast<const char*>(pre_tok) + prefix_bytes);
  const int64_t* pre_fill = reinterpret_cast<const int64_t*>(reinterpret_cast<const char*>(pre_alpha) + prefix_bytes);
  // the fill's ready queue starts empty, its counters at zero
  FillQueue* fill_q = reinterpret_cast<FillQueue*>(static_cast<char*>(c->total.ptr) + 64);
  uint8_t* fill_flags = static_cast<uint8_t*>(c->fill_flags.ptr);
  uint32_t* fill_deps = static_cast<uint32_t*>(c->fill_deps.ptr);
  uint32_t* fill_queue = static_cast<uint32_t*>(c->fill_queue.ptr);
  uint64_t* fill_masks = static_cast<uint64_t*>(c->fill_masks.ptr);
  const unsigned fill_grid = static_cast<unsigned>(std::max<int64_t>(
      1, std::min<int64_t>((c->fill_tiles + kFillThreads / 32 - 1) / (kFillThreads / 32),
                           static_cast<int64_t>(c->num_sms) * 3)));
  // the fill pass: a CTA per tile in flight, as many as fit the SMs
  const unsigned fill_run_grid = static_cast<unsigned>(std::max<int64_t>(
      1, std::min<int64_t>(c->fill_tiles, static_cast<int64_t>(c->num_sms) * 8)));
  if (c->fill_tiles) {
    JXG_CUDA(c, cudaMemsetAsync(fill_queue, 0xFF, c->fill_tiles * 4, s));
    JXG_CUDA(c, cudaMemsetAsync(fill_q, 0, sizeof(FillQueue), s));
  }
  const bool timed = c->timing && !capturing;
  int st;
  if (single) {
    if ((st = launch(c, "k_xyb", timed, [&] {
           k_xyb<<<static_cast<unsigned>(c->xyb_chunks), 256, 0, s>>>(f0);
         })))
      return st;
    if (c->alpha_tiles &&
        ((st = launch(c, "k_alpha_count", timed, [&] {
           k_alpha_count<<<static_cast<unsigned>(c->alpha_tiles), 256, 0, s>>>(f0);
         })) ||
         (st = launch(c, "k_alpha_final", timed, [&] {
           k_alpha_final<<<static_cast<unsigned>(c->alpha_tiles), 256, 0, s>>>(f0);
         })) ||
         (st = launch(c, "k_fill_plan", timed, [&] {
           k_fill_plan<<<fill_grid, kFillThreads, kFillSmemBytes, s>>>(
               f0, c->fill_tiles, fill_flags, fill_deps, fill_masks, fill_queue, fill_q);
         })) ||
         (st = launch(c, "k_fill_invisible", timed, [&] {
           k_fill_invisible<<<fill_run_grid, kFillRunThreads, kFillRunSmemBytes, s>>>(
               f0, fill_flags, fill_deps, fill_masks, fill_queue, fill_q);
         }))))
      return st;
    if ((st = launch(c, "k_adaptive_quant", timed, [&] {
           k_adaptive_quant<<<static_cast<unsigned>(c->total_tiles), 256, 0, s>>>(f0, c->d_exp2);
         })))
      return st;
    if (c->qf_override) {  // the caller's field, and ac_qf_threshold over it
      JXG_CUDA(c, cudaMemcpyAsync(f0.qf, c->qf_override, static_cast<size_t>(f0.a.xb) * f0.a.yb,
                                  cudaMemcpyDeviceToDevice, s));
      if ((st = launch(c, "k_qf_median", timed, [&] { k_qf_median<<<1, 256, 0, s>>>(f0); }))) return st;
    }
    // a searched frame takes only the CfL maps from the tile kernel
    if ((st = launch(c, "k_tile_quantize", timed, [&] {
           k_tile_quantize<<<static_cast<unsigned>(c->total_tiles), kTileThreads, kTileSmemBytes, s>>>(
               f0, c->d_pos, searched ? 1 : 0);
         })))
      return st;
    if (searched && (st = enqueue_search(c, f0, timed))) return st;
  } else {
    if ((st = launch(c, "k_xyb_batch", timed, [&] {
           k_xyb_batch<<<static_cast<unsigned>(c->xyb_chunks), 256, 0, s>>>(frames, pre_xyb, n);
         })))
      return st;
    if (c->alpha_tiles &&
        ((st = launch(c, "k_alpha_count_batch", timed, [&] {
           k_alpha_count_batch<<<static_cast<unsigned>(c->alpha_tiles), 256, 0, s>>>(
               frames, pre_alpha, n);
         })) ||
         (st = launch(c, "k_alpha_final_batch", timed, [&] {
           k_alpha_final_batch<<<static_cast<unsigned>(c->alpha_tiles), 256, 0, s>>>(
               frames, pre_alpha, n);
         })) ||
         (st = launch(c, "k_fill_plan_batch", timed, [&] {
           k_fill_plan_batch<<<fill_grid, kFillThreads, kFillSmemBytes, s>>>(
               frames, pre_fill, n, c->fill_tiles, fill_flags, fill_deps, fill_masks, fill_queue,
               fill_q);
         })) ||
         (st = launch(c, "k_fill_invisible_batch", timed, [&] {
           k_fill_invisible_batch<<<fill_run_grid, kFillRunThreads, kFillRunSmemBytes, s>>>(
               frames, pre_fill, n, fill_flags, fill_deps, fill_masks, fill_queue, fill_q);
         }))))
      return st;
    if ((st = launch(c, "k_adaptive_quant_batch", timed, [&] {
           k_adaptive_quant_batch<<<static_cast<unsigned>(c->total_tiles), 256, 0, s>>>(
               frames, pre_tile, n, c->d_exp2);
         })) ||
        (st = launch(c, "k_tile_quantize_batch", timed, [&] {
           k_tile_quantize_batch<<<static_cast<unsigned>(c->total_tiles), kTileThreads,
                                   kTileSmemBytes, s>>>(frames, pre_tile, n, c->d_pos);
         })))
      return st;
  }
  // token offsets come from the tokenizer's own look-back over its chunks
  TokenScan scan;
  scan.status = static_cast<unsigned long long*>(c->tok_status.ptr);
  scan.chunks = c->token_chunks;
  scan.pass_end = static_cast<uint64_t*>(c->group_offsets.ptr) + c->total_groups;
  if ((st = searched ? launch(c, "k_tokenize_layout", timed, [&] {
         k_tokenize_layout<<<static_cast<unsigned>(c->token_chunks), kLayoutTokThreads, 0, s>>>(
             f0, static_cast<uint2*>(c->tokens.ptr), scan);
       })
       : single ? launch(c, "k_tokenize", timed, [&] {
         k_tokenize<<<static_cast<unsigned>(c->token_chunks), kTokThreads, 0, s>>>(
             f0, static_cast<uint2*>(c->tokens.ptr), scan);
       })
                   : launch(c, "k_tokenize_batch", timed, [&] {
         k_tokenize_batch<<<static_cast<unsigned>(c->token_chunks), kTokThreads, 0, s>>>(
             frames, pre_tok, n, static_cast<uint2*>(c->tokens.ptr), scan);
       })))
    return st;
  c->have_frame = true;
  return JXG_OK;
}

int stage_host_pixels(Context* c, const PassImage* imgs, int n) {
  for (int i = 0; i < n; ++i) {
    const FrameLayout& L = c->layouts[i];
    const size_t bytes = static_cast<size_t>(L.width * L.height) * imgs[i].channels * sample_bytes(imgs[i].bits);
    std::memcpy(static_cast<char*>(c->pixels_host.ptr) + L.pix_off, imgs[i].pixels, bytes);
  }
  return JXG_OK;
}

int wait(Context* c) {
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail(c, JXG_ERR_CUDA, std::string("stream: ") + cudaGetErrorString(e));
  if (!c->pending.empty()) collect_times(c);
  return JXG_OK;
}

// Frame scalars from the frame's distance parameters and its device stats.
void params_from(const FrameLayout& L, const DeviceStats& ds, uint64_t num_tokens,
                 jxg_frame_params* out) {
  std::memset(out, 0, sizeof(*out));
  const DistanceParams& p = L.dp;
  out->distance = p.distance;
  out->global_scale = p.global_scale;
  out->quant_dc = p.quant_dc;
  out->scale = p.scale;
  out->scale_dc = p.scale_dc;
  out->x_qm_scale = p.x_qm_scale;
  out->b_qm_scale = p.b_qm_scale;
  out->epf_iters = p.epf_iters;
  for (int i = 0; i < 3; ++i) out->dc_step[i] = p.dc_step[i];
  out->qf_threshold = ds.qf_threshold;
  out->constant_blocks = ds.constant_blocks;
  const bool screen = is_screen_content(ds.constant_blocks, L.width, L.height);
  out->screen_content = screen;
  out->epf_sharpness = epf_sharpness_id(p.distance, screen);
  out->num_tokens = num_tokens;
}

int check_flags(Context* c, const DeviceStats& ds) {
  if (ds.flags & kFlagFillTimeout)
    return fail(c, JXG_ERR_DEVICE_TIMEOUT, "a bounded device wait of the invisible fill ran out");
  if (ds.flags & kFlagTokenTimeout)
    return fail(c, JXG_ERR_DEVICE_TIMEOUT, "a bounded device wait of the token offsets ran out");
  return JXG_OK;
}

int read_params(Context* c, int index, jxg_frame_params* out) {
  if (!c->have_frame || index < 0 || index >= static_cast<int>(c->layouts.size()))
    return fail(c, JXG_ERR_INVALID_ARGUMENT, "no such frame in the last pass");
  const FrameLayout& L = c->layouts[index];
  DeviceStats ds;
  uint64_t goffs[2];
  JXG_CUDA(c, cudaMemcpyAsync(&ds, static_cast<DeviceStats*>(c->stats.ptr) + index, sizeof(ds),
                              cudaMemcpyDeviceToHost, c->stream));
  JXG_CUDA(c, cudaMemcpyAsync(&goffs[0], static_cast<uint64_t*>(c->group_offsets.ptr) + L.group_off, 8,
                              cudaMemcpyDeviceToHost, c->stream));
  JXG_CUDA(c, cudaMemcpyAsync(&goffs[1],
                              static_cast<uint64_t*>(c->group_offsets.ptr) + L.group_off + L.info.num_groups,
                              8, cudaMemcpyDeviceToHost, c->stream));
  int st = wait(c);
  if (st) return st;
  if ((st = check_flags(c, ds))) return st;
  params_from(L, ds, goffs[1] - goffs[0], out);
  return JXG_OK;
}

// The address kernels use to write caller memory `p`: device memory as is,
// pinned host memory through its mapping, other host memory only where
// the device can reach pageable memory (coherent CPU-GPU systems).
int device_view(Context* c, void* p, void** out) {
  *out = nullptr;
  if (!p) return JXG_OK;
  cudaPointerAttributes attr{};
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    attr.type = cudaMemoryTypeUnregistered;
  }
  if (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged) {
    *out = p;
    return JXG_OK;
  }
  if (attr.type == cudaMemoryTypeHost && attr.devicePointer) {
    *out = attr.devicePointer;
    return JXG_OK;
  }
  int pageable = 0;
  cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, c->device);
  if (pageable) {
    *out = p;
    return JXG_OK;
  }
  return fail(c, JXG_ERR_INVALID_ARGUMENT,
              "asynchronous outputs must be pinned host memory or device memory");
}

// Enqueues every download of frame `index` except the token stream and
// group offsets (fixed sizes; no host synchronisation).
int enqueue_fixed_downloads(Context* c, int index, const jxg_frontend_output* out) {
  const FrameLayout& L = c->layouts[index];
  const jxg_frame_info& fi = L.info;
  const size_t nb = fi.xsize_blocks * fi.ysize_blocks;
  const size_t nt = fi.xsize_tiles * fi.ysize_tiles;
  cudaStream_t s = c->stream;
  auto copy = [&](void* dst, const void* src, size_t bytes) -> int {
    if (!dst || bytes == 0) return JXG_OK;
    JXG_CUDA(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
    return JXG_OK;
  };
  int st;
  if (out->coefficients) {
    if ((st = ensure(c, c->coeffs, nb * 192 * 4))) return st;
    const int64_t count = static_cast<int64_t>(nb) * 192;
    const int grid = static_cast<int>(std::min<int64_t>((count + 255) / 256, 4096));
    st = launch(c, "k_levels_to_raw", c->timing, [&] {
      k_levels_to_raw<<<grid, 256, 0, s>>>(static_cast<const int16_t*>(c->levels.ptr) + 192 * L.block_off,
                                           static_cast<const int32_t*>(c->wide_levels.ptr) + 192 * L.block_off,
                                           L.searched ? c->d_pos_identity : c->d_pos, count,
                                           static_cast<int32_t*>(c->coeffs.ptr));
    });
    if (st) return st;
  }
  if (L.searched && (st = copy(out->ac_strategy, c->search_map.ptr, nb))) return st;
  if ((st = copy(out->quant_field, static_cast<uint8_t*>(c->qf.ptr) + L.block_off, nb)) ||
      (st = copy(out->ytox_map, static_cast<int8_t*>(c->ytox.ptr) + L.tile_off, nt)) ||
      (st = copy(out->ytob_map, static_cast<int8_t*>(c->ytob.ptr) + L.tile_off, nt)) ||
      (st = copy(out->quant_dc, static_cast<int16_t*>(c->quant_dc.ptr) + 3 * L.block_off, 3 * nb * 2)) ||
      (st = copy(out->coefficients, c->coeffs.ptr, nb * 192 * 4)) ||
      (st = copy(out->num_nzeros, static_cast<uint8_t*>(c->nzeros.ptr) + 3 * L.block_off, 3 * nb)) ||
      (st = copy(out->histograms, static_cast<char*>(c->hist.ptr) + index * kHistBytes, kHistBytes)))
    return st;
  if (out->alpha && L.has_alpha &&
      (st = copy(out->alpha, static_cast<uint16_t*>(c->alpha.ptr) + L.alpha_off,
                 L.width * L.height * 2)))
    return st;
  if (out->xyb) {
    const size_t px = L.width * L.height;
    for (int ch = 0; ch < 3; ++ch)
      if ((st = copy(out->xyb + ch * px, static_cast<float*>(c->xyb.ptr) + L.xyb_off + ch * L.plane, px * 4)))
        return st;
  }
  return JXG_OK;
}

// k_pack_tokens over frame `L` of the last pass (see the kernel).
constexpr int kPackCtasPerGroup = 8;
int launch_pack(Context* c, int index, uint32_t* words, uint64_t capacity, uint64_t* word_offsets,
                uint64_t* count_out) {
  const FrameLayout& L = c->layouts[index];
  const int groups = static_cast<int>(L.info.num_groups);
  const dim3 grid(kPackCtasPerGroup, static_cast<unsigned>(std::min(groups, 65535)));
  cudaStream_t s = c->stream;
  return launch(c, "k_pack_tokens", c->timing, [&] {
    k_pack_tokens<<<grid, 256, 0, s>>>(
        static_cast<const uint2*>(c->tokens.ptr),
        static_cast<const uint64_t*>(c->group_offsets.ptr) + L.group_off,
        static_cast<const uint32_t*>(c->group_wide.ptr) + L.group_off,
        &(static_cast<const DeviceStats*>(c->stats.ptr) + index)->any_wide, groups, words, capacity,
        word_offsets, count_out);
  });
}

// The group storage form of frame `index` into host memory through a device
// staging buffer (the caller's memory may be pageable).
int fetch_packed(Context* c, int index, uint64_t num_tokens, jxg_frontend_output* out) {
  const FrameLayout& L = c->layouts[index];
  const uint64_t groups = L.info.num_groups;
  const uint64_t cap = 2 * num_tokens;  // every group wide
  int st;
  if ((st = ensure(c, c->packed, std::max<uint64_t>(cap, 1) * 4)) ||
      (st = ensure(c, c->packed_offs, (groups + 2) * 8)))
    return st;
  uint64_t* offs = static_cast<uint64_t*>(c->packed_offs.ptr);
  if ((st = launch_pack(c, index, out->packed_tokens ? static_cast<uint32_t*>(c->packed.ptr) : nullptr,
                        cap, offs, offs + groups + 1)))
    return st;
  uint64_t words = 0;
  JXG_CUDA(c, cudaMemcpyAsync(&words, offs + groups + 1, 8, cudaMemcpyDeviceToHost, c->stream));
  if ((st = wait(c))) return st;
  if (out->packed_tokens && words > out->packed_capacity)
    return fail(c, JXG_ERR_INVALID_ARGUMENT, "packed token buffer too small");
  if (out->packed_tokens && words)
    JXG_CUDA(c, cudaMemcpyAsync(out->packed_tokens, c->packed.ptr, words * 4, cudaMemcpyDeviceToHost,
                                c->stream));
  if (out->packed_offsets)
    JXG_CUDA(c, cudaMemcpyAsync(out->packed_offsets, offs, (groups + 1) * 8, cudaMemcpyDeviceToHost,
                                c->stream));
  return JXG_OK;
}

int fetch_frame(Context* c, int index, jxg_frontend_output* out) {
  jxg_frame_params p;
  int st = read_params(c, index, &p);
  if (st) return st;
  const FrameLayout& L = c->layouts[index];
  const jxg_frame_info& fi = L.info;
  const size_t nb = fi.xsize_blocks * fi.ysize_blocks;
  cudaStream_t s = c->stream;
  auto copy = [&](void* dst, const void* src, size_t bytes) -> int {
    if (!dst || bytes == 0) return JXG_OK;
    JXG_CUDA(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
    return JXG_OK;
  };
  if (out->tokens && out->token_capacity < p.num_tokens)
    return fail(c, JXG_ERR_INVALID_ARGUMENT, "token buffer too small");
  uint64_t first = 0;
  JXG_CUDA(c, cudaMemcpyAsync(&first, static_cast<uint64_t*>(c->group_offsets.ptr) + L.group_off, 8,
                              cudaMemcpyDeviceToHost, s));
  if ((st = wait(c))) return st;
  if ((st = enqueue_fixed_downloads(c, index, out)) ||
      (st = copy(out->tokens, static_cast<uint2*>(c->tokens.ptr) + first, p.num_tokens * sizeof(jxg_token))) ||
      (st = copy(out->group_offsets, static_cast<uint64_t*>(c->group_offsets.ptr) + L.group_off,
                 (fi.num_groups + 1) * 8)))
    return st;
  if ((out->packed_tokens || out->packed_offsets) &&
      (st = fetch_packed(c, index, p.num_tokens, out)))
    return st;
  if ((st = wait(c))) return st;
  if (out->group_offsets)  // frame-local token offsets
    for (uint64_t g = 0; g <= fi.num_groups; ++g) out->group_offsets[g] -= first;
  if (out->ac_strategy && !L.searched) std::memset(out->ac_strategy, 1, nb);  // all DCT8, first blocks
  return JXG_OK;
}

// Scratch of jxg_token_offsets_noalloc (see include/jxg.h): the chunk sums of
// the scan and the scalars its middle step writes.  A file-scope device array,
// so the entry point never allocates; every call shares it.
constexpr int kNoAllocMaxChunks = 4096;
static_assert(static_cast<int64_t>(kNoAllocMaxChunks) * kScanChunk >=
                  static_cast<int64_t>(JXG_NOALLOC_MAX_GROUPS) * 3 * 1024,
              "scratch must cover the stated group limit");
struct NoAllocScanScratch {
  uint32_t chunk_sums[kNoAllocMaxChunks];
  DeviceStats stats;
};
static __device__ __align__(256) NoAllocScanScratch g_noalloc_scan_scratch;

// Device address of the scratch array per device, looked up on the first
// call with that device current.
constexpr int kMaxDevices = 64;
NoAllocScanScratch* g_noalloc_scratch_ptr[kMaxDevices] = {};
std::mutex g_noalloc_mutex;

int noalloc_scratch(int device, NoAllocScanScratch** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_scratch_ptr[device]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scan_scratch);
    if (e != cudaSuccess || !ptr) return JXG_ERR_CUDA;
    g_noalloc_scratch_ptr[device] = static_cast<NoAllocScanScratch*>(ptr);
  }
  *out = g_noalloc_scratch_ptr[device];
  return JXG_OK;
}

int single_pass(Context* c, const void* pixels, uint64_t w, uint64_t h, int32_t channels,
                int32_t bits, const jxg_config* cfg, bool on_device) {
  if (!cfg) return fail(c, JXG_ERR_INVALID_ARGUMENT, "null config");
  PassImage im{pixels, w, h, channels, bits, *cfg};
  int st = on_device ? check_device_pixels(c, pixels, bits) : JXG_OK;
  if (st) return st;
  st = plan_pass(c, &im, 1, on_device, false);
  if (st) return st;
  return enqueue_pass(c, &im, 1, on_device ? PixelSource::kDevice : PixelSource::kCaller, false);
}

}  // namespace
}  // namespace jxg

namespace {
// Choice (src/epf_filter.rs:577-594); NaN stands for None
struct EpfChoice {
  int iters;
  float quant_mul, pass0;
  int sharpness;
  bool operator==(const EpfChoice& o) const {
    auto same = [](float a, float b) { return (std::isnan(a) && std::isnan(b)) || a == b; };
    return iters == o.iters && same(quant_mul, o.quant_mul) && same(pass0, o.pass0) && sharpness == o.sharpness;
  }
};
EpfChoice epf_candidate(int iters, float strength, float pass0) { return {iters, 0.46f * strength, pass0, 7}; }

// choose (src/epf_filter.rs:599-671), float arithmetic as the reference's
template <class Score>
EpfChoice epf_choose(float distance, EpfChoice baseline, Score&& score) {
  std::vector<std::pair<EpfChoice, float>> rows;
  auto trial = [&](const EpfChoice& c) {
    for (const auto& r : rows)
      if (r.first == c) return r;
    const float loss = score(c);
    rows.push_back({c, std::isfinite(loss) ? loss : INFINITY});
    return rows.back();
  };
  const float nan = std::numeric_limits<float>::quiet_NaN();
  trial(baseline);
  trial(EpfChoice{0, nan, nan, baseline.sharpness});
  const float center = std::min(std::max(2.0f / distance, 0.0625f), 4.0f);
  std::pair<EpfChoice, float> best_pilot{baseline, INFINITY};
  bool first = true;
  const std::pair<int, float> shapes[4] = {{1, nan}, {2, nan}, {3, 0.9f}, {3, 3.6f}};
  for (const auto& sh : shapes) {
    const auto r = trial(epf_candidate(sh.first, center, sh.second));
    if (first || r.second < best_pilot.second) best_pilot = r;  // the first of equal minima
    first = false;
  }
  const EpfChoice pilot = best_pilot.first;
  const float middle = best_pilot.second;
  const float lo = std::max(center / 2.0f, 0.0625f), hi = std::min(center * 2.0f, 4.0f);
  const float low = trial(epf_candidate(pilot.iters, lo, pilot.pass0)).second;
  const float high = trial(epf_candidate(pilot.iters, hi, pilot.pass0)).second;
  if (lo < center && center < hi) {
    const float x0 = std::log2(lo), x1 = std::log2(center), x2 = std::log2(hi);
    const float a = ((middle - low) / (x1 - x0) - (high - middle) / (x2 - x1)) / (x0 - x2);
    const float b = (middle - low) / (x1 - x0) - a * (x0 + x1);
    if (a > 1e-12f) {
      const float v = std::min(std::max(-b / (2.0f * a), x0), x2);
      trial(epf_candidate(pilot.iters, std::pow(2.0f, v), pilot.pass0));
    }
  }
  size_t k = 0;
  for (size_t i = 1; i < rows.size(); ++i)
    if (rows[i].second < rows[k].second) k = i;
  return rows[k].first;
}
}  // namespace

using jxg::Batch;
using jxg::Context;

extern "C" {

int32_t jxg_context_create(int32_t device, void** out_ctx) {
  if (!out_ctx) return JXG_ERR_INVALID_ARGUMENT;
  *out_ctx = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return JXG_ERR_CUDA;
  if (device < 0 || device >= count) return JXG_ERR_INVALID_ARGUMENT;
  if (cudaSetDevice(device) != cudaSuccess) return JXG_ERR_CUDA;
  Context* c = new Context();
  c->device = device;
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return JXG_ERR_CUDA;
  }
  c->stream = c->own_stream;
  if (cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      c->num_sms <= 0)
    c->num_sms = 1;
  float e2[64];
  uint8_t scan[64], pos[64], ident[64];
  jxg::exp2_table(e2);
  jxg::natural_order_8x8(scan, pos);
  for (int i = 0; i < 64; ++i) ident[i] = static_cast<uint8_t>(i);
  std::vector<float> rate(jxg::kRateLog2Entries);
  jxg::rate_log2_table(rate.data());
  bool ok = true;
  for (auto& e : c->plan_uploaded)
    ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
  ok = ok && jxg::transfer_lut(c, 8, 0) != nullptr &&  // the default: 8-bit sRGB
            cudaMalloc(&c->d_exp2, sizeof(e2)) == cudaSuccess &&
            cudaMalloc(&c->d_pos, 64) == cudaSuccess &&
            cudaMemcpy(c->d_exp2, e2, sizeof(e2), cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(c->d_pos, pos, 64, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMalloc(&c->d_pos_identity, 64) == cudaSuccess &&
            cudaMemcpy(c->d_pos_identity, ident, 64, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMalloc(&c->d_rate_log2, rate.size() * 4) == cudaSuccess &&
            cudaMemcpy(c->d_rate_log2, rate.data(), rate.size() * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
            jxg::set_search_attributes() == cudaSuccess &&
            cudaFuncSetAttribute(jxg::k_tile_quantize, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(jxg::kTileSmemBytes)) == cudaSuccess &&
            cudaFuncSetAttribute(jxg::k_tile_quantize_batch,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(jxg::kTileSmemBytes)) == cudaSuccess &&
            cudaFuncSetAttribute(jxg::k_fill_invisible, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(jxg::kFillRunSmemBytes)) == cudaSuccess &&
            cudaFuncSetAttribute(jxg::k_fill_invisible_batch,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(jxg::kFillRunSmemBytes)) == cudaSuccess &&
            cudaFuncSetAttribute(jxg::k_fill_plan, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(jxg::kFillSmemBytes)) == cudaSuccess &&
            cudaFuncSetAttribute(jxg::k_fill_plan_batch,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(jxg::kFillSmemBytes)) == cudaSuccess;
  if (!ok) {
    jxg_context_destroy(c);
    return JXG_ERR_CUDA;
  }
  *out_ctx = c;
  return JXG_OK;
}

void jxg_context_destroy(void* ctx) {
  Context* c = static_cast<Context*>(ctx);
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (jxg::DevBuf* b : {&c->pixels, &c->xyb, &c->qf, &c->ytox, &c->ytob, &c->quant_dc, &c->levels,
                         &c->wide_levels, &c->coeffs, &c->nzeros, &c->nz_packed, &c->counts,
                         &c->tokens, &c->hist, &c->stats,
                         &c->group_offsets, &c->plan, &c->total, &c->op_in, &c->op_out,
                         &c->alpha, &c->alpha_peak, &c->alpha_zero, &c->fill_flags,
                         &c->fill_deps, &c->fill_queue, &c->fill_masks, &c->group_wide, &c->packed,
                         &c->packed_offs, &c->tok_status, &c->search_frame, &c->search_costs,
                         &c->search_map, &c->search_bqf, &c->search_dp, &c->search_sites,
                         &c->search_loss})
    if (b->ptr) cudaFree(b->ptr);
  for (jxg::HostBuf* b : {&c->plan_host, &c->pixels_host, &c->async_slot})
    if (b->ptr) cudaFreeHost(b->ptr);
  for (auto& kv : c->luts) cudaFree(kv.second);
  cudaFree(c->d_exp2);
  cudaFree(c->d_pos);
  cudaFree(c->d_pos_identity);
  cudaFree(c->d_rate_log2);
  for (auto& kv : c->search_tables) cudaFree(kv.second);
  for (auto& p : c->pending) {
    cudaEventDestroy(p.start);
    cudaEventDestroy(p.stop);
  }
  for (auto e : c->spare_events) cudaEventDestroy(e);
  for (auto e : c->plan_uploaded)
    if (e) cudaEventDestroy(e);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
}

int32_t jxg_context_set_stream(void* ctx, void* cuda_stream) {
  Context* c = static_cast<Context*>(ctx);
  if (!c) return JXG_ERR_INVALID_ARGUMENT;
  c->stream = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : c->own_stream;
  return JXG_OK;
}

const char* jxg_context_last_error(void* ctx) {
  Context* c = static_cast<Context*>(ctx);
  return c ? c->last_error.c_str() : "null context";
}

float jxg_distance_from_quality(float quality) { return jxg::distance_from_quality(quality); }

int32_t jxg_frame_info_for(uint64_t width, uint64_t height, jxg_frame_info* out) {
  if (!out) return JXG_ERR_INVALID_ARGUMENT;
  if (width == 0 || height == 0) return JXG_ERR_EMPTY_IMAGE;
  jxg::frame_info(width, height, out);
  return JXG_OK;
}

int32_t jxg_validate_input(uint64_t width, uint64_t height, int32_t channels, int32_t bits,
                           const jxg_config* config) {
  static const uint8_t probe = 0;
  Context scratch;
  return jxg::validate(&scratch, &probe, width, height, channels, bits, config);
}

int32_t jxg_frontend_run_device(void* ctx, const void* pixels, uint64_t width, uint64_t height,
                                int32_t channels, int32_t bits, const jxg_config* config) {
  Context* c = static_cast<Context*>(ctx);
  if (!c) return JXG_ERR_INVALID_ARGUMENT;
  if (c->async_pending) {  // finish the enqueued frame before reusing its buffers
    const int st = jxg_frontend_wait(ctx);
    if (st) return st;
  }
  cudaSetDevice(c->device);
  return jxg::single_pass(c, pixels, width, height, channels, bits, config, true);
}

int32_t jxg_frontend_run(void* ctx, const void* pixels, uint64_t width, uint64_t height,
                         int32_t channels, int32_t bits, const jxg_config* config) {
  Context* c = static_cast<Context*>(ctx);
  if (!c) return JXG_ERR_INVALID_ARGUMENT;
  if (c->async_pending) {
    const int st = jxg_frontend_wait(ctx);
    if (st) return st;
  }
  cudaSetDevice(c->device);
  int st = jxg::single_pass(c, pixels, width, height, channels, bits, config, false);
  if (st) return st;
  return jxg::wait(c);
}

int32_t jxg_frontend_params(void* ctx, jxg_frame_params* out) {
  Context* c = static_cast<Context*>(ctx);
  if (!c || !out) return JXG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  return jxg::read_params(c, 0, out);
}

int32_t jxg_frontend_fetch(void* ctx, jxg_frontend_output* out) {
  Context* c = static_cast<Context*>(ctx);
  if (!c || !out) return JXG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  return jxg::fetch_frame(c, 0, out);
}

int32_t jxg_order_stats(void* ctx, uint32_t* counts, uint32_t* blocks) {
  Context* c = static_cast<Context*>(ctx);
  if (!c || !counts || !blocks) return JXG_ERR_INVALID_ARGUMENT;
  if (!c->have_frame || c->layouts.empty())
    return jxg::fail(c, JXG_ERR_INVALID_ARGUMENT, "no frame in the last pass");
  cudaSetDevice(c->device);
  const jxg::FrameLayout& L = c->layouts[0];
  const int xb = static_cast<int>(L.info.xsize_blocks), yb = static_cast<int>(L.info.ysize_blocks);
  const size_t bytes = (jxg::kOrderCounters + jxg::kOrderSlots) * sizeof(uint32_t);
  int st = jxg::ensure(c, c->order_buf, bytes);
  if (st) return st;
  uint32_t* d_counts = static_cast<uint32_t*>(c->order_buf.ptr);
  uint32_t* d_blocks = d_counts + jxg::kOrderCounters;
  cudaStream_t s = c->stream;
  JXG_CUDA(c, cudaMemsetAsync(d_counts, 0, bytes, s));
  const int64_t nb = static_cast<int64_t>(xb) * yb;
  const int warps = jxg::kOrderStatsThreads / 32;
  const unsigned grid = static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>((nb + warps - 1) / warps, 608)));
  st = jxg::launch(c, "k_order_stats", c->timing, [&] {
    jxg::k_order_stats<<<grid, jxg::kOrderStatsThreads, 0, s>>>(
        static_cast<const int16_t*>(c->levels.ptr) + 192 * L.block_off,
        L.searched ? static_cast<const uint8_t*>(c->search_map.ptr) : nullptr,
        L.searched ? c->d_pos_identity : c->d_pos, xb, yb, d_counts, d_blocks);
  });
  if (st) return st;
  JXG_CUDA(c, cudaMemcpyAsync(counts, d_counts, jxg::kOrderCounters * sizeof(uint32_t),
                              cudaMemcpyDeviceToHost, s));
  JXG_CUDA(c, cudaMemcpyAsync(blocks, d_blocks, jxg::kOrderSlots * sizeof(uint32_t),
                              cudaMemcpyDeviceToHost, s));
  return jxg::wait(c);
}

int32_t jxg_pixel_chromacity(void* ctx, uint32_t* counts, uint32_t* x_steps, uint32_t* b_steps) {
  Context* c = static_cast<Context*>(ctx);
  if (!c) return JXG_ERR_INVALID_ARGUMENT;
  if (!c->have_frame || c->layouts.empty())
    return jxg::fail(c, JXG_ERR_INVALID_ARGUMENT, "no frame in the last pass");
  cudaSetDevice(c->device);
  const jxg::FrameLayout& L = c->layouts[0];
  const int w = static_cast<int>(L.width), h = static_cast<int>(L.height);
  int st = jxg::ensure(c, c->chroma_buf, 7 * sizeof(uint32_t));
  if (st) return st;
  uint32_t* d_counts = static_cast<uint32_t*>(c->chroma_buf.ptr);
  cudaStream_t s = c->stream;
  JXG_CUDA(c, cudaMemsetAsync(d_counts, 0, 7 * sizeof(uint32_t), s));
  if (w >= 2 && h >= 2) {
    const int64_t total = static_cast<int64_t>(w - 1) * (h - 1);
    const unsigned grid = static_cast<unsigned>(
        std::min<int64_t>((total + jxg::kChromacityThreads - 1) / jxg::kChromacityThreads, 1216));
    st = jxg::launch(c, "k_pixel_chromacity", c->timing, [&] {
      jxg::k_pixel_chromacity<<<grid, jxg::kChromacityThreads, 0, s>>>(
          static_cast<const float*>(c->xyb.ptr) + L.xyb_off, w, h, static_cast<int64_t>(L.plane), d_counts);
    });
    if (st) return st;
  }
  uint32_t n[7];
  JXG_CUDA(c, cudaMemcpyAsync(n, d_counts, sizeof(n), cudaMemcpyDeviceToHost, s));
  if ((st = jxg::wait(c))) return st;
  // a level needs PIXEL_CHROMACITY_MIN_PIXELS (4) pixels; the B steps add one
  // for exposed blue once a level is reached (src/frame/chroma.rs:154-163)
  uint32_t lx = 0, lb = 0;
  for (int k = 0; k < 3; ++k) {
    lx += n[k] >= 4u ? 1u : 0u;
    lb += n[3 + k] >= 4u ? 1u : 0u;
  }
  if (counts) std::memcpy(counts, n, sizeof(n));
  if (x_steps) *x_steps = lx;
  if (b_steps) *b_steps = lb == 0 ? 0u : lb - 1u + (n[6] > 0 ? 1u : 0u);
  return JXG_OK;
}

int32_t jxg_derive_orders(const uint32_t* counts, const uint32_t* blocks, uint16_t* used_mask,
                          uint32_t* orders, double* scan_moved) {
  if (!counts || !blocks || !used_mask || !orders) return JXG_ERR_INVALID_ARGUMENT;
  const double moved = jxg::derive_orders(counts, blocks, used_mask, orders);
  if (scan_moved) *scan_moved = moved;
  return JXG_OK;
}

int32_t jxg_frontend_wait(void* ctx) {
  Context* c = static_cast<Context*>(ctx);
  if (!c) return JXG_ERR_INVALID_ARGUMENT;
  if (!c->async_pending) return JXG_OK;
  cudaSetDevice(c->device);
  c->async_pending = false;
  int st = jxg::wait(c);
  if (st) return st;
  const auto* slot = static_cast<const Context::AsyncSlot*>(c->async_slot.ptr);
  if ((st = jxg::check_flags(c, slot->stats))) return st;
  const jxg::FrameLayout& L = c->layouts[0];
  if (c->async_params) jxg::params_from(L, slot->stats, slot->token_count, c->async_params);
  const jxg_frontend_output& out = c->async_out;
  if (out.tokens && slot->token_count > out.token_capacity)
    return jxg::fail(c, JXG_ERR_INVALID_ARGUMENT, "token buffer too small");
  if (out.packed_tokens && slot->packed_count > out.packed_capacity)
    return jxg::fail(c, JXG_ERR_INVALID_ARGUMENT, "packed token buffer too small");
  if (out.ac_strategy && !L.searched)
    std::memset(out.ac_strategy, 1, L.info.xsize_blocks * L.info.ysize_blocks);
  // The token streams, whose lengths the host learns only now, leave the
  // device by the copy engine (a single-frame pass starts at token 0).
  if (out.tokens && slot->token_count)
    JXG_CUDA(c, cudaMemcpyAsync(out.tokens, c->tokens.ptr, slot->token_count * sizeof(jxg_token),
                                cudaMemcpyDefault, c->stream));
  if (out.packed_tokens && slot->packed_count)
    JXG_CUDA(c, cudaMemcpyAsync(out.packed_tokens, c->packed.ptr, slot->packed_count * 4,
                                cudaMemcpyDefault, c->stream));
  if ((out.tokens && slot->token_count) || (out.packed_tokens && slot->packed_count))
    return jxg::wait(c);
  return JXG_OK;
}

int32_t jxg_frontend_enqueue(void* ctx, const void* pixels, uint64_t width, uint64_t height,
                             int32_t channels, int32_t bits, const jxg_config* config,
                             jxg_frame_params* params, jxg_frontend_output* out) {
  Context* c = static_cast<Context*>(ctx);
  if (!c) return JXG_ERR_INVALID_ARGUMENT;
  int st;
  if (c->async_pending && (st = jxg_frontend_wait(ctx))) return st;
  cudaSetDevice(c->device);
  jxg_frontend_output o{};
  if (out) o = *out;
  void* off_dev = nullptr;
  void* woff_dev = nullptr;
  if ((st = jxg::device_view(c, o.group_offsets, &off_dev)) ||
      (st = jxg::device_view(c, o.packed_offsets, &woff_dev)) ||
      (st = jxg::ensure_host(c, c->async_slot, sizeof(Context::AsyncSlot))))
    return st;
  if ((st = jxg::single_pass(c, pixels, width, height, channels, bits, config, false))) return st;
  const jxg::FrameLayout& L = c->layouts[0];
  // packed words are staged on the device; jxg_frontend_wait copies them out
  const uint64_t words_cap = std::min<uint64_t>(o.packed_capacity, 2 * L.info.max_tokens);
  if (o.packed_tokens && (st = jxg::ensure(c, c->packed, std::max<uint64_t>(words_cap, 1) * 4)))
    return st;
  auto* slot = static_cast<Context::AsyncSlot*>(c->async_slot.ptr);
  void* slot_count_dev = nullptr;
  void* slot_words_dev = nullptr;
  if ((st = jxg::device_view(c, &slot->token_count, &slot_count_dev)) ||
      (st = jxg::device_view(c, &slot->packed_count, &slot_words_dev)))
    return st;
  cudaStream_t s = c->stream;
  if ((st = jxg::enqueue_fixed_downloads(c, 0, &o))) return st;
  JXG_CUDA(c, cudaMemcpyAsync(&slot->stats, c->stats.ptr, sizeof(jxg::DeviceStats),
                              cudaMemcpyDeviceToHost, s));
  const unsigned grid = static_cast<unsigned>(std::max(1, std::min(c->num_sms * 4, 1024)));
  st = jxg::launch(c, "k_copy_out_tokens", c->timing, [&] {
    jxg::k_copy_out_tokens<<<grid, 256, 0, s>>>(
        static_cast<const uint2*>(c->tokens.ptr),
        static_cast<const uint64_t*>(c->group_offsets.ptr) + L.group_off,
        static_cast<int>(L.info.num_groups), nullptr, 0, static_cast<uint64_t*>(off_dev),
        static_cast<uint64_t*>(slot_count_dev));
  });
  if (st) return st;
  slot->packed_count = 0;
  if ((o.packed_tokens || o.packed_offsets) &&
      (st = jxg::launch_pack(c, 0, o.packed_tokens ? static_cast<uint32_t*>(c->packed.ptr) : nullptr,
                             o.packed_tokens ? words_cap : 0,
                             static_cast<uint64_t*>(woff_dev),
                             static_cast<uint64_t*>(slot_words_dev))))
    return st;
  c->async_pending = true;
  c->async_params = params;
  c->async_out = o;
  return JXG_OK;
}

int32_t jxg_frontend(void* ctx, const void* pixels, uint64_t width, uint64_t height,
                     int32_t channels, int32_t bits, const jxg_config* config,
                     jxg_frame_params* params, jxg_frontend_output* out) {
  int st = jxg_frontend_run(ctx, pixels, width, height, channels, bits, config);
  if (st) return st;
  if (params && (st = jxg_frontend_params(ctx, params))) return st;
  if (out) return jxg_frontend_fetch(ctx, out);
  return JXG_OK;
}

int32_t jxg_batch_create(void* ctx, int32_t pixels_on_device, void** out_batch) {
  Context* c = static_cast<Context*>(ctx);
  if (!c || !out_batch) return JXG_ERR_INVALID_ARGUMENT;
  Batch* b = new Batch();
  b->ctx = c;
  b->on_device = pixels_on_device != 0;
  *out_batch = b;
  return JXG_OK;
}

static void drop_graph(Batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  b->planned = false;
}

int64_t jxg_batch_add(void* batch, const void* pixels, uint64_t width, uint64_t height,
                      int32_t channels, int32_t bits, const jxg_config* config) {
  Batch* b = static_cast<Batch*>(batch);
  if (!b || !config) return -JXG_ERR_INVALID_ARGUMENT;
  int st = jxg::validate(b->ctx, pixels, width, height, channels, bits, config);
  if (!st && b->on_device) st = jxg::check_device_pixels(b->ctx, pixels, bits);
  if (st) return -st;
  drop_graph(b);
  b->images.push_back(jxg::PassImage{pixels, width, height, channels, bits, *config});
  return static_cast<int64_t>(b->images.size()) - 1;
}

int32_t jxg_batch_run(void* batch, int32_t use_graph) {
  Batch* b = static_cast<Batch*>(batch);
  if (!b || b->images.empty()) return JXG_ERR_INVALID_ARGUMENT;
  Context* c = b->ctx;
  cudaSetDevice(c->device);
  const int n = static_cast<int>(b->images.size());
  int st;
  if (c->async_pending && (st = jxg_frontend_wait(c))) return st;
  if (!b->planned || b->epoch != c->epoch) {
    drop_graph(b);
    if ((st = jxg::plan_pass(c, b->images.data(), n, b->on_device, !b->on_device))) return st;
    b->planned = true;
    b->epoch = c->epoch;
  }
  using jxg::PixelSource;
  if (!use_graph) {
    // host pixels: one copy per image straight from the caller's buffers
    const PixelSource src = b->on_device ? PixelSource::kDevice : PixelSource::kCaller;
    if ((st = jxg::enqueue_pass(c, b->images.data(), n, src, false))) return st;
    return jxg::wait(c);
  }
  // a graph replays fixed copies: host pixels go through the pinned staging buffer
  if (!b->on_device) jxg::stage_host_pixels(c, b->images.data(), n);
  if (!b->exec) {
    // the pass is recorded once and replayed; its buffers stay fixed while
    // the batch is unchanged
    JXG_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    st = jxg::enqueue_pass(c, b->images.data(), n,
                           b->on_device ? PixelSource::kDevice : PixelSource::kStaged, true);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (st) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (e != cudaSuccess) return jxg::fail(c, JXG_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
    b->graph = g;
    JXG_CUDA(c, cudaGraphInstantiate(&b->exec, g, 0));
  }
  JXG_CUDA(c, cudaGraphLaunch(b->exec, c->stream));
  c->have_frame = true;
  return jxg::wait(c);
}

static bool batch_current(const Batch* b) {
  return b->planned && b->epoch == b->ctx->epoch && b->ctx->have_frame;
}

int32_t jxg_batch_result(void* batch, uint64_t index, jxg_frame_params* params,
                         jxg_frontend_output* out) {
  Batch* b = static_cast<Batch*>(batch);
  if (!b) return JXG_ERR_INVALID_ARGUMENT;
  if (!batch_current(b))
    return jxg::fail(b->ctx, JXG_ERR_INVALID_ARGUMENT, "the context ran another pass since this batch");
  if (index >= b->images.size()) return jxg::fail(b->ctx, JXG_ERR_INVALID_ARGUMENT, "index");
  cudaSetDevice(b->ctx->device);
  int st;
  if (params && (st = jxg::read_params(b->ctx, static_cast<int>(index), params))) return st;
  if (out) return jxg::fetch_frame(b->ctx, static_cast<int>(index), out);
  return JXG_OK;
}

void jxg_batch_destroy(void* batch) {
  Batch* b = static_cast<Batch*>(batch);
  if (!b) return;
  cudaSetDevice(b->ctx->device);
  drop_graph(b);
  delete b;
}

int32_t jxg_op_chroma_hf_protection(void* ctx, const float* xyb, uint64_t width, uint64_t height,
                                    float distance, uint8_t* quant_field) {
  Context* c = static_cast<Context*>(ctx);
  if (!c || !xyb || !quant_field) return JXG_ERR_INVALID_ARGUMENT;
  if (width == 0 || height == 0) return JXG_ERR_EMPTY_IMAGE;
  if (!std::isfinite(distance)) return JXG_ERR_INVALID_DISTANCE;
  // ChromaHfFit (src/adaptive_quant.rs:319-342): the boost fades in from
  // distance 0.35 over 0.40 and out from 1.0 over 1.0, at strength 0.40
  auto clamp01 = [](float v) { return v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v); };
  if (distance < 0.35f) return JXG_OK;
  const float fade_in = clamp01((distance - 0.35f) / 0.40f);
  const float fade_out = 1.0f - clamp01((distance - 1.0f) / 1.0f);
  const float strength = 0.40f * fade_in * fade_out;
  if (strength <= 0.0f) return JXG_OK;
  cudaSetDevice(c->device);
  jxg_frame_info fi;
  jxg::frame_info(width, height, &fi);
  const int64_t n = static_cast<int64_t>(width * height);
  const size_t nb = fi.xsize_blocks * fi.ysize_blocks;
  int st;
  if ((st = jxg::ensure(c, c->op_in, jxg::align_up(3 * n * 4, 256))) ||
      (st = jxg::ensure(c, c->op_out, jxg::align_up(nb, 256))))
    return st;
  float* d_xyb = static_cast<float*>(c->op_in.ptr);
  uint8_t* d_field = static_cast<uint8_t*>(c->op_out.ptr);
  cudaStream_t s = c->stream;
  JXG_CUDA(c, cudaMemcpyAsync(d_xyb, xyb, 3 * n * 4, cudaMemcpyHostToDevice, s));
  JXG_CUDA(c, cudaMemcpyAsync(d_field, quant_field, nb, cudaMemcpyHostToDevice, s));
  st = jxg::launch(c, "k_chroma_hf_protection", c->timing, [&] {
    jxg::k_chroma_hf_protection<<<static_cast<unsigned>((nb + 127) / 128), 128, 0, s>>>(
        d_xyb, static_cast<int>(width), static_cast<int>(height), n, static_cast<int>(fi.xsize_blocks),
        static_cast<int>(fi.ysize_blocks), strength, d_field);
  });
  if (st) return st;
  JXG_CUDA(c, cudaMemcpyAsync(quant_field, d_field, nb, cudaMemcpyDeviceToHost, s));
  return jxg::wait(c);
}

int32_t jxg_op_fill_quant_field(void* ctx, const float* xyb, uint64_t width, uint64_t height,
                                float distance, float inv_scale, uint8_t* quant_field) {
  Context* c = static_cast<Context*>(ctx);
  if (!c || !xyb || !quant_field) return JXG_ERR_INVALID_ARGUMENT;
  if (width == 0 || height == 0) return JXG_ERR_EMPTY_IMAGE;
  if (!(distance > 0.0f) || !std::isfinite(distance)) return JXG_ERR_INVALID_DISTANCE;
  cudaSetDevice(c->device);
  // FillQuantFieldFn derives every AQ constant from the distance it is
  // given (src/adaptive_quant.rs:547-727), with no MIN_DISTANCE clamp.
  jxg::DistanceParams dp;
  jxg::compute_distance_params(distance, &dp);
  dp.distance = distance;
  jxg::Frame f;
  std::memset(&f, 0, sizeof(f));
  jxg::KernelArgs& a = f.a;
  jxg::fill_kernel_args(dp, &a);
  a.inv_scale = inv_scale;
  jxg_frame_info fi;
  jxg::frame_info(width, height, &fi);
  a.width = static_cast<int32_t>(width);
  a.height = static_cast<int32_t>(height);
  a.xb = static_cast<int32_t>(fi.xsize_blocks);
  a.yb = static_cast<int32_t>(fi.ysize_blocks);
  a.tiles_x = static_cast<int32_t>(fi.xsize_tiles);
  a.tiles_y = static_cast<int32_t>(fi.ysize_tiles);
  const int64_t n = static_cast<int64_t>(width * height);
  const int64_t plane = (n + 63) / 64 * 64;
  a.plane = static_cast<int32_t>(plane);
  const size_t nb = fi.xsize_blocks * fi.ysize_blocks;
  const int64_t tiles = static_cast<int64_t>(fi.xsize_tiles * fi.ysize_tiles);
  const size_t in_bytes = jxg::align_up(3 * plane * 4, 256);
  const size_t out_bytes = jxg::align_up(nb, 256);
  int st;
  if ((st = jxg::ensure(c, c->op_in, in_bytes)) ||
      (st = jxg::ensure(c, c->op_out, out_bytes + sizeof(jxg::DeviceStats))))
    return st;
  char* in = static_cast<char*>(c->op_in.ptr);
  char* outp = static_cast<char*>(c->op_out.ptr);
  f.xyb = reinterpret_cast<float*>(in);
  f.qf = reinterpret_cast<uint8_t*>(outp);
  f.stats = reinterpret_cast<jxg::DeviceStats*>(outp + out_bytes);
  cudaStream_t s = c->stream;
  for (int ch = 0; ch < 3; ++ch)
    JXG_CUDA(c, cudaMemcpyAsync(f.xyb + ch * plane, xyb + ch * n, n * 4, cudaMemcpyHostToDevice, s));
  JXG_CUDA(c, cudaMemsetAsync(f.stats, 0, sizeof(jxg::DeviceStats), s));
  st = jxg::launch(c, "k_adaptive_quant", c->timing, [&] {
    jxg::k_adaptive_quant<<<static_cast<unsigned>(tiles), 256, 0, s>>>(f, c->d_exp2);
  });
  if (st) return st;
  JXG_CUDA(c, cudaMemcpyAsync(quant_field, f.qf, nb, cudaMemcpyDeviceToHost, s));
  return jxg::wait(c);
}

namespace {
// The gaborish operators: 3 planes in from the host, one launch, 3 planes out.
int32_t gaborish_op(void* ctx, const float* xyb, uint64_t width, uint64_t height, float* out,
                    bool inverse, float mul) {
  Context* c = static_cast<Context*>(ctx);
  if (!c || !xyb || !out) return JXG_ERR_INVALID_ARGUMENT;
  if (width == 0 || height == 0) return JXG_OK;
  if (width > (1u << 20) || height > (1u << 20) || width * height > (1ull << 31))
    return JXG_ERR_DIMENSION_TOO_LARGE;
  if (inverse && !(mul >= 0.0f)) return JXG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  int st;
  const size_t bytes = 3 * width * height * 4;
  if ((st = jxg::ensure(c, c->op_in, bytes)) || (st = jxg::ensure(c, c->op_out, bytes))) return st;
  cudaStream_t s = c->stream;
  JXG_CUDA(c, cudaMemcpyAsync(c->op_in.ptr, xyb, bytes, cudaMemcpyHostToDevice, s));
  jxg::GaborishWeights k{};
  if (inverse) jxg::gaborish_inverse_weights(mul, k.w);
  else jxg::gaborish_weights(k.w);
  const dim3 grid(static_cast<unsigned>((width + jxg::kGabTileX - 1) / jxg::kGabTileX),
                  static_cast<unsigned>((height + jxg::kGabTileY - 1) / jxg::kGabTileY), 3);
  const float* in = static_cast<const float*>(c->op_in.ptr);
  float* o = static_cast<float*>(c->op_out.ptr);
  const int w = static_cast<int>(width), h = static_cast<int>(height);
  st = inverse ? jxg::launch(c, "k_gaborish_inverse", c->timing, [&] {
    jxg::k_gaborish_inverse<<<grid, jxg::kGabThreads, 0, s>>>(in, o, w, h, k);
  })
               : jxg::launch(c, "k_gaborish", c->timing, [&] {
                   jxg::k_gaborish<<<grid, jxg::kGabThreads, 0, s>>>(in, o, w, h, k);
                 });
  if (st) return st;
  JXG_CUDA(c, cudaMemcpyAsync(out, c->op_out.ptr, bytes, cudaMemcpyDeviceToHost, s));
  return jxg::wait(c);
}
}  // namespace

int32_t jxg_op_gaborish_inverse(void* ctx, const float* xyb, uint64_t width, uint64_t height,
                                float mul, float* out) {
  return gaborish_op(ctx, xyb, width, height, out, true, mul);
}

int32_t jxg_op_gaborish(void* ctx, const float* xyb, uint64_t width, uint64_t height, float* out) {
  return gaborish_op(ctx, xyb, width, height, out, false, 0.0f);
}

int32_t jxg_op_epf(void* ctx, const float* xyb, uint64_t width, uint64_t height, const float* sigma_quant,
                   int32_t iters, float quant_mul, float pass0, float pass2, float border_mul,
                   const float* channel_scale, int32_t sharpness, float* out) {
  using namespace jxg;
  Context* c = static_cast<Context*>(ctx);
  if (!c || !xyb || !sigma_quant || !channel_scale || !out) return JXG_ERR_INVALID_ARGUMENT;
  if (width == 0 || height == 0) return fail(c, JXG_ERR_EMPTY_IMAGE, "empty image");
  if (width > kMaxDimension || height > kMaxDimension)
    return fail(c, JXG_ERR_DIMENSION_TOO_LARGE, "dimension too large");
  if (iters < 0 || iters > 3 || sharpness < 0 || sharpness > 7)
    return fail(c, JXG_ERR_INVALID_ARGUMENT, "iters 0..3, sharpness 0..7");
  cudaSetDevice(c->device);
  const int64_t n = static_cast<int64_t>(width) * height;
  const size_t bytes = static_cast<size_t>(n) * 3 * 4;
  if (iters == 0 || sharpness == 0) {  // Epf::apply returns the image itself
    std::memcpy(out, xyb, bytes);
    return JXG_OK;
  }
  RefineArgs r{};
  r.w = static_cast<int32_t>(width);
  r.h = static_cast<int32_t>(height);
  r.xb = static_cast<int32_t>((width + 7) / 8);
  r.yb = static_cast<int32_t>((height + 7) / 8);
  r.epf_border = border_mul;
  for (int k = 0; k < 3; ++k) r.epf_channel[k] = channel_scale[k];
  const int64_t nb = static_cast<int64_t>(r.xb) * r.yb;
  // planes: input, two stage outputs, the largest stage's weights and centre
  // weights; then the per-block sigma values
  const size_t floats = static_cast<size_t>(3 * n * 3 + 13 * n) + 2 * nb + 64;
  int st;
  if ((st = ensure(c, c->op_in, floats * 4))) return st;
  float* in = static_cast<float*>(c->op_in.ptr);
  float* buf[2] = {in + 3 * n, in + 6 * n};
  float* nw = in + 9 * n;
  float* cw = nw + 12 * n;
  float* sq = cw + n;
  r.sigma = sq + nb;
  cudaStream_t s = c->stream;
  JXG_CUDA(c, cudaMemcpyAsync(in, xyb, bytes, cudaMemcpyHostToDevice, s));
  JXG_CUDA(c, cudaMemcpyAsync(sq, sigma_quant, nb * 4, cudaMemcpyHostToDevice, s));
  const float sad_mul = 1.65f;  // SAD_MUL, src/epf_filter.rs:45
  int stages[3], count = 0;
  float sms[3];
  if (iters >= 3) {
    stages[count] = 0;
    sms[count++] = sad_mul * pass0;
  }
  stages[count] = 1;
  sms[count++] = sad_mul;
  if (iters >= 2) {
    stages[count] = 2;
    sms[count++] = sad_mul * pass2;
  }
  st = launch(c, "k_epf_sigma", c->timing, [&] {
    k_epf_sigma<<<static_cast<unsigned>((nb + 255) / 256), 256, 0, s>>>(sq, nb, quant_mul,
                                                                         static_cast<float>(sharpness) / 7.0f, r.sigma);
  });
  if (st) return st;
  const float* src = in;
  for (int k = 0; k < count; ++k) {
    float* dst = buf[k & 1];
    st = launch(c, "k_refine_epf", c->timing, [&] {
      const dim3 grid(static_cast<unsigned>((r.w + kEpfTW - 1) / kEpfTW), static_cast<unsigned>((r.h + kEpfTH - 1) / kEpfTH));
      k_refine_epf<<<grid, 256, 0, s>>>(r, stages[k], sms[k], src, n, r.w, dst, nw, cw);
    });
    if (st) return st;
    src = dst;
  }
  JXG_CUDA(c, cudaMemcpyAsync(out, src, bytes, cudaMemcpyDeviceToHost, s));
  return wait(c);
}

int32_t jxg_op_luma_proxy(void* ctx, const float* source, const float* test, uint64_t width, uint64_t height,
                          double* score, double* terms) {
  using namespace jxg;
  Context* c = static_cast<Context*>(ctx);
  if (!c || !source || !test || !score) return JXG_ERR_INVALID_ARGUMENT;
  if (width < 4 || height < 4) return fail(c, JXG_ERR_INVALID_ARGUMENT, "the proxy needs 4 x 4 pixels");
  if (width > kMaxDimension || height > kMaxDimension)
    return fail(c, JXG_ERR_DIMENSION_TOO_LARGE, "dimension too large");
  cudaSetDevice(c->device);
  const int w = static_cast<int>(width), h = static_cast<int>(height);
  const int64_t n = static_cast<int64_t>(w) * h;
  const int lw[2] = {w / 2, (w / 2) / 2}, lh[2] = {h / 2, (h / 2) / 2};  // half, quarter
  const int64_t m[2] = {static_cast<int64_t>(lw[0]) * lh[0], static_cast<int64_t>(lw[1]) * lh[1]};
  // per level: source values, its mean and variance, test values, two sets of
  // three box planes, s and the three partials; then the slot sums
  const size_t floats = 2 * n + 14 * (m[0] + m[1]) + 2 * kProxySums * kRefineSlots + 64;
  int st;
  if ((st = ensure(c, c->op_in, floats * 4))) return st;
  float* p = static_cast<float*>(c->op_in.ptr);
  float* src = p;
  float* tst = p + n;
  p += 2 * n;
  float *rv[2], *rmv[2], *tv[2], *tmp[2], *box[2], *sm[2], *parts[2];
  for (int l = 0; l < 2; ++l) {
    rv[l] = p;
    rmv[l] = rv[l] + m[l];
    tv[l] = rmv[l] + 2 * m[l];
    tmp[l] = tv[l] + m[l];
    box[l] = tmp[l] + 3 * m[l];
    sm[l] = box[l] + 3 * m[l];
    parts[l] = sm[l] + m[l];
    p = parts[l] + 3 * m[l];
  }
  double* sums = reinterpret_cast<double*>(p + (reinterpret_cast<uintptr_t>(p) & 4 ? 1 : 0));
  cudaStream_t s = c->stream;
  JXG_CUDA(c, cudaMemcpyAsync(src, source, n * 4, cudaMemcpyHostToDevice, s));
  JXG_CUDA(c, cudaMemcpyAsync(tst, test, n * 4, cudaMemcpyHostToDevice, s));
  JXG_CUDA(c, cudaMemsetAsync(sums, 0, kProxySums * kRefineSlots * sizeof(double), s));
  auto grid = [](int64_t k) { return static_cast<unsigned>((k + 255) / 256); };
  st = launch(c, "k_proxy", c->timing, [&] {
    k_proxy_half<<<grid(m[0]), 256, 0, s>>>(src, w, w, h, 1, rv[0]);
    k_proxy_half<<<grid(m[1]), 256, 0, s>>>(rv[0], lw[0], lw[0], lh[0], 0, rv[1]);
    k_proxy_half<<<grid(m[0]), 256, 0, s>>>(tst, w, w, h, 1, tv[0]);
    k_proxy_half<<<grid(m[1]), 256, 0, s>>>(tv[0], lw[0], lw[0], lh[0], 0, tv[1]);
    for (int l = 0; l < 2; ++l) {
      k_proxy_box_v<<<(lw[l] + 127) / 128, 128, 0, s>>>(rv[l], nullptr, lw[l], lh[l], tmp[l]);
      k_proxy_box_h<<<(2 * lh[l] + 127) / 128, 128, 0, s>>>(tmp[l], 2, lw[l], lh[l], rmv[l]);
      k_proxy_variance<<<grid(m[l]), 256, 0, s>>>(rmv[l], m[l]);
      k_proxy_box_v<<<(lw[l] + 127) / 128, 128, 0, s>>>(tv[l], rv[l], lw[l], lh[l], tmp[l]);
      k_proxy_box_h<<<(3 * lh[l] + 127) / 128, 128, 0, s>>>(tmp[l], 3, lw[l], lh[l], box[l]);
      k_proxy_pool<<<grid(m[l]), 256, 0, s>>>(rmv[l], box[l], m[l], sm[l], parts[l], sums + 2 * l * kRefineSlots);
    }
    k_proxy_gradients<<<grid(n), 256, 0, s>>>(src, tst, w, w, h, sums + 4 * kRefineSlots);
  });
  if (st) return st;
  double host[kProxySums * kRefineSlots];
  JXG_CUDA(c, cudaMemcpyAsync(host, sums, sizeof(host), cudaMemcpyDeviceToHost, s));
  if ((st = wait(c))) return st;
  double t[kProxySums];
  for (int q = 0; q < kProxySums; ++q) {
    t[q] = 0.0;
    for (int k = 0; k < kRefineSlots; ++k) t[q] += host[q * kRefineSlots + k];
  }
  const double np = static_cast<double>(h) * (w - 1) + static_cast<double>(h - 1) * w;
  const double v[6] = {t[2] / static_cast<double>(m[1]), t[0] / static_cast<double>(m[0]),
                       std::sqrt(std::sqrt(t[1] / static_cast<double>(m[0]))), t[4] / np, t[5] / np,
                       std::sqrt(std::sqrt(t[6] / np))};
  static const double kW[6] = {109.4163228369586, 4.685925102200196, 2.491781270704224,
                               2.167275675983448, 4.55227651921194,  2.847714678987977};
  double total = 0.0;
  for (int k = 0; k < 6; ++k) {
    total += kW[k] * v[k];
    if (terms) terms[k] = v[k];
  }
  *score = total;
  return JXG_OK;
}

int32_t jxg_op_epf_fit(void* ctx, const float* source_y, const float* recon, uint64_t width, uint64_t height,
                       const float* sigma_quant, float distance, float* choice, double* score) {
  using namespace jxg;
  Context* c = static_cast<Context*>(ctx);
  if (!c || !source_y || !recon || !sigma_quant || !choice || !score) return JXG_ERR_INVALID_ARGUMENT;
  if (width < 4 || height < 4) return fail(c, JXG_ERR_INVALID_ARGUMENT, "the fit needs 4 x 4 pixels");
  if (width > kMaxDimension || height > kMaxDimension)
    return fail(c, JXG_ERR_DIMENSION_TOO_LARGE, "dimension too large");
  if (!(distance > 0.0f) || !std::isfinite(distance)) return fail(c, JXG_ERR_INVALID_DISTANCE, "distance");
  cudaSetDevice(c->device);
  const int w = static_cast<int>(width), h = static_cast<int>(height);
  const int64_t n = static_cast<int64_t>(w) * h;
  const int xb = (w + 7) / 8, yb = (h + 7) / 8;
  const int64_t nb = static_cast<int64_t>(xb) * yb;
  const int lw[2] = {w / 2, (w / 2) / 2}, lh[2] = {h / 2, (h / 2) / 2};
  const int64_t m[2] = {static_cast<int64_t>(lw[0]) * lh[0], static_cast<int64_t>(lw[1]) * lh[1]};
  const size_t floats = 3 * n * 3 + 13 * n + n + 2 * nb + 17 * (m[0] + m[1]) + 2 * kProxySums * kRefineSlots + 64;
  int st;
  if ((st = ensure(c, c->op_in, floats * 4))) return st;
  float* p = static_cast<float*>(c->op_in.ptr);
  float* rec = p;
  float* outb[2] = {p + 3 * n, p + 6 * n};
  float* nw = p + 9 * n;
  float* cw = nw + 12 * n;
  float* src = cw + n;
  float* sq = src + n;
  float* sig = sq + nb;
  p = sig + nb;
  float *rv[2], *rmv[2], *tv[2], *tmp[2], *box[2], *sm[2], *parts[2];
  for (int l = 0; l < 2; ++l) {
    rv[l] = p;
    rmv[l] = rv[l] + m[l];
    tv[l] = rmv[l] + 2 * m[l];
    tmp[l] = tv[l] + m[l];
    box[l] = tmp[l] + 3 * m[l];
    sm[l] = box[l] + 3 * m[l];
    parts[l] = sm[l] + m[l];
    p = parts[l] + 3 * m[l];
  }
  double* sums = reinterpret_cast<double*>(p + (reinterpret_cast<uintptr_t>(p) & 4 ? 1 : 0));
  cudaStream_t s = c->stream;
  JXG_CUDA(c, cudaMemcpyAsync(rec, recon, 3 * n * 4, cudaMemcpyHostToDevice, s));
  JXG_CUDA(c, cudaMemcpyAsync(src, source_y, n * 4, cudaMemcpyHostToDevice, s));
  JXG_CUDA(c, cudaMemcpyAsync(sq, sigma_quant, nb * 4, cudaMemcpyHostToDevice, s));
  auto grid = [](int64_t k) { return static_cast<unsigned>((k + 255) / 256); };
  // the source's proxy levels, once (LumaProxy::new)
  k_proxy_half<<<grid(m[0]), 256, 0, s>>>(src, w, w, h, 1, rv[0]);
  k_proxy_half<<<grid(m[1]), 256, 0, s>>>(rv[0], lw[0], lw[0], lh[0], 0, rv[1]);
  for (int l = 0; l < 2; ++l) {
    k_proxy_box_v<<<(lw[l] + 127) / 128, 128, 0, s>>>(rv[l], nullptr, lw[l], lh[l], tmp[l]);
    k_proxy_box_h<<<(2 * lh[l] + 127) / 128, 128, 0, s>>>(tmp[l], 2, lw[l], lh[l], rmv[l]);
    k_proxy_variance<<<grid(m[l]), 256, 0, s>>>(rmv[l], m[l]);
  }
  JXG_CUDA(c, cudaGetLastError());
  RefineArgs r{};
  r.w = w;
  r.h = h;
  r.xb = xb;
  r.yb = yb;
  r.epf_channel[0] = 40.0f;  // the encoder's XYB channel scales (LoopFilter defaults)
  r.epf_channel[1] = 5.0f;
  r.epf_channel[2] = 3.5f;
  r.sigma = sig;
  const double np_pairs = static_cast<double>(h) * (w - 1) + static_cast<double>(h - 1) * w;
  std::vector<float> host_sigma(nb);
  bool have_unfiltered = false;
  float unfiltered_score = 0.0f;
  int failure = JXG_OK;
  auto proxy_of = [&](const float* y) -> float {
    cudaMemsetAsync(sums, 0, kProxySums * kRefineSlots * sizeof(double), s);
    k_proxy_half<<<grid(m[0]), 256, 0, s>>>(y, w, w, h, 1, tv[0]);
    k_proxy_half<<<grid(m[1]), 256, 0, s>>>(tv[0], lw[0], lw[0], lh[0], 0, tv[1]);
    for (int l = 0; l < 2; ++l) {
      k_proxy_box_v<<<(lw[l] + 127) / 128, 128, 0, s>>>(tv[l], rv[l], lw[l], lh[l], tmp[l]);
      k_proxy_box_h<<<(3 * lh[l] + 127) / 128, 128, 0, s>>>(tmp[l], 3, lw[l], lh[l], box[l]);
      k_proxy_pool<<<grid(m[l]), 256, 0, s>>>(rmv[l], box[l], m[l], sm[l], parts[l], sums + 2 * l * kRefineSlots);
    }
    k_proxy_gradients<<<grid(n), 256, 0, s>>>(src, y, w, w, h, sums + 4 * kRefineSlots);
    double host[kProxySums * kRefineSlots];
    if (cudaMemcpyAsync(host, sums, sizeof(host), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
      failure = fail(c, JXG_ERR_CUDA, "proxy");
      return INFINITY;
    }
    double t[kProxySums];
    for (int q = 0; q < kProxySums; ++q) {
      t[q] = 0.0;
      for (int k = 0; k < kRefineSlots; ++k) t[q] += host[q * kRefineSlots + k];
    }
    static const double kW[6] = {109.4163228369586, 4.685925102200196, 2.491781270704224,
                                 2.167275675983448, 4.55227651921194,  2.847714678987977};
    const double v[6] = {t[2] / static_cast<double>(m[1]), t[0] / static_cast<double>(m[0]),
                         std::sqrt(std::sqrt(t[1] / static_cast<double>(m[0]))), t[4] / np_pairs, t[5] / np_pairs,
                         std::sqrt(std::sqrt(t[6] / np_pairs))};
    double total = 0.0;
    for (int k = 0; k < 6; ++k) total += kW[k] * v[k];
    return static_cast<float>(total);
  };
  auto score_of = [&](const EpfChoice& ch) -> float {
    if (failure) return INFINITY;
    bool unfiltered = ch.iters == 0 || ch.sharpness == 0;
    const float* y = rec + n;
    if (!unfiltered) {
      // LoopFilter::new(iters, pass0, quant_mul, None): a signalled bundle
      // is read back through F16
      float q = 0.46f, p0 = 0.9f, p2 = 6.5f, border = 2.0f / 3.0f;
      const float s0 = !std::isnan(ch.pass0) ? ch.pass0 : (!std::isnan(ch.quant_mul) ? 0.9f : NAN);
      if (!std::isnan(s0)) {
        q = f16_round(!std::isnan(ch.quant_mul) ? ch.quant_mul : 0.46f);
        p0 = f16_round(s0);
        p2 = f16_round(6.5f);
        border = f16_round(2.0f / 3.0f);
      }
      r.epf_border = border;
      k_epf_sigma<<<grid(nb), 256, 0, s>>>(sq, nb, q, static_cast<float>(ch.sharpness) / 7.0f, sig);
      if (cudaMemcpyAsync(host_sigma.data(), sig, nb * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess) {
        failure = fail(c, JXG_ERR_CUDA, "sigma");
        return INFINITY;
      }
      bool any = false;
      for (float v : host_sigma) any = any || v >= -3.905243f;  // MIN_SIGMA
      if (!any) {
        unfiltered = true;
      } else {
        int stages[3], count = 0;
        float sms[3];
        if (ch.iters >= 3) {
          stages[count] = 0;
          sms[count++] = 1.65f * p0;
        }
        stages[count] = 1;
        sms[count++] = 1.65f;
        if (ch.iters >= 2) {
          stages[count] = 2;
          sms[count++] = 1.65f * p2;
        }
        const float* in = rec;
        for (int k = 0; k < count; ++k) {
          const dim3 g(static_cast<unsigned>((w + kEpfTW - 1) / kEpfTW), static_cast<unsigned>((h + kEpfTH - 1) / kEpfTH));
          k_refine_epf<<<g, 256, 0, s>>>(r, stages[k], sms[k], in, n, w, outb[k & 1], nw, cw);
          in = outb[k & 1];
        }
        y = in + n;
      }
    }
    if (unfiltered && have_unfiltered) return unfiltered_score;
    const float v = proxy_of(y);
    if (unfiltered) {
      have_unfiltered = true;
      unfiltered_score = v;
    }
    return v;
  };
  const EpfChoice base{static_cast<int>(choice[0]), choice[1], choice[2], static_cast<int>(choice[3])};
  if (base.iters < 0 || base.iters > 3 || base.sharpness < 0 || base.sharpness > 7)
    return fail(c, JXG_ERR_INVALID_ARGUMENT, "baseline iters 0..3, sharpness 0..7");
  const EpfChoice best = epf_choose(distance, base, score_of);
  if (failure) return failure;
  JXG_CUDA(c, cudaGetLastError());
  choice[0] = static_cast<float>(best.iters);
  choice[1] = best.quant_mul;
  choice[2] = best.pass0;
  choice[3] = static_cast<float>(best.sharpness);
  *score = score_of(best);
  return failure;
}

int32_t jxg_op_dct8x8(void* ctx, const float* blocks, uint64_t count, float* coefficients) {
  Context* c = static_cast<Context*>(ctx);
  if (!c || !blocks || !coefficients) return JXG_ERR_INVALID_ARGUMENT;
  if (count == 0) return JXG_OK;
  cudaSetDevice(c->device);
  int st;
  const size_t bytes = count * 64 * 4;
  if ((st = jxg::ensure(c, c->op_in, bytes)) || (st = jxg::ensure(c, c->op_out, bytes))) return st;
  cudaStream_t s = c->stream;
  JXG_CUDA(c, cudaMemcpyAsync(c->op_in.ptr, blocks, bytes, cudaMemcpyHostToDevice, s));
  const int grid = static_cast<int>((count + 31) / 32);
  st = jxg::launch(c, "k_dct8x8_blocks", c->timing, [&] {
    jxg::k_dct8x8_blocks<<<grid, 256, 0, s>>>(static_cast<const float*>(c->op_in.ptr),
                                              static_cast<int64_t>(count),
                                              static_cast<float*>(c->op_out.ptr));
  });
  if (st) return st;
  JXG_CUDA(c, cudaMemcpyAsync(coefficients, c->op_out.ptr, bytes, cudaMemcpyDeviceToHost, s));
  return jxg::wait(c);
}

int32_t jxg_op_dct(void* ctx, int32_t kind, const float* blocks, uint64_t count,
                   float* coefficients, float* dc_values) {
  Context* c = static_cast<Context*>(ctx);
  static const int kW[15] = {8, 16, 8, 16, 32, 16, 32, 8, 32, 64, 32, 64, 128, 64, 128};
  static const int kH[15] = {8, 8, 16, 16, 16, 32, 32, 32, 8, 64, 64, 32, 128, 128, 64};
  static const int kDc[15] = {1, 2, 2, 4, 8, 8, 16, 4, 4, 64, 32, 32, 256, 128, 128};
  if (!c || !blocks || !coefficients || kind < 0 || kind > 14) return JXG_ERR_INVALID_ARGUMENT;
  if (count == 0) return JXG_OK;
  if (count > (1ull << 31)) return JXG_ERR_DIMENSION_TOO_LARGE;
  cudaSetDevice(c->device);
  const int n = kW[kind] * kH[kind], ndc = kDc[kind];
  const size_t bytes = count * n * 4, dc_bytes = count * ndc * 4;
  int st;
  if ((st = jxg::ensure(c, c->op_in, bytes)) || (st = jxg::ensure(c, c->op_out, bytes + dc_bytes)))
    return st;
  cudaStream_t s = c->stream;
  const float* din = static_cast<const float*>(c->op_in.ptr);
  float* dout = static_cast<float*>(c->op_out.ptr);
  float* ddc = dout + count * n;
  JXG_CUDA(c, cudaMemcpyAsync(c->op_in.ptr, blocks, bytes, cudaMemcpyHostToDevice, s));
  const int64_t cnt = static_cast<int64_t>(count);
  // one warp per block, dct_warps<W, H>() blocks per CTA
  auto run = [&](auto kernel, int warps) {
    kernel<<<static_cast<unsigned>((count + warps - 1) / warps), 32 * warps, 0, s>>>(
        din, cnt, dout, ddc, kind, ndc);
  };
  // the 128-point family: one warp per block, its tile in dynamic shared memory
  auto run_large = [&](auto kernel, size_t smem) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(smem));
    kernel<<<static_cast<unsigned>(count), 32, smem, s>>>(din, cnt, dout, ddc, kind, ndc);
  };
  st = jxg::launch(c, "k_dct_blocks", c->timing, [&] {
    using namespace jxg;
    switch (kind) {
      case kDct8x8:
        k_dct8x8_blocks<<<static_cast<unsigned>((count + 31) / 32), 256, 0, s>>>(din, cnt, dout);
        break;
      case kDct8x16: run(k_dct_blocks<16, 8, false>, dct_warps<16, 8>()); break;
      case kDct16x8: run(k_dct_blocks<8, 16, true>, dct_warps<8, 16>()); break;
      case kDct16x16: run(k_dct_blocks<16, 16, true>, dct_warps<16, 16>()); break;
      case kDct16x32: run(k_dct_blocks<32, 16, false>, dct_warps<32, 16>()); break;
      case kDct32x16: run(k_dct_blocks<16, 32, true>, dct_warps<16, 32>()); break;
      case kDct32x32: run(k_dct_blocks<32, 32, true>, dct_warps<32, 32>()); break;
      case kDct32x8: run(k_dct_blocks<8, 32, true>, dct_warps<8, 32>()); break;
      case kDct8x32: run(k_dct_blocks<32, 8, false>, dct_warps<32, 8>()); break;
      case kDct64x64: run(k_dct_blocks<64, 64, true>, dct_warps<64, 64>()); break;
      case kDct64x32: run(k_dct_blocks<32, 64, true>, dct_warps<32, 64>()); break;
      case kDct32x64: run(k_dct_blocks<64, 32, false>, dct_warps<64, 32>()); break;
      case kDct128x128:
        run_large(k_dct_large_blocks<128, 128, true>, large_dct_smem<128, 128>());
        break;
      case kDct128x64:
        run_large(k_dct_large_blocks<64, 128, true>, large_dct_smem<64, 128>());
        break;
      default:  // 64x128
        run_large(k_dct_large_blocks<128, 64, false>, large_dct_smem<128, 64>());
    }
  });
  if (st) return st;
  JXG_CUDA(c, cudaMemcpyAsync(coefficients, dout, bytes, cudaMemcpyDeviceToHost, s));
  if (dc_values && kind != jxg::kDct8x8)
    JXG_CUDA(c, cudaMemcpyAsync(dc_values, ddc, dc_bytes, cudaMemcpyDeviceToHost, s));
  if ((st = jxg::wait(c))) return st;
  if (dc_values && kind == jxg::kDct8x8)  // an 8x8 block's DC is its first coefficient
    for (uint64_t i = 0; i < count; ++i) dc_values[i] = coefficients[i * 64];
  return JXG_OK;
}

int32_t jxg_op_idct(void* ctx, int32_t kind, const float* coefficients, uint64_t count,
                    float* blocks) {
  Context* c = static_cast<Context*>(ctx);
  static const int kW[15] = {8, 16, 8, 16, 32, 16, 32, 8, 32, 64, 32, 64, 128, 64, 128};
  static const int kH[15] = {8, 8, 16, 16, 16, 32, 32, 32, 8, 64, 64, 32, 128, 128, 64};
  if (!c || !coefficients || !blocks || kind < 0 || kind > 14) return JXG_ERR_INVALID_ARGUMENT;
  if (count == 0) return JXG_OK;
  if (count > (1ull << 31)) return JXG_ERR_DIMENSION_TOO_LARGE;
  cudaSetDevice(c->device);
  const size_t bytes = count * kW[kind] * kH[kind] * 4;
  int st;
  if ((st = jxg::ensure(c, c->op_in, bytes)) || (st = jxg::ensure(c, c->op_out, bytes))) return st;
  cudaStream_t s = c->stream;
  const float* din = static_cast<const float*>(c->op_in.ptr);
  float* dout = static_cast<float*>(c->op_out.ptr);
  JXG_CUDA(c, cudaMemcpyAsync(c->op_in.ptr, coefficients, bytes, cudaMemcpyHostToDevice, s));
  const int64_t cnt = static_cast<int64_t>(count);
  auto run = [&](auto kernel, int warps) {
    kernel<<<static_cast<unsigned>((count + warps - 1) / warps), 32 * warps, 0, s>>>(din, cnt, dout);
  };
  auto run_large = [&](auto kernel, size_t smem) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(smem));
    kernel<<<static_cast<unsigned>(count), 32, smem, s>>>(din, cnt, dout);
  };
  st = jxg::launch(c, "k_idct_blocks", c->timing, [&] {
    using namespace jxg;
    switch (kind) {
      case kDct8x8: run(k_idct_blocks<8, 8, kIdctSquare>, dct_warps<8, 8>()); break;
      case kDct8x16: run(k_idct_blocks<16, 8, kIdctRowsFirst>, dct_warps<16, 8>()); break;
      case kDct16x8: run(k_idct_blocks<8, 16, kIdctColsFirst>, dct_warps<8, 16>()); break;
      case kDct16x16: run(k_idct_blocks<16, 16, kIdctSquare>, dct_warps<16, 16>()); break;
      case kDct16x32: run(k_idct_blocks<32, 16, kIdctRowsFirst>, dct_warps<32, 16>()); break;
      case kDct32x16: run(k_idct_blocks<16, 32, kIdctColsFirst>, dct_warps<16, 32>()); break;
      case kDct32x32: run(k_idct_blocks<32, 32, kIdctSquare>, dct_warps<32, 32>()); break;
      case kDct32x8: run(k_idct_blocks<8, 32, kIdctColsFirst>, dct_warps<8, 32>()); break;
      case kDct8x32: run(k_idct_blocks<32, 8, kIdctRowsFirst>, dct_warps<32, 8>()); break;
      case kDct64x64: run(k_idct_blocks<64, 64, kIdctSquare>, dct_warps<64, 64>()); break;
      case kDct64x32: run(k_idct_blocks<32, 64, kIdctColsFirst>, dct_warps<32, 64>()); break;
      case kDct32x64: run(k_idct_blocks<64, 32, kIdctRowsFirst>, dct_warps<64, 32>()); break;
      case kDct128x128:
        run_large(k_idct_large_blocks<128, 128, kIdctSquare>, large_dct_smem<128, 128>());
        break;
      case kDct128x64:
        run_large(k_idct_large_blocks<64, 128, kIdctColsFirst>, large_dct_smem<64, 128>());
        break;
      default:  // 64x128
        run_large(k_idct_large_blocks<128, 64, kIdctRowsFirst>, large_dct_smem<128, 64>());
    }
  });
  if (st) return st;
  JXG_CUDA(c, cudaMemcpyAsync(blocks, dout, bytes, cudaMemcpyDeviceToHost, s));
  return jxg::wait(c);
}

int32_t jxg_op_small_transform(void* ctx, int32_t kind, const float* blocks, uint64_t count,
                               float* out) {
  Context* c = static_cast<Context*>(ctx);
  if (!c || !blocks || !out || kind < 0 || kind > 10) return JXG_ERR_INVALID_ARGUMENT;
  if (count == 0) return JXG_OK;
  if (count > (1ull << 31)) return JXG_ERR_DIMENSION_TOO_LARGE;
  cudaSetDevice(c->device);
  const size_t bytes = count * 64 * 4;
  int st;
  if ((st = jxg::ensure(c, c->op_in, bytes)) || (st = jxg::ensure(c, c->op_out, bytes))) return st;
  cudaStream_t s = c->stream;
  JXG_CUDA(c, cudaMemcpyAsync(c->op_in.ptr, blocks, bytes, cudaMemcpyHostToDevice, s));
  st = jxg::launch(c, "k_small_transform_blocks", c->timing, [&] {
    jxg::k_small_transform_blocks<<<static_cast<unsigned>((count + 127) / 128), 128, 0, s>>>(
        kind, static_cast<const float*>(c->op_in.ptr), static_cast<int64_t>(count),
        static_cast<float*>(c->op_out.ptr));
  });
  if (st) return st;
  JXG_CUDA(c, cudaMemcpyAsync(out, c->op_out.ptr, bytes, cudaMemcpyDeviceToHost, s));
  return jxg::wait(c);
}

int32_t jxg_op_pack_tokens(void* ctx, const jxg_token* tokens, const uint64_t* group_offsets,
                           uint64_t num_groups, uint32_t* words, uint64_t capacity,
                           uint64_t* word_offsets) {
  Context* c = static_cast<Context*>(ctx);
  if (!c || !group_offsets || num_groups == 0 || num_groups > 0x7FFFFFFFull)
    return JXG_ERR_INVALID_ARGUMENT;
  for (uint64_t g = 0; g < num_groups; ++g)
    if (group_offsets[g + 1] < group_offsets[g]) return JXG_ERR_INVALID_ARGUMENT;
  const uint64_t first = group_offsets[0];
  const uint64_t n = group_offsets[num_groups] - first;
  if (n && !tokens) return JXG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  const size_t tok_bytes = (n * 8 + 15) / 16 * 16, off_bytes = (num_groups + 1) * 8;
  const size_t flag_bytes = (num_groups * 4 + 15) / 16 * 16;
  const uint64_t cap = std::min<uint64_t>(capacity, 2 * n);
  int st;
  if ((st = jxg::ensure(c, c->op_in, tok_bytes + off_bytes + flag_bytes)) ||
      (st = jxg::ensure(c, c->op_out, (cap * 4 + 15) / 16 * 16 + off_bytes + 8)))
    return st;
  char* in = static_cast<char*>(c->op_in.ptr);
  uint2* d_tok = reinterpret_cast<uint2*>(in);
  uint64_t* d_goffs = reinterpret_cast<uint64_t*>(in + tok_bytes);
  uint32_t* d_wide = reinterpret_cast<uint32_t*>(in + tok_bytes + off_bytes);
  char* outp = static_cast<char*>(c->op_out.ptr);
  uint32_t* d_words = reinterpret_cast<uint32_t*>(outp);
  uint64_t* d_woffs = reinterpret_cast<uint64_t*>(outp + (cap * 4 + 15) / 16 * 16);
  uint64_t* d_count = d_woffs + num_groups + 1;
  cudaStream_t s = c->stream;
  if (n) JXG_CUDA(c, cudaMemcpyAsync(d_tok, tokens + first, n * 8, cudaMemcpyHostToDevice, s));
  std::vector<uint64_t> rebased(group_offsets, group_offsets + num_groups + 1);
  for (uint64_t& o : rebased) o -= first;
  JXG_CUDA(c, cudaMemcpyAsync(d_goffs, rebased.data(), off_bytes, cudaMemcpyHostToDevice, s));
  JXG_CUDA(c, cudaMemsetAsync(d_wide, 0, num_groups * 4, s));
  const dim3 grid(jxg::kPackCtasPerGroup, static_cast<unsigned>(std::min<uint64_t>(num_groups, 65535)));
  if ((st = jxg::launch(c, "k_token_group_flags", c->timing, [&] {
         jxg::k_token_group_flags<<<grid, 256, 0, s>>>(d_tok, d_goffs, static_cast<int>(num_groups),
                                                       d_wide);
       })) ||
      (st = jxg::launch(c, "k_pack_tokens", c->timing, [&] {
         jxg::k_pack_tokens<<<grid, 256, 0, s>>>(d_tok, d_goffs, d_wide, nullptr,
                                                 static_cast<int>(num_groups),
                                                 words ? d_words : nullptr, cap, d_woffs, d_count);
       })))
    return st;
  uint64_t count = 0;
  JXG_CUDA(c, cudaMemcpyAsync(&count, d_count, 8, cudaMemcpyDeviceToHost, s));
  if ((st = jxg::wait(c))) return st;
  if (word_offsets)
    JXG_CUDA(c, cudaMemcpyAsync(word_offsets, d_woffs, off_bytes, cudaMemcpyDeviceToHost, s));
  if (words && count > capacity) {
    if ((st = jxg::wait(c))) return st;
    return jxg::fail(c, JXG_ERR_INVALID_ARGUMENT, "packed token buffer too small");
  }
  if (words && count)
    JXG_CUDA(c, cudaMemcpyAsync(words, d_words, count * 4, cudaMemcpyDeviceToHost, s));
  return jxg::wait(c);
}

int32_t jxg_token_offsets_noalloc(const uint32_t* counts, uint64_t num_groups, uint32_t* offsets,
                                  uint64_t* group_offsets, void* cuda_stream) {
  if (!counts || !offsets || !group_offsets || num_groups == 0) return JXG_ERR_INVALID_ARGUMENT;
  if (num_groups > JXG_NOALLOC_MAX_GROUPS) return JXG_ERR_DIMENSION_TOO_LARGE;
  int device = -1;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= jxg::kMaxDevices)
    return JXG_ERR_CUDA;
  jxg::NoAllocScanScratch* scratch = nullptr;
  int st = jxg::noalloc_scratch(device, &scratch);
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  const int64_t n = static_cast<int64_t>(num_groups) * 3 * 1024;
  const int chunks = static_cast<int>((n + jxg::kScanChunk - 1) / jxg::kScanChunk);
  // the middle step writes the pass scalars: start them from zero
  if (cudaMemsetAsync(&scratch->stats, 0, sizeof(scratch->stats), s) != cudaSuccess)
    return JXG_ERR_CUDA;
  jxg::k_scan_reduce<<<chunks, jxg::kScanThreads, 0, s>>>(counts, n, scratch->chunk_sums);
  jxg::k_scan_chunks<<<1, jxg::kScanThreads, 0, s>>>(scratch->chunk_sums, chunks,
                                                     &scratch->stats.num_tokens, group_offsets,
                                                     static_cast<int>(num_groups));
  jxg::k_scan_apply<<<chunks, jxg::kScanThreads, 0, s>>>(counts, n, scratch->chunk_sums, offsets,
                                                         group_offsets, 3 * 1024);
  return cudaGetLastError() == cudaSuccess ? JXG_OK : JXG_ERR_CUDA;
}

int32_t jxg_selftest_bounded_wait(void* ctx, uint32_t polls) {
  Context* c = static_cast<Context*>(ctx);
  if (!c) return JXG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  int st;
  if ((st = jxg::ensure(c, c->op_out, 256))) return st;
  uint32_t* flag = static_cast<uint32_t*>(c->op_out.ptr);  // never set
  uint32_t* result = flag + 1;
  JXG_CUDA(c, cudaMemsetAsync(flag, 0, 8, c->stream));
  jxg::k_wait_selftest<<<1, 32, 0, c->stream>>>(flag, polls, result);
  JXG_CUDA(c, cudaGetLastError());
  uint32_t r = 0;
  JXG_CUDA(c, cudaMemcpyAsync(&r, result, 4, cudaMemcpyDeviceToHost, c->stream));
  if ((st = jxg::wait(c))) return st;
  if (r == 2u) return jxg::fail(c, JXG_ERR_DEVICE_TIMEOUT, "bounded wait ran out (self-test)");
  return r == 1u ? JXG_OK : JXG_ERR_CUDA;
}

int32_t jxg_selftest_token_lookback(void* ctx, uint32_t polls) {
  Context* c = static_cast<Context*>(ctx);
  if (!c) return JXG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  int st;
  if ((st = jxg::ensure(c, c->op_out, 256))) return st;
  auto* status = static_cast<unsigned long long*>(c->op_out.ptr);  // ticket, chunk 0, chunk 1
  auto* flags = reinterpret_cast<uint32_t*>(status + 4);
  JXG_CUDA(c, cudaMemsetAsync(status, 0, 64, c->stream));
  jxg::k_lookback_selftest<<<1, 32, 0, c->stream>>>(status, polls, flags);
  JXG_CUDA(c, cudaGetLastError());
  uint32_t r = 0;
  JXG_CUDA(c, cudaMemcpyAsync(&r, flags, 4, cudaMemcpyDeviceToHost, c->stream));
  if ((st = jxg::wait(c))) return st;
  if (r & jxg::kFlagTokenTimeout)
    return jxg::fail(c, JXG_ERR_DEVICE_TIMEOUT, "token look-back wait ran out (self-test)");
  return JXG_ERR_CUDA;
}

int32_t jxg_selftest_math(void* ctx, int32_t which, uint32_t lo_bits, uint32_t hi_bits,
                          uint64_t* mismatches, uint32_t* first_bad) {
  Context* c = static_cast<Context*>(ctx);
  if (!c || !mismatches || !first_bad || hi_bits < lo_bits || which < 0 || which > 8)
    return JXG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  int st;
  if ((st = jxg::ensure(c, c->op_out, 256))) return st;
  auto* count = static_cast<unsigned long long*>(c->op_out.ptr);
  auto* first = reinterpret_cast<uint32_t*>(count + 1);
  // masking_sqrt's multiplier as the front end computes it
  jxg::DistanceParams dp;
  jxg::compute_distance_params(1.0f, &dp);
  jxg::KernelArgs ka;
  jxg::fill_kernel_args(dp, &ka);
  JXG_CUDA(c, cudaMemsetAsync(count, 0, 8, c->stream));
  JXG_CUDA(c, cudaMemsetAsync(first, 0xFF, 4, c->stream));
  jxg::k_math_selftest<<<c->num_sms * 8, 256, 0, c->stream>>>(which, ka.aq_masking_sqrt_mul, lo_bits,
                                                               hi_bits, count, first);
  JXG_CUDA(c, cudaGetLastError());
  unsigned long long n = 0;
  JXG_CUDA(c, cudaMemcpyAsync(&n, count, 8, cudaMemcpyDeviceToHost, c->stream));
  JXG_CUDA(c, cudaMemcpyAsync(first_bad, first, 4, cudaMemcpyDeviceToHost, c->stream));
  if ((st = jxg::wait(c))) return st;
  *mismatches = n;
  return JXG_OK;
}

int32_t jxg_frontend_run_with_field(void* ctx, const void* pixels, uint64_t width, uint64_t height,
                                    int32_t channels, int32_t bits, const jxg_config* config,
                                    const uint8_t* quant_field, int32_t pixels_on_device) {
  using namespace jxg;
  Context* c = static_cast<Context*>(ctx);
  if (!c || !quant_field || !config) return JXG_ERR_INVALID_ARGUMENT;
  if (config->speed != JXG_SPEED_ULTRAFAST)
    return fail(c, JXG_ERR_UNSUPPORTED, "a caller's quant field needs the UltraFast gates");
  if (c->async_pending) {
    const int st = jxg_frontend_wait(ctx);
    if (st) return st;
  }
  cudaSetDevice(c->device);
  int st;
  if ((st = validate(c, pixels, width, height, channels, bits, config))) return st;
  const size_t nb = static_cast<size_t>((width + 7) / 8) * ((height + 7) / 8);
  if ((st = ensure(c, c->field_buf, nb))) return st;
  cudaPointerAttributes at{};
  const bool device_field =
      cudaPointerGetAttributes(&at, quant_field) == cudaSuccess && at.type == cudaMemoryTypeDevice;
  cudaGetLastError();  // a host pointer may leave an error behind on some drivers
  JXG_CUDA(c, cudaMemcpyAsync(c->field_buf.ptr, quant_field, nb,
                              device_field ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->stream));
  c->qf_override = static_cast<const uint8_t*>(c->field_buf.ptr);
  st = single_pass(c, pixels, width, height, channels, bits, config, pixels_on_device != 0);
  c->qf_override = nullptr;
  if (st || pixels_on_device) return st;
  return wait(c);
}

namespace {
int refine_grid(int64_t n) { return static_cast<int>((n + 255) / 256); }
}  // namespace

int32_t jxg_refine_begin(void* ctx, uint64_t* width, uint64_t* height) {
  using namespace jxg;
  Context* c = static_cast<Context*>(ctx);
  if (!c || !width || !height) return JXG_ERR_INVALID_ARGUMENT;
  if (c->async_pending) {
    const int st = jxg_frontend_wait(ctx);
    if (st) return st;
  }
  c->refine_ready = false;
  if (!c->have_frame || c->layouts.size() != 1 || c->layouts[0].searched)
    return fail(c, JXG_ERR_UNSUPPORTED, "refinement needs a one-frame UltraFast pass on the context first");
  cudaSetDevice(c->device);
  int st;
  if ((st = wait(c))) return st;
  const Frame& f0 = *reinterpret_cast<const Frame*>(static_cast<const char*>(c->plan_host.ptr) +
                                                    c->plan_slot * c->plan_slot_cap);
  const KernelArgs& a = f0.a;
  RefineArgs& r = c->refine;
  r = RefineArgs{};
  r.w = a.width;
  r.h = a.height;
  r.xb = a.xb;
  r.yb = a.yb;
  r.pw = a.xb * 8;
  r.plane = a.plane;
  r.xyb = f0.xyb;  // read by this call only
  r.tiles_x = a.tiles_x;
  r.scale = a.scale;
  std::memcpy(r.qm_mul, a.qm_mul, sizeof(r.qm_mul));
  std::memcpy(r.matrix, a.matrix, sizeof(r.matrix));
  std::memcpy(r.inv_matrix, a.inv_matrix, sizeof(r.inv_matrix));
  std::memcpy(r.thresholds, a.thresholds, sizeof(r.thresholds));
  const int64_t nb = static_cast<int64_t>(r.xb) * r.yb, pp = static_cast<int64_t>(r.pw) * r.yb * 8;
  for (int k = 0; k < 3; ++k) {
    c->refine_w[k] = r.w >> k;
    c->refine_h[k] = r.h >> k;
    c->refine_n[k] = static_cast<int64_t>(c->refine_w[k]) * c->refine_h[k];
  }
  const int64_t n = c->refine_n[0], n1 = c->refine_n[1], n2 = c->refine_n[2];
  // one allocation: coef, chat, levels (nb x 192), recon and its gradient
  // (3 pp), bits, M, the linear planes and gradients per scale, the moment,
  // blur and gradient maps, four f64 sums
  const int64_t tiles = static_cast<int64_t>(a.tiles_x) * a.tiles_y;
  // the decoder's EPF at this frame's loop-filter settings
  jxg_frame_params fp{};
  if ((st = read_params(c, 0, &fp))) return st;
  LoopFilterParams lfp{};
  loop_filter_params(a.distance, &lfp);
  r.epf_stages = 0;
  if (fp.epf_iters > 0 && fp.epf_sharpness > 0 && r.w >= 4 && r.h >= 4) {
    const float sad_mul = 1.65f;  // SAD_MUL, src/epf_filter.rs:45
    if (fp.epf_iters == 1) {
      r.epf_stages = 1;
      r.epf_stage[0] = 1;
      r.epf_sm[0] = sad_mul;
    } else if (fp.epf_iters == 2) {
      r.epf_stages = 2;
      r.epf_stage[0] = 1;
      r.epf_sm[0] = sad_mul;
      r.epf_stage[1] = 2;
      r.epf_sm[1] = sad_mul * lfp.pass2;
    } else {
      r.epf_stages = 3;
      r.epf_stage[0] = 0;
      r.epf_sm[0] = sad_mul * lfp.pass0;
      r.epf_stage[1] = 1;
      r.epf_sm[1] = sad_mul;
      r.epf_stage[2] = 2;
      r.epf_sm[2] = sad_mul * lfp.pass2;
    }
  }
  r.epf_border = lfp.border;
  std::memcpy(r.epf_channel, lfp.channel_scale, sizeof(r.epf_channel));
  r.epf_quant_mul = lfp.quant_mul;
  r.epf_lut = static_cast<float>(fp.epf_sharpness) / 7.0f;
  r.epf_quant_scale = a.scale;
  const int64_t epf_planes = r.epf_stages ? 3 * r.epf_stages + 20 + r.epf_stages : 0;
  // the luma proxy's levels (half and quarter) and the source's Y plane
  c->refine_proxy = r.w >= 4 && r.h >= 4;
  const int64_t w2 = r.w / 2, h2 = r.h / 2, w4 = w2 / 2, h4 = h2 / 2;
  const int64_t proxy_floats = c->refine_proxy ? n + 20 * (w2 * h2 + w4 * h4) : 0;
  // one allocation: source coefficients (nb x 192), the decoded XYB planes
  // (3 pp), M and M^T, the source and decoded linear planes and the gradient
  // per scale, the f64 sums, theta, its gradient and Adam moments, copies of
  // the field and the colour maps; each piece rounded up to 64 floats
  const size_t floats = nb * 192 + 3 * nb + 3 * pp + 2 * 4096 + 3 * 3 * (n + n1 + n2) + 2 * 4 * kRefineSlots +
                        4 * nb + (nb + 2 * tiles) / 4 + nb + epf_planes * n + 6 * n + proxy_floats +
                        2 * kProxySums * kRefineSlots + 64 + 64 * 90;
  if ((st = ensure(c, c->refine_buf, floats * 4 + 256))) return st;
  float* base = static_cast<float*>(c->refine_buf.ptr);
  auto take = [&](int64_t count) {
    float* p = base;
    base += (count + 63) / 64 * 64;
    return p;
  };
  r.coef = take(nb * 192);
  r.dc = take(3 * nb);
  r.sigma = take(nb);
  for (int k = 0; k < r.epf_stages; ++k) {
    const int nn = r.epf_stage[k] == 0 ? 12 : 4;
    c->refine_epf_out[k] = take(3 * n);
    c->refine_epf_nw[k] = take(nn * n);
    c->refine_epf_cw[k] = take(n);
  }
  c->refine_epf_g[0] = take(3 * n);
  c->refine_epf_g[1] = take(3 * n);
  c->refine_proxy_sums = reinterpret_cast<double*>(take(2 * kProxySums * kRefineSlots));
  c->refine_proxy_k = reinterpret_cast<ProxyScalars*>(take(64));
  if (c->refine_proxy) {
    c->refine_src_y = take(n);
    const int64_t dims[2][2] = {{w2, h2}, {w4, h4}};
    for (int l = 0; l < 2; ++l) {
      auto& L = c->refine_pl[l];
      L.w = static_cast<int>(dims[l][0]);
      L.h = static_cast<int>(dims[l][1]);
      const int64_t m = dims[l][0] * dims[l][1];
      L.ref_vals = take(m);
      L.ref_mv = take(2 * m);
      L.vals = take(m);
      L.tmp = take(3 * m);
      L.box = take(3 * m);
      L.s = take(m);
      L.parts = take(3 * m);
      L.g = take(3 * m);
      L.gtmp = take(3 * m);
      L.gv = take(m);
    }
  }
  r.recon = take(3 * pp);
  r.m = take(4096);
  r.mt = take(4096);
  for (int k = 0; k < 3; ++k) {
    c->refine_lin[0][k] = take(3 * c->refine_n[k]);
    c->refine_lin[1][k] = take(3 * c->refine_n[k]);
    c->refine_glin[k] = take(3 * c->refine_n[k]);
  }
  c->refine_sums = reinterpret_cast<double*>(take(2 * 4 * kRefineSlots));
  c->refine_theta = take(nb);
  c->refine_grad = take(nb);
  c->refine_adam = take(2 * nb);
  // the pass's field and colour maps, copied: a later pass on the context
  // may overwrite or move its own buffers
  uint8_t* qf = reinterpret_cast<uint8_t*>(take((nb + 3) / 4));
  int8_t* ytox = reinterpret_cast<int8_t*>(take((tiles + 3) / 4));
  int8_t* ytob = reinterpret_cast<int8_t*>(take((tiles + 3) / 4));
  cudaStream_t s = c->stream;
  JXG_CUDA(c, cudaMemcpyAsync(qf, f0.qf, nb, cudaMemcpyDeviceToDevice, s));
  JXG_CUDA(c, cudaMemcpyAsync(ytox, f0.ytox, tiles, cudaMemcpyDeviceToDevice, s));
  JXG_CUDA(c, cudaMemcpyAsync(ytob, f0.ytob, tiles, cudaMemcpyDeviceToDevice, s));
  JXG_CUDA(c, cudaMemsetAsync(c->refine_theta, 0, nb * 4, s));
  r.qf = qf;
  r.ytox = ytox;
  r.ytob = ytob;
  c->refine_steps = 0;
  // M: the library's 8x8 inverse of each unit coefficient vector
  std::vector<float> unit(64 * 64, 0.0f), cols(64 * 64);
  for (int j = 0; j < 64; ++j) unit[j * 64 + j] = 1.0f;
  if ((st = ensure(c, c->op_in, unit.size() * 4)) || (st = ensure(c, c->op_out, unit.size() * 4))) return st;
  JXG_CUDA(c, cudaMemcpyAsync(c->op_in.ptr, unit.data(), unit.size() * 4, cudaMemcpyHostToDevice, s));
  k_idct_blocks<8, 8, kIdctSquare><<<(64 + dct_warps<8, 8>() - 1) / dct_warps<8, 8>(), 32 * dct_warps<8, 8>(), 0, s>>>(
      static_cast<const float*>(c->op_in.ptr), 64, static_cast<float*>(c->op_out.ptr));
  JXG_CUDA(c, cudaGetLastError());
  JXG_CUDA(c, cudaMemcpyAsync(cols.data(), c->op_out.ptr, cols.size() * 4, cudaMemcpyDeviceToHost, s));
  if ((st = wait(c))) return st;
  // cols[j][p] is the image of coefficient j: M[p][j], M^T[j][p]
  std::vector<float> m(4096);
  for (int j = 0; j < 64; ++j)
    for (int p = 0; p < 64; ++p) m[p * 64 + j] = cols[j * 64 + p];
  JXG_CUDA(c, cudaMemcpyAsync(r.m, m.data(), 4096 * 4, cudaMemcpyHostToDevice, s));
  JXG_CUDA(c, cudaMemcpyAsync(r.mt, cols.data(), 4096 * 4, cudaMemcpyHostToDevice, s));
  const bool timed = c->timing;
  if ((st = launch(c, "k_refine_dct", timed, [&] {
         k_refine_dct<<<static_cast<unsigned>((nb + 7) / 8), 256, 0, s>>>(r);
       })) ||
      (st = launch(c, "k_refine_dc", timed, [&] {
         k_refine_dc<<<refine_grid(nb), 256, 0, s>>>(f0.quant_dc, nb, a.inv_dc_factor[0], a.inv_dc_factor[1],
                                                     a.inv_dc_factor[2], a.cfl_dc_factor_x, a.cfl_dc_factor_b, r.dc);
       })) ||
      (st = launch(c, "k_refine_linear", timed, [&] {
         k_refine_linear<<<refine_grid(n), 256, 0, s>>>(r.xyb, r.plane, r.w, c->refine_lin[0][0], r.w, r.h);
       })))
    return st;
  for (int k = 1; k < 3; ++k)
    if (c->refine_n[k] && (st = launch(c, "k_refine_down", timed, [&] {
                             k_refine_down<<<refine_grid(3 * c->refine_n[k]), 256, 0, s>>>(
                                 c->refine_lin[0][k - 1], c->refine_lin[0][k], c->refine_w[k - 1], c->refine_h[k - 1]);
                           })))
      return st;
  if (c->refine_proxy) {
    // the source's Y plane and its proxy levels: values, box mean and variance
    JXG_CUDA(c, cudaMemcpyAsync(c->refine_src_y, r.xyb + r.plane, n * 4, cudaMemcpyDeviceToDevice, s));
    auto& H = c->refine_pl[0];
    auto& Q = c->refine_pl[1];
    k_proxy_half<<<refine_grid(static_cast<int64_t>(H.w) * H.h), 256, 0, s>>>(c->refine_src_y, r.w, r.w, r.h, 1,
                                                                              H.ref_vals);
    k_proxy_half<<<refine_grid(static_cast<int64_t>(Q.w) * Q.h), 256, 0, s>>>(H.ref_vals, H.w, H.w, H.h, 0,
                                                                              Q.ref_vals);
    for (auto* L : {&H, &Q}) {
      const int64_t m = static_cast<int64_t>(L->w) * L->h;
      k_proxy_box_v_par<<<refine_grid(m), 256, 0, s>>>(L->ref_vals, nullptr, L->w, L->h, L->tmp);
      k_proxy_box_h_par<<<refine_grid(2 * m), 256, 0, s>>>(L->tmp, 2, L->w, L->h, L->ref_mv);
      k_proxy_variance<<<refine_grid(m), 256, 0, s>>>(L->ref_mv, m);
    }
    JXG_CUDA(c, cudaGetLastError());
  }
  if ((st = wait(c))) return st;
  r.xyb = nullptr;
  c->refine_ready = true;
  *width = static_cast<uint64_t>(r.w);
  *height = static_cast<uint64_t>(r.h);
  return JXG_OK;
}

int32_t jxg_refine_eval(void* ctx, const float* theta, float rate_lambda, float* grad, double* loss3,
                        int32_t* levels) {
  using namespace jxg;
  Context* c = static_cast<Context*>(ctx);
  if (!c || !loss3) return JXG_ERR_INVALID_ARGUMENT;
  if (!c->refine_ready) return fail(c, JXG_ERR_INVALID_ARGUMENT, "jxg_refine_begin first");
  if (!theta) theta = c->refine_theta;
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  const RefineArgs& r = c->refine;
  const int64_t nb = static_cast<int64_t>(r.xb) * r.yb;
  const int64_t n = c->refine_n[0];
  const int64_t pp = static_cast<int64_t>(r.pw) * r.yb * 8;
  int st;
  int32_t* dlev = nullptr;
  if (levels) {
    if ((st = ensure(c, c->refine_levels, nb * 192 * 4))) return st;
    dlev = static_cast<int32_t*>(c->refine_levels.ptr);
  }
  const bool timed = c->timing;
  double* sums = c->refine_sums;
  double* psums = c->refine_proxy_sums;
  const bool use_ssim = c->refine_w_ssim > 0.0f;
  const bool use_proxy = c->refine_proxy && c->refine_w_proxy > 0.0f;
  JXG_CUDA(c, cudaMemsetAsync(sums, 0, 4 * kRefineSlots * sizeof(double), s));
  if (use_proxy) JXG_CUDA(c, cudaMemsetAsync(psums, 0, kProxySums * kRefineSlots * sizeof(double), s));
  const unsigned block_ctas = static_cast<unsigned>((nb + 7) / 8);
  const bool epf = r.epf_stages > 0;
  if ((epf && (st = launch(c, "k_refine_sigma", timed, [&] {
                 k_refine_sigma<<<refine_grid(nb), 256, 0, s>>>(r, theta);
               }))) ||
      (st = launch(c, "k_refine_forward", timed, [&] {
         k_refine_forward<<<block_ctas, 256, 0, s>>>(r, theta, dlev, epf ? nullptr : c->refine_lin[1][0],
                                                     sums + 3 * kRefineSlots);
       })))
    return st;
  // the decoded XYB the distortion sees: after the EPF, or the padded recon
  const float* dec = r.recon;
  int64_t dec_plane = pp;
  int dec_stride = r.pw;
  if (epf) {
    for (int k = 0; k < r.epf_stages; ++k) {
      const float* in = k == 0 ? r.recon : c->refine_epf_out[k - 1];
      const int64_t plane = k == 0 ? pp : n;
      const int stride = k == 0 ? r.pw : r.w;
      if ((st = launch(c, "k_refine_epf", timed, [&] {
             const dim3 grid(static_cast<unsigned>((r.w + kEpfTW - 1) / kEpfTW),
                             static_cast<unsigned>((r.h + kEpfTH - 1) / kEpfTH));
             k_refine_epf<<<grid, 256, 0, s>>>(r, r.epf_stage[k], r.epf_sm[k], in, plane, stride,
                                               c->refine_epf_out[k], c->refine_epf_nw[k], c->refine_epf_cw[k]);
           })))
        return st;
    }
    dec = c->refine_epf_out[r.epf_stages - 1];
    dec_plane = n;
    dec_stride = r.w;
    if (use_ssim && (st = launch(c, "k_refine_linear", timed, [&] {
                       k_refine_linear<<<refine_grid(n), 256, 0, s>>>(dec, n, r.w, c->refine_lin[1][0], r.w, r.h);
                     })))
      return st;
  }
  if (use_ssim) {
    for (int k = 1; k < 3; ++k)
      if (c->refine_n[k] && (st = launch(c, "k_refine_down", timed, [&] {
                               k_refine_down<<<refine_grid(3 * c->refine_n[k]), 256, 0, s>>>(
                                   c->refine_lin[1][k - 1], c->refine_lin[1][k], c->refine_w[k - 1],
                                   c->refine_h[k - 1]);
                             })))
        return st;
    for (int k = 0; k < 3; ++k) {
      const int64_t nk = c->refine_n[k];
      if (!nk) continue;
      const int w = c->refine_w[k], h = c->refine_h[k];
      // L_k = w_ssim sum(1 - SSIM) / (3 channels * pixels * 3 scales)
      const float weight = static_cast<float>(c->refine_w_ssim / (9.0 * static_cast<double>(nk)));
      const dim3 grid(static_cast<unsigned>((w + kSsimTW - 1) / kSsimTW),
                      static_cast<unsigned>((h + kSsimTH - 1) / kSsimTH), 3);
      if ((st = launch(c, "k_refine_ssim", timed, [&] {
             k_refine_ssim<<<grid, 256, 0, s>>>(c->refine_lin[0][k], c->refine_lin[1][k], w, h, weight,
                                                c->refine_glin[k], sums + k * kRefineSlots);
           })))
        return st;
    }
  }
  // the luma proxy on the decoded Y plane
  const float* dec_y = dec + dec_plane;
  auto& PH = c->refine_pl[0];
  auto& PQ = c->refine_pl[1];
  const int64_t npairs = static_cast<int64_t>(r.h) * (r.w - 1) + static_cast<int64_t>(r.h - 1) * r.w;
  if (use_proxy &&
      (st = launch(c, "k_refine_proxy", timed, [&] {
         k_proxy_half<<<refine_grid(static_cast<int64_t>(PH.w) * PH.h), 256, 0, s>>>(dec_y, dec_stride, r.w, r.h, 1,
                                                                                     PH.vals);
         k_proxy_half<<<refine_grid(static_cast<int64_t>(PQ.w) * PQ.h), 256, 0, s>>>(PH.vals, PH.w, PH.w, PH.h, 0,
                                                                                     PQ.vals);
         for (int l = 0; l < 2; ++l) {
           auto& L = c->refine_pl[l];
           const int64_t m = static_cast<int64_t>(L.w) * L.h;
           k_proxy_box_v_par<<<refine_grid(m), 256, 0, s>>>(L.vals, L.ref_vals, L.w, L.h, L.tmp);
           k_proxy_box_h_par<<<refine_grid(3 * m), 256, 0, s>>>(L.tmp, 3, L.w, L.h, L.box);
           k_proxy_pool<<<refine_grid(m), 256, 0, s>>>(L.ref_mv, L.box, m, L.s, L.parts,
                                                       psums + 2 * l * kRefineSlots);
         }
         k_proxy_gradients<<<refine_grid(n), 256, 0, s>>>(c->refine_src_y, dec_y, dec_stride, r.w, r.h,
                                                          psums + 4 * kRefineSlots);
       })))
    return st;
  const float rate_weight = static_cast<float>(static_cast<double>(rate_lambda) / static_cast<double>(n));
  if (grad) {
    if (use_ssim && c->refine_n[2] && (st = launch(c, "k_refine_up_add", timed, [&] {
                                         k_refine_up_add<<<refine_grid(3 * c->refine_n[1]), 256, 0, s>>>(
                                             c->refine_glin[2], c->refine_glin[1], c->refine_w[1], c->refine_h[1]);
                                       })))
      return st;
    const float* gx = nullptr;
    if (epf || use_proxy || !use_ssim) {
      // the decoded-XYB gradient as planes: SSIM's through XYB -> linear,
      // plus the proxy's on Y, then back through each EPF stage
      int cur = 0;
      float* g = c->refine_epf_g[cur];
      if (use_ssim) {
        if ((st = launch(c, "k_refine_linear_adjoint", timed, [&] {
               k_refine_linear_adjoint<<<refine_grid(n), 256, 0, s>>>(dec, dec_plane, dec_stride, c->refine_glin[0],
                                                                      c->refine_glin[1], r.w, r.h, c->refine_w[1],
                                                                      c->refine_h[1], g);
             })))
          return st;
      } else {
        JXG_CUDA(c, cudaMemsetAsync(g, 0, 3 * n * sizeof(float), s));
      }
      if (use_proxy &&
          (st = launch(c, "k_refine_proxy_adjoint", timed, [&] {
             const double n2 = static_cast<double>(PH.w) * PH.h, n4 = static_cast<double>(PQ.w) * PQ.h;
             k_proxy_finalize<<<1, 32, 0, s>>>(psums, n2, n4, static_cast<double>(npairs), c->refine_w_proxy,
                                               c->refine_proxy_k);
             for (int l = 0; l < 2; ++l) {
               auto& L = c->refine_pl[l];
               const int64_t m = static_cast<int64_t>(L.w) * L.h;
               k_proxy_pool_grad<<<refine_grid(m), 256, 0, s>>>(L.s, L.parts, m, c->refine_proxy_k, l, L.g);
               k_proxy_box_adjoint_h<<<refine_grid(3 * m), 256, 0, s>>>(L.g, L.w, L.h, L.gtmp);
               cudaMemsetAsync(L.gv, 0, m * sizeof(float), s);
               k_proxy_box_adjoint_v<<<refine_grid(m), 256, 0, s>>>(L.gtmp, L.vals, L.ref_vals, L.w, L.h, L.gv);
             }
             k_proxy_up<<<refine_grid(static_cast<int64_t>(PH.w) * PH.h), 256, 0, s>>>(PQ.gv, PQ.w, PQ.h, PH.gv,
                                                                                        PH.w, PH.h, PH.w);
             k_proxy_up<<<refine_grid(n), 256, 0, s>>>(PH.gv, PH.w, PH.h, g + n, r.w, r.h, r.w);
             k_proxy_gradients_adjoint<<<refine_grid(n), 256, 0, s>>>(c->refine_src_y, dec_y, dec_stride, r.w, r.h,
                                                                      c->refine_proxy_k, g + n, r.w);
           })))
        return st;
      for (int k = r.epf_stages - 1; k >= 0; --k) {
        if ((st = launch(c, "k_refine_epf_adjoint", timed, [&] {
               k_refine_epf_adjoint<<<refine_grid(n), 256, 0, s>>>(r, r.epf_stage[k], c->refine_epf_g[cur],
                                                                   c->refine_epf_nw[k], c->refine_epf_cw[k],
                                                                   c->refine_epf_g[1 - cur]);
             })))
          return st;
        cur = 1 - cur;
      }
      gx = c->refine_epf_g[cur];
    }
    if ((st = launch(c, "k_refine_backward", timed, [&] {
           k_refine_backward<<<block_ctas, 256, 0, s>>>(r, theta, c->refine_glin[0], c->refine_glin[1],
                                                        c->refine_w[1], c->refine_h[1], gx, rate_weight, grad);
         })))
      return st;
  }
  double host[4 * kRefineSlots], phost[kProxySums * kRefineSlots];
  JXG_CUDA(c, cudaMemcpyAsync(host, sums, sizeof(host), cudaMemcpyDeviceToHost, s));
  if (use_proxy) JXG_CUDA(c, cudaMemcpyAsync(phost, psums, sizeof(phost), cudaMemcpyDeviceToHost, s));
  if (levels) JXG_CUDA(c, cudaMemcpyAsync(levels, dlev, nb * 192 * 4, cudaMemcpyDeviceToHost, s));
  if ((st = wait(c))) return st;
  double total[4] = {0.0, 0.0, 0.0, 0.0};
  for (int q = 0; q < 4; ++q)
    for (int k = 0; k < kRefineSlots; ++k) total[q] += host[q * kRefineSlots + k];
  double dist = 0.0;
  if (use_ssim)
    for (int k = 0; k < 3; ++k)
      if (c->refine_n[k]) dist += c->refine_w_ssim * total[k] / (9.0 * static_cast<double>(c->refine_n[k]));
  if (use_proxy) {
    double t[kProxySums];
    for (int q = 0; q < kProxySums; ++q) {
      t[q] = 0.0;
      for (int k = 0; k < kRefineSlots; ++k) t[q] += phost[q * kRefineSlots + k];
    }
    const double n2 = static_cast<double>(PH.w) * PH.h, n4 = static_cast<double>(PQ.w) * PQ.h;
    const double np = static_cast<double>(npairs);
    // src/epf_proxy.rs:181-199 (the weights, as kProxyWeights)
    static const double kW[6] = {109.4163228369586, 4.685925102200196, 2.491781270704224,
                                 2.167275675983448, 4.55227651921194,  2.847714678987977};
    const double terms[6] = {t[2] / n4, t[0] / n2, std::sqrt(std::sqrt(t[1] / n2)), t[4] / np, t[5] / np,
                             std::sqrt(std::sqrt(t[6] / np))};
    double proxy = 0.0;
    for (int k = 0; k < 6; ++k) proxy += kW[k] * terms[k];
    dist += c->refine_w_proxy * proxy;
  }
  loss3[0] = dist + static_cast<double>(rate_lambda) * total[3] / static_cast<double>(n);
  loss3[1] = dist;
  loss3[2] = total[3];
  return JXG_OK;
}

int32_t jxg_refine_set_weights(void* ctx, float ssim_weight, float proxy_weight) {
  Context* c = static_cast<Context*>(ctx);
  if (!c) return JXG_ERR_INVALID_ARGUMENT;
  if (!std::isfinite(ssim_weight) || !std::isfinite(proxy_weight) || ssim_weight < 0.0f || proxy_weight < 0.0f ||
      (ssim_weight == 0.0f && proxy_weight == 0.0f))
    return jxg::fail(c, JXG_ERR_INVALID_ARGUMENT, "weights finite, non-negative and not both zero");
  c->refine_w_ssim = ssim_weight;
  c->refine_w_proxy = proxy_weight;
  return JXG_OK;
}

int32_t jxg_refine_decoded(void* ctx, const float* theta, float* xyb) {
  using namespace jxg;
  Context* c = static_cast<Context*>(ctx);
  if (!c || !xyb) return JXG_ERR_INVALID_ARGUMENT;
  if (!c->refine_ready) return fail(c, JXG_ERR_INVALID_ARGUMENT, "jxg_refine_begin first");
  double loss3[3];
  int st;
  if ((st = jxg_refine_eval(ctx, theta, 0.0f, nullptr, loss3, nullptr))) return st;
  const RefineArgs& r = c->refine;
  const int64_t n = static_cast<int64_t>(r.w) * r.h, pp = static_cast<int64_t>(r.pw) * r.yb * 8;
  for (int k = 0; k < 3; ++k) {
    if (r.epf_stages)
      JXG_CUDA(c, cudaMemcpyAsync(xyb + k * n, c->refine_epf_out[r.epf_stages - 1] + k * n, n * 4,
                                  cudaMemcpyDeviceToHost, c->stream));
    else
      JXG_CUDA(c, cudaMemcpy2DAsync(xyb + k * n, static_cast<size_t>(r.w) * 4, r.recon + k * pp,
                                    static_cast<size_t>(r.pw) * 4, static_cast<size_t>(r.w) * 4, r.h,
                                    cudaMemcpyDeviceToHost, c->stream));
  }
  return wait(c);
}

int32_t jxg_refine_field(void* ctx, const float* theta, uint8_t* quant_field) {
  using namespace jxg;
  Context* c = static_cast<Context*>(ctx);
  if (!c || !quant_field) return JXG_ERR_INVALID_ARGUMENT;
  if (!c->refine_ready) return fail(c, JXG_ERR_INVALID_ARGUMENT, "jxg_refine_begin first");
  if (!theta) theta = c->refine_theta;
  cudaSetDevice(c->device);
  const int64_t nb = static_cast<int64_t>(c->refine.xb) * c->refine.yb;
  cudaPointerAttributes at{};
  const bool on_device =
      cudaPointerGetAttributes(&at, quant_field) == cudaSuccess && at.type == cudaMemoryTypeDevice;
  cudaGetLastError();
  int st;
  if (!on_device && (st = ensure(c, c->field_buf, nb))) return st;
  uint8_t* out = on_device ? quant_field : static_cast<uint8_t*>(c->field_buf.ptr);
  k_refine_field<<<refine_grid(nb), 256, 0, c->stream>>>(c->refine.qf, theta, nb, out);
  JXG_CUDA(c, cudaGetLastError());
  if (!on_device) JXG_CUDA(c, cudaMemcpyAsync(quant_field, out, nb, cudaMemcpyDeviceToHost, c->stream));
  return wait(c);
}

int32_t jxg_refine_step(void* ctx, float rate_lambda, float learning_rate, double* loss3) {
  using namespace jxg;
  Context* c = static_cast<Context*>(ctx);
  if (!c || !loss3) return JXG_ERR_INVALID_ARGUMENT;
  if (!c->refine_ready) return fail(c, JXG_ERR_INVALID_ARGUMENT, "jxg_refine_begin first");
  if (!(learning_rate > 0.0f) || !std::isfinite(learning_rate) || !(rate_lambda >= 0.0f) ||
      !std::isfinite(rate_lambda))
    return fail(c, JXG_ERR_INVALID_ARGUMENT, "learning rate > 0 and lambda >= 0, both finite");
  const int64_t nb = static_cast<int64_t>(c->refine.xb) * c->refine.yb;
  int st = jxg_refine_eval(ctx, c->refine_theta, rate_lambda, c->refine_grad, loss3, nullptr);
  if (st) return st;
  if (c->refine_steps == 0) JXG_CUDA(c, cudaMemsetAsync(c->refine_adam, 0, 2 * nb * 4, c->stream));
  const int t = ++c->refine_steps;
  const float c1 = static_cast<float>(1.0 / (1.0 - std::pow(kAdamBeta1, t)));
  const float c2 = static_cast<float>(1.0 / (1.0 - std::pow(kAdamBeta2, t)));
  k_refine_adam<<<refine_grid(nb), 256, 0, c->stream>>>(c->refine.qf, c->refine_grad, nb, learning_rate, c1, c2,
                                                        c->refine_adam, c->refine_theta);
  JXG_CUDA(c, cudaGetLastError());
  return wait(c);
}

int32_t jxg_refine_theta(void* ctx, float* theta, int32_t to_context) {
  using namespace jxg;
  Context* c = static_cast<Context*>(ctx);
  if (!c || !theta) return JXG_ERR_INVALID_ARGUMENT;
  if (!c->refine_ready) return fail(c, JXG_ERR_INVALID_ARGUMENT, "jxg_refine_begin first");
  const size_t bytes = static_cast<size_t>(c->refine.xb) * c->refine.yb * 4;
  if (to_context) {
    JXG_CUDA(c, cudaMemcpyAsync(c->refine_theta, theta, bytes, cudaMemcpyDefault, c->stream));
    c->refine_steps = 0;
  } else {
    JXG_CUDA(c, cudaMemcpyAsync(theta, c->refine_theta, bytes, cudaMemcpyDefault, c->stream));
  }
  return wait(c);
}

int32_t jxg_refine_model(void* ctx, float* constants, float* coefficients, float* inverse, float* dc) {
  using namespace jxg;
  Context* c = static_cast<Context*>(ctx);
  if (!c || !constants) return JXG_ERR_INVALID_ARGUMENT;
  if (!c->refine_ready) return fail(c, JXG_ERR_INVALID_ARGUMENT, "jxg_refine_begin first");
  cudaSetDevice(c->device);
  const RefineArgs& r = c->refine;
  float* o = constants;
  *o++ = r.scale;
  for (int k = 0; k < 3; ++k) *o++ = r.qm_mul[k];
  std::memcpy(o, r.matrix, sizeof(r.matrix));
  o += 192;
  std::memcpy(o, r.inv_matrix, sizeof(r.inv_matrix));
  o += 192;
  std::memcpy(o, r.thresholds, sizeof(r.thresholds));
  o += 12;
  // the EPF model: stages, their ids and SAD multipliers, border multiplier,
  // channel scales, quant_mul, sharpness / 7, quantizer scale
  *o++ = static_cast<float>(r.epf_stages);
  for (int k = 0; k < 3; ++k) *o++ = k < r.epf_stages ? static_cast<float>(r.epf_stage[k]) : -1.0f;
  for (int k = 0; k < 3; ++k) *o++ = k < r.epf_stages ? r.epf_sm[k] : 0.0f;
  *o++ = r.epf_border;
  for (int k = 0; k < 3; ++k) *o++ = r.epf_channel[k];
  *o++ = r.epf_quant_mul;
  *o++ = r.epf_lut;
  *o++ = r.epf_quant_scale;
  const int64_t nb = static_cast<int64_t>(r.xb) * r.yb;
  if (coefficients)
    JXG_CUDA(c, cudaMemcpyAsync(coefficients, r.coef, nb * 192 * 4, cudaMemcpyDeviceToHost, c->stream));
  if (inverse) JXG_CUDA(c, cudaMemcpyAsync(inverse, r.m, 4096 * 4, cudaMemcpyDeviceToHost, c->stream));
  if (dc) JXG_CUDA(c, cudaMemcpyAsync(dc, r.dc, nb * 3 * 4, cudaMemcpyDeviceToHost, c->stream));
  return wait(c);
}

int32_t jxg_get_launch_geometry(void* ctx, uint8_t* warps) {
  Context* c = static_cast<Context*>(ctx);
  if (!c || !warps) return JXG_ERR_INVALID_ARGUMENT;
  std::memcpy(warps, c->tune, jxg::kTuneKernels);
  return JXG_OK;
}

int32_t jxg_set_launch_geometry(void* ctx, const uint8_t* warps) {
  Context* c = static_cast<Context*>(ctx);
  if (!c || !warps) return JXG_ERR_INVALID_ARGUMENT;
  for (int k = 0; k < jxg::kTuneKernels; ++k)
    if (warps[k] != 1 && warps[k] != 2 && warps[k] != 4 && warps[k] != 8)
      return jxg::fail(c, JXG_ERR_INVALID_ARGUMENT, "warps per CTA must be 1, 2, 4 or 8");
  std::memcpy(c->tune, warps, jxg::kTuneKernels);
  return JXG_OK;
}

int32_t jxg_autotune(void* ctx, const void* pixels, uint64_t width, uint64_t height,
                     int32_t channels, int32_t bits, const jxg_config* config, int32_t rounds,
                     double* times_ms) {
  Context* c = static_cast<Context*>(ctx);
  if (!c || !pixels || !config || rounds < 1) return JXG_ERR_INVALID_ARGUMENT;
  if (c->async_pending) {
    const int st = jxg_frontend_wait(ctx);
    if (st) return st;
  }
  cudaSetDevice(c->device);
  static const char* const kNames[jxg::kTuneKernels] = {
      "k_cost_dct8",   "k_cost_16x8",   "k_cost_8x16",   "k_cost_16x16", "k_layout_dct8",
      "k_layout_16x8", "k_layout_8x16", "k_layout_16x16", "k_retile",    "k_site"};
  static const uint8_t kCandidates[4] = {1, 2, 4, 8};
  const bool was_timing = c->timing;
  uint8_t pick[jxg::kTuneKernels];
  double best[jxg::kTuneKernels];
  std::memcpy(pick, c->tune, sizeof(pick));
  for (double& b : best) b = INFINITY;
  int st = JXG_OK;
  for (int ci = 0; ci < 4 && st == JXG_OK; ++ci) {
    std::memset(c->tune, kCandidates[ci], sizeof(c->tune));
    c->timing = false;  // one untimed pass first
    if ((st = jxg::single_pass(c, pixels, width, height, channels, bits, config, true)) ||
        (st = jxg::wait(c)))
      break;
    jxg::collect_times(c);
    c->times.clear();
    c->timing = true;
    for (int r = 0; r < rounds && st == JXG_OK; ++r)
      st = jxg::single_pass(c, pixels, width, height, channels, bits, config, true);
    if (st || (st = jxg::wait(c))) break;
    jxg::collect_times(c);
    for (int k = 0; k < jxg::kTuneKernels; ++k) {
      const auto it = c->times.find(kNames[k]);
      const double ms = it == c->times.end() || it->second.launches == 0
                            ? NAN
                            : it->second.total_ms / static_cast<double>(it->second.launches);
      if (times_ms) times_ms[k * 4 + ci] = ms;
      if (ms < best[k]) {
        best[k] = ms;
        pick[k] = kCandidates[ci];
      }
    }
  }
  c->times.clear();
  c->timing = was_timing;
  std::memcpy(c->tune, pick, sizeof(pick));
  return st;
}

int32_t jxg_enable_kernel_timing(void* ctx, int32_t enable) {
  Context* c = static_cast<Context*>(ctx);
  if (!c) return JXG_ERR_INVALID_ARGUMENT;
  c->timing = enable != 0;
  return JXG_OK;
}

int32_t jxg_kernel_times(void* ctx, const char** names, double* total_ms, uint64_t* launches,
                         int32_t capacity) {
  Context* c = static_cast<Context*>(ctx);
  if (!c) return JXG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  if (cudaStreamSynchronize(c->stream) == cudaSuccess) jxg::collect_times(c);
  c->time_names.clear();
  int i = 0;
  for (auto& kv : c->times) {
    c->time_names.push_back(kv.first);
    if (i < capacity) {
      if (total_ms) total_ms[i] = kv.second.total_ms;
      if (launches) launches[i] = kv.second.launches;
    }
    ++i;
  }
  for (int k = 0; k < i && k < capacity; ++k)
    if (names) names[k] = c->time_names[k].c_str();
  return i;
}

int32_t jxg_reset_kernel_times(void* ctx) {
  Context* c = static_cast<Context*>(ctx);
  if (!c) return JXG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  if (cudaStreamSynchronize(c->stream) == cudaSuccess) jxg::collect_times(c);
  c->times.clear();
  return JXG_OK;
}

}  // extern "C"
