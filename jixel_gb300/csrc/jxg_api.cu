// C ABI of the GB300 VarDCT front end: context, buffers, launches, fetch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/jxg.h"
#include "frame_params.h"
#include "jxg_kernels.cuh"

namespace jxg {
namespace {

constexpr uint64_t kMaxDimension = 0x3FFFFFFFull;  // MAX_DIMENSION, src/encode_image.rs:99

struct DevBuf {
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

}  // namespace

struct Context {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::string last_error;
  // constant tables
  float* d_lut = nullptr;       // sRGB -> linear, 256
  float* d_exp2 = nullptr;      // fast_exp2 table, 64
  uint8_t* d_scan = nullptr;    // natural 8x8 order, 64
  uint8_t* d_pos = nullptr;     // its inverse, 64
  // frame buffers
  DevBuf pixels, xyb, qf, ytox, ytob, quant_dc, levels, wide_levels, coeffs, nzeros, nz_packed, counts,
      offsets, chunks, tokens, hist, stats, group_offsets, op_in, op_out;
  // last pass
  bool have_frame = false;
  uint64_t width = 0, height = 0;
  jxg_frame_info info{};
  DistanceParams dp{};
  KernelArgs args{};
  int64_t plane = 0;
  // timing
  bool timing = false;
  std::vector<PendingEvent> pending;
  std::vector<cudaEvent_t> spare_events;
  std::map<std::string, TimedKernel> times;
  std::vector<std::string> time_names;
};

namespace {

int fail(Context* c, int code, const std::string& msg) {
  if (c) c->last_error = msg;
  return code;
}

#define JXG_CUDA(ctx, call)                                                              \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
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
int launch(Context* c, const char* name, Launch&& fn) {
  cudaEvent_t s = nullptr, e = nullptr;
  if (c->timing) {
    s = take_event(c);
    e = take_event(c);
    cudaEventRecord(s, c->stream);
  }
  fn();
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return fail(c, JXG_ERR_CUDA, std::string(name) + ": " + cudaGetErrorString(err));
  if (c->timing) {
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

int sm_count(int device) {
  int n = 0;
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device);
  return n > 0 ? n : 1;
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
  if (channels != 3 && channels != 4) return fail(c, JXG_ERR_BAD_CHANNEL_COUNT, "channels");
  if (bits != 8 && bits != 16) return fail(c, JXG_ERR_BAD_BIT_DEPTH, "bits");
  if (!std::isfinite(cfg->distance) || cfg->distance <= 0.0f)
    return fail(c, JXG_ERR_INVALID_DISTANCE, "distance must be positive and finite");
  if (cfg->speed != JXG_SPEED_ULTRAFAST)
    return fail(c, JXG_ERR_UNSUPPORTED, "only Speed::UltraFast gates are built");
  if (w * h > (1ull << 31))
    return fail(c, JXG_ERR_DIMENSION_TOO_LARGE, "frames above 2^31 pixels are not supported");
  return JXG_OK;
}

// Enqueue the whole pass on the context's stream; `pixels` is device memory.
int enqueue_frontend(Context* c, const void* pixels, uint64_t w, uint64_t h, int32_t channels,
                     int32_t bits, const jxg_config* cfg) {
  int st = validate(c, pixels, w, h, channels, bits, cfg);
  if (st) return st;
  DistanceParams dp;
  if (compute_distance_params(cfg->distance, &dp))
    return fail(c, JXG_ERR_INVALID_DISTANCE, "distance");
  KernelArgs& a = c->args;
  std::memset(&a, 0, sizeof(a));
  dct8_tables(dp.distance, a.matrix, a.inv_matrix);
  fill_kernel_args(dp, &a);
  jxg_frame_info& fi = c->info;
  frame_info(w, h, &fi);
  a.width = static_cast<int32_t>(w);
  a.height = static_cast<int32_t>(h);
  a.xb = static_cast<int32_t>(fi.xsize_blocks);
  a.yb = static_cast<int32_t>(fi.ysize_blocks);
  a.tiles_x = static_cast<int32_t>(fi.xsize_tiles);
  a.tiles_y = static_cast<int32_t>(fi.ysize_tiles);
  a.groups_x = static_cast<int32_t>(fi.xsize_groups);
  a.groups_y = static_cast<int32_t>(fi.ysize_groups);
  const int64_t n = static_cast<int64_t>(w * h);
  const int64_t plane = (n + 63) / 64 * 64;
  a.plane = static_cast<int32_t>(plane);
  c->plane = plane;
  c->dp = dp;
  c->width = w;
  c->height = h;
  const int64_t nb = static_cast<int64_t>(fi.xsize_blocks * fi.ysize_blocks);
  const int64_t ntiles = static_cast<int64_t>(fi.xsize_tiles * fi.ysize_tiles);
  const int64_t ncounts = static_cast<int64_t>(fi.num_groups) * 1024 * 4;
  const int64_t nchunks = (ncounts + kScanChunk - 1) / kScanChunk;
  if ((st = ensure(c, c->xyb, 3 * plane * sizeof(float))) ||
      (st = ensure(c, c->qf, nb)) || (st = ensure(c, c->ytox, ntiles)) ||
      (st = ensure(c, c->ytob, ntiles)) || (st = ensure(c, c->quant_dc, 3 * nb * 2)) ||
      (st = ensure(c, c->levels, nb * 192 * 2)) || (st = ensure(c, c->wide_levels, nb * 192 * 4)) ||
      (st = ensure(c, c->nzeros, 3 * nb)) || (st = ensure(c, c->nz_packed, 4 * nb)) ||
      (st = ensure(c, c->counts, ncounts * 4)) || (st = ensure(c, c->offsets, ncounts * 4)) ||
      (st = ensure(c, c->chunks, nchunks * 4)) ||
      (st = ensure(c, c->tokens, fi.max_tokens * sizeof(uint2))) ||
      (st = ensure(c, c->hist, (size_t)kNumFineAcContexts * kAlphabet * 4)) ||
      (st = ensure(c, c->stats, sizeof(DeviceStats))) ||
      (st = ensure(c, c->group_offsets, (fi.num_groups + 1) * 8)))
    return st;
  cudaStream_t s = c->stream;
  JXG_CUDA(c, cudaMemsetAsync(c->stats.ptr, 0, sizeof(DeviceStats), s));
  JXG_CUDA(c, cudaMemsetAsync(c->hist.ptr, 0, (size_t)kNumFineAcContexts * kAlphabet * 4, s));
  JXG_CUDA(c, cudaMemsetAsync(c->counts.ptr, 0, ncounts * 4, s));
  const int sms = sm_count(c->device);
  float* xyb = static_cast<float*>(c->xyb.ptr);
  DeviceStats* stats = static_cast<DeviceStats*>(c->stats.ptr);
  // 1. linearise + XYB
  XybArgs xa;
  opsin_matrix(xa.opsin);
  xa.pixels = n;
  xa.plane = plane;
  const bool fast_rgb8 = bits == 8 && channels == 3 &&
                         (reinterpret_cast<uintptr_t>(pixels) & 3u) == 0;
  if (fast_rgb8) {
    const int64_t quads = n / 4;
    const int grid = static_cast<int>(std::min<int64_t>((quads + 255) / 256 + 1, sms * 8));
    st = launch(c, "k_xyb_rgb8", [&] {
      k_xyb_rgb8<<<grid, 256, 0, s>>>(xa, static_cast<const uint8_t*>(pixels), c->d_lut, xyb);
    });
  } else {
    const int grid = static_cast<int>(std::min<int64_t>((n + 255) / 256, sms * 8));
    st = launch(c, "k_xyb_generic", [&] {
      k_xyb_generic<<<grid, 256, 0, s>>>(xa, pixels, bits / 8, channels, c->d_lut, xyb);
    });
  }
  if (st) return st;
  // 3. adaptive quant field per DC group
  {
    dim3 grid(a.tiles_x, a.tiles_y);
    st = launch(c, "k_adaptive_quant", [&] {
      k_adaptive_quant<<<grid, 256, 0, s>>>(a, xyb, c->d_exp2, static_cast<uint8_t*>(c->qf.ptr),
                                            stats);
    });
    if (st) return st;
  }
  // 4. CfL tiles + DCT8 quantisation
  {
    TileOutputs to;
    to.ytox = static_cast<int8_t*>(c->ytox.ptr);
    to.ytob = static_cast<int8_t*>(c->ytob.ptr);
    to.qf = static_cast<const uint8_t*>(c->qf.ptr);
    to.levels = static_cast<int16_t*>(c->levels.ptr);
    to.wide_levels = static_cast<int32_t*>(c->wide_levels.ptr);
    to.quant_dc = static_cast<int16_t*>(c->quant_dc.ptr);
    to.nzeros = static_cast<uint8_t*>(c->nzeros.ptr);
    to.nz_packed = static_cast<uint32_t*>(c->nz_packed.ptr);
    to.token_counts = static_cast<uint32_t*>(c->counts.ptr);
    to.stats = stats;
    dim3 grid(a.tiles_x, a.tiles_y);
    st = launch(c, "k_tile_quantize", [&] {
      k_tile_quantize<<<grid, kTileThreads, kTileSmemBytes, s>>>(a, xyb, c->d_pos, to);
    });
    if (st) return st;
  }
  // 5. token offsets (+ qf threshold)
  {
    uint32_t* counts = static_cast<uint32_t*>(c->counts.ptr);
    uint32_t* offs = static_cast<uint32_t*>(c->offsets.ptr);
    uint32_t* chunks = static_cast<uint32_t*>(c->chunks.ptr);
    uint64_t* goffs = static_cast<uint64_t*>(c->group_offsets.ptr);
    const int ch = static_cast<int>(nchunks);
    if ((st = launch(c, "k_scan_reduce", [&] {
           k_scan_reduce<<<ch, kScanThreads, 0, s>>>(counts, ncounts, chunks);
         })) ||
        (st = launch(c, "k_scan_chunks", [&] {
           k_scan_chunks<<<1, kScanThreads, 0, s>>>(chunks, ch, stats, goffs,
                                                     static_cast<int>(fi.num_groups));
         })) ||
        (st = launch(c, "k_scan_apply", [&] {
           k_scan_apply<<<ch, kScanThreads, 0, s>>>(counts, ncounts, chunks, offs, goffs, 4 * 1024);
         })))
      return st;
  }
  // 6. tokens + histograms
  {
    TokenArgs ta;
    ta.xb = a.xb;
    ta.yb = a.yb;
    ta.groups_x = a.groups_x;
    ta.levels = static_cast<const int16_t*>(c->levels.ptr);
    ta.wide_levels = static_cast<const int32_t*>(c->wide_levels.ptr);
    ta.nz_packed = static_cast<const uint32_t*>(c->nz_packed.ptr);
    ta.qf = static_cast<const uint8_t*>(c->qf.ptr);
    ta.offsets = static_cast<const uint32_t*>(c->offsets.ptr);
    ta.stats = stats;
    ta.tokens = static_cast<uint2*>(c->tokens.ptr);
    ta.histograms = static_cast<uint32_t*>(c->hist.ptr);
    const int64_t warps = nb;
    const int grid = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>((warps + 7) / 8, sms * 16)));
    st = launch(c, "k_tokenize", [&] { k_tokenize<<<grid, 256, 0, s>>>(ta); });
    if (st) return st;
  }
  c->have_frame = true;
  return JXG_OK;
}

int wait(Context* c) {
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail(c, JXG_ERR_CUDA, std::string("stream: ") + cudaGetErrorString(e));
  if (c->timing) collect_times(c);
  return JXG_OK;
}

int read_params(Context* c, jxg_frame_params* out) {
  DeviceStats ds;
  JXG_CUDA(c, cudaMemcpyAsync(&ds, c->stats.ptr, sizeof(ds), cudaMemcpyDeviceToHost, c->stream));
  int st = wait(c);
  if (st) return st;
  std::memset(out, 0, sizeof(*out));
  const DistanceParams& p = c->dp;
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
  bool screen = is_screen_content(ds.constant_blocks, c->width, c->height);
  out->screen_content = screen;
  out->epf_sharpness = epf_sharpness_id(p.distance, screen);
  out->num_tokens = ds.num_tokens;
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

}  // namespace
}  // namespace jxg

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
  float lut[256], e2[64];
  uint8_t scan[64], pos[64];
  jxg::srgb_to_linear_table(lut);
  jxg::exp2_table(e2);
  jxg::natural_order_8x8(scan, pos);
  bool ok = cudaMalloc(&c->d_lut, sizeof(lut)) == cudaSuccess &&
            cudaMalloc(&c->d_exp2, sizeof(e2)) == cudaSuccess &&
            cudaMalloc(&c->d_scan, 64) == cudaSuccess && cudaMalloc(&c->d_pos, 64) == cudaSuccess &&
            cudaMemcpy(c->d_lut, lut, sizeof(lut), cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(c->d_exp2, e2, sizeof(e2), cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(c->d_scan, scan, 64, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(c->d_pos, pos, 64, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaFuncSetAttribute(jxg::k_tile_quantize, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(jxg::kTileSmemBytes)) == cudaSuccess;
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
  for (jxg::DevBuf* b : {&c->pixels, &c->xyb, &c->qf, &c->ytox, &c->ytob, &c->quant_dc, &c->coeffs,
                         &c->levels, &c->wide_levels, &c->nz_packed,
                         &c->nzeros, &c->counts, &c->offsets, &c->chunks, &c->tokens, &c->hist,
                         &c->stats, &c->group_offsets, &c->op_in, &c->op_out})
    if (b->ptr) cudaFree(b->ptr);
  cudaFree(c->d_lut);
  cudaFree(c->d_exp2);
  cudaFree(c->d_scan);
  cudaFree(c->d_pos);
  for (auto& p : c->pending) {
    cudaEventDestroy(p.start);
    cudaEventDestroy(p.stop);
  }
  for (auto e : c->spare_events) cudaEventDestroy(e);
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
  cudaSetDevice(c->device);
  return jxg::enqueue_frontend(c, pixels, width, height, channels, bits, config);
}

int32_t jxg_frontend_run(void* ctx, const void* pixels, uint64_t width, uint64_t height,
                         int32_t channels, int32_t bits, const jxg_config* config) {
  Context* c = static_cast<Context*>(ctx);
  if (!c) return JXG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  int st = jxg::validate(c, pixels, width, height, channels, bits, config);
  if (st) return st;
  const size_t bytes = static_cast<size_t>(width * height) * channels * (bits / 8);
  if ((st = jxg::ensure(c, c->pixels, bytes))) return st;
  JXG_CUDA(c, cudaMemcpyAsync(c->pixels.ptr, pixels, bytes, cudaMemcpyHostToDevice, c->stream));
  st = jxg::enqueue_frontend(c, c->pixels.ptr, width, height, channels, bits, config);
  if (st) return st;
  return jxg::wait(c);
}

int32_t jxg_frontend_params(void* ctx, jxg_frame_params* out) {
  Context* c = static_cast<Context*>(ctx);
  if (!c || !out) return JXG_ERR_INVALID_ARGUMENT;
  if (!c->have_frame) return jxg::fail(c, JXG_ERR_INVALID_ARGUMENT, "no front-end pass yet");
  cudaSetDevice(c->device);
  return jxg::read_params(c, out);
}

int32_t jxg_frontend_fetch(void* ctx, jxg_frontend_output* out) {
  Context* c = static_cast<Context*>(ctx);
  if (!c || !out) return JXG_ERR_INVALID_ARGUMENT;
  if (!c->have_frame) return jxg::fail(c, JXG_ERR_INVALID_ARGUMENT, "no front-end pass yet");
  cudaSetDevice(c->device);
  jxg_frame_params p;
  int st = jxg::read_params(c, &p);
  if (st) return st;
  const jxg_frame_info& fi = c->info;
  const size_t nb = fi.xsize_blocks * fi.ysize_blocks;
  const size_t nt = fi.xsize_tiles * fi.ysize_tiles;
  cudaStream_t s = c->stream;
  auto copy = [&](void* dst, const void* src, size_t bytes) -> int {
    if (!dst || bytes == 0) return JXG_OK;
    JXG_CUDA(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
    return JXG_OK;
  };
  if (out->tokens && out->token_capacity < p.num_tokens)
    return jxg::fail(c, JXG_ERR_INVALID_ARGUMENT, "token buffer too small");
  if (out->coefficients) {
    if ((st = jxg::ensure(c, c->coeffs, nb * 192 * 4))) return st;
    const int64_t count = static_cast<int64_t>(nb) * 192;
    const int grid = static_cast<int>(std::min<int64_t>((count + 255) / 256, 4096));
    st = jxg::launch(c, "k_levels_to_raw", [&] {
      jxg::k_levels_to_raw<<<grid, 256, 0, s>>>(static_cast<const int16_t*>(c->levels.ptr),
                                                static_cast<const int32_t*>(c->wide_levels.ptr),
                                                c->d_pos, count, static_cast<int32_t*>(c->coeffs.ptr));
    });
    if (st) return st;
  }
  if ((st = copy(out->quant_field, c->qf.ptr, nb)) || (st = copy(out->ytox_map, c->ytox.ptr, nt)) ||
      (st = copy(out->ytob_map, c->ytob.ptr, nt)) ||
      (st = copy(out->quant_dc, c->quant_dc.ptr, 3 * nb * 2)) ||
      (st = copy(out->coefficients, c->coeffs.ptr, nb * 192 * 4)) ||
      (st = copy(out->num_nzeros, c->nzeros.ptr, 3 * nb)) ||
      (st = copy(out->tokens, c->tokens.ptr, p.num_tokens * sizeof(jxg_token))) ||
      (st = copy(out->group_offsets, c->group_offsets.ptr, (fi.num_groups + 1) * 8)) ||
      (st = copy(out->histograms, c->hist.ptr, (size_t)jxg::kNumFineAcContexts * jxg::kAlphabet * 4)))
    return st;
  if (out->xyb) {
    const size_t n = c->width * c->height;
    for (int ch = 0; ch < 3; ++ch)
      if ((st = copy(out->xyb + ch * n, static_cast<float*>(c->xyb.ptr) + ch * c->plane, n * 4)))
        return st;
  }
  if (out->ac_strategy) std::memset(out->ac_strategy, 1, nb);  // all DCT8, first blocks
  return jxg::wait(c);
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
  jxg::KernelArgs a;
  std::memset(&a, 0, sizeof(a));
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
  int st;
  if ((st = jxg::ensure(c, c->op_in, 3 * plane * 4)) || (st = jxg::ensure(c, c->op_out, nb)) ||
      (st = jxg::ensure(c, c->stats, sizeof(jxg::DeviceStats))))
    return st;
  cudaStream_t s = c->stream;
  for (int ch = 0; ch < 3; ++ch)
    JXG_CUDA(c, cudaMemcpyAsync(static_cast<float*>(c->op_in.ptr) + ch * plane, xyb + ch * n, n * 4,
                                cudaMemcpyHostToDevice, s));
  JXG_CUDA(c, cudaMemsetAsync(c->stats.ptr, 0, sizeof(jxg::DeviceStats), s));
  dim3 grid(a.tiles_x, a.tiles_y);
  st = jxg::launch(c, "k_adaptive_quant", [&] {
    jxg::k_adaptive_quant<<<grid, 256, 0, s>>>(a, static_cast<float*>(c->op_in.ptr), c->d_exp2,
                                               static_cast<uint8_t*>(c->op_out.ptr),
                                               static_cast<jxg::DeviceStats*>(c->stats.ptr));
  });
  if (st) return st;
  JXG_CUDA(c, cudaMemcpyAsync(quant_field, c->op_out.ptr, nb, cudaMemcpyDeviceToHost, s));
  return jxg::wait(c);
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
  st = jxg::launch(c, "k_dct8x8_blocks", [&] {
    jxg::k_dct8x8_blocks<<<grid, 256, 0, s>>>(static_cast<const float*>(c->op_in.ptr),
                                              static_cast<int64_t>(count),
                                              static_cast<float*>(c->op_out.ptr));
  });
  if (st) return st;
  JXG_CUDA(c, cudaMemcpyAsync(coefficients, c->op_out.ptr, bytes, cudaMemcpyDeviceToHost, s));
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
  // the middle step reads the pass scalars: start them from zero
  if (cudaMemsetAsync(&scratch->stats, 0, sizeof(scratch->stats), s) != cudaSuccess)
    return JXG_ERR_CUDA;
  jxg::k_scan_reduce<<<chunks, jxg::kScanThreads, 0, s>>>(counts, n, scratch->chunk_sums);
  jxg::k_scan_chunks<<<1, jxg::kScanThreads, 0, s>>>(scratch->chunk_sums, chunks, &scratch->stats,
                                                     group_offsets, static_cast<int>(num_groups));
  jxg::k_scan_apply<<<chunks, jxg::kScanThreads, 0, s>>>(counts, n, scratch->chunk_sums, offsets,
                                                         group_offsets, 3 * 1024);
  return cudaGetLastError() == cudaSuccess ? JXG_OK : JXG_ERR_CUDA;
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
