/*
 * jxg.h -- C ABI of the GB300 VarDCT front end.
 *
 * Plain pointers and sizes only.  One jxg_context owns one CUDA stream and the
 * device buffers of one frame; calls on different contexts are thread-safe,
 * calls on one context are serialised by the caller.  Status codes mirror the
 * reference's `EncodeError` variants (src/util.rs:129-160); 0 is success.
 *
 * Each entry point names the reference interface it stands in for.
 */
#ifndef JXG_H_
#define JXG_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes: EncodeError (src/util.rs:129-160) plus device failures. */
#define JXG_OK 0
#define JXG_ERR_EMPTY_IMAGE 1         /* EncodeError::EmptyImage */
#define JXG_ERR_INPUT_SIZE_MISMATCH 2 /* EncodeError::InputSizeMismatch */
#define JXG_ERR_ALPHA_SIZE_MISMATCH 3 /* EncodeError::AlphaSizeMismatch */
#define JXG_ERR_INVALID_DISTANCE 4    /* EncodeError::InvalidDistance */
#define JXG_ERR_QUALITY_IS_NAN 5      /* EncodeError::QualityIsNaN */
#define JXG_ERR_DIMENSION_TOO_LARGE 6 /* EncodeError::DimensionTooLarge */
#define JXG_ERR_ALLOCATION_FAILED 7   /* EncodeError::AllocationFailed */
#define JXG_ERR_UNSUPPORTED 8         /* EncodeError::Unsupported */
#define JXG_ERR_BAD_CHANNEL_COUNT 9   /* EncodeError::BadChannelCount */
#define JXG_ERR_BAD_BIT_DEPTH 10      /* EncodeError::BadBitDepth */
#define JXG_ERR_INVALID_ARGUMENT 100  /* null pointer, short output buffer, ... */
#define JXG_ERR_CUDA 101              /* a CUDA runtime call failed */
#define JXG_ERR_DEVICE_TIMEOUT 102    /* a bounded device wait gave up */

/* Speed (src/encode_image.rs:256-286).  This build runs UltraFast's gates
 * (src/effort.rs:305-309) and Fastest's (:311-320) for one frame per pass:
 * the square-merge search over 16x16 / 32x32 DCTs, the coefficient-model
 * re-tiling with 16x8 / 8x16 pairs, the quant-field aggregation and the
 * matrix-header accounting, with the layout's DC/AC coding and tokens.
 * Fastest at distances up to 1.709, where the reference also reranks merges
 * in the reconstruction domain (FAST_RERANK_MAX_DISTANCE,
 * src/ac_strategy.rs:67), Fastest in a batch of several frames, and every
 * slower tier return JXG_ERR_UNSUPPORTED.  At distances up to 0.0567 the
 * reference's Fastest keeps every block DCT8 (src/ac_strategy.rs:73-80), as
 * UltraFast does. */
#define JXG_SPEED_ULTRAFAST 0
#define JXG_SPEED_FASTEST 1
#define JXG_SPEED_FAST 2
#define JXG_SPEED_MEDIUM 3
#define JXG_SPEED_MEDIUM_SLOW 4
#define JXG_SPEED_SLOW 5
#define JXG_SPEED_EXTRA_SLOW 6

/* The part of `EncodeConfig` (src/encode_image.rs:326-588) the front end
 * reads: distance (set it from a quality with jxg_distance_from_quality, as
 * `with_quality`, src/encode_image.rs:986, does), speed, the host thread
 * budget (`with_num_threads`, :1251) and the samples' transfer function
 * (`color_encoding.transfer`, an H.273 transfer-characteristics code as
 * TransferFunction, src/color_encoding.rs:99-160).  The device result never
 * depends on num_threads.  `transfer` 0 means "not set": a zero-initialised
 * config is the default encoding, sRGB (13), whose 8-bit table is the f64
 * formula of srgb_to_linear_u8_ref (src/color.rs:35-42, :315-318).  It is not
 * H.273's Reserved code: the reference decodes Reserved like Unspecified (2),
 * through the f32 sRGB formula, so a caller that means Reserved passes 2.
 * 1, 6, 14, 15 decode as BT.709, 4 BT.470M, 5 BT.470BG, 7 SMPTE 240,
 * 8 linear, 17 SMPTE 428, and 2, 9-12 through the f32 sRGB formula
 * (select_transfer, src/color.rs:201-222); PQ (16) and HLG (18) return
 * JXG_ERR_UNSUPPORTED. */
typedef struct jxg_config {
  float distance;
  int32_t speed;
  int32_t num_threads;
  int32_t transfer;
  int32_t reserved[4];
} jxg_config;

#define JXG_TRANSFER_SRGB 13
#define JXG_TRANSFER_LINEAR 8
#define JXG_TRANSFER_BT709 1

/* Frame geometry (`ImageDim`, src/frame.rs:84-124). */
typedef struct jxg_frame_info {
  uint64_t width, height;
  uint64_t xsize_blocks, ysize_blocks; /* 8x8 blocks */
  uint64_t xsize_tiles, ysize_tiles;   /* 64x64 chroma-from-luma tiles */
  uint64_t xsize_groups, ysize_groups; /* 256x256 AC groups */
  uint64_t num_groups, num_dc_groups;  /* groups; 2048x2048 DC groups */
  uint64_t max_tokens;                 /* upper bound of the token count */
} jxg_frame_info;

/* Per-frame scalars: `DistanceParams` (src/frame/quantization.rs:35-48)
 * after the frame's chroma gates, plus what pass one derives. */
typedef struct jxg_frame_params {
  float distance;
  int32_t global_scale;
  int32_t quant_dc;
  float scale;
  float scale_dc;
  uint32_t x_qm_scale;
  uint32_t b_qm_scale;
  uint32_t epf_iters;
  float dc_step[3];
  uint32_t qf_threshold;    /* ac_qf_threshold, src/frame/ac_groups.rs:92 */
  uint32_t screen_content;  /* is_screen_content, src/frame/chroma.rs:42 */
  int32_t epf_sharpness;    /* epf_sharpness_id, src/frame/quantization.rs:218 */
  uint32_t reserved;
  uint64_t constant_blocks; /* numerator of constant_block_fraction */
  uint64_t num_tokens;
} jxg_frame_params;

/* `Token` (src/entropy/token.rs:30-34): fine AC context and value. */
typedef struct jxg_token {
  uint32_t context;
  uint32_t value;
} jxg_token;

/* Number of fine AC contexts (`K_NUM_FINE_AC_CONTEXTS`,
 * src/ac_context.rs:113-114) and the histogram alphabet (`ALPHABET_SIZE`,
 * src/entropy/prefix_code.rs:30). */
#define JXG_NUM_FINE_AC_CONTEXTS 14850
#define JXG_ALPHABET_SIZE 128

/* Caller-allocated outputs of one front-end pass; NULL members are skipped.
 * Sizes follow jxg_frame_info.  Block maps are image rasters of blocks;
 * the tile maps are rasters of 64x64 tiles. */
typedef struct jxg_frontend_output {
  uint8_t* quant_field;    /* xb*yb raw quant field (DcGroupData::raw_quant_field) */
  uint8_t* ac_strategy;    /* xb*yb (raw << 1) | first (AcStrategyImage cells) */
  int8_t* ytox_map;        /* tiles */
  int8_t* ytob_map;        /* tiles */
  int16_t* quant_dc;       /* 3 planes X, Y, B of xb*yb (DcGroupData::quant_dc) */
  int32_t* coefficients;   /* xb*yb*192: per block X, Y, B, 64 levels each, in raw
                              coefficient order; a transform covering several
                              blocks spreads its channel's levels in runs of 64:
                              run t of a transform at (bx, by) covering cx
                              blocks across sits at block (bx + t % cx, by + t / cx) */
  uint8_t* num_nzeros;     /* 3 planes of xb*yb */
  float* xyb;              /* 3 planes of w*h (the opsin image) */
  jxg_token* tokens;       /* pass-one tokens, groups in raster order */
  uint64_t token_capacity; /* entries available in `tokens` */
  uint64_t* group_offsets; /* num_groups + 1 token offsets */
  uint32_t* histograms;    /* JXG_NUM_FINE_AC_CONTEXTS * JXG_ALPHABET_SIZE */
  uint16_t* alpha;         /* RGBA input: w*h alpha after fringe clearing (the
                              plane the extra channel codes); untouched for RGB */
  /* The same tokens in the groups' storage form (AcTokens,
   * src/entropy/token_stream.rs:37-76, as PendingAcGroup holds them,
   * src/frame/ac_groups.rs:78-82): a group whose contexts all fit 14 bits
   * and values 18 bits is one word per token, context << 18 | value; any
   * other group is two words per token, context then value. */
  uint32_t* packed_tokens;
  uint64_t packed_capacity; /* words available in `packed_tokens` */
  uint64_t* packed_offsets; /* num_groups + 1 word offsets; a group is wide when
                               it holds twice as many words as tokens */
} jxg_frontend_output;

/* Library lifetime ---------------------------------------------------- */

/* EncodingContext::new (src/encoding_context.rs:609): device state of one
 * encoder on `device`. */
int32_t jxg_context_create(int32_t device, void** out_ctx);
void jxg_context_destroy(void* ctx);
/* Run this context's launches on `cuda_stream` (a cudaStream_t; NULL
 * restores the context's own stream). */
int32_t jxg_context_set_stream(void* ctx, void* cuda_stream);
/* Text of the last error on this context (empty when none). */
const char* jxg_context_last_error(void* ctx);

/* distance_from_quality (src/encode_image.rs:1321-1338). */
float jxg_distance_from_quality(float quality);
/* ImageDim::new (src/frame.rs:100-123). */
int32_t jxg_frame_info_for(uint64_t width, uint64_t height, jxg_frame_info* out);
/* The input checks of encode_image_rgb / encode_with_coded_planes
 * (src/encode_image.rs:1785-1801, :4818-4827) plus this build's limits,
 * without touching a device: returns the status jxg_frontend_run would. */
int32_t jxg_validate_input(uint64_t width, uint64_t height, int32_t channels, int32_t bits,
                           const jxg_config* config);

/* Front end ------------------------------------------------------------
 * Pass one of encode_frame_core_inner (src/frame/vardct_encoder.rs:798-1100)
 * at the configured speed: linearise + XYB (src/encode_image.rs:1498,
 * src/xyb.rs:439), chroma gates (src/frame/chroma.rs:389), per-DC-group
 * setup_dc_group (src/frame/dc_groups.rs:127: fill_quant_field, fill_cmap,
 * fill_ac_strategy), ac_qf_threshold (src/frame/ac_groups.rs:92) and every
 * process_ac_group (src/frame/ac_groups.rs:116 -> write_ac_group,
 * src/group.rs:1259), with the tokens' per-context histograms
 * (build_histograms_with, src/entropy/write.rs:840).
 *
 * `pixels`: interleaved samples, `channels` 1 (grey, as encode_image_gray
 * on its lossy path: the luma decoded into all three planes,
 * src/encode_image.rs:1571-1600; the caller keeps the reference's bi-level
 * and few-level checks, which route such images to the lossless coder),
 * 2 (grey + alpha), 3 (RGB) or 4 (RGBA; alpha in the last channel, as
 * encode_image_with_alpha / _16bit with their defaults: lossy alpha, so the
 * near-transparent fringe is cleared (src/alpha_fringe.rs:78), zero-alpha
 * colours are filled from their neighbours (src/invisible.rs:34) and a
 * non-constant alpha scales each block's quant field by its peak alpha
 * (src/adaptive_quant.rs:953-1070)), `bits` 8 (bytes, as encode_image) or
 * 10, 12, 16 (16-bit words, as encode_image_10bit / _12bit / _16bit and
 * their _with_alpha forms, src/encode_image.rs:3752-3850, 4230: samples
 * above the largest code decode to 0, alpha is capped to it), decoded by
 * config->transfer (sRGB primaries). */

/* Host input: copies the pixels in, runs, and waits for the device. */
int32_t jxg_frontend_run(void* ctx, const void* pixels, uint64_t width, uint64_t height,
                         int32_t channels, int32_t bits, const jxg_config* config);
/* Device input (`pixels` in this device's memory): enqueues the pass on the
 * context's stream and returns without waiting. */
int32_t jxg_frontend_run_device(void* ctx, const void* pixels, uint64_t width, uint64_t height,
                                int32_t channels, int32_t bits, const jxg_config* config);
/* Waits for the pass and returns its scalars. */
int32_t jxg_frontend_params(void* ctx, jxg_frame_params* out);
/* Waits for the pass and copies the requested outputs to host memory. */
int32_t jxg_frontend_fetch(void* ctx, jxg_frontend_output* out);
/* jxg_frontend_run + jxg_frontend_params + jxg_frontend_fetch. */
int32_t jxg_frontend(void* ctx, const void* pixels, uint64_t width, uint64_t height,
                     int32_t channels, int32_t bits, const jxg_config* config,
                     jxg_frame_params* params, jxg_frontend_output* out);

/* Coefficient-order statistics --------------------------------------------
 * The first AC pass's tally for custom coefficient orders (OrderStats,
 * src/coeff_order.rs:511-540, tallied by the tokeniser at
 * src/group.rs:2555-2574; the reference collects it from Speed::Fast up and
 * derives the orders with derive_orders, src/frame/vardct_encoder.rs:1147-1153).
 * The order groups are ORDER_SPECS (src/coeff_order.rs:117-125): slot
 * s = 0..6 holds order group s with 64, 64, 256, 1024, 128, 256 and 512
 * coefficients (DCT8; the 8x8-sized transforms; DCT16X16; DCT32X32;
 * DCT16X8 / DCT8X16; DCT32X8 / DCT8X32; DCT32X16 / DCT16X32).  Counters
 * are laid out [slot][channel X, Y, B][raw coefficient index], slot s
 * starting at 3 x the sizes of the slots before it, JXG_ORDER_COUNTERS in
 * all; orders use the same layout with scan position in place of raw index. */
#define JXG_ORDER_SLOTS 7
#define JXG_ORDER_COUNTERS 6912
/* The order statistics of the context's last pass (its first frame): per
 * slot, channel and raw index the transforms whose level there is non-zero,
 * counted over the whole transform; `blocks` per slot the transforms.
 * `counts` holds JXG_ORDER_COUNTERS, `blocks` JXG_ORDER_SLOTS.  Waits. */
int32_t jxg_order_stats(void* ctx, uint32_t* counts, uint32_t* blocks);
/* pixel_chromacity_steps (src/frame/chroma.rs:89-165; the reference runs it
 * in configure_chroma, :389-450, from Speed::Fast up at distances from
 * PIXEL_CHROMACITY_MIN_DISTANCE, to raise the X and B quant-scale floors) on
 * the context's last pass (its first frame's XYB, after the invisible fill
 * and the grey snap, as the reference's).  `counts` (7, optional): the X
 * steps reaching 0.015 / 0.022 / 0.026, the B - Y steps above 0.28 / 0.33 /
 * 0.38, the strongly exposed blue pixels; `x_steps` / `b_steps` (optional):
 * the extra steps.  Waits. */
int32_t jxg_pixel_chromacity(void* ctx, uint32_t* counts, uint32_t* x_steps, uint32_t* b_steps);
/* derive_orders (src/coeff_order.rs:621-673), on the host: from statistics
 * laid out as jxg_order_stats writes them, the used-order mask (bit = order
 * group), every slot's three orders (scan position -> raw index; natural
 * where not adopted; JXG_ORDER_COUNTERS entries) and, when `scan_moved` is
 * set, the share of the expected scan walk the adopted orders remove.  Needs
 * no device. */
int32_t jxg_derive_orders(const uint32_t* counts, const uint32_t* blocks, uint16_t* used_mask,
                          uint32_t* orders, double* scan_moved);

/* Asynchronous front end --------------------------------------------------
 * jxg_frontend_enqueue enqueues on the context's stream the upload of
 * `pixels`, the pass, and the download of `params` and every requested
 * output, then returns without waiting; jxg_frontend_wait completes it
 * (params, status).  The group and word offsets are written by the device
 * itself (the group sizes are known only there), so `out->group_offsets`
 * and `out->packed_offsets` must be memory the device can write: pinned
 * host memory (cudaHostAlloc / cudaHostRegister), device memory, or any
 * host memory on systems with coherent CPU-GPU access.  The token streams
 * (`tokens`, `packed_tokens`), whose lengths the host learns at the wait,
 * are copied by the wait, which returns once they have landed.  Upload and
 * downloads run asynchronously when `pixels` and the outputs are pinned.  A context
 * holds one frame in flight (enqueueing again waits for the previous one);
 * two contexts on one device overlap one frame's transfers with the other's
 * kernels.  `pixels` and the outputs must stay valid until the wait. */
int32_t jxg_frontend_enqueue(void* ctx, const void* pixels, uint64_t width, uint64_t height,
                             int32_t channels, int32_t bits, const jxg_config* config,
                             jxg_frame_params* params, jxg_frontend_output* out);
int32_t jxg_frontend_wait(void* ctx);

/* Batch -----------------------------------------------------------------
 * Many frames of any sizes, layouts and distances in one pass: each stage is
 * one launch over the (frame, work unit) list of the whole batch, and the
 * pass can be recorded once as a CUDA graph and replayed.  Every frame's
 * results equal those of a one-frame jxg_frontend call on it.  The reference
 * encodes one image per call (encode_image, src/encode_image.rs:1610); a
 * caller with many images calls this instead of looping.
 *
 * jxg_batch_create: `pixels_on_device` nonzero = the pixel pointers given to
 *   jxg_batch_add are device memory of the context's GPU, else host memory.
 * jxg_batch_add: appends one frame (arguments as jxg_frontend_run); returns
 *   its index, or the negated status when the input is rejected.  The
 *   pointer is read at every jxg_batch_run, so it must stay valid.
 * jxg_batch_run: runs the pass and waits.  `use_graph` nonzero records the
 *   pass as a CUDA graph on the first run and replays it afterwards; adding
 *   a frame, or running another pass on the context, re-records it.
 * jxg_batch_result: scalars and outputs of frame `index` of the last run
 *   (either pointer may be NULL); as jxg_frontend_params + _fetch.
 * One context holds one pass at a time: results of a batch are readable
 * until the context runs another pass. */
int32_t jxg_batch_create(void* ctx, int32_t pixels_on_device, void** out_batch);
int64_t jxg_batch_add(void* batch, const void* pixels, uint64_t width, uint64_t height,
                      int32_t channels, int32_t bits, const jxg_config* config);
int32_t jxg_batch_run(void* batch, int32_t use_graph);
int32_t jxg_batch_result(void* batch, uint64_t index, jxg_frame_params* params,
                         jxg_frontend_output* out);
void jxg_batch_destroy(void* batch);

/* Operator table --------------------------------------------------------
 * Single-stage entry points standing in for the reference's kernel
 * dispatch table (EncodingContext, src/encoding_context.rs:224-294).  They
 * take host buffers and run the same device kernels as the front end. */

/* FillQuantFieldFn (src/adaptive_quant.rs:474) over every DC group of an XYB
 * image: `xyb` is 3 planes of w*h floats; writes xb*yb raw field values. */
int32_t jxg_op_fill_quant_field(void* ctx, const float* xyb, uint64_t width, uint64_t height,
                                float distance, float inv_scale, uint8_t* quant_field);
/* apply_chroma_hf_protection (src/adaptive_quant.rs:303-402; the reference
 * runs it after the field, per DC group, when the Slow chroma policy marks
 * the frame X- or B-heavy, src/frame/dc_groups.rs:100-108) over a whole
 * frame: `xyb` is 3 planes of w*h floats, `quant_field` the xb*yb raw field,
 * raised in place where a block's edges are mostly chromatic.  Outside
 * distances 0.35 to 2 the field is left as it is. */
int32_t jxg_op_chroma_hf_protection(void* ctx, const float* xyb, uint64_t width, uint64_t height,
                                    float distance, uint8_t* quant_field);
/* gaborish_inverse (src/gaborish.rs:44; the encoder's pre-inversion that
 * gaborize, src/frame/quantization.rs:240-245, runs with mul 0.9908511 when
 * Gaborish is enabled): `xyb` is 3 planes of w*h floats, `out` receives the
 * filtered planes (a symmetric 5x5 with mirror-reflected edges, every output
 * from the source pixels).  `mul` must be non-negative. */
int32_t jxg_op_gaborish_inverse(void* ctx, const float* xyb, uint64_t width, uint64_t height,
                                float mul, float* out);
/* The decoder's Gaborish (src/epf_filter.rs:165, gaborish_pixel
 * src/epf_filter/kernels.rs:134): the 3x3 with clamped edges and the
 * default weights, products fused into the sums as the NEON and AVX2+FMA
 * backends do. */
int32_t jxg_op_gaborish(void* ctx, const float* xyb, uint64_t width, uint64_t height, float* out);
/* The decoder's edge-preserving filter (Epf::apply, src/epf_filter.rs:268-350):
 * `xyb` 3 planes of w*h floats in, `out` the filtered planes.  `sigma_quant`
 * holds one value per 8x8 block (xb*yb, FrameBlocks::sigma_quant: the
 * quantizer scale x the block's field x -1.1715729); `iters` 0..3 picks the
 * stages (1: the 4-neighbour patch stage; 2: + the single-pixel stage at
 * `pass2`; 3: the 12-neighbour stage at `pass0` first); `quant_mul`,
 * `border_mul` and `channel_scale` are LoopFilter's fields as the decoder
 * reads them; `sharpness` 0..7 (0, like iters 0, leaves the planes as they
 * are).  Products and sums round separately, as the reference's scalar
 * backend. */
int32_t jxg_op_epf(void* ctx, const float* xyb, uint64_t width, uint64_t height, const float* sigma_quant,
                   int32_t iters, float quant_mul, float pass0, float pass2, float border_mul,
                   const float* channel_scale, int32_t sharpness, float* out);
/* The reference's six-term luma proxy (LumaProxy::new / compare,
 * src/epf_proxy.rs:148-214): `source` and `test` Y planes of w*h floats
 * (both at least 4 x 4); `terms` (6 floats, may be NULL) receives the
 * quarter-resolution structure mean, the half-resolution structure mean and
 * fourth-power pool, and the adjacent-gradient error, excess and
 * fourth-power pool; `score` their weighted sum.  The pools are parallel
 * sums (the reference's are sequential): equal to rounding. */
int32_t jxg_op_luma_proxy(void* ctx, const float* source, const float* test, uint64_t width, uint64_t height,
                          double* score, double* terms);
/* The encoder's EPF fit (fit and choose, src/epf_filter.rs:599-671,
 * :807-873; MediumSlow and up in the reference): candidate loop-filter
 * settings rendered over `recon` (3 planes of w*h) with the EPF and ranked
 * by the luma proxy of their Y plane against `source_y` (w*h): the
 * baseline, no filtering, four shape pilots at strength 2 / distance, the
 * best pilot's endpoints and a log-quadratic vertex.  A setting is {iters,
 * quant_mul, pass0, sharpness} with NaN for an unset quant_mul or pass0;
 * `choice` (4 floats) carries the baseline in and the chosen setting out,
 * `score` its proxy score.  Frames of at least 4 x 4 pixels. */
int32_t jxg_op_epf_fit(void* ctx, const float* source_y, const float* recon, uint64_t width, uint64_t height,
                       const float* sigma_quant, float distance, float* choice, double* score);
/* DctFn<8, 8, 64> (src/dct.rs:172, scalar dct8x8 :631): `count` blocks of 64
 * row-major samples in, 64 coefficients (transposed storage, 1/64 scale) out. */
int32_t jxg_op_dct8x8(void* ctx, const float* blocks, uint64_t count, float* coefficients);
/* DctFn<W, H, N> of the larger blocks (src/dct.rs: dct8x16 :823, dct16x8
 * :904, dct16x16 :1010, dct32x32 :1980, dct32x16 :2251, dct16x32 :2340,
 * dct32x8 :1742, dct8x32 :1777, dct64x64 :2576, dct64x32 :2659, dct32x64
 * :2689; src/dct128.rs dct128x128 :385, dct128x64 :416, dct64x128 :446;
 * kind 0 is dct8x8 as jxg_op_dct8x8) with the DC values of every covered
 * 8x8 block (dc_from_dct*, src/dct.rs:930-2806, src/dct128.rs:561-636).
 * `blocks` holds `count` row-major blocks of H rows of W samples;
 * `coefficients` receives W H coefficients per block in the reference's
 * order, `dc_values` (optional) one value per covered 8x8 block (1, 2, 2,
 * 4, 8, 8, 16, 4, 4, 64, 32, 32, 256, 128, 128 for kinds 0..14) in raster
 * order of those blocks. */
#define JXG_DCT8X8 0
#define JXG_DCT8X16 1  /* 8 rows x 16 columns */
#define JXG_DCT16X8 2
#define JXG_DCT16X16 3
#define JXG_DCT16X32 4
#define JXG_DCT32X16 5
#define JXG_DCT32X32 6
#define JXG_DCT32X8 7   /* 32 rows x 8 columns */
#define JXG_DCT8X32 8
#define JXG_DCT64X64 9
#define JXG_DCT64X32 10 /* 64 rows x 32 columns */
#define JXG_DCT32X64 11
#define JXG_DCT128X128 12
#define JXG_DCT128X64 13 /* 128 rows x 64 columns */
#define JXG_DCT64X128 14
int32_t jxg_op_dct(void* ctx, int32_t kind, const float* blocks, uint64_t count,
                   float* coefficients, float* dc_values);
/* The inverse transforms (IdctMethods, src/dct.rs:358-416; inv_dct8x16
 * :1634, inv_dct16x8 :1658, inv_dct16x32 :1683, inv_dct32x16 :1705,
 * inv_dct8x32 :1804, inv_dct32x8 :1833, inv_dct64x32 :2710, inv_dct32x64
 * :2735, the square inverses :1590-1627; src/dct128.rs:473-555): `count`
 * blocks of W H
 * coefficients in jxg_op_dct's order back to row-major H x W samples. */
int32_t jxg_op_idct(void* ctx, int32_t kind, const float* coefficients, uint64_t count,
                    float* blocks);
/* The 8x8-sized transforms besides DCT8 on `count` row-major 8x8 blocks:
 * kind 0 identity8x8 (src/dct.rs:185), 1 dct2x2_8x8 (:306), 2 dct4x4
 * (:1163), 3 dct4x8 (:1238), 4 dct8x4 (:1319), 5 inv_identity8x8 (:225),
 * 6 inv_dct2x2_8x8 (:345), 7..10 afv_from_pixels kinds 0..3 (src/afv.rs:207;
 * AFV corner at the left/right, top/bottom of the block by kind bits 0/1);
 * 64 values out per block. */
int32_t jxg_op_small_transform(void* ctx, int32_t kind, const float* blocks, uint64_t count,
                               float* out);
/* AcTokens::from (src/entropy/token_stream.rs:59-76) per group: `tokens`
 * from group_offsets[0] to group_offsets[num_groups] (host arrays) into the
 * storage form of jxg_frontend_output.packed_tokens; `word_offsets` gets
 * num_groups + 1 offsets from zero.  At most `capacity` words are written;
 * a larger stream returns JXG_ERR_INVALID_ARGUMENT after the offsets. */
int32_t jxg_op_pack_tokens(void* ctx, const jxg_token* tokens, const uint64_t* group_offsets,
                           uint64_t num_groups, uint32_t* words, uint64_t capacity,
                           uint64_t* word_offsets);

/* Allocation-free token offsets -----------------------------------------
 * This entry point has no counterpart in the reference encoder.  It is for
 * callers that cannot allocate device memory at encode time: a host that
 * owns every device buffer through its own pool or arena, a real-time
 * pipeline that forbids allocation after start-up, or code that enqueues
 * work where a cudaMalloc would stall or serialise other streams.  It runs
 * the same exclusive scan the front end uses to place tokens (token counts
 * in the [group][1024 blocks][Y, X, B] layout -> per-entry offsets, per-group
 * offsets and, in group_offsets[num_groups], the token total), reading and
 * writing only the caller's device buffers plus one fixed scratch array
 * compiled into the library (a file-scope __device__ array of 16 KiB of
 * chunk sums and 1 KiB of pass scalars, held by every GPU that loads the
 * library until the process exits).
 *
 * - counts:        device, num_groups * 3072 uint32 token counts;
 * - offsets:       device, num_groups * 3072 uint32 exclusive offsets out;
 * - group_offsets: device, num_groups + 1 uint64 out;
 * - cuda_stream:   a cudaStream_t (NULL = the legacy default stream).
 * Limit: num_groups <= JXG_NOALLOC_MAX_GROUPS groups of 256x256 pixels
 * (frames up to about 0.72 gigapixels); larger requests return JXG_ERR_DIMENSION_TOO_LARGE.  The call
 * only enqueues work on the stream; it calls no cudaMalloc, cudaFree or
 * allocating library routine.  The first call on a device looks up the
 * scratch array's device address (cudaGetSymbolAddress) with that device
 * current; make that first call before any stream capture.  All calls share
 * the one scratch array, which keeps the last call's contents: calls whose
 * work overlaps on the GPU (different streams, or different host threads on
 * one device) race and must be serialised by the caller. */
#define JXG_NOALLOC_MAX_GROUPS 10922
int32_t jxg_token_offsets_noalloc(const uint32_t* counts, uint64_t num_groups, uint32_t* offsets,
                                  uint64_t* group_offsets, void* cuda_stream);

/* Bounded device waits ---------------------------------------------------
 * The invisible-colour fill lets a warp wait for neighbouring tiles that
 * other warps fill; every such wait polls at most a fixed number of times
 * and, when that runs out, records JXG_ERR_DEVICE_TIMEOUT for the frame
 * instead of spinning on.  This entry point runs the same wait on a flag
 * that is never set, for `polls` polls, and returns JXG_ERR_DEVICE_TIMEOUT:
 * the error path, exercised without faulting or hanging the device. */
int32_t jxg_selftest_bounded_wait(void* ctx, uint32_t polls);
/* The tokenizer's look-back on token offsets waiting on a chunk that never
 * publishes, for `polls` polls: returns JXG_ERR_DEVICE_TIMEOUT with the
 * context still usable. */
int32_t jxg_selftest_token_lookback(void* ctx, uint32_t polls);

/* The XYB cube root and the AQ pre-pass and gamma terms divide and take
 * square roots with fused-multiply-add sequences instead of the IEEE
 * operations, on input ranges where they give the same results.  This entry
 * point compares both on the device for every float bit pattern in
 * [lo_bits, hi_bits): `which` 0 = the cube root (XYB inputs lie in
 * [0, 0x40000000)), 1 / 2 = the AQ gamma ratio inverted / direct (inputs in
 * [0, 0x44800000)), 3 = the AQ masking square root (inputs in
 * [0, 0x3E4CCCCD]), 4 = the cube root on the packed two-lane FP32 path,
 * 5 = a 16-bit sample over 65535 (here [lo, hi) are sample values, 0..65536),
 * 6 / 7 / 8 = the gamma ratio inverted / direct and the masking square root
 * on the packed two-lane FP32 path.
 * It returns the number of differing results and the
 * smallest differing pattern (0xFFFFFFFF when none). */
int32_t jxg_selftest_math(void* ctx, int32_t which, uint32_t lo_bits, uint32_t hi_bits,
                          uint64_t* mismatches, uint32_t* first_bad);

/* Quant-field refinement -------------------------------------------------
 * No counterpart in the reference, which has no gradients anywhere: the
 * per-block quant field of an all-DCT8 frame is refined by gradient steps on
 * a differentiable model of its coding.  Parameters theta are one log quant
 * scale per 8x8 block: block b quantises at scale * qf_b * exp(theta_b), qf
 * the frame's adaptive field.  The model (FP32) quantises and dequantises the
 * AC coefficients exactly as the front end does (with CfL and the decoder's
 * bias; the DC slot holds the pass's decoded DC), inverts the 8x8 DCT,
 * applies the decoder's EPF at the frame's settings (its adjoint with the
 * weights held), converts XYB to linear RGB and scores 1 - SSIM
 * against the source at three scales, plus a rate model (1.6 + log2(1 +
 * |level|) bits per non-zero AC level, 2.6 (|v| / max(threshold, 0.5))^4 per
 * level v that rounds to zero); rounding is straight-through in the backward
 * pass.  Gaborish (off in the reference's encoder) and DC smoothing are not
 * modelled.
 *
 * jxg_refine_begin takes the frame of the context's last pass (one frame,
 * Speed::UltraFast), copies what the model needs (a later pass does not
 * disturb it), sets the context's own theta to zero and returns the
 * frame's size (theta holds one value per 8x8 block: ceil(width / 8) x
 * ceil(height / 8)); the others need it. */
int32_t jxg_refine_begin(void* ctx, uint64_t* width, uint64_t* height);
/* Loss at `theta` (device memory, xb*yb floats; NULL: the context's own):
 * loss3 = {distortion + rate_lambda * bits / pixels, distortion, bits} on the
 * host; `grad` (device, xb*yb floats, or NULL) receives d loss / d theta from
 * the hand-written adjoint kernels; `levels` (host, xb*yb*192, or NULL) the AC
 * levels per block, channel X, Y, B and raw coefficient index (row * 8 + col,
 * the DC slot 0). */
int32_t jxg_refine_eval(void* ctx, const float* theta, float rate_lambda, float* grad, double* loss3,
                        int32_t* levels);
/* The distortion's mix: ssim_weight x (1 - SSIM, as above) + proxy_weight x
 * the reference's six-term luma proxy (LumaProxy, src/epf_proxy.rs:132-214:
 * structure terms of the decoded XYB Y plane at half and quarter resolution
 * and its adjacent gradients, against the source's; frames of at least 4 x 4
 * pixels).  Defaults 1 and 0.1; both finite, non-negative, not both zero. */
int32_t jxg_refine_set_weights(void* ctx, float ssim_weight, float proxy_weight);
/* One Adam step (beta 0.9 / 0.999) on the context's own theta: loss3 at the
 * theta before the step, as jxg_refine_eval.  theta stays where
 * qf * exp(theta) is within 1..255. */
int32_t jxg_refine_step(void* ctx, float rate_lambda, float learning_rate, double* loss3);
/* Copy the context's own theta out to `theta` (to_context 0) or in from it
 * (1; restarts Adam); host or device memory, xb*yb floats. */
int32_t jxg_refine_theta(void* ctx, float* theta, int32_t to_context);
/* The model's decoded frame at `theta` (NULL: the context's own): the XYB
 * planes after dequantisation, the inverse transforms, the decoded DC and
 * the EPF, 3 planes of w*h floats on the host (a decoder's reconstruction
 * of the all-DCT8 frame, short of DC smoothing). */
int32_t jxg_refine_decoded(void* ctx, const float* theta, float* xyb);
/* The integer field of `theta` (NULL: the context's own): round(qf *
 * exp(theta)) clamped to 1..255, xb*yb bytes into host or device memory. */
int32_t jxg_refine_field(void* ctx, const float* theta, uint8_t* quant_field);
/* The model's constants for an outside check: constants = {scale, qm_mul[3],
 * matrix[3][64], inv_matrix[3][64], thresholds[3][4], then the EPF's stage
 * count, stage ids[3] (-1 unused), SAD multipliers[3], border multiplier,
 * channel scales[3], quant_mul, sharpness / 7, quantizer scale} (414 floats); the
 * source coefficients (xb*yb*192, raw order), the 64 x 64 inverse transform
 * [pixel][coefficient] and the decoded DC per block (xb*yb*3: X, Y, B; the
 * pass's DC levels dequantised, which the model's DC slot holds); any of the
 * last three may be NULL; all on the host. */
int32_t jxg_refine_model(void* ctx, float* constants, float* coefficients, float* inverse, float* dc);
/* One UltraFast pass with the caller's quant field (xb*yb values 1..255, host
 * or device memory; e.g. a refined field) in place of the adaptive one; the
 * AC thresholds' median stage runs over it.  Host pixels: runs and waits, as
 * jxg_frontend_run; device pixels: enqueues, as jxg_frontend_run_device. */
int32_t jxg_frontend_run_with_field(void* ctx, const void* pixels, uint64_t width, uint64_t height,
                                    int32_t channels, int32_t bits, const jxg_config* config,
                                    const uint8_t* quant_field, int32_t pixels_on_device);

/* Launch geometry and its autotuner ---------------------------------------
 * Warps per CTA of the Speed::Fastest kernels whose warps work
 * independently (each warp a candidate transform, a placed transform, a
 * re-tiling tile or a strip of merge sites), in this order: the DCT8,
 * 16x8, 8x16 and 16x16 costs, the DCT8, 16x8, 8x16 and 16x16 layout
 * coding, the re-tiling DP, the site variance.  Results never depend on it;
 * its speed does, by occupancy and tail against the GPU's shared memory and
 * SM count.  It has no counterpart in the reference, whose thread pool needs
 * no tuning. */
#define JXG_TUNE_KERNELS 10
/* The context's current warps per CTA (JXG_TUNE_KERNELS bytes). */
int32_t jxg_get_launch_geometry(void* ctx, uint8_t* warps);
/* Sets them (each 1, 2, 4 or 8), e.g. from a choice saved for this GPU. */
int32_t jxg_set_launch_geometry(void* ctx, const uint8_t* warps);
/* Times every candidate (1, 2, 4, 8 warps per CTA, all kernels at once) on
 * `rounds` passes of the given frame (device pixels, as
 * jxg_frontend_run_device; a Speed::Fastest config, the only one that
 * launches these kernels) after one untimed pass each, with CUDA events per
 * launch, and keeps each kernel's fastest.  `times_ms`, if not NULL,
 * receives JXG_TUNE_KERNELS x 4 average launch times (NaN where a kernel did
 * not run).  The passes reuse the context's buffers; the context's
 * previous outputs are overwritten. */
int32_t jxg_autotune(void* ctx, const void* pixels, uint64_t width, uint64_t height,
                     int32_t channels, int32_t bits, const jxg_config* config, int32_t rounds,
                     double* times_ms);

/* Kernel timing -------------------------------------------------------- */
/* With `enable`, every launch of this context is bracketed by CUDA events on
 * its stream; jxg_kernel_times sums their durations per kernel. */
int32_t jxg_enable_kernel_timing(void* ctx, int32_t enable);
/* Fills up to `capacity` entries of names (static strings), total
 * milliseconds and launch counts; returns the number of kernels. */
int32_t jxg_kernel_times(void* ctx, const char** names, double* total_ms, uint64_t* launches,
                         int32_t capacity);
int32_t jxg_reset_kernel_times(void* ctx);

#ifdef __cplusplus
}
#endif

#endif /* JXG_H_ */
