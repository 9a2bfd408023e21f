/*
 * cuimg_gb300 -- C ABI of the GB300 (sm_103a) semi-dense tracking path.
 *
 * This is the drop-in boundary for cuimg's per-frame tracker
 *   cuimg::tracker<tracking_strategies::bc2s_fast_gradient_cpu>::run(frame)
 * (cuimg/tracking2/tracker.hpp:72-91): a C++ strategy object or any FFI calls
 * these functions instead of running the reference's OpenMP functors.  All
 * signatures use plain pointers and sizes.  Every function returns a status
 * code (GBT_OK == 0); no exception crosses the ABI.  One context is driven by
 * one host thread; all its GPU work is ordered on the context's CUDA stream.
 *
 * Geometry follows the reference: level s has floor(rows / 2^s) x
 * floor(cols / 2^s) pixels (obox2d operator/, cuimg/obox2d.h:69-72); points
 * are (row, col).
 */
#ifndef CUIMG_GB300_H_
#define CUIMG_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define GBT_OK 0
#define GBT_E_INVALID 1   /* bad argument or unsupported size */
#define GBT_E_CUDA 2      /* a CUDA runtime call failed (see gbt_last_error) */
#define GBT_E_OOM 3       /* device or pinned allocation failed */
#define GBT_E_CAPACITY 4  /* a particle set outgrew its preallocated capacity */
#define GBT_E_TIMEOUT 5   /* a bounded device-side wait gave up */
#define GBT_E_TOO_LARGE 6 /* request exceeds the fixed scratch of an allocation-free entry point */

typedef struct gbt_ctx gbt_ctx;

/* One video stream's tracker settings.  Mirrors the reference's constructor
 * tracker<F>(obox2d(rows, cols), nscales) and the setters of
 * generic_strategy (tracking_strategies.hpp:56-91) and fast_detector
 * (fast_detector.hpp:170-193). */
typedef struct {
  int32_t rows, cols;           /* level-0 frame size */
  int32_t nscales;              /* number of pyramid levels / tracker scales (1..9) */
  int32_t detector_threshold;   /* fast_detector::set_fast_threshold (>= 0) */
  int32_t detector_n;           /* fast_detector::set_n (arc length, default 9) */
  int32_t detector_frequency;   /* generic_strategy::set_detector_frequency */
  int32_t filtering_frequency;  /* generic_strategy::set_filtering_frequency */
  int32_t k;                    /* generic_strategy::set_k (default 300) */
  int32_t with_merge;           /* generic_strategy::set_with_merge (default 1) */
  int32_t detector;             /* GBT_DETECTOR_*: the strategy's detector (default FAST) */
  int32_t detector_step;        /* regular_detector::set_step (default 1) */
  int32_t detector_grad_th;     /* regular_detector::set_grad_th (default 1) */
  int32_t matcher;              /* GBT_MATCHER_*: the strategy's matcher (default BC2S) */
} gbt_config;

/* Matchers.  GBT_MATCHER_BC2S is the generic strategy's BC2S feature descent
 * (bc2s_fast_gradient_cpu and the other detectors above).  GBT_MATCHER_LK is
 * the reference's pyramidal LK tracker strategy,
 * pyrlk_cpu<fast_detector<cpu>, iterative_lk_match_5x5>
 * (cuimg/tracking2/pyrlk_tracker.h:16-82, pyrlk_tracker.hpp:772-1063):
 * sub-pixel particles (gbt_get_particles_f) matched by LK with an 11x11
 * window, the 25 strongest gradients, 30 iterations and the coarse-to-fine
 * prediction of get_flow_at, FAST births, compaction and merge; no BC2S
 * features or flow bins.  All streams of a context use the same matcher.  LK
 * contexts take gray frames (GBT_FRAMES_HOST / GBT_FRAMES_DEVICE) and keep the
 * stages INPUT (the strategy's image, border up to 3), SALIENCY, MASK and
 * SPARSE; input slots, graphs, tuning, trajectories, checkpoints, flow bins,
 * profiling and RGB input return GBT_E_INVALID for them.  The FAST detector
 * is the only detector of the LK strategy. */
#define GBT_MATCHER_BC2S 0
#define GBT_MATCHER_LK 1

/* Detectors of the reference's generic strategy (tracking_strategies.h):
 * bc2s_fast_gradient_cpu (fast_detector), bc2s_regular_gradient_cpu
 * (regular_detector: a particle at every `step`-th pixel of every row and
 * column whose 8-neighbour contrast at distance 2, averaged, reaches
 * `grad_th`, regular_detector.hpp:62-103) and bc2s_dense_gradient_cpu
 * (dense_detector: a particle at every pixel without one,
 * dense_detector.hpp:19-31).  Births are added in raster order before the
 * compaction, like the FAST births.  The particle capacity of a level is
 * H*W/6 + 4096 for FAST, 4 * ceil(H/step) * ceil(W/step) + 4096 for regular
 * and 4*H*W + 4096 for dense (neither checks for particles already at a
 * pixel the way FAST does, so the reference's counts grow without bound);
 * births beyond it are dropped and gbt_sync reports GBT_E_CAPACITY. */
#define GBT_DETECTOR_FAST 0
#define GBT_DETECTOR_REGULAR 1
#define GBT_DETECTOR_DENSE 2

/* Fills `cfg` with the reference defaults for a rows x cols stream. */
void gbt_config_default(gbt_config* cfg, int32_t rows, int32_t cols, int32_t nscales);

/* Returns 1 if the tracker accepts this geometry: every level at least
 * 16 x 16 and every 8x8 flow bin's parent bin inside the next level (the
 * reference reads outside its upper flow image otherwise,
 * tracking_strategies.hpp:596-599). */
int gbt_sizes_ok(int32_t rows, int32_t cols, int32_t nscales);

/* Creates a context that advances `nstreams` independent streams (each with
 * its own configuration and resolution) by one frame per gbt_run call.
 * Replaces constructing one tracker<F> per stream (tracker.hpp:11-26). */
int gbt_create(const gbt_config* cfgs, int32_t nstreams, int32_t device, gbt_ctx** out);

/* The same with the number of stream groups chosen by the caller (0: the
 * default, min(4, nstreams)).  The streams are split into groups balanced by
 * pixels per frame; each group is a complete tracker over its streams with its
 * own device buffers, CUDA streams and graphs, so the latency-bound stages of
 * one group run while another group's matcher or blurs fill the GPU.  Results
 * do not depend on the grouping.  No counterpart in the reference. */
int gbt_create_ex(const gbt_config* cfgs, int32_t nstreams, int32_t device, int32_t groups, gbt_ctx** out);
int gbt_groups(gbt_ctx* ctx, int32_t* groups);
int gbt_destroy(gbt_ctx* ctx);

/* Message of the last error on this context (NUL-terminated). */
int gbt_last_error(gbt_ctx* ctx, char* buf, size_t len);

/* Frame input.  `frames[i]` is stream i's gray uint8 frame with row pitch
 * `pitches[i]` bytes; `location` says where the pointers live.  With
 * GBT_FRAMES_HOST the frames are staged through the context's pinned buffers
 * (host copy + one H2D copy per stream, ordered on the context stream).  With
 * GBT_FRAMES_DEVICE (and GBT_FRAMES_DEVICE_RGB) the frame's first kernel reads
 * the caller's buffers directly, with no copy: they must hold the frame when
 * the context's streams reach it and stay unchanged until the frame is done
 * (gbt_sync, or an event recorded on gbt_stream after this call).
 * Replaces tracker<F>::run(const I& in) (tracker.hpp:72-80). */
#define GBT_FRAMES_HOST 0
#define GBT_FRAMES_DEVICE 1
#define GBT_FRAMES_HOST_RGB 2   /* interleaved RGB on the host */
#define GBT_FRAMES_DEVICE_RGB 3 /* interleaved RGB on the device */
int gbt_run(gbt_ctx* ctx, const uint8_t* const* frames, const int64_t* pitches, int32_t location);

/* RGB frames are copied to the device as they are (3 bytes per pixel; one
 * H2D copy straight from pinned host memory) and turned into gray inside the
 * pyramid kernel, which writes level 0 and the coarser levels in one pass.
 * GBT_RGB_CHANNEL0 (default) tracks channel 0, as the reference's sample does
 * (get_x, dsl/get_comp.h:105; samples/tracking/main.cc:117); GBT_RGB_BT601
 * tracks the luma (77 R + 150 G + 29 B + 128) >> 8 (not a reference path). */
#define GBT_RGB_CHANNEL0 0
#define GBT_RGB_BT601 1
int gbt_set_rgb_to_gray(gbt_ctx* ctx, int32_t mode);

/* Runs one frame for all streams from frames already placed in the
 * context's input slots (gbt_input_slot); used for CUDA-graph replay. */
int gbt_run_resident(gbt_ctx* ctx);

/* Device pointer and pitch of stream `s`'s level-0 input slot for the next
 * frame.  Consecutive frames alternate between two slots (the front end of
 * one frame runs while the back end of the previous one still reads the other
 * slot's images), so ask again before every frame; write the slot on the
 * context stream (gbt_stream) or synchronously. */
int gbt_input_slot(gbt_ctx* ctx, int32_t stream, uint8_t** dptr, int64_t* pitch);

/* Capture the per-frame launch sequences into CUDA graphs and replay them
 * from then on (1), or launch stage by stage (0).  Each stream group keeps a
 * front-end graph per frame parity and a back-end graph per frame kind
 * (detector and filter frames or not) and parity. */
int gbt_use_graphs(gbt_ctx* ctx, int32_t enable);

/* Waits for all queued work; returns GBT_E_CAPACITY/GBT_E_TIMEOUT if a
 * device-side check has failed in this context (the flags stay set: the
 * particle state is no longer the reference's from then on). */
int gbt_sync(gbt_ctx* ctx);

/* Test hook for the bounded device-side waits (no reference counterpart).
 * With `enable` set, the tiled matcher arms each tile's barrier but issues no
 * copy, so every tile's wait gives up (after 0.5 s of the GPU's global timer,
 * counted while the CTA is resident), leaves the tile's particles unmatched and
 * flags the context: the next gbt_sync returns GBT_E_TIMEOUT.  (Outside the
 * hook, a tile whose copies were issued and still had not landed after a
 * second 0.5 s wait also reports "copy still in flight" in gbt_last_error:
 * destroy that context, since the copies may land in another tile's shared
 * memory.)  Nothing faults; the device and other
 * contexts stay usable.  GBT_E_INVALID when the context does not stage tiles
 * by TMA (another matcher variant, or no tensor maps). */
int gbt_test_withhold_tile_copies(gbt_ctx* ctx, int32_t enable);

/* Test hook (no reference counterpart): the tiled matcher bins each frame's
 * particles into a fixed-capacity list per 64 x 128 tile (1024 particles) and
 * matches the particles beyond a full tile's capacity from global memory in a
 * second kernel; this sets a smaller capacity (1 .. 1024) so that the
 * overflow path carries most particles.  Results do not change. */
int gbt_test_tile_capacity(gbt_ctx* ctx, int32_t cap);

/* Test hook (no reference counterpart): the number of particles the tiled
 * matcher with slim margins (GBT_TUNE_MATCH_TILE 4..7) has matched again from
 * global memory because their descent would have left the staged tile, summed
 * over the context's frames so far; waits for queued work. */
int gbt_test_tile_fallbacks(gbt_ctx* ctx, int64_t* count);

/* The CUDA stream (cudaStream_t) that follows the context's work: after every
 * call that queues work it waits for all of that work, so an event recorded
 * on it (or work queued on it) comes after the frames queued so far, and input
 * the caller writes on it is waited for.  (Each stream group works on its own
 * internal streams; a frame's input copy, pyramid and blurs overlap the
 * previous frame's matching and filtering.  The matching and filtering
 * streams have the device's greatest priority and the input, pyramid and
 * blur streams its least (the default priority), so a caller's own work at
 * the default priority shares the GPU with the latter.) */
int gbt_stream(gbt_ctx* ctx, void** cuda_stream);

/* Runtime setters, callable between frames at any time, as the reference's
 * strategy and detector setters are: generic_strategy::set_detector_frequency,
 * set_filtering_frequency, set_k, set_with_merge
 * (cuimg/tracking2/tracking_strategies.hpp:56-91), fast_detector::set_n and
 * set_fast_threshold (cuimg/tracking2/fast_detector.hpp:170-193) and
 * regular_detector::set_grad_th (cuimg/tracking2/regular_detector.hpp:25-40).
 * `scale` selects one scale of the stream (the reference's
 * tracker.scale(s).strategy()...) or, with -1, every scale and the stream's
 * configuration.  gbt_set_param waits for the context's queued work; the
 * frames queued after it use the new value.  Ranges as gbt_create: threshold,
 * k and grad_th >= 0, n in 1..16, frequencies >= 1, with_merge 0 or 1.
 * Values set for one scale only are not part of a checkpoint's configuration
 * check: set them again on the context a checkpoint is loaded into. */
#define GBT_PARAM_DETECTOR_THRESHOLD 0
#define GBT_PARAM_DETECTOR_N 1
#define GBT_PARAM_DETECTOR_FREQUENCY 2
#define GBT_PARAM_FILTERING_FREQUENCY 3
#define GBT_PARAM_K 4
#define GBT_PARAM_WITH_MERGE 5
#define GBT_PARAM_DETECTOR_GRAD_TH 6
int gbt_set_param(gbt_ctx* ctx, int32_t stream, int32_t scale, int32_t key, int32_t value);
int gbt_get_param(gbt_ctx* ctx, int32_t stream, int32_t scale, int32_t key, int32_t* value);

/* Particle set of (stream, scale): dense slot count (tombstones included,
 * as particle_container::size(), particle_container.h:137). */
int gbt_nparticles(gbt_ctx* ctx, int32_t stream, int32_t scale, int32_t* n);

/* Copies the particle set to host arrays sized for gbt_nparticles entries:
 * speed (2 floats: row, col), pos (2 int16: row, col), age (uint16),
 * features (16 bytes: s1 ring samples then s2 ring samples; the reference's
 * 16 weights are the constant 255 on this path).  `matches` (size >= the
 * pre-compaction slot count, returned in *nmatches) is the
 * old-slot -> new-slot map of the last compaction, -1 for dead slots
 * (particle_container::matches(), particle_container.hpp:215-252);
 * *compact_has_run says whether this frame compacted.  Any pointer may be
 * NULL.  Replaces pset().dense_particles()/features()/matches(). */
int gbt_get_particles(gbt_ctx* ctx, int32_t stream, int32_t scale, float* speed, int16_t* pos,
                      uint16_t* age, uint8_t* features, int32_t* matches, int32_t* nmatches,
                      int32_t* compact_has_run);

/* The particle set with sub-pixel positions: pos and speed as 2 floats
 * (row, col) per slot, the rest as gbt_get_particles.  For the LK matcher the
 * positions are the particle_f<translation_transform> positions
 * (particle_container.h:45-57); gbt_get_particles gives them truncated to
 * int16 (the reference's i_int2 conversion) and zero features.  For the BC2S
 * matcher they are the integral positions as floats. */
int gbt_get_particles_f(gbt_ctx* ctx, int32_t stream, int32_t scale, float* pos, float* speed, uint16_t* age,
                        int32_t* matches, int32_t* nmatches, int32_t* compact_has_run);

/* Stage images of (stream, scale) after the last frame, for checks and
 * debugging.  Sizes: level rows x cols (+2*border for the bordered ones). */
#define GBT_STAGE_INPUT 0     /* uint8, border b: pyramid level (clamped border) */
#define GBT_STAGE_S1 1        /* uint8, border b: BC2S blur 1 */
#define GBT_STAGE_S2 2        /* uint8, border b: BC2S blur 2 */
#define GBT_STAGE_CONTRAST 3  /* uint32: contrast_kernel value */
#define GBT_STAGE_SALIENCY 4  /* uint8: FAST saliency (valid right after a detector frame) */
#define GBT_STAGE_MASK 5      /* uint8: detector mask (valid right after a detector frame) */
#define GBT_STAGE_SPARSE 6    /* uint32: particle index per pixel, 0xFFFFFFFF = none */
int gbt_get_stage(gbt_ctx* ctx, int32_t stream, int32_t scale, int32_t stage, int32_t border, void* out);

/* Flow bins (8x8 px) of (stream, scale): bin grid size, then flow (2 floats
 * per bin, NO_FLOW = -500), multiscale count, stats count and stats speed
 * (2 int32 per bin).  compute_flow_stats_kernel / flow_fusion_kernel
 * (tracking_strategies.hpp:525-639). */
int gbt_bins(gbt_ctx* ctx, int32_t stream, int32_t scale, int32_t* rows, int32_t* cols);
int gbt_get_bins(gbt_ctx* ctx, int32_t stream, int32_t scale, float* flow, uint32_t* count,
                 int32_t* stat_n, int32_t* stat_speed);

/* Particle slot counts of every (stream, scale) unit in one device read
 * (units ordered stream-major, scales ascending); waits for queued work. */
int gbt_read_counts(gbt_ctx* ctx, int32_t* counts, int32_t n);

/* The same read queued on the context stream (gbt_stream) after the frames
 * queued so far; returns at once.  `counts` is host memory (pinned, for the
 * copy to be asynchronous) that holds the values once the stream has reached
 * this point, so a caller can read frame t's counts while frame t + 1 runs. */
int gbt_read_counts_async(gbt_ctx* ctx, int32_t* counts, int32_t n);

/* Frame counter of (stream, scale) (generic_strategy::frame_cpt_). */
int gbt_frame_count(gbt_ctx* ctx, int32_t stream, int32_t scale, int32_t* n);

/* Device-side trajectories (the sample's per-particle position history,
 * samples/tracking/main.cc:39-57,125-127, kept in step with the particle slots
 * as particle_container::sync_attributes does, particle_container.hpp:514-553).
 * Once enabled, every frame appends each live particle's position (keeping the
 * last `history` <= 255), clears dead slots' histories, and moves histories to
 * their new slots when a compaction renumbers them; births start empty.  The
 * history buffers stay on the GPU: no per-frame copy of the particle vectors.
 * gbt_get_trajectories fills xy[n][history][2] (row, col; oldest first, zero
 * padded) and len[n] for the current slots; with xy and len NULL it only
 * returns n and history. */
int gbt_trajectories_enable(gbt_ctx* ctx, int32_t history);
int gbt_get_trajectories(gbt_ctx* ctx, int32_t stream, int32_t scale, int16_t* xy, uint8_t* len, int32_t* n,
                         int32_t* history);

/* Checkpoint / resume.  The carried state of every stream and scale (the
 * particle_container's particles, features, matches and counters,
 * particle_container.h:171-182; the frame counter, tracking_strategies.h:84-106;
 * the device-side trajectories) as one byte blob.  gbt_checkpoint_load accepts
 * only a blob saved from a context with the same stream configurations and
 * continues bit for bit where the saved context stood. */
int gbt_checkpoint_size(gbt_ctx* ctx, size_t* bytes);
int gbt_checkpoint_save(gbt_ctx* ctx, void* buf, size_t cap, size_t* written);
int gbt_checkpoint_load(gbt_ctx* ctx, const void* buf, size_t len);

/* Tuning knobs (results are identical for every setting; only speed
 * changes).  GBT_TUNE_MATCHER: 0 = particles binned by prediction into
 * 64 x 128 tiles, one CTA per tile matching from shared memory, 1 = one warp
 * per particle with the sweep candidates spread over its lanes, 2 = one thread
 * per particle with ring offsets computed from each level's pitch, 3 = one
 * thread per particle with compile-time ring offsets.  0 and 3 need every
 * stream to be at most 4064 pixels wide (fixed s1/s2 pitch) and fall back to 2
 * otherwise.
 * GBT_TUNE_BLUR_ROWS: height of the strip one warp walks in the BC2S blur.
 * GBT_TUNE_MATCH_TILE (matcher 0 only): 0 = 256 threads per tile CTA, each
 * taking every 256th particle of the tile; 1 / 2 / 3 = 128 / 64 / 256 threads
 * taking the tile's particles one at a time from a shared counter; 4 / 5 / 6 =
 * 128 / 256 / 192 threads likewise, with the tile staged with slim margins (14
 * rows and 16 columns instead of 26 and 32, so more CTAs fit on an SM; the few
 * particles whose descent would leave the staged area are matched again from
 * global memory); 7 = 160 threads likewise, compiled for six CTAs per SM (the
 * same 30 warps as 6 in smaller CTAs), the default.  The package's autotuner
 * (cuimg_gb300/autotune.py) times the settings on the caller's workload and
 * caches the winner. */
#define GBT_TUNE_MATCHER 0
#define GBT_TUNE_BLUR_ROWS 1   /* rows per warp strip of the BC2S blur: 16, 32 or 64 */
#define GBT_TUNE_MATCH_TILE 2  /* tiled matcher CTA shape and staged margins: 0..7 */
int gbt_set_tuning(gbt_ctx* ctx, int32_t knob, int32_t value);
int gbt_get_tuning(gbt_ctx* ctx, int32_t knob, int32_t* value);

/* Per-stage launch counters and device time of the last frame (for tests
 * and the benchmark): number of kernel launches issued per frame. */
int gbt_kernels_per_frame(gbt_ctx* ctx, int32_t* n);
/* Kernels this context has launched since gbt_create (frame-graph replays
 * count every kernel node they run). */
int gbt_kernel_launches(gbt_ctx* ctx, int64_t* total);

/* Per-kernel device-time accounting with CUDA events on the context stream
 * (eager launches; graph replays are not split).  gbt_profile_read returns
 * the number of entries and fills entry i: kernel name, accumulated
 * milliseconds and launch count. */
int gbt_profile_enable(gbt_ctx* ctx, int32_t enable);
int gbt_profile_read(gbt_ctx* ctx, int32_t i, char* name, size_t len, double* total_ms, int32_t* launches);

/* ------------------------------------------------------------------------
 * Separable fp32 Gaussian (meta_convolve_row2d + meta_convolve_col2d,
 * cuimg/gpu/meta_convolve.h:131-161,288-314; taps of
 * tools/make_meta_gaussian for integer sigma, cuimg/gaussian_kernel.h:13-18
 * otherwise; radius ceil(3 sigma); clamp-to-edge borders).
 * `in`/`out` are device pointers to rows x cols fp32 images with row pitch in
 * bytes; `stream` is a cudaStream_t (NULL = default stream).
 */
int gbt_gaussian_taps(float sigma, float* taps, int32_t* radius);
int gbt_gaussian_f32(const float* in, int64_t in_pitch, float* out, int64_t out_pitch, int32_t rows,
                     int32_t cols, float sigma, void* stream);

/* Same filter over `nimg` images of one size in one launch; image i starts
 * at byte offset i * in_img_bytes (in) and i * out_img_bytes (out). */
int gbt_gaussian_f32_batch(const float* in, int64_t in_pitch, int64_t in_img_bytes, float* out,
                           int64_t out_pitch, int64_t out_img_bytes, int32_t rows, int32_t cols,
                           int32_t nimg, float sigma, void* stream);

/* Gaussian pyramid option: sigma-1 blur then keep every second pixel
 * (the disabled pyramid of cuimg/gpu/mipmap.h:94-108,229-246), levels
 * 1..nlevels-1 written back to back (level l: floor(rows/2^l) x
 * floor(cols/2^l), dense rows) into `out`. */
int gbt_gaussian_pyramid_f32(const float* in, int64_t in_pitch, int32_t rows, int32_t cols,
                             int32_t nlevels, float* out, void* stream);

/* 2x2 floor-mean uint8 pyramid alone (subsample/mipmap_kernel,
 * cuimg/gpu/mipmap.h:24-49,206-227): levels 1..nlevels-1, dense rows, back
 * to back. */
int gbt_pyramid_u8(const uint8_t* in, int64_t in_pitch, int32_t rows, int32_t cols, int32_t nlevels,
                   uint8_t* out, void* stream);

/* ------------------------------------------------------------------------
 * Pyramidal Lucas-Kanade (iterative_lk_match_5x5::match,
 * cuimg/tracking2/pyrlk_tracker.hpp:165-334, with get_flow_at's coarse-to-fine
 * prediction :1027-1063 and pyrlk_match_particles_kernel's acceptance
 * :677-769).  The reference hard-codes window 11, 25 masked pixels, 30
 * iterations, step threshold 0.1 and error bound k = 300. */
typedef struct {
  int32_t window;    /* odd window size, 3..15 */
  int32_t npix;      /* strongest-gradient pixels used in the normal equations */
  int32_t max_iter;  /* Gauss-Newton iterations at most */
  float eps;         /* stop when the step norm falls below eps */
  float max_err;     /* accept when the mean residual is below max_err */
  int32_t warps_per_block;  /* CTA size of the tracking kernel (one warp per point): 2, 4 or 8;
                               0 = 8.  Speed only (the package's autotuner picks it). */
} gbt_lk_params;

void gbt_lk_params_default(gbt_lk_params* p);

/* Scratch bytes gbt_lk_track_batch uses for npairs rows x cols pairs. */
int64_t gbt_lk_scratch_bytes(int32_t rows, int32_t cols, int32_t nlevels, int32_t npairs);

/* Tracks npts points per pair through npairs frame pairs in one batch.
 * Device pointers: prev / cur hold npairs images (image p at byte offset
 * p * img_bytes, rows of `pitch` bytes), uint8 when is_u8 (2x2 floor-mean
 * pyramid, uint8 template: the reference's gl8u path) or fp32 otherwise
 * (sigma-1 Gaussian pyramid); pts / out are npairs * npts (row, col) pairs in
 * level-0 pixels, status is 1 when the track is accepted, err the matcher's
 * mean residual.  Allocates (and caches) its scratch arena on the current
 * device. */
int gbt_lk_track_batch(const void* prev, const void* cur, int64_t pitch, int64_t img_bytes, int32_t rows,
                       int32_t cols, int32_t is_u8, int32_t nlevels, const gbt_lk_params* params,
                       int32_t npairs, const float* pts, int32_t npts, float* out, int32_t* status,
                       float* err, void* stream);

/* ------------------------------------------------------------------------
 * Differentiable LK residual and its adjoint (new: the reference has no
 * gradients).  Forward per point: the translational LK of
 * iterative_lk_match_5x5 (cuimg/tracking2/pyrlk_tracker.hpp:165-334) made
 * differentiable -- sigma-1 Gaussian pyramids of both fp32 frames, Sobel/8
 * gradients, the full window, exactly `iters` Gauss-Newton steps per level,
 * coarse-to-fine from the initial flow u0 (level-0 pixels) -- and
 * loss = sum over the level-0 window of (I0-level(p + o) - I1-level(v + o))^2
 * at the final position v.  The backward pass recomputes the pyramids
 * (nothing is kept between the two calls) and returns the gradients of
 * sum_i dloss_i * loss_i with respect to I0, I1 (dense npairs x rows x cols)
 * and u0.  Image and point layouts as gbt_lk_track_batch (fp32 only). */
int64_t gbt_lkd_scratch_bytes(int32_t rows, int32_t cols, int32_t nlevels, int32_t npairs);
int gbt_lkd_forward(const float* I0, const float* I1, int64_t pitch, int64_t img_bytes, int32_t rows, int32_t cols,
                    int32_t nlevels, int32_t window, int32_t iters, int32_t npairs, const float* pts,
                    const float* u0, int32_t npts, float* loss, float* vfinal, void* stream);
int gbt_lkd_backward(const float* I0, const float* I1, int64_t pitch, int64_t img_bytes, int32_t rows,
                     int32_t cols, int32_t nlevels, int32_t window, int32_t iters, int32_t npairs,
                     const float* pts, const float* u0, int32_t npts, const float* dloss, float* dI0,
                     float* dI1, float* du0, void* stream);

/* The same pair with a tape (no counterpart in the reference): the forward
 * records, per point, every level's normal-matrix inverse and the iterates
 * with their right-hand sides (gbt_lkd_tape_bytes of device memory); the
 * backward given that tape reads them instead of replaying the forward.  The
 * tape belongs to the same images, points, u0 and configuration. */
int64_t gbt_lkd_tape_bytes(int32_t nlevels, int32_t iters, int32_t npairs, int32_t npts);
int gbt_lkd_forward_tape(const float* I0, const float* I1, int64_t pitch, int64_t img_bytes, int32_t rows,
                         int32_t cols, int32_t nlevels, int32_t window, int32_t iters, int32_t npairs,
                         const float* pts, const float* u0, int32_t npts, float* loss, float* vfinal, void* tape,
                         void* stream);
int gbt_lkd_backward_tape(const float* I0, const float* I1, int64_t pitch, int64_t img_bytes, int32_t rows,
                          int32_t cols, int32_t nlevels, int32_t window, int32_t iters, int32_t npairs,
                          const float* pts, const float* u0, int32_t npts, const float* dloss, float* dI0,
                          float* dI1, float* du0, const void* tape, void* stream);

/* Allocation-free variant of gbt_lk_track_batch (no counterpart in the
 * reference).  For callers that must not allocate device memory (their own
 * device pool or budget, a plugin that may not touch the CUDA heap): same
 * arguments and results, but the scratch lives in a fixed static device
 * array of gbt_lk_noalloc_max_bytes() bytes (48 MiB) that every GPU loading
 * this library holds until exit.  Requests needing more scratch than that
 * (gbt_lk_scratch_bytes) return GBT_E_TOO_LARGE.  The first call on a device
 * (and the first after its context is re-created by cudaDeviceReset) looks up
 * the array's address, so make it before any stream capture.  All calls share
 * the array and overwrite what it holds: calls queued one after another on one
 * stream are ordered and safe; calls whose GPU work overlaps race. */
int64_t gbt_lk_noalloc_max_bytes(void);
int gbt_lk_track_batch_noalloc(const void* prev, const void* cur, int64_t pitch, int64_t img_bytes, int32_t rows,
                               int32_t cols, int32_t is_u8, int32_t nlevels, const gbt_lk_params* params,
                               int32_t npairs, const float* pts, int32_t npts, float* out, int32_t* status,
                               float* err, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* CUIMG_GB300_H_ */
