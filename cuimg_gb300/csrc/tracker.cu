// Host side of the GB300 tracker: context, HBM layout, per-frame launch
// sequence (optionally replayed from CUDA graphs) and the C ABI declared in
// include/cuimg_gb300.h.
//
// One gbt_run advances every stream of the context by one frame, the batched
// equivalent of calling tracker<F>::run(frame) (cuimg/tracking2/tracker.hpp:72-91)
// on each stream: pyramid, then for all scales at once the BC2S blurs,
// matcher, flow statistics, detector/births/compaction on detector frames, and
// filter/merge on filtering frames.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cuimg_gb300.h"
#include "pyrlk.h"
#include "tracker_kernels.cuh"

using namespace gbt;

namespace {

inline int round_up(int v, int m) { return (v + m - 1) / m * m; }

struct StreamInfo {
  gbt_config cfg;
  int unit0;
  uint8_t* pinned;  // staging buffer for pageable host frames
  size_t pinned_bytes;
  uint8_t* d_rgb = nullptr;  // device RGB frame, allocated on the first RGB input
  int64_t rgb_pitch = 0;
};

}  // namespace

struct Group {
  int device = 0;
  int nsm = 0;
  cudaStream_t stream = nullptr;
  // Frame pipeline.  The front end of a frame (its input copy, the pyramid
  // and the blurs) runs on `pre` into the image buffers of the frame's parity
  // while the back end of the previous frame (matcher to tick) still runs on
  // `stream` over the other parity's images.  The back end waits for its
  // front end (ev_front); a front end waits for the back end that last read
  // its parity's images (ev_back).  With per-kernel timing on, both run on
  // `stream`.
  cudaStream_t pre = nullptr;
  cudaEvent_t ev_front = nullptr;
  cudaEvent_t ev_back[2] = {nullptr, nullptr};
  Unit* d_units_v[2] = {nullptr, nullptr};  // unit tables whose images are the parity-0 / parity-1 buffers
  std::vector<Unit> units_odd;           // host copy of the parity-1 table
  std::vector<StreamInfo> streams;
  std::vector<Unit> units;
  Unit* d_units = nullptr;
  UState* d_state = nullptr;
  Frame* d_frame = nullptr;
  int* d_counts = nullptr;  // gbt_read_counts_async staging
  int host_frame = 0;
  // static work tables (device)
  int* d_stream_unit0 = nullptr;
  int* d_pyr_prefix[2] = {nullptr, nullptr};
  int pyr_tiles[2] = {0, 0};
  int* d_blur_prefix = nullptr;  // for blur_rows
  int blur_tiles = 0;
  int* d_blur_prefix_v[3] = {nullptr, nullptr, nullptr};  // strips of 16, 32, 64 rows
  int blur_tiles_v[3] = {0, 0, 0};
  int blur_rows = BL_SR;
  int* d_bin_prefix = nullptr;
  int* d_cap_table = nullptr;  // particle-capacity chunks per unit (trajectories)
  Ingest* d_ingest = nullptr;   // per stream: how k_pyramid gets level 0
  // Pinned host tables for d_ingest, INGEST_RING of them: a changed table is
  // written into the next one, whose upload to d_ingest has completed (its
  // event), so that per-frame source pointers need no host synchronisation.
  Ingest* h_ingest_ring = nullptr;
  Ingest* h_ingest = nullptr;   // the table being edited / last uploaded
  int ingest_slot = 0;
  cudaEvent_t ingest_ev[4] = {};
  bool ingest_dirty = true;
  int rgb_mode = GBT_RGB_CHANNEL0;
  int traj_T = 0;              // trajectory history length, 0 = off
  int nbins = 0;
  int* d_det_prefix = nullptr;
  int det_blocks = 0;
  int* d_btable = nullptr;
  // dynamic chunk tables
  int* d_pre = nullptr;
  // tiled matcher: tiles over all units, per-tile counts (then the overflow count), tile lists
  int mt_tiles = 0;
  long long mt_list_cap = 0;  // particle slots of all units: the overflow list never needs more
  int* d_mt_prefix = nullptr;
  int* d_mt_cnt = nullptr;
  unsigned long long* d_mt_fallback = nullptr;  // particles the slim-margin tiled matcher finished from global memory
  int* d_mt_list = nullptr;  // mt_tiles lists of MT_LIST_CAP slots (k_mt_list)
  int2* d_mt_ovf = nullptr;  // (unit, slot) of the particles beyond a tile's list capacity
  int mt_cap = MT_LIST_CAP;  // list capacity in use (test hook: smaller, to force the overflow path)
  int* d_post = nullptr;
  // bulk buffers cleared per frame
  void* occ_all = nullptr;
  size_t occ_bytes = 0;
  void* pmask_all = nullptr;
  void* ppos_all = nullptr;
  size_t pmask_bytes = 0;
  std::vector<void*> allocs;
  // graphs: back ends keyed by (any detector unit, any filtering unit,
  // parity), front ends by parity
  bool use_graphs = false;
  cudaGraphExec_t graph[8] = {};
  cudaGraphExec_t front_graph[2] = {nullptr, nullptr};
  int launches_per_frame = 0;   // kernels of the last frame enqueued (memsets not counted)
  int graph_launches[8] = {};   // kernels in each captured back-end graph
  int front_launches = 0;       // kernels in a captured front-end graph
  long long kernels_total = 0;  // kernels launched by this context, graph nodes included
  int match_variant = 0;  // GBT_TUNE_MATCHER
  int mt_shape = 7;       // GBT_TUNE_MATCH_TILE: tiled matcher threads, particle assignment and margins
  int withhold_tiles = 0; // test hook: the tiled matcher's tile copies are not issued
  int fm_grid = 0;        // k_filter_merge CTAs: the ones all SMs hold at once
  // TMA descriptors of every unit's s1 and s2 for the tiled matcher, parity 0
  // then 1 (null when the driver cannot encode them: the matcher then stages
  // its tiles with cp.async)
  CUtensorMap* d_tmaps = nullptr;
  bool fixed_fpitch = true;  // every unit's s1/s2 pitch is FIXED_FPITCH
  bool any_alt_detector = false;  // a stream uses the regular or the dense detector
  std::string err;
  // scratch for stage dumps
  void* dump_buf = nullptr;
  size_t dump_bytes = 0;
  // per-kernel event timing (eager launches only)
  bool profiling = false;
  struct Prof {
    std::string name;
    double ms = 0;
    int launches = 0;
  };
  std::vector<Prof> prof;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  std::vector<cudaEvent_t> event_pool;
  size_t event_next = 0;
};

static int set_err(Group* c, int code, const char* fmt, ...) {
  if (c) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    c->err = buf;
  }
  return code;
}

#define CK(call)                                                                                 \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess)                                                                       \
      return set_err(ctx, GBT_E_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                     __FILE__, __LINE__);                                                        \
  } while (0)

static int dalloc(Group* ctx, void** p, size_t bytes, bool zero) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) return set_err(ctx, GBT_E_OOM, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
  ctx->allocs.push_back(*p);
  if (zero) CK(cudaMemset(*p, 0, bytes));
  return GBT_OK;
}

template <typename T>
static int dalloc_t(Group* ctx, T** p, size_t n, bool zero = true) {
  return dalloc(ctx, (void**)p, n * sizeof(T), zero);
}

static int upload_table(Group* ctx, int** d, const std::vector<int>& h) {
  int r = dalloc_t(ctx, d, h.size(), false);
  if (r) return r;
  CK(cudaMemcpy(*d, h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice));
  return GBT_OK;
}

extern "C" void gbt_config_default(gbt_config* cfg, int32_t rows, int32_t cols, int32_t nscales) {
  cfg->rows = rows;
  cfg->cols = cols;
  cfg->nscales = nscales;
  cfg->detector_threshold = 20;
  cfg->detector_n = 9;
  cfg->detector_frequency = 1;   // generic_strategy defaults (tracking_strategies.hpp:45-48)
  cfg->filtering_frequency = 1;
  cfg->k = 300;
  cfg->with_merge = 1;
  cfg->detector = GBT_DETECTOR_FAST;
  cfg->detector_step = 1;   // regular_detector defaults (regular_detector.hpp:12-17)
  cfg->detector_grad_th = 1;
  cfg->matcher = GBT_MATCHER_BC2S;
}

extern "C" int gbt_sizes_ok(int32_t rows, int32_t cols, int32_t nscales) {
  if (nscales < 1 || nscales > 9 || rows > 32767 || cols > 32767) return 0;
  int H = rows, W = cols;
  for (int s = 0; s < nscales; s++) {
    if (H < 16 || W < 16) return 0;
    if (s + 1 < nscales) {
      int bh = (H + 7) / 8, bw = (W + 7) / 8, ubh = (H / 2 + 7) / 8, ubw = (W / 2 + 7) / 8;
      if ((bh - 1) / 2 >= ubh || (bw - 1) / 2 >= ubw) return 0;
    }
    H /= 2;
    W /= 2;
  }
  return 1;
}

static void free_ctx(Group* ctx) {
  if (!ctx) return;
  if (ctx->device >= 0) cudaSetDevice(ctx->device);
  for (auto e : ctx->event_pool) cudaEventDestroy(e);
  for (auto& g : ctx->graph)
    if (g) cudaGraphExecDestroy(g);
  for (auto& g : ctx->front_graph)
    if (g) cudaGraphExecDestroy(g);
  for (void* p : ctx->allocs) cudaFree(p);
  for (auto& s : ctx->streams)
    if (s.pinned) cudaFreeHost(s.pinned);
  if (ctx->h_ingest_ring) cudaFreeHost(ctx->h_ingest_ring);
  for (cudaEvent_t e : ctx->ingest_ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : {ctx->ev_front, ctx->ev_back[0], ctx->ev_back[1]})
    if (e) cudaEventDestroy(e);
  if (ctx->pre) cudaStreamDestroy(ctx->pre);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

// Unit `ui` with the image buffers of frame parity `par`.
static Unit unit_view(const Group* ctx, size_t ui, int par) {
  Unit u = ctx->units[ui];
  if (par) {
    const Unit& o = ctx->units_odd[ui];
    u.img = o.img;
    u.s1 = o.s1;
    u.s2 = o.s2;
  }
  return u;
}

// Uploads both parities' unit tables after a change of ctx->units.
static int upload_units(Group* ctx) {
  const size_t n = ctx->units.size();
  std::vector<Unit> v(n);
  for (int par = 0; par < 2; par++) {
    for (size_t i = 0; i < n; i++) v[i] = unit_view(ctx, i, par);
    CK(cudaMemcpy(ctx->d_units_v[par], v.data(), n * sizeof(Unit), cudaMemcpyHostToDevice));
  }
  return GBT_OK;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (the
// library does not link the driver API).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// 2-D uint8 maps over the bordered s1 / s2 (FIXED_FPITCH bytes by H + 2 RB
// rows, row stride FIXED_FPITCH) with the matcher's staged boxes: the full
// margins' (MT_SC bytes by MT_SR rows) at d_tmaps[((0 * 2 + par) * nunits +
// unit) * 2 + image], the slim margins' after them (geometry 1).  Leaves
// d_tmaps null when the entry point or an encoding is unavailable.
static int encode_tile_maps(Group* ctx) {
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn) {
    cudaGetLastError();
    return GBT_OK;
  }
  const EncodeTiledFn encode = (EncodeTiledFn)fn;
  const size_t nunits = ctx->units.size();
  std::vector<CUtensorMap> maps(2 * 2 * nunits * 2);
  for (int geom = 0; geom < 2; geom++)
    for (int par = 0; par < 2; par++)
      for (size_t ui = 0; ui < nunits; ui++) {
        const Unit v = unit_view(ctx, ui, par);
        const cuuint64_t dims[2] = {(cuuint64_t)FIXED_FPITCH, (cuuint64_t)(v.H + 2 * RB)};
        const cuuint64_t strides[1] = {(cuuint64_t)FIXED_FPITCH};
        const cuuint32_t box[2] = {(cuuint32_t)(geom ? MT_C + 2 * MT_MC_SLIM : MT_SC),
                                   (cuuint32_t)(geom ? MT_R + 2 * MT_MR_SLIM : MT_SR)};
        const cuuint32_t estr[2] = {1, 1};
        uint8_t* img[2] = {v.s1, v.s2};
        for (int k = 0; k < 2; k++)
          if (encode(&maps[((geom * 2 + par) * nunits + ui) * 2 + k], CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, img[k], dims,
                     strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return GBT_OK;
      }
  int r;
  if ((r = dalloc_t(ctx, &ctx->d_tmaps, maps.size(), false))) return r;
  CK(cudaMemcpy(ctx->d_tmaps, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice));
  return GBT_OK;
}

static bool split_front(const Group* ctx) { return !ctx->profiling; }
static cudaStream_t front_stream(const Group* ctx) { return split_front(ctx) ? ctx->pre : ctx->stream; }

// Orders the next frame's input writes after the back end that last read the
// images of its parity.
static int prepare_front(Group* ctx) {
  if (split_front(ctx)) CK(cudaStreamWaitEvent(ctx->pre, ctx->ev_back[ctx->host_frame & 1], 0));
  return GBT_OK;
}

static int sync_all(Group* ctx) {
  CK(cudaStreamSynchronize(ctx->pre));
  CK(cudaStreamSynchronize(ctx->stream));
  return GBT_OK;
}

static int build(Group* ctx, const gbt_config* cfgs, int nstreams) {
  CK(cudaSetDevice(ctx->device));
  CK(cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, ctx->device));
  {
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_filter_merge, FM_THREADS, 0));
    ctx->fm_grid = ctx->nsm * std::max(1, per_sm);
  }
  {
    // The back end carries the frame-to-frame dependency, so its blocks are
    // dispatched first; the front end (next frame's pyramid and blurs) fills
    // the SMs the back end leaves idle.  Graph launches take their stream's
    // priority.
    int least = 0, greatest = 0;
    CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    CK(cudaStreamCreateWithPriority(&ctx->stream, cudaStreamNonBlocking, greatest));
    CK(cudaStreamCreateWithPriority(&ctx->pre, cudaStreamNonBlocking, least));
  }
  for (cudaEvent_t* e : {&ctx->ev_front, &ctx->ev_back[0], &ctx->ev_back[1]})
    CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  // Units: streams in order, scales 0..L-1 of each stream contiguous.
  size_t occ_words = 0;
  for (int s = 0; s < nstreams; s++) {
    StreamInfo si{};
    si.cfg = cfgs[s];
    si.unit0 = (int)ctx->units.size();
    const gbt_config& c = cfgs[s];
    int H = c.rows, W = c.cols;
    for (int l = 0; l < c.nscales; l++) {
      Unit u{};
      u.H = H;
      u.W = W;
      u.stream = s;
      u.scale = l;
      u.nscales = c.nscales;
      u.upper = l + 1 < c.nscales ? si.unit0 + l + 1 : -1;
      u.threshold = c.detector_threshold;
      u.nfast = c.detector_n;
      u.k = c.k;
      u.det_freq = c.detector_frequency;
      u.filt_freq = c.filtering_frequency;
      u.with_merge = c.with_merge;
      u.det_kind = c.detector;
      u.det_step = c.detector_step;
      u.det_grad_th = c.detector_grad_th;
      u.BH = (H + 7) / 8;
      u.BW = (W + 7) / 8;
      u.TH = H / 3;
      u.TW = W / 3;
      occ_words += (size_t)u.BH * u.BW;
      ctx->units.push_back(u);
      H /= 2;
      W /= 2;
    }
    ctx->streams.push_back(si);
  }
  const int nunits = (int)ctx->units.size();
  ctx->occ_bytes = occ_words * 8;
  ctx->pmask_bytes = occ_words * 8;
  int r;
  if ((r = dalloc(ctx, &ctx->occ_all, ctx->occ_bytes, true))) return r;
  if ((r = dalloc(ctx, &ctx->pmask_all, ctx->pmask_bytes, true))) return r;
  if ((r = dalloc(ctx, &ctx->ppos_all, ctx->pmask_bytes, true))) return r;
  size_t woff = 0;
  for (auto& u : ctx->units) {
    size_t nb = (size_t)u.BH * u.BW;
    u.occ = (unsigned long long*)ctx->occ_all + woff;
    u.pmask = (unsigned long long*)ctx->pmask_all + woff;
    u.ppos = (unsigned long long*)ctx->ppos_all + woff;
    woff += nb;
    u.ipitch = round_up(u.W, 64);
    if ((r = dalloc(ctx, (void**)&u.img, (size_t)u.ipitch * u.H, true))) return r;
    u.fpitch = u.W + 2 * CB <= FIXED_FPITCH ? FIXED_FPITCH : round_up(u.W + 2 * CB, 64);
    if (u.fpitch != FIXED_FPITCH) ctx->fixed_fpitch = false;
    if ((r = dalloc(ctx, (void**)&u.s1, (size_t)u.fpitch * (u.H + 2 * RB), true))) return r;
    if ((r = dalloc(ctx, (void**)&u.s2, (size_t)u.fpitch * (u.H + 2 * RB), true))) return r;
    Unit o{};  // parity-1 images (zeroed like the parity-0 ones: the s1/s2 borders stay zero)
    if ((r = dalloc(ctx, (void**)&o.img, (size_t)u.ipitch * u.H, true))) return r;
    if ((r = dalloc(ctx, (void**)&o.s1, (size_t)u.fpitch * (u.H + 2 * RB), true))) return r;
    if ((r = dalloc(ctx, (void**)&o.s2, (size_t)u.fpitch * (u.H + 2 * RB), true))) return r;
    ctx->units_odd.push_back(o);
    if ((r = dalloc_t(ctx, &u.idx, (size_t)u.H * u.W))) return r;
    if ((r = dalloc_t(ctx, &u.st_n, nb))) return r;
    if ((r = dalloc_t(ctx, &u.st_sp, nb))) return r;
    if ((r = dalloc_t(ctx, &u.flow, nb))) return r;
    if ((r = dalloc_t(ctx, &u.msc, nb))) return r;
    if (u.det_kind == GBT_DETECTOR_FAST) {
      u.max_births = u.TH * u.TW;
      u.birth_items = 3 * u.TH * u.TW;
      u.cap = u.H * u.W / 6 + 4096;
    } else {
      u.max_births = u.det_kind == GBT_DETECTOR_DENSE
                         ? u.H * u.W
                         : ((u.H + u.det_step - 1) / u.det_step) * ((u.W + u.det_step - 1) / u.det_step);
      u.birth_items = u.H * u.W;
      u.cap = 4 * u.max_births + 4096;  // both detectors add particles where some already are
    }
    if (u.det_kind != GBT_DETECTOR_FAST) ctx->any_alt_detector = true;
    u.cap = round_up(u.cap, CHUNK);
    u.max_chunks = u.cap / CHUNK;
    u.MTR = (u.H + MT_R - 1) / MT_R;
    u.MTC = (u.W + MT_C - 1) / MT_C;
    u.mt_base = ctx->mt_tiles;
    ctx->mt_tiles += u.MTR * u.MTC;
    ctx->mt_list_cap += u.cap;
    for (int b = 0; b < 2; b++) {
      if ((r = dalloc_t(ctx, &u.pos[b], u.cap))) return r;
      if ((r = dalloc_t(ctx, &u.spd[b], u.cap))) return r;
      if ((r = dalloc_t(ctx, &u.age[b], u.cap))) return r;
      if ((r = dalloc_t(ctx, &u.feat[b], u.cap))) return r;
    }
    if ((r = dalloc_t(ctx, &u.matches, (size_t)u.cap + (size_t)u.max_births))) return r;
    if ((r = dalloc_t(ctx, &u.chunk_cnt, (size_t)u.cap / 32 + 1))) return r;
    if ((r = dalloc_t(ctx, &u.tilecode, (size_t)u.TH * u.TW + 1))) return r;
    u.birth_chunks = (u.birth_items + CHUNK - 1) / CHUNK;
    if ((r = dalloc_t(ctx, &u.birth_cnt, (size_t)u.birth_items / 32 + 2))) return r;
    if ((r = dalloc_t(ctx, &u.act_cnt, (size_t)u.cap / 32 + 1))) return r;
    if ((r = dalloc_t(ctx, &u.cmask, u.cap))) return r;
    if ((r = dalloc_t(ctx, &u.act_list, u.cap))) return r;
    if ((r = dalloc_t(ctx, &u.act_cand, (size_t)u.cap * 8, false))) return r;
  }
  if ((r = dalloc_t(ctx, &ctx->d_units_v[0], nunits, false))) return r;
  if ((r = dalloc_t(ctx, &ctx->d_units_v[1], nunits, false))) return r;
  ctx->d_units = ctx->d_units_v[0];
  if ((r = upload_units(ctx))) return r;
  if (ctx->fixed_fpitch && (r = encode_tile_maps(ctx))) return r;
  if ((r = dalloc_t(ctx, &ctx->d_state, nunits))) return r;
  if ((r = dalloc_t(ctx, &ctx->d_frame, 1))) return r;
  if ((r = dalloc_t(ctx, &ctx->d_counts, nunits))) return r;
  if ((r = dalloc_t(ctx, &ctx->d_pre, nunits + 1))) return r;
  if ((r = dalloc_t(ctx, &ctx->d_mt_cnt, ctx->mt_tiles + 1))) return r;
  if ((r = dalloc_t(ctx, &ctx->d_mt_fallback, 1))) return r;
  if ((r = dalloc_t(ctx, &ctx->d_mt_list, (size_t)ctx->mt_tiles * MT_LIST_CAP, false))) return r;
  if ((r = dalloc_t(ctx, &ctx->d_mt_ovf, ctx->mt_list_cap, false))) return r;
  if ((r = dalloc_t(ctx, &ctx->d_post, nunits + 1))) return r;

  // Static tables.
  std::vector<int> su0, pyr0(1, 0), pyr1(1, 0);
  for (auto& s : ctx->streams) {
    su0.push_back(s.unit0);
    const Unit& b0 = ctx->units[s.unit0];
    pyr0.push_back(pyr0.back() + ((b0.H + PYR_TR - 1) / PYR_TR) * ((b0.W + PYR_TC - 1) / PYR_TC));
    int t1 = 0;
    if (s.cfg.nscales > 6) {
      const Unit& b5 = ctx->units[s.unit0 + 5];
      t1 = ((b5.H + PYR_TR - 1) / PYR_TR) * ((b5.W + PYR_TC - 1) / PYR_TC);
    }
    pyr1.push_back(pyr1.back() + t1);
  }
  ctx->pyr_tiles[0] = pyr0.back();
  ctx->pyr_tiles[1] = pyr1.back();
  std::vector<int> bins(1, 0), det(1, 0), bt(1, 0);
  for (int v = 0; v < 3; v++) {
    const int sr = 16 << v;
    std::vector<int> blur(1, 0);
    for (auto& u : ctx->units) blur.push_back(blur.back() + ((u.H + sr - 1) / sr) * ((u.W + BL_OC - 1) / BL_OC));
    ctx->blur_tiles_v[v] = blur.back();
    if ((r = upload_table(ctx, &ctx->d_blur_prefix_v[v], blur))) return r;
  }
  ctx->d_blur_prefix = ctx->d_blur_prefix_v[2];
  ctx->blur_tiles = ctx->blur_tiles_v[2];
  for (auto& u : ctx->units) {
    bins.push_back(bins.back() + u.BH * u.BW);
    det.push_back(det.back() + ((u.TH + DT_R - 1) / DT_R) * ((u.TW + DT_C - 1) / DT_C));
    bt.push_back(bt.back() + u.birth_chunks);
  }
  ctx->nbins = bins.back();
  ctx->det_blocks = det.back();
  if ((r = upload_table(ctx, &ctx->d_stream_unit0, su0))) return r;
  if ((r = upload_table(ctx, &ctx->d_pyr_prefix[0], pyr0))) return r;
  if ((r = upload_table(ctx, &ctx->d_pyr_prefix[1], pyr1))) return r;
  if ((r = upload_table(ctx, &ctx->d_bin_prefix, bins))) return r;
  if ((r = upload_table(ctx, &ctx->d_det_prefix, det))) return r;
  if ((r = upload_table(ctx, &ctx->d_btable, bt))) return r;
  {
    std::vector<int> capt(1, 0);
    for (auto& u : ctx->units) capt.push_back(capt.back() + u.max_chunks);
    if ((r = upload_table(ctx, &ctx->d_cap_table, capt))) return r;
  }
  {
    std::vector<int> mt;
    for (auto& u : ctx->units) mt.push_back(u.mt_base);
    mt.push_back(ctx->mt_tiles);
    if ((r = upload_table(ctx, &ctx->d_mt_prefix, mt))) return r;
  }
  for (auto& s : ctx->streams) {
    const Unit& u = ctx->units[s.unit0];
    s.pinned_bytes = (size_t)u.H * u.W * 3;
    CK(cudaMallocHost((void**)&s.pinned, s.pinned_bytes));
  }
  if ((r = dalloc_t(ctx, &ctx->d_ingest, nstreams))) return r;
  CK(cudaMallocHost((void**)&ctx->h_ingest_ring, sizeof(Ingest) * nstreams * 4));
  memset(ctx->h_ingest_ring, 0, sizeof(Ingest) * nstreams * 4);
  ctx->h_ingest = ctx->h_ingest_ring;
  for (cudaEvent_t& e : ctx->ingest_ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  CK(cudaDeviceSynchronize());
  return GBT_OK;
}

static int grp_create(const gbt_config* cfgs, int32_t nstreams, int32_t device, Group** out) {
  if (!out) return GBT_E_INVALID;
  *out = nullptr;
  if (!cfgs || nstreams < 1) return GBT_E_INVALID;
  for (int s = 0; s < nstreams; s++) {
    const gbt_config& c = cfgs[s];
    if (!gbt_sizes_ok(c.rows, c.cols, c.nscales) || c.detector_frequency < 1 || c.filtering_frequency < 1 ||
        c.detector_n < 1 || c.detector_n > 16 || c.detector_threshold < 0 || c.detector < GBT_DETECTOR_FAST ||
        c.detector > GBT_DETECTOR_DENSE || c.detector_step < 1)
      return GBT_E_INVALID;
  }
  Group* ctx = new Group;
  ctx->device = device;
  int r = build(ctx, cfgs, nstreams);
  if (r) {
    fprintf(stderr, "gbt_create: %s\n", ctx->err.c_str());
    free_ctx(ctx);
    return r;
  }
  *out = ctx;
  return GBT_OK;
}

static int grp_destroy(Group* ctx) {
  if (!ctx) return GBT_E_INVALID;
  cudaSetDevice(ctx->device);
  if (ctx->pre) cudaStreamSynchronize(ctx->pre);
  cudaStreamSynchronize(ctx->stream);
  free_ctx(ctx);
  return GBT_OK;
}

static int grp_input_slot(Group* ctx, int32_t stream, uint8_t** dptr, int64_t* pitch) {
  if (!ctx || stream < 0 || stream >= (int)ctx->streams.size()) return GBT_E_INVALID;
  const Unit u = unit_view(ctx, ctx->streams[stream].unit0, ctx->host_frame & 1);  // the next frame's slot
  if (dptr) *dptr = u.img;
  if (pitch) *pitch = u.ipitch;
  return GBT_OK;
}

// Frame kind of the frame about to run (per unit: gbt_set_param may give the
// scales of a stream different frequencies, as the reference's per-scale
// setters can).
static void frame_kind(Group* ctx, bool& any_det, bool& any_filt) {
  any_det = any_filt = false;
  for (const Unit& u : ctx->units) {
    if (ctx->host_frame % u.det_freq == 0) any_det = true;
    if (ctx->host_frame % u.filt_freq == 0) any_filt = true;
  }
}

// The unit field a gbt_set_param key addresses, with its accepted range.
static int* param_field(Unit& u, int key, int& lo, int& hi) {
  lo = 0;
  hi = 1 << 30;
  switch (key) {
    case GBT_PARAM_DETECTOR_THRESHOLD: return &u.threshold;
    case GBT_PARAM_DETECTOR_N: lo = 1; hi = 16; return &u.nfast;
    case GBT_PARAM_DETECTOR_FREQUENCY: lo = 1; return &u.det_freq;
    case GBT_PARAM_FILTERING_FREQUENCY: lo = 1; return &u.filt_freq;
    case GBT_PARAM_K: return &u.k;
    case GBT_PARAM_WITH_MERGE: hi = 1; return &u.with_merge;
    case GBT_PARAM_DETECTOR_GRAD_TH: return &u.det_grad_th;
    default: return nullptr;
  }
}

static int* config_field(gbt_config& c, int key) {
  switch (key) {
    case GBT_PARAM_DETECTOR_THRESHOLD: return &c.detector_threshold;
    case GBT_PARAM_DETECTOR_N: return &c.detector_n;
    case GBT_PARAM_DETECTOR_FREQUENCY: return &c.detector_frequency;
    case GBT_PARAM_FILTERING_FREQUENCY: return &c.filtering_frequency;
    case GBT_PARAM_K: return &c.k;
    case GBT_PARAM_WITH_MERGE: return &c.with_merge;
    case GBT_PARAM_DETECTOR_GRAD_TH: return &c.detector_grad_th;
    default: return nullptr;
  }
}

// Waits for the group's queued work, changes the parameter of the stream's
// scale (every scale when scale is -1, which also updates the stream's
// configuration) and re-uploads the unit tables; frames run from then on use
// the new value.
static int grp_set_param(Group* ctx, int32_t stream, int32_t scale, int32_t key, int32_t value) {
  if (!ctx || stream < 0 || stream >= (int)ctx->streams.size()) return GBT_E_INVALID;
  StreamInfo& si = ctx->streams[stream];
  if (scale < -1 || scale >= si.cfg.nscales) return GBT_E_INVALID;
  int lo, hi;
  if (!param_field(ctx->units[si.unit0], key, lo, hi)) return set_err(ctx, GBT_E_INVALID, "unknown parameter %d", key);
  if (value < lo || value > hi) return set_err(ctx, GBT_E_INVALID, "parameter %d out of range: %d", key, value);
  CK(cudaSetDevice(ctx->device));
  int r = sync_all(ctx);
  if (r) return r;
  const int l0 = scale < 0 ? 0 : scale, l1 = scale < 0 ? si.cfg.nscales : scale + 1;
  for (int l = l0; l < l1; l++) *param_field(ctx->units[si.unit0 + l], key, lo, hi) = value;
  if (scale < 0) *config_field(si.cfg, key) = value;
  return upload_units(ctx);
}

static int grp_get_param(Group* ctx, int32_t stream, int32_t scale, int32_t key, int32_t* value) {
  if (!ctx || !value || stream < 0 || stream >= (int)ctx->streams.size()) return GBT_E_INVALID;
  const StreamInfo& si = ctx->streams[stream];
  if (scale < 0 || scale >= si.cfg.nscales) return GBT_E_INVALID;
  int lo, hi;
  const int* f = param_field(ctx->units[si.unit0 + scale], key, lo, hi);
  if (!f) return GBT_E_INVALID;
  *value = *f;
  return GBT_OK;
}

// An event from the profiling pool, or null when none could be created (the
// launch is then not timed).
static cudaEvent_t next_event(Group* ctx) {
  if (ctx->event_next == ctx->event_pool.size()) {
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    ctx->event_pool.push_back(e);
  }
  return ctx->event_pool[ctx->event_next++];
}

static int prof_slot(Group* ctx, const char* name) {
  for (size_t i = 0; i < ctx->prof.size(); i++)
    if (ctx->prof[i].name == name) return (int)i;
  Group::Prof p;
  p.name = name;
  ctx->prof.push_back(p);
  return (int)ctx->prof.size() - 1;
}

// Brackets one launch with events when profiling (never inside a capture).
struct ProfScope {
  Group* ctx;
  int slot = -1;
  cudaEvent_t a = nullptr;
  ProfScope(Group* c, const char* name) : ctx(c) {
    if (!ctx->profiling) return;
    a = next_event(ctx);
    if (!a) return;
    slot = prof_slot(ctx, name);
    cudaEventRecord(a, ctx->stream);
  }
  ~ProfScope() {
    if (slot < 0) return;
    cudaEvent_t b = next_event(ctx);
    if (!b) return;
    cudaEventRecord(b, ctx->stream);
    ctx->pending.push_back({slot, {a, b}});
  }
};

static void prof_collect(Group* ctx) {
  if (ctx->pending.empty()) return;
  cudaStreamSynchronize(ctx->stream);
  for (auto& p : ctx->pending) {
    float ms = 0;
    cudaEventElapsedTime(&ms, p.second.first, p.second.second);
    ctx->prof[p.first].ms += ms;
    ctx->prof[p.first].launches++;
  }
  ctx->pending.clear();
  ctx->event_next = 0;
}

#define PROF(name) ProfScope prof_scope_##__LINE__(ctx, name)

// Front end of a frame on `st`: the pyramid (with the fused RGB ingest) and
// the BC2S blurs, into the image buffers of parity `par`.
static int enqueue_front(Group* ctx, int par, cudaStream_t st, int& n) {
  const int nunits = (int)ctx->units.size();
  const int nstreams = (int)ctx->streams.size();
  const Unit* du = ctx->d_units_v[par];
  n = 0;
  { PROF("k_pyramid"); k_pyramid<<<ctx->pyr_tiles[0], PYR_THREADS, 0, st>>>(du, ctx->d_stream_unit0, ctx->d_pyr_prefix[0], nstreams, 0, ctx->d_ingest); }
  n++;
  if (ctx->pyr_tiles[1] > 0) {
    PROF("k_pyramid5");
    k_pyramid<<<ctx->pyr_tiles[1], PYR_THREADS, 0, st>>>(du, ctx->d_stream_unit0, ctx->d_pyr_prefix[1], nstreams, 5, ctx->d_ingest);
    n++;
  }
  {
    PROF("k_blur");
    const int nb = (ctx->blur_tiles + BL_WARPS - 1) / BL_WARPS;
    if (ctx->blur_rows == 16)
      k_blur<16><<<nb, 32 * BL_WARPS, 0, st>>>(du, ctx->d_blur_prefix, nunits);
    else if (ctx->blur_rows == 32)
      k_blur<32><<<nb, 32 * BL_WARPS, 0, st>>>(du, ctx->d_blur_prefix, nunits);
    else
      k_blur<64><<<nb, 32 * BL_WARPS, 0, st>>>(du, ctx->d_blur_prefix, nunits);
    n++;
  }
  CK(cudaGetLastError());
  return GBT_OK;
}

// Back end of a frame on the context stream: matching, flow statistics,
// detection, filtering, merging, trajectories and the frame tick, over the
// images of parity `par`.
static int enqueue_back(Group* ctx, bool any_det, bool any_filt, int par, int& n) {
  const int nunits = (int)ctx->units.size();
  const int pgrid = std::max(1, ctx->nsm * 2);
  const Unit* du = ctx->d_units_v[par];
  cudaStream_t st = ctx->stream;
  n = 0;
  CK(cudaMemsetAsync(ctx->occ_all, 0, ctx->occ_bytes, st));
  if (ctx->match_variant == 0 && ctx->fixed_fpitch) {
    CK(cudaMemsetAsync(ctx->d_mt_cnt, 0, (size_t)(ctx->mt_tiles + 1) * sizeof(int), st));  // + the overflow count
    {
      PROF("k_mt_list");
      k_mt_list<<<pgrid, CHUNK, 0, st>>>(du, ctx->d_state, ctx->d_pre, nunits, ctx->d_mt_cnt, ctx->mt_tiles,
                                         ctx->mt_cap, ctx->d_mt_list, ctx->d_mt_ovf);
    }
    const bool slim = ctx->mt_shape >= 4;
    const CUtensorMap* tm = ctx->d_tmaps ? ctx->d_tmaps + ((size_t)(slim ? 2 : 0) + par) * nunits * 2 : nullptr;
    int* err = &ctx->d_frame->err;
    unsigned long long* fb = ctx->d_mt_fallback;
#define GBT_MT_ARGS du, ctx->d_state, ctx->d_frame, ctx->d_mt_prefix, nunits, ctx->d_mt_cnt, ctx->mt_cap, ctx->d_mt_list, tm, err, ctx->withhold_tiles, fb
    constexpr int FR = MT_MR, FC = MT_MC, SR_ = MT_MR_SLIM, SC_ = MT_MC_SLIM;
    {
    PROF("k_match_tiled");
    switch (ctx->mt_shape) {
      case 1: k_match_tiled<128, true, 8, FR, FC><<<ctx->mt_tiles, 128, 0, st>>>(GBT_MT_ARGS); break;
      case 2: k_match_tiled<64, true, 10, FR, FC><<<ctx->mt_tiles, 64, 0, st>>>(GBT_MT_ARGS); break;
      case 3: k_match_tiled<256, true, 4, FR, FC><<<ctx->mt_tiles, 256, 0, st>>>(GBT_MT_ARGS); break;
      case 4: k_match_tiled<128, true, 7, SR_, SC_><<<ctx->mt_tiles, 128, 0, st>>>(GBT_MT_ARGS); break;
      case 5: k_match_tiled<256, true, 4, SR_, SC_><<<ctx->mt_tiles, 256, 0, st>>>(GBT_MT_ARGS); break;
      case 6: k_match_tiled<192, true, 5, SR_, SC_><<<ctx->mt_tiles, 192, 0, st>>>(GBT_MT_ARGS); break;
      case 7: k_match_tiled<160, true, 6, SR_, SC_><<<ctx->mt_tiles, 160, 0, st>>>(GBT_MT_ARGS); break;
      default: k_match_tiled<MT_THREADS, false, 4, FR, FC><<<ctx->mt_tiles, MT_THREADS, 0, st>>>(GBT_MT_ARGS); break;
    }
    }
#undef GBT_MT_ARGS
    {
      PROF("k_match_overflow");
      k_match_overflow<<<ctx->nsm, 256, 0, st>>>(du, ctx->d_state, ctx->d_frame, ctx->d_mt_cnt + ctx->mt_tiles,
                                                  ctx->d_mt_ovf);
    }
    n += 3;
  } else if (ctx->match_variant == 1) {
    PROF("k_match_warp");
    k_match_warp<<<ctx->nsm * 4, 32 * MW_WARPS, 0, st>>>(du, ctx->d_state, ctx->d_frame, ctx->d_pre, nunits);
    n++;
  } else {
    PROF("k_match");
    const dim3 g(ctx->nsm * 8);
    if (ctx->match_variant == 3 && ctx->fixed_fpitch)
      k_match<FeatFP<FIXED_FPITCH>><<<g, MATCH_BLOCK, 0, st>>>(du, ctx->d_state, ctx->d_frame, ctx->d_pre, nunits);
    else
      k_match<Feat><<<g, MATCH_BLOCK, 0, st>>>(du, ctx->d_state, ctx->d_frame, ctx->d_pre, nunits);
    n++;
  }
  { PROF("k_stats"); k_stats<<<(ctx->nbins + 255) / 256, 256, 0, st>>>(du, ctx->d_state, ctx->d_bin_prefix, nunits); }
  n++;
  if (any_det) {
    CK(cudaMemsetAsync(ctx->ppos_all, 0, ctx->pmask_bytes, st));
    { PROF("k_pmask"); k_pmask<<<pgrid, CHUNK, 0, st>>>(du, ctx->d_state, ctx->d_frame, ctx->d_pre, nunits); }
    { PROF("k_pmask_dilate"); k_pmask_dilate<<<(ctx->nbins + 255) / 256, 256, 0, st>>>(du, ctx->d_frame, ctx->d_bin_prefix, nunits); }
    { PROF("k_detect"); k_detect<<<ctx->det_blocks, 256, 0, st>>>(du, ctx->d_frame, ctx->d_det_prefix, nunits); }
    if (ctx->any_alt_detector) {
      PROF("k_detect_alt");
      k_detect_alt<<<(ctx->nbins + 255) / 256, 256, 0, st>>>(du, ctx->d_frame, ctx->d_bin_prefix, nunits);
      n++;
    }
    { PROF("k_det_count"); k_det_count<<<pgrid, CHUNK, 0, st>>>(du, ctx->d_state, ctx->d_frame, ctx->d_pre, ctx->d_btable, nunits); }
    { PROF("k_unit_scan"); k_unit_scan<<<nunits, 1024, 0, st>>>(du, ctx->d_state, ctx->d_frame); }
    { PROF("k_det_scatter"); k_det_scatter<<<pgrid, CHUNK, 0, st>>>(du, ctx->d_state, ctx->d_frame, ctx->d_pre, ctx->d_btable, nunits); }
    { PROF("k_commit"); k_commit<<<1, 1024, 0, st>>>(du, ctx->d_state, ctx->d_frame, ctx->d_post, nunits); }
    n += 7;
  }
  int* table = any_det ? ctx->d_post : ctx->d_pre;
  if (any_filt) {
    const int fgrid = ctx->fm_grid;
    { PROF("k_filter_merge"); k_filter_merge<<<fgrid, FM_THREADS, 0, st>>>(du, ctx->d_state, ctx->d_frame, table, nunits); }
    { PROF("k_merge_unit"); k_merge_unit<<<nunits, MU_THREADS, 0, st>>>(du, ctx->d_state, ctx->d_frame); }
    n += 2;
  }
  if (ctx->traj_T) {
    PROF("k_traj");
    k_traj<<<ctx->nsm * 4, CHUNK, 0, st>>>(du, ctx->d_state, ctx->d_cap_table, nunits, ctx->traj_T);
    n++;
  }
  { PROF("k_tick"); k_tick<<<1, 1024, 0, st>>>(du, ctx->d_state, ctx->d_frame, ctx->d_pre, nunits); }
  n++;
  CK(cudaGetLastError());
  return GBT_OK;
}

// Captures (once) and launches a graph of what `issue` enqueues on `st`.
template <class F>
static int launch_graph(Group* ctx, cudaGraphExec_t& exec, int& launches, cudaStream_t st, F issue) {
  if (!exec) {
    cudaGraph_t g;
    int n = 0;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int r = issue(n);
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (r) return r;
    if (e != cudaSuccess) return set_err(ctx, GBT_E_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return set_err(ctx, GBT_E_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
    launches = n;
  }
  CK(cudaGraphLaunch(exec, st));
  return GBT_OK;
}

// Queues one frame whose input is in place (ordered on the front-end stream).
static int run_frame(Group* ctx) {
  bool any_det, any_filt;
  frame_kind(ctx, any_det, any_filt);
  const int par = ctx->host_frame & 1;
  const bool split = split_front(ctx);
  cudaStream_t fs = split ? ctx->pre : ctx->stream;
  int nf = 0, nb = 0, r;
  if (ctx->use_graphs) {
    r = launch_graph(ctx, ctx->front_graph[par], ctx->front_launches, fs,
                     [&](int& n) { return enqueue_front(ctx, par, fs, n); });
    nf = ctx->front_launches;
  } else {
    r = enqueue_front(ctx, par, fs, nf);
  }
  if (r) return r;
  if (split) {
    CK(cudaEventRecord(ctx->ev_front, fs));
    CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_front, 0));
  }
  const int key = (any_det ? 1 : 0) | (any_filt ? 2 : 0) | (par << 2);
  if (ctx->use_graphs) {
    r = launch_graph(ctx, ctx->graph[key], ctx->graph_launches[key], ctx->stream,
                     [&](int& n) { return enqueue_back(ctx, any_det, any_filt, par, n); });
    nb = ctx->graph_launches[key];
  } else {
    r = enqueue_back(ctx, any_det, any_filt, par, nb);
  }
  if (r) return r;
  CK(cudaEventRecord(ctx->ev_back[par], ctx->stream));
  if (!ctx->use_graphs) prof_collect(ctx);
  ctx->launches_per_frame = nf + nb;
  ctx->kernels_total += ctx->launches_per_frame;
  ctx->host_frame++;
  return GBT_OK;
}

// Drops every captured graph (the next frames capture them again).
static void drop_graphs(Group* ctx) {
  for (auto& g : ctx->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  for (auto& g : ctx->front_graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

static int grp_set_tuning(Group* ctx, int32_t knob, int32_t value) {
  if (!ctx) return GBT_E_INVALID;
  if (knob == GBT_TUNE_MATCHER && value >= 0 && value <= 3) {
    if (ctx->match_variant != value) drop_graphs(ctx);
    ctx->match_variant = value;
    return GBT_OK;
  }
  if (knob == GBT_TUNE_BLUR_ROWS && (value == 16 || value == 32 || value == 64)) {
    const int v = value == 16 ? 0 : (value == 32 ? 1 : 2);
    if (ctx->blur_rows != value) drop_graphs(ctx);
    ctx->blur_rows = value;
    ctx->d_blur_prefix = ctx->d_blur_prefix_v[v];
    ctx->blur_tiles = ctx->blur_tiles_v[v];
    return GBT_OK;
  }
  if (knob == GBT_TUNE_MATCH_TILE && value >= 0 && value <= 7) {
    if (ctx->mt_shape != value) drop_graphs(ctx);
    ctx->mt_shape = value;
    return GBT_OK;
  }
  return GBT_E_INVALID;
}

static int grp_get_tuning(Group* ctx, int32_t knob, int32_t* value) {
  if (!ctx || !value) return GBT_E_INVALID;
  if (knob == GBT_TUNE_MATCHER) {
    *value = ctx->match_variant;
    return GBT_OK;
  }
  if (knob == GBT_TUNE_BLUR_ROWS) {
    *value = ctx->blur_rows;
    return GBT_OK;
  }
  if (knob == GBT_TUNE_MATCH_TILE) {
    *value = ctx->mt_shape;
    return GBT_OK;
  }
  return GBT_E_INVALID;
}

// Sets stream s's ingest (mode, and the source for modes 1 - 3) for the next
// frame.  d_ingest is rewritten on the front stream before the frame's
// kernels, after every earlier frame's pyramid, so only the host table needs
// care: once uploaded it may still feed a copy in flight, so a change after an
// upload goes into the next table of the ring.
static int set_ingest(Group* ctx, size_t s, int mode, const uint8_t* src, int64_t pitch) {
  const Ingest want{src, mode ? (long long)pitch : 0, mode, 0};
  const Ingest& cur = ctx->h_ingest[s];
  if (cur.rgb == want.rgb && cur.pitch == want.pitch && cur.mode == want.mode) return GBT_OK;
  if (!ctx->ingest_dirty) {
    const size_t n = ctx->streams.size();
    const int next = (ctx->ingest_slot + 1) % 4;
    CK(cudaEventSynchronize(ctx->ingest_ev[next]));  // its last upload (long done, as a rule)
    Ingest* t = ctx->h_ingest_ring + (size_t)next * n;
    memcpy(t, ctx->h_ingest, sizeof(Ingest) * n);
    ctx->h_ingest = t;
    ctx->ingest_slot = next;
    ctx->ingest_dirty = true;
  }
  ctx->h_ingest[s] = want;
  return GBT_OK;
}

static int flush_ingest(Group* ctx) {
  if (ctx->ingest_dirty) {
    CK(cudaMemcpyAsync(ctx->d_ingest, ctx->h_ingest, sizeof(Ingest) * ctx->streams.size(), cudaMemcpyHostToDevice,
                       front_stream(ctx)));
    CK(cudaEventRecord(ctx->ingest_ev[ctx->ingest_slot], front_stream(ctx)));
    ctx->ingest_dirty = false;
  }
  return GBT_OK;
}

static int grp_trajectories_enable(Group* ctx, int32_t history) {
  if (!ctx || history < 1 || history > 255) return GBT_E_INVALID;
  if (ctx->traj_T) return ctx->traj_T == history ? GBT_OK : GBT_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  int r = sync_all(ctx);
  if (r) return r;
  for (auto& u : ctx->units)
    for (int b = 0; b < 2; b++) {
      if ((r = dalloc_t(ctx, &u.tpos[b], (size_t)history * u.cap))) return r;
      if ((r = dalloc_t(ctx, &u.thead[b], u.cap))) return r;
      if ((r = dalloc_t(ctx, &u.tlen[b], u.cap))) return r;
    }
  int r2 = upload_units(ctx);
  if (r2) return r2;
  drop_graphs(ctx);
  ctx->traj_T = history;
  return GBT_OK;
}

static int grp_test_withhold_tile_copies(Group* ctx, int32_t enable) {
  if (!ctx) return GBT_E_INVALID;
  if (!ctx->d_tmaps || ctx->match_variant != 0 || !ctx->fixed_fpitch)
    return set_err(ctx, GBT_E_INVALID, "the tiled matcher does not stage its tiles by TMA in this context");
  if (ctx->withhold_tiles != (enable != 0)) drop_graphs(ctx);
  ctx->withhold_tiles = enable != 0;
  return GBT_OK;
}

static int grp_test_tile_capacity(Group* ctx, int32_t cap) {
  if (!ctx || cap < 1 || cap > MT_LIST_CAP) return GBT_E_INVALID;
  if (ctx->mt_cap != cap) drop_graphs(ctx);
  ctx->mt_cap = cap;
  return GBT_OK;
}

static int grp_use_graphs(Group* ctx, int32_t enable) {
  if (!ctx) return GBT_E_INVALID;
  ctx->use_graphs = enable != 0;
  return GBT_OK;
}

// `user`: the caller's input writes (recorded on the stream it wrote them on).
static int grp_run_resident(Group* ctx, cudaEvent_t user) {
  if (!ctx) return GBT_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  int r0 = prepare_front(ctx);
  if (r0) return r0;
  if (user) CK(cudaStreamWaitEvent(front_stream(ctx), user, 0));
  for (size_t s = 0; s < ctx->streams.size(); s++) {
    int r = set_ingest(ctx, s, 0, nullptr, 0);
    if (r) return r;
  }
  int r = flush_ingest(ctx);
  if (r) return r;
  return run_frame(ctx);
}

static int grp_run(Group* ctx, const uint8_t* const* frames, const int64_t* pitches, int32_t location) {
  if (!ctx || !frames) return GBT_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  int r0 = prepare_front(ctx);
  if (r0) return r0;
  cudaStream_t in = front_stream(ctx);  // input copies go with the frame's front end
  for (size_t s = 0; s < ctx->streams.size(); s++) {
    StreamInfo& si = ctx->streams[s];
    const Unit u = unit_view(ctx, si.unit0, ctx->host_frame & 1);
    const uint8_t* src = frames[s];
    int mode = 0;
    const uint8_t* isrc = nullptr;  // the pyramid's source for modes 1 - 3
    int64_t ipitch = 0;
    if (!src) return set_err(ctx, GBT_E_INVALID, "frame %zu is NULL", s);
    if (location == GBT_FRAMES_DEVICE) {
      int64_t p = pitches ? pitches[s] : u.W;
      if (p < u.W) return set_err(ctx, GBT_E_INVALID, "pitch %lld < cols %d", (long long)p, u.W);
      // Read by the frame's pyramid kernel straight from the caller's buffer.
      mode = 3;
      isrc = src;
      ipitch = p;
    } else if (location == GBT_FRAMES_HOST) {
      int64_t p = pitches ? pitches[s] : u.W;
      if (p < u.W) return set_err(ctx, GBT_E_INVALID, "pitch %lld < cols %d", (long long)p, u.W);
      cudaPointerAttributes at;
      bool pinned = cudaPointerGetAttributes(&at, src) == cudaSuccess && at.type == cudaMemoryTypeHost;
      cudaGetLastError();
      if (pinned) {
        CK(cudaMemcpy2DAsync(u.img, u.ipitch, src, p, u.W, u.H, cudaMemcpyHostToDevice, in));
      } else {
        // The staging buffer may still feed the previous frame's copy.
        CK(cudaStreamSynchronize(in));
        for (int r = 0; r < u.H; r++) memcpy(si.pinned + (size_t)r * u.W, src + (size_t)r * p, u.W);
        CK(cudaMemcpy2DAsync(u.img, u.ipitch, si.pinned, u.W, u.W, u.H, cudaMemcpyHostToDevice, in));
      }
    } else if (location == GBT_FRAMES_HOST_RGB || location == GBT_FRAMES_DEVICE_RGB) {
      const int64_t row = (int64_t)u.W * 3;
      int64_t p = pitches ? pitches[s] : row;
      if (p < row) return set_err(ctx, GBT_E_INVALID, "pitch %lld too small for RGB", (long long)p);
      if (location == GBT_FRAMES_DEVICE_RGB) {
        // Read by the frame's pyramid kernel straight from the caller's buffer.
        isrc = src;
        ipitch = p;
      } else {
        if (!si.d_rgb) {
          si.rgb_pitch = (row + 15) / 16 * 16;
          int r = dalloc(ctx, (void**)&si.d_rgb, (size_t)si.rgb_pitch * u.H, false);
          if (r) return r;
        }
        cudaPointerAttributes at;
        bool pinned = cudaPointerGetAttributes(&at, src) == cudaSuccess && at.type == cudaMemoryTypeHost;
        cudaGetLastError();
        if (!pinned) {
          // The staging buffer may still feed the previous frame's copy.
          CK(cudaStreamSynchronize(in));
          for (int rr = 0; rr < u.H; rr++) memcpy(si.pinned + (size_t)rr * row, src + (size_t)rr * p, row);
          src = si.pinned;
          p = row;
        }
        CK(cudaMemcpy2DAsync(si.d_rgb, si.rgb_pitch, src, p, row, u.H, cudaMemcpyHostToDevice, in));
        isrc = si.d_rgb;
        ipitch = si.rgb_pitch;
      }
      mode = ctx->rgb_mode == GBT_RGB_BT601 ? 2 : 1;
    } else {
      return set_err(ctx, GBT_E_INVALID, "bad frame location %d", location);
    }
    int r = set_ingest(ctx, s, mode, isrc, ipitch);
    if (r) return r;
  }
  int r = flush_ingest(ctx);
  if (r) return r;
  return run_frame(ctx);
}

static int grp_set_rgb_to_gray(Group* ctx, int32_t mode) {
  if (!ctx || (mode != GBT_RGB_CHANNEL0 && mode != GBT_RGB_BT601)) return GBT_E_INVALID;
  ctx->rgb_mode = mode;
  return GBT_OK;
}

static int grp_sync(Group* ctx) {
  if (!ctx) return GBT_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  int r = sync_all(ctx);
  if (r) return r;
  Frame f;
  CK(cudaMemcpy(&f, ctx->d_frame, sizeof f, cudaMemcpyDeviceToHost));
  if (f.err & ERR_CAPACITY) return set_err(ctx, GBT_E_CAPACITY, "particle capacity exceeded");
  if (f.err & ERR_COPY_INFLIGHT)
    return set_err(ctx, GBT_E_TIMEOUT,
                   "a bounded wait on an asynchronous copy gave up with the copy still in flight; "
                   "destroy this context");
  if (f.err & ERR_TIMEOUT) return set_err(ctx, GBT_E_TIMEOUT, "a bounded wait on an asynchronous copy gave up");
  return GBT_OK;
}

static int grp_kernel_launches(Group* ctx, int64_t* total) {
  if (!ctx || !total) return GBT_E_INVALID;
  *total = ctx->kernels_total;
  return GBT_OK;
}

static int grp_kernels_per_frame(Group* ctx, int32_t* n) {
  if (!ctx || !n) return GBT_E_INVALID;
  *n = ctx->launches_per_frame;
  return GBT_OK;
}

static int unit_of(Group* ctx, int stream, int scale) {
  if (!ctx || stream < 0 || stream >= (int)ctx->streams.size()) return -1;
  if (scale < 0 || scale >= ctx->streams[stream].cfg.nscales) return -1;
  return ctx->streams[stream].unit0 + scale;
}

static int read_state(Group* ctx, int ui, UState* s) {
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpy(s, ctx->d_state + ui, sizeof(UState), cudaMemcpyDeviceToHost));
  return GBT_OK;
}

static int grp_nparticles(Group* ctx, int32_t stream, int32_t scale, int32_t* n) {
  int ui = unit_of(ctx, stream, scale);
  if (ui < 0 || !n) return GBT_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  UState s;
  int r = read_state(ctx, ui, &s);
  if (r) return r;
  *n = s.n;
  return GBT_OK;
}

static int grp_read_counts(Group* ctx, int32_t* counts, int32_t n) {
  if (!ctx || !counts || n < (int)ctx->units.size()) return GBT_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  std::vector<UState> st(ctx->units.size());
  CK(cudaMemcpyAsync(st.data(), ctx->d_state, st.size() * sizeof(UState), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (size_t i = 0; i < st.size(); i++) counts[i] = st[i].n;
  return GBT_OK;
}

static int grp_frame_count(Group* ctx, int32_t stream, int32_t scale, int32_t* n) {
  if (unit_of(ctx, stream, scale) < 0 || !n) return GBT_E_INVALID;
  *n = ctx->host_frame;
  return GBT_OK;
}

static int grp_get_particles(Group* ctx, int32_t stream, int32_t scale, float* speed, int16_t* pos,
                                 uint16_t* age, uint8_t* features, int32_t* matches, int32_t* nmatches,
                                 int32_t* compact_has_run) {
  int ui = unit_of(ctx, stream, scale);
  if (ui < 0) return GBT_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  UState s;
  int r = read_state(ctx, ui, &s);
  if (r) return r;
  const Unit& u = ctx->units[ui];
  const int n = s.n, b = s.cur;
  if (speed) {
    std::vector<short2> v(n);
    if (n) CK(cudaMemcpy(v.data(), u.spd[b], n * sizeof(short2), cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; i++) {
      speed[2 * i] = v[i].x;
      speed[2 * i + 1] = v[i].y;
    }
  }
  if (pos && n) CK(cudaMemcpy(pos, u.pos[b], n * sizeof(short2), cudaMemcpyDeviceToHost));
  if (age && n) CK(cudaMemcpy(age, u.age[b], n * sizeof(uint16_t), cudaMemcpyDeviceToHost));
  if (features && n) CK(cudaMemcpy(features, u.feat[b], n * 16, cudaMemcpyDeviceToHost));
  if (nmatches) *nmatches = s.nmatches;
  if (matches && s.nmatches)
    CK(cudaMemcpy(matches, u.matches, (size_t)s.nmatches * 4, cudaMemcpyDeviceToHost));
  if (compact_has_run) *compact_has_run = s.compact;
  return GBT_OK;
}

static int grp_get_trajectories(Group* ctx, int32_t stream, int32_t scale, int16_t* xy, uint8_t* len,
                                    int32_t* n, int32_t* history) {
  int ui = unit_of(ctx, stream, scale);
  if (ui < 0 || !n || !ctx->traj_T) return GBT_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  UState s;
  int r = read_state(ctx, ui, &s);
  if (r) return r;
  const Unit& u = ctx->units[ui];
  const int T = ctx->traj_T, np = s.n, b = s.cur;
  *n = np;
  if (history) *history = T;
  if ((!xy && !len) || np == 0) return GBT_OK;
  std::vector<uint8_t> hl(np), hh(np);
  std::vector<short2> hp((size_t)T * np);
  CK(cudaMemcpy(hl.data(), u.tlen[b], np, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hh.data(), u.thead[b], np, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy2D(hp.data(), (size_t)np * sizeof(short2), u.tpos[b], (size_t)u.cap * sizeof(short2),
                  (size_t)np * sizeof(short2), T, cudaMemcpyDeviceToHost));
  for (int j = 0; j < np; j++) {
    const int L = hl[j], h = hh[j];
    if (len) len[j] = (uint8_t)L;
    if (!xy) continue;
    int16_t* o = xy + (size_t)j * T * 2;
    for (int m = 0; m < T; m++) {
      if (m < L) {
        const short2 p = hp[(size_t)((h - L + m + T) % T) * np + j];
        o[2 * m] = p.x;
        o[2 * m + 1] = p.y;
      } else {
        o[2 * m] = o[2 * m + 1] = 0;
      }
    }
  }
  return GBT_OK;
}

// ---------------------------------------------------------------------------
// Checkpoint / resume: the tracker's whole carried state (particle_container:
// particles, features, matches, counters, particle_container.h:171-182; the
// strategy's frame counter, tracking_strategies.h:84-106; the device-side
// trajectories) as one byte blob.
namespace {
struct CkHeader {
  char magic[8];
  uint32_t version;
  int32_t nstreams, nunits, traj_T, host_frame, dev_f, dev_err, reserved;
};
constexpr char CK_MAGIC[8] = {'G', 'B', 'T', 'C', 'K', 'P', 'T', '1'};

size_t unit_blob_bytes(const UState& s, int T) {
  size_t n = (size_t)s.n;
  return sizeof(UState) + n * (sizeof(short2) * 2 + sizeof(uint16_t) + sizeof(uint4)) + (size_t)s.nmatches * 4 +
         (T ? n * (2 + (size_t)T * sizeof(short2)) : 0);
}
}  // namespace

static int read_all_states(Group* ctx, std::vector<UState>& st) {
  st.resize(ctx->units.size());
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpy(st.data(), ctx->d_state, st.size() * sizeof(UState), cudaMemcpyDeviceToHost));
  return GBT_OK;
}

static int grp_checkpoint_size(Group* ctx, size_t* bytes) {
  if (!ctx || !bytes) return GBT_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  std::vector<UState> st;
  int r = read_all_states(ctx, st);
  if (r) return r;
  size_t b = sizeof(CkHeader) + ctx->streams.size() * sizeof(gbt_config);
  for (auto& s : st) b += unit_blob_bytes(s, ctx->traj_T);
  *bytes = b;
  return GBT_OK;
}

static int grp_checkpoint_save(Group* ctx, void* buf, size_t cap, size_t* written) {
  if (!ctx || !buf) return GBT_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  size_t need;
  int r = grp_checkpoint_size(ctx, &need);
  if (r) return r;
  if (cap < need) return set_err(ctx, GBT_E_INVALID, "checkpoint needs %zu bytes", need);
  std::vector<UState> st;
  if ((r = read_all_states(ctx, st))) return r;
  Frame fr;
  CK(cudaMemcpy(&fr, ctx->d_frame, sizeof(Frame), cudaMemcpyDeviceToHost));
  uint8_t* o = (uint8_t*)buf;
  CkHeader h{};
  memcpy(h.magic, CK_MAGIC, 8);
  h.version = 1;
  h.nstreams = (int32_t)ctx->streams.size();
  h.nunits = (int32_t)ctx->units.size();
  h.traj_T = ctx->traj_T;
  h.host_frame = ctx->host_frame;
  h.dev_f = fr.f;
  h.dev_err = fr.err;
  memcpy(o, &h, sizeof h);
  o += sizeof h;
  for (auto& si : ctx->streams) {
    memcpy(o, &si.cfg, sizeof(gbt_config));
    o += sizeof(gbt_config);
  }
  const int T = ctx->traj_T;
  for (size_t k = 0; k < ctx->units.size(); k++) {
    const Unit& u = ctx->units[k];
    UState s = st[k];
    const int b = s.cur, n = s.n;
    s.cur = 0;  // stored as buffer 0
    memcpy(o, &s, sizeof s);
    o += sizeof s;
    auto get = [&](const void* src, size_t bytes) -> int {
      if (bytes) CK(cudaMemcpy(o, src, bytes, cudaMemcpyDeviceToHost));
      o += bytes;
      return GBT_OK;
    };
    if ((r = get(u.pos[b], n * sizeof(short2))) || (r = get(u.spd[b], n * sizeof(short2))) ||
        (r = get(u.age[b], n * sizeof(uint16_t))) || (r = get(u.feat[b], n * sizeof(uint4))) ||
        (r = get(u.matches, (size_t)s.nmatches * 4)))
      return r;
    if (T) {
      if ((r = get(u.tlen[b], n)) || (r = get(u.thead[b], n))) return r;
      if (n) CK(cudaMemcpy2D(o, n * sizeof(short2), u.tpos[b], (size_t)u.cap * sizeof(short2), n * sizeof(short2), T,
                             cudaMemcpyDeviceToHost));
      o += (size_t)T * n * sizeof(short2);
    }
  }
  if (written) *written = (size_t)(o - (uint8_t*)buf);
  return GBT_OK;
}

static int grp_checkpoint_load(Group* ctx, const void* buf, size_t len) {
  if (!ctx || !buf || len < sizeof(CkHeader)) return GBT_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  const uint8_t* p = (const uint8_t*)buf;
  const uint8_t* end = p + len;
  CkHeader h;
  memcpy(&h, p, sizeof h);
  p += sizeof h;
  if (memcmp(h.magic, CK_MAGIC, 8) != 0 || h.version != 1 || h.nstreams != (int32_t)ctx->streams.size() ||
      h.nunits != (int32_t)ctx->units.size())
    return set_err(ctx, GBT_E_INVALID, "checkpoint does not belong to a context of this shape");
  if ((size_t)(end - p) < ctx->streams.size() * sizeof(gbt_config)) return GBT_E_INVALID;
  for (auto& si : ctx->streams) {
    if (memcmp(p, &si.cfg, sizeof(gbt_config)) != 0)
      return set_err(ctx, GBT_E_INVALID, "checkpoint stream configuration differs");
    p += sizeof(gbt_config);
  }
  const int T = h.traj_T;
  if (T < 0 || T > 255 || (ctx->traj_T && T && ctx->traj_T != T))
    return set_err(ctx, GBT_E_INVALID, "checkpoint trajectory length differs");
  // Validate every unit before changing anything.
  {
    const uint8_t* q = p;
    for (size_t k = 0; k < ctx->units.size(); k++) {
      const Unit& u = ctx->units[k];
      UState s;
      if ((size_t)(end - q) < sizeof(UState)) return set_err(ctx, GBT_E_INVALID, "checkpoint is truncated");
      memcpy(&s, q, sizeof s);
      if (s.n < 0 || s.n > u.cap || s.nmatches < 0 || s.nmatches > u.cap + u.max_births || s.cur != 0)
        return set_err(ctx, GBT_E_INVALID, "checkpoint unit %zu is inconsistent", k);
      if ((size_t)(end - q) < unit_blob_bytes(s, T)) return set_err(ctx, GBT_E_INVALID, "checkpoint is truncated");
      q += unit_blob_bytes(s, T);
    }
  }
  if (T && ctx->traj_T != T) {
    int r = grp_trajectories_enable(ctx, T);
    if (r) return r;
  }
  CK(cudaStreamSynchronize(ctx->stream));
  std::vector<UState> st(ctx->units.size());
  for (size_t k = 0; k < ctx->units.size(); k++) {
    const Unit& u = ctx->units[k];
    UState s;
    memcpy(&s, p, sizeof s);
    p += sizeof s;
    const int n = s.n;
    auto put = [&](void* dst, size_t bytes) -> int {
      if (bytes) CK(cudaMemcpy(dst, p, bytes, cudaMemcpyHostToDevice));
      p += bytes;
      return GBT_OK;
    };
    int r;
    if ((r = put(u.pos[0], n * sizeof(short2))) || (r = put(u.spd[0], n * sizeof(short2))) ||
        (r = put(u.age[0], n * sizeof(uint16_t))) || (r = put(u.feat[0], n * sizeof(uint4))) ||
        (r = put(u.matches, (size_t)s.nmatches * 4)))
      return r;
    if (T) {
      if ((r = put(u.tlen[0], n)) || (r = put(u.thead[0], n))) return r;
      if (n) CK(cudaMemcpy2D(u.tpos[0], (size_t)u.cap * sizeof(short2), p, n * sizeof(short2), n * sizeof(short2), T,
                             cudaMemcpyHostToDevice));
      p += (size_t)T * n * sizeof(short2);
    }
    if (ctx->traj_T && !T) {  // a blob without trajectories: histories start empty
      CK(cudaMemset(u.tlen[0], 0, u.cap));
      CK(cudaMemset(u.thead[0], 0, u.cap));
    }
    // Sparse-index entries of this context's own earlier frames could carry
    // the stamps of the frames to come: start from "nothing current".
    CK(cudaMemset(u.idx, 0, (size_t)u.H * u.W * sizeof(unsigned long long)));
    st[k] = s;
  }
  CK(cudaMemcpy(ctx->d_state, st.data(), st.size() * sizeof(UState), cudaMemcpyHostToDevice));
  Frame fr{h.dev_f, h.dev_err};
  CK(cudaMemcpy(ctx->d_frame, &fr, sizeof fr, cudaMemcpyHostToDevice));
  // The chunk table of the first frame after the load follows the new counts.
  k_tick_table<<<1, 1024, 0, ctx->stream>>>(ctx->d_units, ctx->d_state, (int)ctx->units.size(), ctx->d_pre);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->host_frame = h.host_frame;
  return GBT_OK;
}

static int grp_bins(Group* ctx, int32_t stream, int32_t scale, int32_t* rows, int32_t* cols) {
  int ui = unit_of(ctx, stream, scale);
  if (ui < 0) return GBT_E_INVALID;
  if (rows) *rows = ctx->units[ui].BH;
  if (cols) *cols = ctx->units[ui].BW;
  return GBT_OK;
}

static int grp_get_bins(Group* ctx, int32_t stream, int32_t scale, float* flow, uint32_t* count,
                            int32_t* stat_n, int32_t* stat_speed) {
  int ui = unit_of(ctx, stream, scale);
  if (ui < 0) return GBT_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  const Unit& u = ctx->units[ui];
  size_t nb = (size_t)u.BH * u.BW;
  if (flow) CK(cudaMemcpy(flow, u.flow, nb * 8, cudaMemcpyDeviceToHost));
  if (count) CK(cudaMemcpy(count, u.msc, nb * 4, cudaMemcpyDeviceToHost));
  if (stat_n) CK(cudaMemcpy(stat_n, u.st_n, nb * 4, cudaMemcpyDeviceToHost));
  if (stat_speed) CK(cudaMemcpy(stat_speed, u.st_sp, nb * 8, cudaMemcpyDeviceToHost));
  return GBT_OK;
}

// Stage images computed on demand from the resident state (checks only).
namespace gbt {
__global__ void k_dump(const Unit* __restrict__ units, const UState* __restrict__ st, const Frame* __restrict__ fr,
                       int ui, int what, void* out) {
  const Unit& u = units[ui];
  const int total = u.H * u.W;
  const int flast = fr->f - 1;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    int r = t / u.W, c = t % u.W;
    if (what == GBT_STAGE_CONTRAST) {
      ((uint32_t*)out)[t] = (uint32_t)contrast_at(u, r, c);
    } else if (what == GBT_STAGE_SPARSE) {
      unsigned long long e = u.idx[t];
      ((uint32_t*)out)[t] = idx_current(e, flast) ? (uint32_t)(e & 0xffffffffu) : 0xffffffffu;
    } else {
      bool masked = (u.pmask[bin_word(u, r, c)] & bin_bit(r, c)) != 0 || contrast_at(u, r, c) < 5;
      if (what == GBT_STAGE_MASK) {
        ((uint8_t*)out)[t] = masked ? 0 : 255;
      } else {
        uint8_t v = 0;
        if (!masked) {
          uint8_t win[7][7];
          for (int a = 0; a < 7; a++)
            for (int b = 0; b < 7; b++) win[a][b] = (uint8_t)img_at(u, r - 3 + a, c - 3 + b);
          v = (uint8_t)fast_saliency_bf<7>(&win[3][3], u.nfast, u.threshold);
        }
        ((uint8_t*)out)[t] = v;
      }
    }
  }
}
}  // namespace gbt

static int grp_get_stage(Group* ctx, int32_t stream, int32_t scale, int32_t stage, int32_t border, void* out) {
  int ui = unit_of(ctx, stream, scale);
  if (ui < 0 || !out || border < 0 || border > 6) return GBT_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  const int lp = (ctx->host_frame + 1) & 1;  // parity of the last frame run
  const Unit u = unit_view(ctx, ui, lp);
  const int H = u.H, W = u.W, b = border;
  if (stage == GBT_STAGE_INPUT) {
    std::vector<uint8_t> dom((size_t)H * W);
    CK(cudaMemcpy2D(dom.data(), W, u.img, u.ipitch, W, H, cudaMemcpyDeviceToHost));
    uint8_t* o = (uint8_t*)out;
    size_t k = 0;
    for (int r = -b; r < H + b; r++)
      for (int c = -b; c < W + b; c++) {
        int rr = std::min(std::max(r, 0), H - 1), cc = std::min(std::max(c, 0), W - 1);
        o[k++] = dom[(size_t)rr * W + cc];
      }
    return GBT_OK;
  }
  if (stage == GBT_STAGE_S1 || stage == GBT_STAGE_S2) {
    const uint8_t* base = (stage == GBT_STAGE_S1 ? u.s1 : u.s2) + (size_t)(RB - b) * u.fpitch + (CB - b);
    CK(cudaMemcpy2D(out, W + 2 * b, base, u.fpitch, W + 2 * b, H + 2 * b, cudaMemcpyDeviceToHost));
    return GBT_OK;
  }
  size_t bytes = (size_t)H * W * 4;
  if (ctx->dump_bytes < bytes) {
    void* p;
    int r = dalloc(ctx, &p, bytes, false);
    if (r) return r;
    ctx->dump_buf = p;
    ctx->dump_bytes = bytes;
  }
  if (stage != GBT_STAGE_CONTRAST && stage != GBT_STAGE_SALIENCY && stage != GBT_STAGE_MASK &&
      stage != GBT_STAGE_SPARSE)
    return GBT_E_INVALID;
  k_dump<<<256, 256, 0, ctx->stream>>>(ctx->d_units_v[lp], ctx->d_state, ctx->d_frame, ui, stage, ctx->dump_buf);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  size_t es = (stage == GBT_STAGE_CONTRAST || stage == GBT_STAGE_SPARSE) ? 4 : 1;
  CK(cudaMemcpy(out, ctx->dump_buf, (size_t)H * W * es, cudaMemcpyDeviceToHost));
  return GBT_OK;
}

static int grp_profile_enable(Group* ctx, int32_t enable) {
  if (!ctx) return GBT_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  int r = sync_all(ctx);  // the front end changes streams
  if (r) return r;
  ctx->profiling = enable != 0;
  if (ctx->profiling) ctx->prof.clear();
  return GBT_OK;
}

static int grp_profile_read(Group* ctx, int32_t i, char* name, size_t len, double* total_ms, int32_t* launches) {
  if (!ctx) return -1;
  if (i < 0 || i >= (int)ctx->prof.size()) return (int)ctx->prof.size();
  if (name && len) snprintf(name, len, "%s", ctx->prof[i].name.c_str());
  if (total_ms) *total_ms = ctx->prof[i].ms;
  if (launches) *launches = ctx->prof[i].launches;
  return (int)ctx->prof.size();
}

// ---------------------------------------------------------------------------
// The context: its streams split into groups, each a complete tracker over its
// streams (units, work tables, CUDA streams, graphs).  Groups share nothing,
// so the latency-bound stages of one group (scans, the merge replay, the tick)
// run while another group's matcher or blurs fill the GPU.  The stream callers
// see (gbt_stream) is `join`: every call that queues work ends with `join`
// waiting for each group's context stream, and input the caller writes on
// `join` is waited for by the groups.  Results do not depend on the grouping.
struct gbt_ctx {
  int device = 0;
  std::vector<Group*> g;
  std::vector<int> grp, local;             // per stream: its group and its index there
  std::vector<std::vector<int>> members;   // per group: its streams, ascending
  std::vector<int> nscales, unit0;         // per stream: scales, first unit (context order)
  std::vector<int> gunit0;                 // per stream: first unit inside its group
  int nunits = 0;
  cudaStream_t join = nullptr;
  std::vector<cudaEvent_t> ev;             // per group: its latest queued work
  cudaEvent_t ev_join = nullptr;
  bool profiling = false;                  // per-kernel timing: groups run one after another
  std::string err;
  PkTracker* pk = nullptr;                 // the LK matcher's engine (gbt_config.matcher == GBT_MATCHER_LK)
};

// Entry points of an LK-matcher context: the engine's status, with its message.
static int pk_adopt(gbt_ctx* c, int r) {
  if (r) c->err = pk_error(c->pk);
  return r;
}
static int pk_unsupported(gbt_ctx* c, const char* what) {
  c->err = std::string(what) + " is not available with the LK matcher";
  return GBT_E_INVALID;
}
#define LK_ONLY(call) \
  if (c && c->pk) return pk_adopt(c, (call))
#define LK_NOT(name) \
  if (c && c->pk) return pk_unsupported(c, name)

#define CKO(call)                                                                              \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) {                                                                   \
      c->err = std::string(#call) + " failed: " + cudaGetErrorString(e_);                      \
      return GBT_E_CUDA;                                                                       \
    }                                                                                          \
  } while (0)

static int adopt(gbt_ctx* c, Group* g, int r) {
  if (r && g) c->err = g->err;
  return r;
}

static int join_groups(gbt_ctx* c) {
  for (size_t k = 0; k < c->g.size(); k++) {
    CKO(cudaEventRecord(c->ev[k], c->g[k]->stream));
    CKO(cudaStreamWaitEvent(c->join, c->ev[k], 0));
  }
  return GBT_OK;
}

// With per-kernel timing on, group k's work waits for group k - 1's, so that
// every event pair times one kernel alone.
static int serialize_group(gbt_ctx* c, size_t k) {
  if (!c->profiling || k == 0) return GBT_OK;
  CKO(cudaEventRecord(c->ev[k - 1], c->g[k - 1]->stream));
  CKO(cudaStreamWaitEvent(c->g[k]->stream, c->ev[k - 1], 0));
  return GBT_OK;
}

static void free_outer(gbt_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  for (Group* g : c->g) grp_destroy(g);
  for (cudaEvent_t e : c->ev)
    if (e) cudaEventDestroy(e);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  if (c->join) cudaStreamDestroy(c->join);
  delete c;
}

// Streams to groups: longest-processing-time-first by pixels per frame, ties
// to the lower group; each group keeps its streams in ascending order.
static void partition(const gbt_config* cfgs, int n, int G, std::vector<std::vector<int>>& members) {
  std::vector<int> order(n);
  for (int s = 0; s < n; s++) order[s] = s;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return (long long)cfgs[a].rows * cfgs[a].cols > (long long)cfgs[b].rows * cfgs[b].cols;
  });
  std::vector<long long> load(G, 0);
  members.assign(G, {});
  for (int s : order) {
    int k = 0;
    for (int j = 1; j < G; j++)
      if (load[j] < load[k]) k = j;
    members[k].push_back(s);
    load[k] += (long long)cfgs[s].rows * cfgs[s].cols;
  }
  for (auto& m : members) std::sort(m.begin(), m.end());
}

static bool lk_config_ok(const gbt_config& c) {
  if (c.nscales < 1 || c.nscales > 9 || c.detector_frequency < 1 || c.filtering_frequency < 1 || c.detector_n < 1 ||
      c.detector_n > 16 || c.detector_threshold < 0 || c.k < 0 || c.detector != GBT_DETECTOR_FAST)
    return false;
  for (int l = 0; l < c.nscales; l++)
    if ((c.rows >> l) < 16 || (c.cols >> l) < 16) return false;
  return true;
}

extern "C" int gbt_create_ex(const gbt_config* cfgs, int32_t nstreams, int32_t device, int32_t groups,
                             gbt_ctx** out) {
  if (!out) return GBT_E_INVALID;
  *out = nullptr;
  if (!cfgs || nstreams < 1) return GBT_E_INVALID;
  for (int s = 0; s < nstreams; s++)
    if (cfgs[s].matcher != cfgs[0].matcher || (cfgs[s].matcher != GBT_MATCHER_BC2S && cfgs[s].matcher != GBT_MATCHER_LK))
      return GBT_E_INVALID;
  if (cfgs[0].matcher == GBT_MATCHER_LK) {
    for (int s = 0; s < nstreams; s++)
      if (!lk_config_ok(cfgs[s])) return GBT_E_INVALID;
    gbt_ctx* c = new gbt_ctx;
    c->device = device;
    std::string err;
    int r = pk_create(cfgs, nstreams, device, &c->pk, err);
    if (r) {
      fprintf(stderr, "gbt_create: %s\n", err.c_str());
      delete c;
      return r;
    }
    c->nunits = 0;
    for (int s = 0; s < nstreams; s++) {
      c->nscales.push_back(cfgs[s].nscales);
      c->unit0.push_back(c->nunits);
      c->nunits += cfgs[s].nscales;
    }
    *out = c;
    return GBT_OK;
  }
  int G = groups > 0 ? groups : 4;
  G = std::max(1, std::min(G, (int)nstreams));
  gbt_ctx* c = new gbt_ctx;
  c->device = device;
  partition(cfgs, nstreams, G, c->members);
  c->grp.assign(nstreams, 0);
  c->local.assign(nstreams, 0);
  c->nscales.assign(nstreams, 0);
  c->unit0.assign(nstreams, 0);
  c->gunit0.assign(nstreams, 0);
  for (int s = 0; s < nstreams; s++) {
    c->nscales[s] = cfgs[s].nscales;
    c->unit0[s] = c->nunits;
    c->nunits += cfgs[s].nscales;
  }
  for (int k = 0; k < G; k++) {
    std::vector<gbt_config> sub;
    int u = 0;
    for (size_t i = 0; i < c->members[k].size(); i++) {
      const int s = c->members[k][i];
      c->grp[s] = k;
      c->local[s] = (int)i;
      c->gunit0[s] = u;
      u += cfgs[s].nscales;
      sub.push_back(cfgs[s]);
    }
    Group* g = nullptr;
    int r = grp_create(sub.data(), (int32_t)sub.size(), device, &g);
    if (r) {
      free_outer(c);
      return r;
    }
    c->g.push_back(g);
  }
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->join, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
  c->ev.assign(G, nullptr);
  for (int k = 0; k < G && e == cudaSuccess; k++) e = cudaEventCreateWithFlags(&c->ev[k], cudaEventDisableTiming);
  if (e != cudaSuccess) {
    fprintf(stderr, "gbt_create: %s\n", cudaGetErrorString(e));
    free_outer(c);
    return GBT_E_CUDA;
  }
  *out = c;
  return GBT_OK;
}

extern "C" int gbt_create(const gbt_config* cfgs, int32_t nstreams, int32_t device, gbt_ctx** out) {
  return gbt_create_ex(cfgs, nstreams, device, 0, out);
}

extern "C" int gbt_groups(gbt_ctx* c, int32_t* groups) {
  if (c && c->pk && groups) {
    *groups = 1;
    return GBT_OK;
  }
  if (!c || !groups) return GBT_E_INVALID;
  *groups = (int32_t)c->g.size();
  return GBT_OK;
}

extern "C" int gbt_destroy(gbt_ctx* c) {
  if (c && c->pk) {
    pk_destroy(c->pk);
    delete c;
    return GBT_OK;
  }
  if (!c) return GBT_E_INVALID;
  cudaSetDevice(c->device);
  if (c->join) cudaStreamSynchronize(c->join);
  free_outer(c);
  return GBT_OK;
}

extern "C" int gbt_last_error(gbt_ctx* c, char* buf, size_t len) {
  if (!c || !buf || !len) return GBT_E_INVALID;
  snprintf(buf, len, "%s", c->err.c_str());
  return GBT_OK;
}

extern "C" int gbt_stream(gbt_ctx* c, void** s) {
  if (c && c->pk && s) {
    *s = (void*)pk_stream(c->pk);
    return GBT_OK;
  }
  if (!c || !s) return GBT_E_INVALID;
  *s = (void*)c->join;
  return GBT_OK;
}

static bool stream_ok(const gbt_ctx* c, int32_t s) { return c && s >= 0 && s < (int32_t)c->grp.size(); }

extern "C" int gbt_input_slot(gbt_ctx* c, int32_t stream, uint8_t** dptr, int64_t* pitch) {
  LK_NOT("gbt_input_slot");
  if (!stream_ok(c, stream)) return GBT_E_INVALID;
  Group* g = c->g[c->grp[stream]];
  return adopt(c, g, grp_input_slot(g, c->local[stream], dptr, pitch));
}

extern "C" int gbt_set_tuning(gbt_ctx* c, int32_t knob, int32_t value) {
  LK_NOT("gbt_set_tuning");
  if (!c) return GBT_E_INVALID;
  for (Group* g : c->g) {
    int r = grp_set_tuning(g, knob, value);
    if (r) return adopt(c, g, r);
  }
  return GBT_OK;
}

extern "C" int gbt_get_tuning(gbt_ctx* c, int32_t knob, int32_t* value) {
  LK_NOT("gbt_get_tuning");
  if (!c) return GBT_E_INVALID;
  return adopt(c, c->g[0], grp_get_tuning(c->g[0], knob, value));
}

extern "C" int gbt_trajectories_enable(gbt_ctx* c, int32_t history) {
  LK_NOT("device-side trajectories");
  if (!c) return GBT_E_INVALID;
  for (Group* g : c->g) {
    int r = grp_trajectories_enable(g, history);
    if (r) return adopt(c, g, r);
  }
  return GBT_OK;
}

extern "C" int gbt_use_graphs(gbt_ctx* c, int32_t enable) {
  LK_NOT("gbt_use_graphs");
  if (!c) return GBT_E_INVALID;
  for (Group* g : c->g) grp_use_graphs(g, enable);
  return GBT_OK;
}

extern "C" int gbt_test_withhold_tile_copies(gbt_ctx* c, int32_t enable) {
  LK_NOT("gbt_test_withhold_tile_copies");
  if (!c) return GBT_E_INVALID;
  for (Group* g : c->g) {
    int r = grp_test_withhold_tile_copies(g, enable);
    if (r) return adopt(c, g, r);
  }
  return GBT_OK;
}

extern "C" int gbt_test_tile_capacity(gbt_ctx* c, int32_t cap) {
  LK_NOT("gbt_test_tile_capacity");
  if (!c) return GBT_E_INVALID;
  for (Group* g : c->g) {
    int r = grp_test_tile_capacity(g, cap);
    if (r) return adopt(c, g, r);
  }
  return GBT_OK;
}

extern "C" int gbt_test_tile_fallbacks(gbt_ctx* c, int64_t* count) {
  LK_NOT("gbt_test_tile_fallbacks");
  if (!c || !count) return GBT_E_INVALID;
  int64_t total = 0;
  for (Group* g : c->g) {
    if (cudaSetDevice(g->device) != cudaSuccess) return adopt(c, g, set_err(g, GBT_E_CUDA, "cudaSetDevice failed"));
    int r = sync_all(g);
    if (r) return adopt(c, g, r);
    unsigned long long n = 0;
    if (cudaMemcpy(&n, g->d_mt_fallback, sizeof n, cudaMemcpyDeviceToHost) != cudaSuccess)
      return adopt(c, g, set_err(g, GBT_E_CUDA, "reading the tiled matcher's fallback count failed"));
    total += (int64_t)n;
  }
  *count = total;
  return GBT_OK;
}

extern "C" int gbt_set_rgb_to_gray(gbt_ctx* c, int32_t mode) {
  LK_NOT("RGB input");
  if (!c) return GBT_E_INVALID;
  for (Group* g : c->g) {
    int r = grp_set_rgb_to_gray(g, mode);
    if (r) return adopt(c, g, r);
  }
  return GBT_OK;
}

extern "C" int gbt_run_resident(gbt_ctx* c) {
  LK_NOT("gbt_run_resident");
  if (!c) return GBT_E_INVALID;
  CKO(cudaSetDevice(c->device));
  CKO(cudaEventRecord(c->ev_join, c->join));  // the caller's slot writes on gbt_stream
  for (size_t k = 0; k < c->g.size(); k++) {
    int r = serialize_group(c, k);
    if (!r) r = adopt(c, c->g[k], grp_run_resident(c->g[k], c->ev_join));
    if (r) return r;
  }
  return join_groups(c);
}

extern "C" int gbt_run(gbt_ctx* c, const uint8_t* const* frames, const int64_t* pitches, int32_t location) {
  LK_ONLY(pk_run(c->pk, frames, pitches, location));
  if (!c || !frames) return GBT_E_INVALID;
  CKO(cudaSetDevice(c->device));
  for (size_t k = 0; k < c->g.size(); k++) {
    const auto& m = c->members[k];
    std::vector<const uint8_t*> f(m.size());
    std::vector<int64_t> p(m.size());
    for (size_t i = 0; i < m.size(); i++) {
      f[i] = frames[m[i]];
      if (pitches) p[i] = pitches[m[i]];
    }
    int r = serialize_group(c, k);
    if (!r) r = adopt(c, c->g[k], grp_run(c->g[k], f.data(), pitches ? p.data() : nullptr, location));
    if (r) return r;
  }
  return join_groups(c);
}

extern "C" int gbt_sync(gbt_ctx* c) {
  LK_ONLY(pk_sync(c->pk));
  if (!c) return GBT_E_INVALID;
  int first = GBT_OK;
  for (Group* g : c->g) {
    int r = grp_sync(g);
    if (r && !first) first = adopt(c, g, r);
  }
  CKO(cudaStreamSynchronize(c->join));
  return first;
}

extern "C" int gbt_kernel_launches(gbt_ctx* c, int64_t* total) {
  LK_ONLY(pk_kernel_launches(c->pk, total));
  if (!c || !total) return GBT_E_INVALID;
  int64_t t = 0;
  for (Group* g : c->g) {
    int64_t x = 0;
    grp_kernel_launches(g, &x);
    t += x;
  }
  *total = t;
  return GBT_OK;
}

extern "C" int gbt_kernels_per_frame(gbt_ctx* c, int32_t* n) {
  LK_ONLY(pk_kernels_per_frame(c->pk, n));
  if (!c || !n) return GBT_E_INVALID;
  int32_t t = 0;
  for (Group* g : c->g) {
    int32_t x = 0;
    grp_kernels_per_frame(g, &x);
    t += x;
  }
  *n = t;
  return GBT_OK;
}

#define DISPATCH(call_with_local)                        \
  if (!stream_ok(c, stream)) return GBT_E_INVALID;       \
  Group* g = c->g[c->grp[stream]];                       \
  const int32_t ls = c->local[stream];                   \
  return adopt(c, g, call_with_local)

extern "C" int gbt_set_param(gbt_ctx* c, int32_t stream, int32_t scale, int32_t key, int32_t value) {
  LK_ONLY(pk_set_param(c->pk, stream, scale, key, value));
  DISPATCH(grp_set_param(g, ls, scale, key, value));
}

extern "C" int gbt_get_param(gbt_ctx* c, int32_t stream, int32_t scale, int32_t key, int32_t* value) {
  LK_ONLY(pk_get_param(c->pk, stream, scale, key, value));
  DISPATCH(grp_get_param(g, ls, scale, key, value));
}

extern "C" int gbt_nparticles(gbt_ctx* c, int32_t stream, int32_t scale, int32_t* n) {
  LK_ONLY(pk_nparticles(c->pk, stream, scale, n));
  DISPATCH(grp_nparticles(g, ls, scale, n));
}

extern "C" int gbt_frame_count(gbt_ctx* c, int32_t stream, int32_t scale, int32_t* n) {
  LK_ONLY(pk_frame_count(c->pk, stream, scale, n));
  DISPATCH(grp_frame_count(g, ls, scale, n));
}

extern "C" int gbt_get_particles(gbt_ctx* c, int32_t stream, int32_t scale, float* speed, int16_t* pos,
                                 uint16_t* age, uint8_t* features, int32_t* matches, int32_t* nmatches,
                                 int32_t* compact_has_run) {
  if (c && c->pk) {  // integral positions (i_int2 truncation), no features
    int32_t n = 0;
    int r = pk_adopt(c, pk_nparticles(c->pk, stream, scale, &n));
    if (r) return r;
    std::vector<float> p(2 * (size_t)n);
    r = pk_adopt(c, pk_get_particles(c->pk, stream, scale, p.data(), speed, age, matches, nmatches, compact_has_run));
    if (r) return r;
    for (size_t i = 0; pos && i < p.size(); i++) pos[i] = (int16_t)(int)p[i];
    if (features) memset(features, 0, 16 * (size_t)n);
    return GBT_OK;
  }
  DISPATCH(grp_get_particles(g, ls, scale, speed, pos, age, features, matches, nmatches, compact_has_run));
}

extern "C" int gbt_get_particles_f(gbt_ctx* c, int32_t stream, int32_t scale, float* pos, float* speed, uint16_t* age,
                                   int32_t* matches, int32_t* nmatches, int32_t* compact_has_run) {
  LK_ONLY(pk_get_particles(c->pk, stream, scale, pos, speed, age, matches, nmatches, compact_has_run));
  int32_t n = 0;
  int r = gbt_nparticles(c, stream, scale, &n);
  if (r) return r;
  std::vector<int16_t> p(2 * (size_t)n);
  r = gbt_get_particles(c, stream, scale, speed, p.data(), age, nullptr, matches, nmatches, compact_has_run);
  if (r) return r;
  for (size_t i = 0; pos && i < p.size(); i++) pos[i] = (float)p[i];
  return GBT_OK;
}

extern "C" int gbt_get_trajectories(gbt_ctx* c, int32_t stream, int32_t scale, int16_t* xy, uint8_t* len,
                                    int32_t* n, int32_t* history) {
  LK_NOT("device-side trajectories");
  DISPATCH(grp_get_trajectories(g, ls, scale, xy, len, n, history));
}

extern "C" int gbt_bins(gbt_ctx* c, int32_t stream, int32_t scale, int32_t* rows, int32_t* cols) {
  LK_NOT("flow bins");
  DISPATCH(grp_bins(g, ls, scale, rows, cols));
}

extern "C" int gbt_get_bins(gbt_ctx* c, int32_t stream, int32_t scale, float* flow, uint32_t* count,
                            int32_t* stat_n, int32_t* stat_speed) {
  LK_NOT("flow bins");
  DISPATCH(grp_get_bins(g, ls, scale, flow, count, stat_n, stat_speed));
}

extern "C" int gbt_get_stage(gbt_ctx* c, int32_t stream, int32_t scale, int32_t stage, int32_t border, void* out) {
  LK_ONLY(pk_get_stage(c->pk, stream, scale, stage, border, out));
  DISPATCH(grp_get_stage(g, ls, scale, stage, border, out));
}

extern "C" int gbt_read_counts(gbt_ctx* c, int32_t* counts, int32_t n) {
  LK_ONLY(pk_read_counts(c->pk, counts, n, false));
  if (!c || !counts || n < c->nunits) return GBT_E_INVALID;
  for (size_t k = 0; k < c->g.size(); k++) {
    Group* g = c->g[k];
    std::vector<int32_t> tmp(g->units.size());
    int r = grp_read_counts(g, tmp.data(), (int32_t)tmp.size());
    if (r) return adopt(c, g, r);
    for (int s : c->members[k])
      for (int l = 0; l < c->nscales[s]; l++) counts[c->unit0[s] + l] = tmp[c->gunit0[s] + l];
  }
  return GBT_OK;
}

extern "C" int gbt_read_counts_async(gbt_ctx* c, int32_t* counts, int32_t n) {
  LK_ONLY(pk_read_counts(c->pk, counts, n, true));
  if (!c || !counts || n < c->nunits) return GBT_E_INVALID;
  CKO(cudaSetDevice(c->device));
  for (size_t k = 0; k < c->g.size(); k++) {
    Group* g = c->g[k];
    const int nu = (int)g->units.size();
    k_counts<<<(nu + 255) / 256, 256, 0, g->stream>>>(g->d_state, nu, g->d_counts);
    CKO(cudaGetLastError());
    for (int s : c->members[k])
      CKO(cudaMemcpyAsync(counts + c->unit0[s], g->d_counts + c->gunit0[s], (size_t)c->nscales[s] * sizeof(int32_t),
                          cudaMemcpyDeviceToHost, g->stream));
  }
  return join_groups(c);
}

// Checkpoint of a grouped context: a header with the grouping, then each
// group's blob (its own header, configurations and units) with its size.
namespace {
const char CKG_MAGIC[8] = {'G', 'B', 'T', 'C', 'K', 'P', 'G', '1'};
struct CkgHeader {
  char magic[8];
  int32_t version, ngroups, nstreams, pad;
};
}  // namespace

extern "C" int gbt_checkpoint_size(gbt_ctx* c, size_t* bytes) {
  LK_NOT("checkpointing");
  if (!c || !bytes) return GBT_E_INVALID;
  size_t b = sizeof(CkgHeader) + c->grp.size() * sizeof(int32_t) + c->g.size() * sizeof(uint64_t);
  for (Group* g : c->g) {
    size_t x = 0;
    int r = grp_checkpoint_size(g, &x);
    if (r) return adopt(c, g, r);
    b += x;
  }
  *bytes = b;
  return GBT_OK;
}

extern "C" int gbt_checkpoint_save(gbt_ctx* c, void* buf, size_t cap, size_t* written) {
  LK_NOT("checkpointing");
  if (!c || !buf) return GBT_E_INVALID;
  size_t need = 0;
  int r = gbt_checkpoint_size(c, &need);
  if (r) return r;
  if (cap < need) return GBT_E_INVALID;
  uint8_t* p = (uint8_t*)buf;
  CkgHeader h{};
  memcpy(h.magic, CKG_MAGIC, 8);
  h.version = 1;
  h.ngroups = (int32_t)c->g.size();
  h.nstreams = (int32_t)c->grp.size();
  memcpy(p, &h, sizeof h);
  p += sizeof h;
  for (int s = 0; s < h.nstreams; s++) {
    const int32_t k = c->grp[s];
    memcpy(p, &k, sizeof k);
    p += sizeof k;
  }
  for (Group* g : c->g) {
    size_t x = 0, w = 0;
    if ((r = grp_checkpoint_size(g, &x))) return adopt(c, g, r);
    const uint64_t x64 = x;
    memcpy(p, &x64, sizeof x64);
    p += sizeof x64;
    if ((r = grp_checkpoint_save(g, p, x, &w))) return adopt(c, g, r);
    p += x;
  }
  if (written) *written = (size_t)(p - (uint8_t*)buf);
  return GBT_OK;
}

extern "C" int gbt_checkpoint_load(gbt_ctx* c, const void* buf, size_t len) {
  LK_NOT("checkpointing");
  if (!c || !buf || len < sizeof(CkgHeader)) return GBT_E_INVALID;
  const uint8_t* p = (const uint8_t*)buf;
  const uint8_t* end = p + len;
  CkgHeader h;
  memcpy(&h, p, sizeof h);
  p += sizeof h;
  if (memcmp(h.magic, CKG_MAGIC, 8) != 0 || h.version != 1 || h.ngroups != (int32_t)c->g.size() ||
      h.nstreams != (int32_t)c->grp.size() || (size_t)(end - p) < (size_t)h.nstreams * sizeof(int32_t)) {
    c->err = "checkpoint does not belong to a context of this shape";
    return GBT_E_INVALID;
  }
  for (int s = 0; s < h.nstreams; s++) {
    int32_t k;
    memcpy(&k, p, sizeof k);
    p += sizeof k;
    if (k != c->grp[s]) {
      c->err = "checkpoint groups its streams differently";
      return GBT_E_INVALID;
    }
  }
  // Every group's blob is checked by its own loader before it changes anything;
  // first make sure all the blobs are there.
  std::vector<std::pair<const uint8_t*, size_t>> blobs;
  for (size_t k = 0; k < c->g.size(); k++) {
    uint64_t x;
    if ((size_t)(end - p) < sizeof x) return GBT_E_INVALID;
    memcpy(&x, p, sizeof x);
    p += sizeof x;
    if ((uint64_t)(end - p) < x) return GBT_E_INVALID;
    blobs.push_back({p, (size_t)x});
    p += x;
  }
  for (size_t k = 0; k < c->g.size(); k++) {
    int r = grp_checkpoint_load(c->g[k], blobs[k].first, blobs[k].second);
    if (r) return adopt(c, c->g[k], r);
  }
  return GBT_OK;
}

extern "C" int gbt_profile_enable(gbt_ctx* c, int32_t enable) {
  LK_NOT("per-kernel profiling");
  if (!c) return GBT_E_INVALID;
  for (Group* g : c->g) {
    int r = grp_profile_enable(g, enable);
    if (r) return adopt(c, g, r);
  }
  c->profiling = enable != 0;
  return GBT_OK;
}

// Per-kernel entries of all groups, merged by kernel name (first-seen order).
extern "C" int gbt_profile_read(gbt_ctx* c, int32_t i, char* name, size_t len, double* total_ms, int32_t* launches) {
  LK_NOT("per-kernel profiling");
  if (!c) return -1;
  std::vector<std::string> names;
  std::vector<double> ms;
  std::vector<int> cnt;
  char nb[128];
  for (Group* g : c->g) {
    double t = 0;
    int32_t n = 0;
    const int m = grp_profile_read(g, -1, nullptr, 0, nullptr, nullptr);
    for (int k = 0; k < m; k++) {
      grp_profile_read(g, k, nb, sizeof nb, &t, &n);
      size_t j = 0;
      while (j < names.size() && names[j] != nb) j++;
      if (j == names.size()) {
        names.push_back(nb);
        ms.push_back(0);
        cnt.push_back(0);
      }
      ms[j] += t;
      cnt[j] += n;
    }
  }
  if (i < 0 || i >= (int)names.size()) return (int)names.size();
  if (name && len) snprintf(name, len, "%s", names[i].c_str());
  if (total_ms) *total_ms = ms[i];
  if (launches) *launches = cnt[i];
  return (int)names.size();
}
