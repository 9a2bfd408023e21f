/*
 * cuimg_gb300_strategy.hpp -- the GB300 path as strategies of cuimg's
 * unchanged tracker<F> (cuimg/tracking2/tracker.h:10-47).
 *
 * tracker<F> builds one strategy object per scale and, every frame, calls
 * update(input, pset) on each scale, coarsest first (tracker.hpp:83-91).
 * Two strategies:
 *   bc2s_fast_gradient_gb300 -- bc2s_fast_gradient_cpu
 *     (cuimg/tracking2/tracking_strategies.h:138-151): the strategy concept of
 *     generic_strategy (:28-107);
 *   pyrlk_gb300 -- pyrlk_cpu<fast_detector<cpu>, iterative_lk_match_5x5>
 *     (cuimg/tracking2/pyrlk_tracker.h:16-82): sub-pixel particle_f particles
 *     tracked by pyramidal LK.
 * Both provide the types input / particles_type / particle_type /
 * architecture, construction from the scale's obox2d, set_upper, upper, init,
 * update, clear, border_needed, detector() with set_n / set_fast_threshold
 * (fast_detector.hpp:170-193), and the frequency / k / merge setters, which
 * take effect at any time with the reference's scope (pyrlk_cpu's set_k sets
 * its own scale only; generic_strategy's forwards to the coarser scales).
 *
 * The scales share one GPU context.  The finest scale's update() uploads the
 * frame and advances every scale in one gbt_run; the coarser scales' update()
 * calls (which come first) only remember their particle containers.  After the
 * run, every scale's pset() is loaded from the GPU -- particles, features,
 * matches, compact_has_run() and the sparse index -- so that callers read
 * dense_particles(), features(), matches(), call sync_attributes()
 * (particle_container.hpp:514-553) and nparticles() exactly as with
 * bc2s_fast_gradient_cpu.  Errors throw std::runtime_error, as the reference's
 * check_cuda_error() does (cuimg/error.h:17-29).
 *
 * Use: include the cuimg headers as usual, then this file; change the
 * strategy name, e.g. in samples/tracking/main.cc:101
 *     typedef tracker<tracking_strategies::bc2s_fast_gradient_gb300> T1;
 * and link libcuimg_gb300.so.  Nothing else in the caller changes.  (pyrlk_gb300's
 * particle set has the reference's particle_f<translation_transform>
 * particles and an empty feature of its own, gb300::no_feature, in place of
 * pyrlk_tracker.h's dummy_feature, so that this header needs no Eigen.)
 *
 * The host pyramid that tracker<F>::update_input still builds
 * (tracker.hpp:53-69) is not used by the GPU path.
 */
#ifndef CUIMG_GB300_STRATEGY_HPP_
#define CUIMG_GB300_STRATEGY_HPP_

#include <cmath>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuimg/cpu/host_image2d.h>
#include <cuimg/gl.h>
#include <cuimg/tracking2/tracker.h>

#include "cuimg_gb300.h"

namespace cuimg {
namespace tracking_strategies {
namespace gb300 {

// Throws std::runtime_error with the context's last error when a call fails.
inline void check(int status, gbt_ctx* ctx, const char* what) {
  if (status == GBT_OK) return;
  std::string msg = std::string("cuimg_gb300: ") + what + " failed (status " + std::to_string(status) + ")";
  if (ctx) {
    char buf[512] = {0};
    gbt_last_error(ctx, buf, sizeof buf);
    if (buf[0]) msg += std::string(": ") + buf;
  }
  throw std::runtime_error(msg);
}

// One scale's particle state as the C ABI returns it after a frame.
struct scale_state {
  std::vector<float> speed;      // 2 per slot (row, col)
  std::vector<int16_t> pos;      // 2 per slot (row, col)
  std::vector<uint16_t> age;     // 1 per slot; 0 = dead slot
  std::vector<uint8_t> features; // 16 per slot: s1 ring samples, then s2 ring samples
  std::vector<int32_t> matches;  // old slot -> new slot of the last compaction, -1 = died
  bool compacted = false;        // the frame ran a compaction (compact_has_run())
  int rows = 0, cols = 0;
  std::vector<uint32_t> sparse;  // slot index per pixel, 0xFFFFFFFF = none
};

// Reads (stream, scale) of a context into `st`.
inline void read_scale_state(gbt_ctx* ctx, int stream, int scale, int rows, int cols, scale_state& st) {
  int32_t n = 0, nm = 0, comp = 0;
  check(gbt_nparticles(ctx, stream, scale, &n), ctx, "gbt_nparticles");
  check(gbt_get_particles(ctx, stream, scale, nullptr, nullptr, nullptr, nullptr, nullptr, &nm, &comp), ctx,
        "gbt_get_particles");
  st.speed.resize(2 * (size_t)n);
  st.pos.resize(2 * (size_t)n);
  st.age.resize(n);
  st.features.resize(16 * (size_t)n);
  st.matches.resize(nm);
  check(gbt_get_particles(ctx, stream, scale, st.speed.data(), st.pos.data(), st.age.data(), st.features.data(),
                          st.matches.data(), &nm, &comp),
        ctx, "gbt_get_particles");
  st.matches.resize(nm);
  st.compacted = comp != 0;
  st.rows = rows;
  st.cols = cols;
  st.sparse.resize((size_t)rows * cols);
  check(gbt_get_stage(ctx, stream, scale, GBT_STAGE_SPARSE, 0, st.sparse.data()), ctx, "gbt_get_stage");
}

// Makes the reference's particle_container `pset` hold `st` as it would
// after the same frame on the CPU strategy.  compact_has_run() can only be
// set by the container itself: before_matching() clears it
// (particle_container.hpp:188-193) and compact() sets it and rebuilds
// matches() (:217-252).  So a compacting frame is replayed: the slots are laid
// out as they stood before the compaction (each survivor at its old slot,
// other slots empty) and the container compacts them; survivors the filter
// removed after the compaction keep a live age through it and get their final
// age afterwards.
template <typename PS>
void load_pset(const scale_state& st, PS& pset) {
  typedef typename PS::particle_type P;
  typedef typename PS::feature_type FV;
  const size_t n = st.age.size();
  auto particle_of = [&](size_t j) {
    P p;
    p.speed = i_float2(st.speed[2 * j], st.speed[2 * j + 1]);
    p.pos = i_short2(st.pos[2 * j], st.pos[2 * j + 1]);
    p.age = st.age[j];
    p.fault = 0;
    p.prev_match_time = 0;
    p.next_match_time = 0;
    return p;
  };
  auto feature_of = [&](size_t j) {
    FV f;
    for (int k = 0; k < 16; k++) {
      f.distances[k] = st.features[16 * j + k];
      f.weights[k] = 255;
    }
    return f;
  };
  pset.before_matching();
  auto& parts = pset.dense_particles();
  auto& feats = pset.features();
  if (st.compacted) {
    const size_t m = st.matches.size();
    parts.assign(m, P());
    feats.assign(m, FV());
    for (size_t i = 0; i < m; i++) {
      const int j = st.matches[i];
      if (j < 0) continue;
      if ((size_t)j >= n) throw std::runtime_error("cuimg_gb300: compaction map points past the particles");
      parts[i] = particle_of(j);
      parts[i].age = 1;  // alive through the compaction; final age below
      feats[i] = feature_of(j);
    }
    pset.compact();
    if (parts.size() != n) throw std::runtime_error("cuimg_gb300: compaction map does not match the particles");
    for (size_t j = 0; j < n; j++) parts[j].age = st.age[j];
  } else {
    parts.resize(n);
    feats.resize(n);
    for (size_t j = 0; j < n; j++) {
      parts[j] = particle_of(j);
      feats[j] = feature_of(j);
    }
    auto& mv = pset.matches();  // the last compaction's map, as the CPU strategy keeps it
    mv.resize(st.matches.size());
    for (size_t i = 0; i < st.matches.size(); i++) mv[i] = (unsigned)st.matches[i];
  }
  auto& sp = pset.sparse_particles();
  for (int r = 0; r < st.rows; r++)
    for (int c = 0; c < st.cols; c++) sp(r, c) = st.sparse[(size_t)r * st.cols + c];
  pset.tick();
}

// The LK matcher's particles: sub-pixel positions and speeds.
struct lk_scale_state {
  std::vector<float> pos, speed;  // 2 per slot (row, col)
  std::vector<uint16_t> age;
  std::vector<int32_t> matches;
  bool compacted = false;
  int rows = 0, cols = 0;
  std::vector<uint32_t> sparse;
};

inline void read_scale_state(gbt_ctx* ctx, int stream, int scale, int rows, int cols, lk_scale_state& st) {
  int32_t n = 0, nm = 0, comp = 0;
  check(gbt_nparticles(ctx, stream, scale, &n), ctx, "gbt_nparticles");
  check(gbt_get_particles_f(ctx, stream, scale, nullptr, nullptr, nullptr, nullptr, &nm, &comp), ctx,
        "gbt_get_particles_f");
  st.pos.resize(2 * (size_t)n);
  st.speed.resize(2 * (size_t)n);
  st.age.resize(n);
  st.matches.resize(nm);
  check(gbt_get_particles_f(ctx, stream, scale, st.pos.data(), st.speed.data(), st.age.data(), st.matches.data(),
                            &nm, &comp),
        ctx, "gbt_get_particles_f");
  st.matches.resize(nm);
  st.compacted = comp != 0;
  st.rows = rows;
  st.cols = cols;
  st.sparse.resize((size_t)rows * cols);
  check(gbt_get_stage(ctx, stream, scale, GBT_STAGE_SPARSE, 0, st.sparse.data()), ctx, "gbt_get_stage");
}

// The empty feature of pyrlk_gb300's particle set (pyrlk_tracker.h:13-17's
// dummy_feature, restated so that this header needs no Eigen).
struct no_feature {
  typedef int value_type;
  int operator()(i_int2) const { return 0; }
};

// load_pset for particle_f particles (particle_container.h:45-57), the same
// compaction replay.
template <typename PS>
void load_pset(const lk_scale_state& st, PS& pset) {
  typedef typename PS::particle_type P;
  typedef typename PS::feature_type FV;
  const size_t n = st.age.size();
  auto particle_of = [&](size_t j) {
    P p;
    p.speed = i_float2(st.speed[2 * j], st.speed[2 * j + 1]);
    p.pos = i_float2(st.pos[2 * j], st.pos[2 * j + 1]);
    p.age = st.age[j];
    return p;
  };
  pset.before_matching();
  auto& parts = pset.dense_particles();
  auto& feats = pset.features();
  if (st.compacted) {
    const size_t m = st.matches.size();
    parts.assign(m, P());
    feats.assign(m, FV());
    for (size_t i = 0; i < m; i++) {
      const int j = st.matches[i];
      if (j < 0) continue;
      if ((size_t)j >= n) throw std::runtime_error("cuimg_gb300: compaction map points past the particles");
      parts[i] = particle_of(j);
      parts[i].age = 1;  // alive through the compaction; final age below
    }
    pset.compact();
    if (parts.size() != n) throw std::runtime_error("cuimg_gb300: compaction map does not match the particles");
    for (size_t j = 0; j < n; j++) parts[j].age = st.age[j];
  } else {
    parts.resize(n);
    feats.assign(n, FV());
    for (size_t j = 0; j < n; j++) parts[j] = particle_of(j);
    auto& mv = pset.matches();
    mv.resize(st.matches.size());
    for (size_t i = 0; i < st.matches.size(); i++) mv[i] = (unsigned)st.matches[i];
  }
  auto& sp = pset.sparse_particles();
  for (int r = 0; r < st.rows; r++)
    for (int c = 0; c < st.cols; c++) sp(r, c) = st.sparse[(size_t)r * st.cols + c];
  pset.tick();
}

// Per-scale settings, as generic_strategy and fast_detector hold them.
struct scale_params {
  int threshold = 20;  // fast_detector's threshold (the reference leaves it unset until set_fast_threshold)
  int n = 9;
  int detector_frequency = 1;
  int filtering_frequency = 1;
  int k = 300;
  int with_merge = 1;
};

// The GPU context shared by a tracker's scales (scale 0 = finest).
struct engine {
  std::vector<scale_params> params;
  std::vector<void*> psets;  // each scale's particles_type, remembered at its update()
  std::vector<obox2d> domains;
  gbt_ctx* ctx = nullptr;
  int device = 0;
  int matcher = GBT_MATCHER_BC2S;

  ~engine() {
    if (ctx) gbt_destroy(ctx);
  }

  // Sets `key` to `value` on scales [from, to) and, once the context runs,
  // on the GPU too.
  void set(int from, int to, int key, int value) {
    for (int s = from; s < to; s++) {
      int* f = field(params[s], key);
      *f = value;
      if (ctx) check(gbt_set_param(ctx, 0, s, key, value), ctx, "gbt_set_param");
    }
  }

  static int* field(scale_params& p, int key) {
    switch (key) {
      case GBT_PARAM_DETECTOR_THRESHOLD: return &p.threshold;
      case GBT_PARAM_DETECTOR_N: return &p.n;
      case GBT_PARAM_DETECTOR_FREQUENCY: return &p.detector_frequency;
      case GBT_PARAM_FILTERING_FREQUENCY: return &p.filtering_frequency;
      case GBT_PARAM_K: return &p.k;
      default: return &p.with_merge;
    }
  }

  void create() {
    const int L = (int)params.size();
    gbt_config c;
    gbt_config_default(&c, domains[0].nrows(), domains[0].ncols(), L);
    const scale_params& p0 = params[0];
    c.detector_threshold = p0.threshold;
    c.detector_n = p0.n;
    c.detector_frequency = p0.detector_frequency;
    c.filtering_frequency = p0.filtering_frequency;
    c.k = p0.k;
    c.with_merge = p0.with_merge;
    c.matcher = matcher;
    check(gbt_create(&c, 1, device, &ctx), nullptr, "gbt_create");
    static const int keys[] = {GBT_PARAM_DETECTOR_THRESHOLD, GBT_PARAM_DETECTOR_N, GBT_PARAM_DETECTOR_FREQUENCY,
                               GBT_PARAM_FILTERING_FREQUENCY, GBT_PARAM_K, GBT_PARAM_WITH_MERGE};
    for (int s = 1; s < L; s++)
      for (int key : keys) {
        const int v = *field(params[s], key), v0 = *field(params[0], key);
        if (v != v0) check(gbt_set_param(ctx, 0, s, key, v), ctx, "gbt_set_param");
      }
  }

  void destroy() {
    if (ctx) gbt_destroy(ctx);
    ctx = nullptr;
  }
};

}  // namespace gb300

// The detector() handle of a GB300 scale: fast_detector's setters, applied to
// this scale only, as the reference's per-scale detector objects are.
class gb300_fast_detector {
 public:
  gb300_fast_detector& set_n(unsigned n) {
    eng_->set(scale_, scale_ + 1, GBT_PARAM_DETECTOR_N, (int)n);
    return *this;
  }
  // The reference stores a float and compares the saliency with it truncated
  // (fast_detector.hpp:28,75) and births against it as a float (:251); both
  // agree for whole numbers, which is what this path takes.
  gb300_fast_detector& set_fast_threshold(float f) {
    if (!(f >= 0.f) || std::floor(f) != f)
      throw std::invalid_argument("cuimg_gb300: the FAST threshold must be a whole number >= 0");
    eng_->set(scale_, scale_ + 1, GBT_PARAM_DETECTOR_THRESHOLD, (int)f);
    return *this;
  }
  int border_needed() const { return 3; }

 private:
  template <typename T>
  friend class basic_gb300_strategy;
  gb300::engine* eng_ = nullptr;
  int scale_ = 0;
};

namespace gb300 {

// bc2s_fast_gradient_cpu's types and scopes.
struct bc2s_traits {
  typedef particle_container<bc2s_feature<cpu>, particle, cpu> particles_type;
  typedef scale_state state_type;
  static constexpr int matcher = GBT_MATCHER_BC2S;
  static constexpr int border = 6;        // bc2s_feature's 6 (bc2s_feature.h:85) > fast_detector's 3
  static constexpr bool k_forwards = true;  // generic_strategy::set_k (tracking_strategies.hpp:66-74)
};

// pyrlk_cpu<fast_detector<cpu>, iterative_lk_match_5x5>'s.
struct pyrlk_traits {
  typedef particle_container<no_feature, particle_f<translation_transform>, cpu> particles_type;
  typedef lk_scale_state state_type;
  static constexpr int matcher = GBT_MATCHER_LK;
  static constexpr int border = 3;          // pyrlk_cpu::border_needed: the detector's (pyrlk_tracker.hpp:822-827)
  static constexpr bool k_forwards = false;  // pyrlk_cpu::set_k (pyrlk_tracker.h:44)
};

}  // namespace gb300

template <typename T>
class basic_gb300_strategy {
 public:
  typedef basic_gb300_strategy<T> self;
  typedef host_image2d<gl8u> input;
  typedef typename T::particles_type particles_type;
  typedef typename particles_type::particle_type particle_type;
  typedef cpu architecture;
  typedef gb300_fast_detector detector_t;

  explicit basic_gb300_strategy(const obox2d& d) : eng_(std::make_shared<gb300::engine>()) {
    eng_->params.resize(1);
    eng_->psets.assign(1, nullptr);
    eng_->domains.assign(1, d);
    eng_->matcher = T::matcher;
    bind();
  }
  basic_gb300_strategy(const self&) = delete;
  self& operator=(const self&) = delete;

  // tracker<F> links scale s to scale s + 1 after building the coarser
  // trackers (tracker.hpp:11-43), so the finest scale joins last: it takes
  // over the coarser scales' shared state as its scale 0.
  void set_upper(self* u) {
    upper_ = u;
    u->lower_ = this;
    std::shared_ptr<gb300::engine> e = u->eng_;
    e->params.insert(e->params.begin(), eng_->params[0]);
    e->psets.insert(e->psets.begin(), nullptr);
    e->domains.insert(e->domains.begin(), eng_->domains[0]);
    eng_ = e;
    scale_ = 0;
    for (self* p = u; p; p = p->upper_) p->scale_++;
    for (self* p = this; p; p = p->upper_) p->bind();
  }
  self* upper() { return upper_; }
  void init() {}

  // The frequencies apply to this scale and every coarser one
  // (tracking_strategies.hpp:56-82, pyrlk_tracker.hpp:795-815), with_merge to
  // this scale, k as the traits say.
  self& set_detector_frequency(unsigned nframe) {
    eng_->set(scale_, (int)eng_->params.size(), GBT_PARAM_DETECTOR_FREQUENCY, (int)nframe);
    return *this;
  }
  self& set_filtering_frequency(unsigned nframe) {
    eng_->set(scale_, (int)eng_->params.size(), GBT_PARAM_FILTERING_FREQUENCY, (int)nframe);
    return *this;
  }
  self& set_k(int k) {
    eng_->set(scale_, T::k_forwards ? (int)eng_->params.size() : scale_ + 1, GBT_PARAM_K, k);
    return *this;
  }
  void set_with_merge(bool b) { eng_->set(scale_, scale_ + 1, GBT_PARAM_WITH_MERGE, b ? 1 : 0); }
  // The GPU the scales run on (default 0); takes effect at the next context.
  void set_device(int device) { eng_->device = device; }

  detector_t& detector() { return detector_; }
  int border_needed() const { return T::border; }

  void update(const input& in, particles_type& pset) {
    gb300::engine& e = *eng_;
    e.psets[scale_] = &pset;
    if (scale_ != 0) return;  // coarser scales run inside the finest scale's gbt_run
    if (!e.ctx) e.create();
    const uint8_t* frame = (const uint8_t*)&in(0, 0);
    const int64_t pitch = (int64_t)in.pitch();
    gb300::check(gbt_run(e.ctx, &frame, &pitch, GBT_FRAMES_HOST), e.ctx, "gbt_run");
    for (size_t s = 0; s < e.params.size(); s++) {
      if (!e.psets[s]) continue;
      gb300::read_scale_state(e.ctx, 0, (int)s, e.domains[s].nrows(), e.domains[s].ncols(), state_);
      gb300::load_pset(state_, *(particles_type*)e.psets[s]);
    }
  }

  // tracker<F>::clear (tracker.hpp:94-102) clears every scale's strategy and
  // particle set; the next frame starts a fresh context (frame counter 0).
  void clear() {
    if (scale_ == 0) eng_->destroy();
  }

  // The shared GPU context (for callers that also want the C ABI's extras:
  // device-side trajectories, checkpoints, stage images).
  gbt_ctx* context() const { return eng_->ctx; }

 private:
  void bind() {
    detector_.eng_ = eng_.get();
    detector_.scale_ = scale_;
  }

  std::shared_ptr<gb300::engine> eng_;
  int scale_ = 0;
  self* upper_ = nullptr;
  self* lower_ = nullptr;
  detector_t detector_;
  typename T::state_type state_;
};

typedef basic_gb300_strategy<gb300::bc2s_traits> bc2s_fast_gradient_gb300;
typedef basic_gb300_strategy<gb300::pyrlk_traits> pyrlk_gb300;

}  // namespace tracking_strategies
}  // namespace cuimg

#endif  // CUIMG_GB300_STRATEGY_HPP_
