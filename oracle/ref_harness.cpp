// Reference harness -- TEST INFRASTRUCTURE ONLY (never shipped).
//
// Compiles matt-42/cuimg's own CPU tracker
// `tracker<tracking_strategies::bc2s_fast_gradient_cpu>`
// (cuimg/tracking2/tracker.hpp, cuimg/tracking2/tracking_strategies.hpp) unchanged,
// from the reference sources where they lie, with the self-written compat
// shim in oracle/shim (Boost / Eigen stand-ins), and exposes it through a
// small C ABI so the Python tests can drive it with ctypes and read every
// intermediate stage back.  Built by oracle/Makefile into oracle/_ref/.
//
// Build flags mirror the reference's CPU configuration: -DNO_CUDA -DNDEBUG,
// no WITH_OPENCV (so bc2s_feature<cpu>::update takes the integer binomial
// blur branch, cuimg/tracking2/bc2s_feature.hpp:248-251), OpenMP enabled but
// run with one thread (the reference's parallel matcher and merge are racy,
// so the single-threaded order is the deterministic semantics).
//
// Uninitialised memory: the reference allocates images with `new char[]`
// (cuimg/cpu/host_image2d.hpp:97) and never writes the outer ring of the
// binomial blur outputs (cuimg/cpu/gaussian_blur.h:17,30).  This harness
// replaces the global allocation operators with zero-filling ones, which
// pins those never-written pixels to 0.  The CUDA path reproduces exactly
// that.

#include <cassert>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <new>

void* operator new(std::size_t n) {
  void* p = std::calloc(1, n ? n : 1);
  if (!p) throw std::bad_alloc();
  return p;
}
void* operator new[](std::size_t n) {
  void* p = std::calloc(1, n ? n : 1);
  if (!p) throw std::bad_alloc();
  return p;
}
void operator delete(void* p) noexcept { std::free(p); }
void operator delete[](void* p) noexcept { std::free(p); }
void operator delete(void* p, std::size_t) noexcept { std::free(p); }
void operator delete[](void* p, std::size_t) noexcept { std::free(p); }

#include <cuimg/profiler.h>
#include <cuimg/dsl/all.h>
#include <cuimg/cpu/host_image2d.h>
#include <cuimg/cpu/fill.h>
#include <cuimg/tracking2/tracker.h>
#include <cuimg/tracking2/pyrlk_tracker.h>

using namespace cuimg;

typedef tracking_strategies::bc2s_fast_gradient_cpu S;
typedef tracker<S> T;
typedef S::super G;  // generic_strategy<...>

// Legal access to the strategy's protected stage buffers: a pointer to a
// protected base member may be formed inside a derived class.
struct peek : public S {
  static host_image2d<unsigned int> G::*contrast() { return &peek::contrast_; }
  static host_image2d<gl8u> G::*mask() { return &peek::mask_; }
  static host_image2d<i_float2> G::*flow() { return &peek::flow_; }
  static host_image2d<unsigned int> G::*mscount() { return &peek::multiscale_count_; }
  static host_image2d<std::pair<int, i_int2> > G::*stats() { return &peek::flow_stats_; }
  static int G::*frame() { return &peek::frame_cpt_; }
};

struct ref_ctx {
  T* tr;
  int nscales;
  obox2d dom;
};

// Copy rows [-b, nrows+b) x cols [-b, ncols+b) of an image into `out`.
template <typename V, typename O>
static void dump(const host_image2d<V>& img, int b, O* out) {
  int nr = img.nrows(), nc = img.ncols();
  size_t k = 0;
  for (int r = -b; r < nr + b; r++)
    for (int cc = -b; cc < nc + b; cc++)
      out[k++] = (O)img(r, cc).x;
}

extern "C" {

void* ref_create(int rows, int cols, int nscales, int threshold,
                 int detector_frequency, int filtering_frequency) {
  ref_ctx* c = new ref_ctx;
  c->dom = obox2d(rows, cols);
  c->nscales = nscales;
  c->tr = new T(c->dom, nscales);
  c->tr->strategy().set_detector_frequency(detector_frequency);
  c->tr->strategy().set_filtering_frequency(filtering_frequency);
  for (int s = 0; s < nscales; s++)
    c->tr->scale(s).strategy().detector().set_n(9).set_fast_threshold(threshold);
  return c;
}

void ref_destroy(void* h) {
  ref_ctx* c = (ref_ctx*)h;
  delete c->tr;
  delete c;
}

// The reference's own setter of scale `scale`, called between frames: 0
// detector().set_fast_threshold, 1 detector().set_n, 2 set_detector_frequency,
// 3 set_filtering_frequency, 4 set_k (these three also set every coarser
// scale, tracking_strategies.hpp:56-82), 5 set_with_merge.
int ref_set_param(void* h, int scale, int key, int value) {
  ref_ctx* c = (ref_ctx*)h;
  if (scale < 0 || scale >= c->nscales) return -1;
  S& st = c->tr->scale(scale).strategy();
  switch (key) {
    case 0: st.detector().set_fast_threshold(value); break;
    case 1: st.detector().set_n(value); break;
    case 2: st.set_detector_frequency(value); break;
    case 3: st.set_filtering_frequency(value); break;
    case 4: st.set_k(value); break;
    case 5: st.set_with_merge(value != 0); break;
    default: return -1;
  }
  return 0;
}

void ref_run(void* h, const uint8_t* frame) {
  ref_ctx* c = (ref_ctx*)h;
  host_image2d<gl8u> in(c->dom);
  for (int r = 0; r < c->dom.nrows(); r++)
    std::memcpy(&in(r, 0), frame + (size_t)r * c->dom.ncols(), c->dom.ncols());
  c->tr->run(in);
}

void ref_dims(void* h, int scale, int* rows, int* cols) {
  ref_ctx* c = (ref_ctx*)h;
  const obox2d& d = c->tr->scale(scale).domain();
  *rows = d.nrows();
  *cols = d.ncols();
}

// Pyramid level (tracker input) with `b` border pixels.
void ref_get_input(void* h, int scale, int b, uint8_t* out) {
  ref_ctx* c = (ref_ctx*)h;
  dump(c->tr->scale(scale).input(), b, out);
}

void ref_get_s1(void* h, int scale, int b, uint8_t* out) {
  ref_ctx* c = (ref_ctx*)h;
  dump(c->tr->scale(scale).strategy().feature().s1(), b, out);
}

void ref_get_s2(void* h, int scale, int b, uint8_t* out) {
  ref_ctx* c = (ref_ctx*)h;
  dump(c->tr->scale(scale).strategy().feature().s2(), b, out);
}

void ref_get_saliency(void* h, int scale, uint8_t* out) {
  ref_ctx* c = (ref_ctx*)h;
  dump(c->tr->scale(scale).strategy().detector().saliency(), 0, out);
}

void ref_get_contrast(void* h, int scale, uint32_t* out) {
  ref_ctx* c = (ref_ctx*)h;
  G& g = c->tr->scale(scale).strategy();
  const host_image2d<unsigned int>& img = g.*peek::contrast();
  for (int r = 0; r < img.nrows(); r++)
    for (int cc = 0; cc < img.ncols(); cc++)
      out[(size_t)r * img.ncols() + cc] = img(r, cc);
}

void ref_get_mask(void* h, int scale, uint8_t* out) {
  ref_ctx* c = (ref_ctx*)h;
  G& g = c->tr->scale(scale).strategy();
  dump(g.*peek::mask(), 0, out);
}

// Flow-bin images: flow (float2), multiscale count, stats (count, last speed).
void ref_bins(void* h, int scale, int* rows, int* cols) {
  ref_ctx* c = (ref_ctx*)h;
  G& g = c->tr->scale(scale).strategy();
  *rows = (g.*peek::flow()).nrows();
  *cols = (g.*peek::flow()).ncols();
}

void ref_get_bins(void* h, int scale, float* flow, uint32_t* count,
                  int32_t* stat_n, int32_t* stat_speed) {
  ref_ctx* c = (ref_ctx*)h;
  G& g = c->tr->scale(scale).strategy();
  const host_image2d<i_float2>& f = g.*peek::flow();
  const host_image2d<unsigned int>& m = g.*peek::mscount();
  const host_image2d<std::pair<int, i_int2> >& st = g.*peek::stats();
  size_t k = 0;
  for (int r = 0; r < f.nrows(); r++)
    for (int cc = 0; cc < f.ncols(); cc++, k++) {
      flow[2 * k] = f(r, cc).x;
      flow[2 * k + 1] = f(r, cc).y;
      count[k] = m(r, cc);
      stat_n[k] = st(r, cc).first;
      stat_speed[2 * k] = st(r, cc).second.x;
      stat_speed[2 * k + 1] = st(r, cc).second.y;
    }
}

int ref_frame_count(void* h, int scale) {
  ref_ctx* c = (ref_ctx*)h;
  G& g = c->tr->scale(scale).strategy();
  return g.*peek::frame();
}

int ref_nparticles(void* h, int scale) {
  ref_ctx* c = (ref_ctx*)h;
  return c->tr->scale(scale).pset().size();
}

int ref_total_particles(void* h) {
  ref_ctx* c = (ref_ctx*)h;
  return c->tr->nparticles();
}

int ref_compact_has_run(void* h, int scale) {
  ref_ctx* c = (ref_ctx*)h;
  return c->tr->scale(scale).pset().compact_has_run();
}

// Particle state: speed (2 floats), pos (2 int16: row, col), age (uint16).
// Features: 16 distances + 16 weights (uint8).  Matches: int32 per slot.
void ref_get_particles(void* h, int scale, float* speed, int16_t* pos,
                       uint16_t* age, uint8_t* feat, int32_t* matches,
                       int* nmatches) {
  ref_ctx* c = (ref_ctx*)h;
  auto& ps = c->tr->scale(scale).pset();
  const auto& P = ps.dense_particles();
  const auto& F = ps.features();
  for (size_t i = 0; i < P.size(); i++) {
    speed[2 * i] = P[i].speed.x;
    speed[2 * i + 1] = P[i].speed.y;
    pos[2 * i] = P[i].pos.x;
    pos[2 * i + 1] = P[i].pos.y;
    age[i] = P[i].age;
    for (int j = 0; j < 16; j++) {
      feat[32 * i + j] = F[i].distances[j];
      feat[32 * i + 16 + j] = F[i].weights[j];
    }
  }
  const auto& M = ps.matches();
  *nmatches = (int)M.size();
  if (matches)
    for (size_t i = 0; i < M.size(); i++) matches[i] = (int32_t)M[i];
}

// Sparse index image over the domain (uint32, 0xFFFFFFFF = empty).
void ref_get_sparse(void* h, int scale, uint32_t* out) {
  ref_ctx* c = (ref_ctx*)h;
  const auto& sp = c->tr->scale(scale).pset().sparse_particles();
  for (int r = 0; r < sp.nrows(); r++)
    for (int cc = 0; cc < sp.ncols(); cc++)
      out[(size_t)r * sp.ncols() + cc] = sp(r, cc);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// The reference's pyramidal LK tracker, tracker<pyrlk_cpu<fast_detector<cpu>,
// iterative_lk_match_5x5>> (cuimg/tracking2/pyrlk_tracker.h:16-82; never
// instantiated upstream).  Used with births on the first frame only and no
// filtering or merging, so that after the second frame a particle's age and
// position are exactly the LK acceptance and result for the detected point.
typedef tracking_strategies::pyrlk_cpu<fast_detector<cpu>, tracking_strategies::iterative_lk_match_5x5> LKS;
typedef tracker<LKS> LKT;

struct reflk_ctx {
  LKT* tr;
  obox2d dom;
};

extern "C" {

void* reflk_create(int rows, int cols, int nscales, int threshold) {
  reflk_ctx* c = new reflk_ctx;
  c->dom = obox2d(rows, cols);
  c->tr = new LKT(c->dom, nscales);
  c->tr->strategy().set_detector_frequency(1000);
  c->tr->strategy().set_filtering_frequency(1000);
  for (int s = 0; s < nscales; s++) {
    c->tr->scale(s).strategy().set_with_merge(false);
    c->tr->scale(s).strategy().detector().set_n(9).set_fast_threshold(threshold);
  }
  return c;
}

void reflk_destroy(void* h) {
  reflk_ctx* c = (reflk_ctx*)h;
  delete c->tr;
  delete c;
}

void reflk_run(void* h, const uint8_t* frame) {
  reflk_ctx* c = (reflk_ctx*)h;
  host_image2d<gl8u> in(c->dom);
  for (int r = 0; r < c->dom.nrows(); r++)
    std::memcpy(&in(r, 0), frame + (size_t)r * c->dom.ncols(), c->dom.ncols());
  c->tr->run(in);
}

int reflk_nparticles(void* h, int scale) {
  reflk_ctx* c = (reflk_ctx*)h;
  return c->tr->scale(scale).pset().size();
}

void reflk_get(void* h, int scale, float* pos, uint16_t* age) {
  reflk_ctx* c = (reflk_ctx*)h;
  const auto& P = c->tr->scale(scale).pset().dense_particles();
  for (size_t i = 0; i < P.size(); i++) {
    pos[2 * i] = P[i].pos.x;
    pos[2 * i + 1] = P[i].pos.y;
    age[i] = P[i].age;
  }
}

// The LK tracker as the sample would run it: detector every `det_freq`
// frames, filtering (and merging, when `with_merge`) every `filt_freq`.
void* reflk_create_full(int rows, int cols, int nscales, int threshold, int det_freq, int filt_freq, int with_merge) {
  reflk_ctx* c = new reflk_ctx;
  c->dom = obox2d(rows, cols);
  c->tr = new LKT(c->dom, nscales);
  c->tr->strategy().set_detector_frequency(det_freq);
  c->tr->strategy().set_filtering_frequency(filt_freq);
  for (int s = 0; s < nscales; s++) {
    c->tr->scale(s).strategy().set_with_merge(with_merge != 0);
    c->tr->scale(s).strategy().detector().set_n(9).set_fast_threshold(threshold);
  }
  return c;
}

// Full particle state of a scale: pos, speed (2 floats each), age, the last
// compaction's matches and whether this frame compacted.
void reflk_get_full(void* h, int scale, float* pos, float* speed, uint16_t* age, int32_t* matches, int* nmatches,
                    int* compact_has_run) {
  reflk_ctx* c = (reflk_ctx*)h;
  auto& ps = c->tr->scale(scale).pset();
  const auto& P = ps.dense_particles();
  for (size_t i = 0; i < P.size(); i++) {
    if (pos) {
      pos[2 * i] = P[i].pos.x;
      pos[2 * i + 1] = P[i].pos.y;
    }
    if (speed) {
      speed[2 * i] = P[i].speed.x;
      speed[2 * i + 1] = P[i].speed.y;
    }
    if (age) age[i] = P[i].age;
  }
  const auto& M = ps.matches();
  *nmatches = (int)M.size();
  if (matches)
    for (size_t i = 0; i < M.size(); i++) matches[i] = (int32_t)M[i];
  *compact_has_run = ps.compact_has_run();
}

void reflk_get_sparse(void* h, int scale, uint32_t* out) {
  reflk_ctx* c = (reflk_ctx*)h;
  const auto& sp = c->tr->scale(scale).pset().sparse_particles();
  for (int r = 0; r < sp.nrows(); r++)
    for (int cc = 0; cc < sp.ncols(); cc++) out[(size_t)r * sp.ncols() + cc] = sp(r, cc);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// The generic strategy with the reference's other detectors:
// tracker<bc2s_regular_gradient_cpu> (regular_detector) and
// tracker<bc2s_dense_gradient_cpu> (dense_detector),
// cuimg/tracking2/tracking_strategies.h:169-181,216-227.  Particles, features
// and matches only.
struct refx_base {
  virtual ~refx_base() {}
  virtual void run(const host_image2d<gl8u>& in) = 0;
  virtual int nparticles(int s) = 0;
  virtual int compact_has_run(int s) = 0;
  virtual void get(int s, float* speed, int16_t* pos, uint16_t* age, uint8_t* feat, int32_t* matches,
                   int* nmatches) = 0;
  obox2d dom;
};

template <typename ST>
struct refx_impl : refx_base {
  tracker<ST>* tr;
  ~refx_impl() { delete tr; }
  void run(const host_image2d<gl8u>& in) { tr->run(in); }
  int nparticles(int s) { return tr->scale(s).pset().size(); }
  int compact_has_run(int s) { return tr->scale(s).pset().compact_has_run(); }
  void get(int s, float* speed, int16_t* pos, uint16_t* age, uint8_t* feat, int32_t* matches, int* nmatches) {
    auto& ps = tr->scale(s).pset();
    const auto& P = ps.dense_particles();
    const auto& F = ps.features();
    for (size_t i = 0; i < P.size(); i++) {
      speed[2 * i] = P[i].speed.x;
      speed[2 * i + 1] = P[i].speed.y;
      pos[2 * i] = P[i].pos.x;
      pos[2 * i + 1] = P[i].pos.y;
      age[i] = P[i].age;
      for (int j = 0; j < 16; j++) {
        feat[32 * i + j] = F[i].distances[j];
        feat[32 * i + 16 + j] = F[i].weights[j];
      }
    }
    const auto& M = ps.matches();
    *nmatches = (int)M.size();
    if (matches)
      for (size_t i = 0; i < M.size(); i++) matches[i] = (int32_t)M[i];
  }
};

extern "C" {

// kind 1: regular (step, grad_th), kind 2: dense.
void* refx_create(int kind, int rows, int cols, int nscales, int detector_frequency, int filtering_frequency,
                  int step, int grad_th) {
  refx_base* b = nullptr;
  obox2d dom(rows, cols);
  if (kind == 1) {
    auto* x = new refx_impl<tracking_strategies::bc2s_regular_gradient_cpu>;
    x->tr = new tracker<tracking_strategies::bc2s_regular_gradient_cpu>(dom, nscales);
    x->tr->strategy().set_detector_frequency(detector_frequency);
    x->tr->strategy().set_filtering_frequency(filtering_frequency);
    for (int s = 0; s < nscales; s++) x->tr->scale(s).strategy().detector().set_step(step).set_grad_th(grad_th);
    b = x;
  } else if (kind == 2) {
    auto* x = new refx_impl<tracking_strategies::bc2s_dense_gradient_cpu>;
    x->tr = new tracker<tracking_strategies::bc2s_dense_gradient_cpu>(dom, nscales);
    x->tr->strategy().set_detector_frequency(detector_frequency);
    x->tr->strategy().set_filtering_frequency(filtering_frequency);
    b = x;
  }
  if (b) b->dom = dom;
  return b;
}

void refx_destroy(void* h) { delete (refx_base*)h; }

void refx_run(void* h, const uint8_t* frame) {
  refx_base* b = (refx_base*)h;
  host_image2d<gl8u> in(b->dom);
  for (int r = 0; r < b->dom.nrows(); r++)
    std::memcpy(&in(r, 0), frame + (size_t)r * b->dom.ncols(), b->dom.ncols());
  b->run(in);
}

int refx_nparticles(void* h, int s) { return ((refx_base*)h)->nparticles(s); }
int refx_compact_has_run(void* h, int s) { return ((refx_base*)h)->compact_has_run(s); }
void refx_get_particles(void* h, int s, float* speed, int16_t* pos, uint16_t* age, uint8_t* feat,
                        int32_t* matches, int* nmatches) {
  ((refx_base*)h)->get(s, speed, pos, age, feat, matches, nmatches);
}

}  // extern "C"
