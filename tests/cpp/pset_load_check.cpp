// Checks the GB300 strategy's particle-set loader (gb300::load_pset in
// include/cuimg_gb300_strategy.hpp) against the reference's own containers.
//
// Built by tests/test_cpp_boundary.py against the reference headers (with the
// oracle/shim stand-ins for Boost / Eigen) and the oracle library.  For every
// frame of a seeded clip it runs the reference's CPU tracker
// (tracker<bc2s_fast_gradient_cpu>) and the oracle side by side; it turns the
// oracle's state into the per-scale view the C ABI returns (gbt_get_particles
// + the sparse stage image: the GPU returns exactly the oracle's state, which
// the GPU parity tests check), loads it into one particle_container per scale
// with load_pset, and compares that container with the reference tracker's
// pset() of the same scale: dense particles, features, matches,
// compact_has_run(), the sparse index and frame_cpt().  It also runs the
// sample's trajectory bookkeeping (samples/tracking/main.cc:39-57,125-127:
// sync_attributes, then one history step per live particle) on both and
// compares the histories.  Exit status 0 when every frame and scale agrees.
#include <cassert>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <new>
#include <vector>

// Zero-filled allocations, as in oracle/ref_harness.cpp: the reference never
// writes the outer ring of its blur outputs, and the oracle pins it to 0.
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

#include "cuimg_gb300_strategy.hpp"

extern "C" {
void* oracle_create(int rows, int cols, int nscales, int threshold, int det_freq, int filt_freq);
void oracle_destroy(void* h);
int oracle_run(void* h, const uint8_t* frame);
int oracle_nparticles(void* h, int s);
int oracle_compact_has_run(void* h, int s);
void oracle_get_particles(void* h, int s, float* speed, int16_t* pos, uint16_t* age, uint8_t* feat,
                          int32_t* matches, int* nmatches);
void oracle_get_sparse(void* h, int s, uint32_t* out);
}

using namespace cuimg;

// A short position history per particle slot, kept in step with the slots.
struct history {
  std::deque<i_int2> pts;
};

template <typename PS>
static void step_histories(std::vector<history>& v, const PS& pset) {
  pset.sync_attributes(v, history());
  const auto& parts = pset.dense_particles();
  for (size_t i = 0; i < v.size(); i++) {
    if (parts[i].age > 0) {
      v[i].pts.push_back(i_int2(parts[i].pos));
      if (v[i].pts.size() > 20) v[i].pts.pop_front();
    } else {
      v[i].pts.clear();
    }
  }
}

static int fail(int t, int s, const char* what) {
  std::printf("MISMATCH frame %d scale %d: %s\n", t, s, what);
  return 1;
}

int main(int argc, char** argv) {
  if (argc != 7) {
    std::fprintf(stderr, "usage: %s rows cols nscales det_freq nframes frames.raw\n", argv[0]);
    return 2;
  }
  const int rows = std::atoi(argv[1]), cols = std::atoi(argv[2]), L = std::atoi(argv[3]);
  const int det_freq = std::atoi(argv[4]), nframes = std::atoi(argv[5]);
  std::vector<uint8_t> clip((size_t)rows * cols * nframes);
  FILE* f = std::fopen(argv[6], "rb");
  if (!f || std::fread(clip.data(), 1, clip.size(), f) != clip.size()) return 2;
  std::fclose(f);

  typedef tracking_strategies::bc2s_fast_gradient_cpu S;
  typedef tracker<S> T;
  typedef S::particles_type PS;
  const obox2d dom(rows, cols);
  T ref(dom, L);
  ref.strategy().set_detector_frequency(det_freq);
  ref.strategy().set_filtering_frequency(1);
  for (int s = 0; s < L; s++) ref.scale(s).strategy().detector().set_n(9).set_fast_threshold(20);
  void* o = oracle_create(rows, cols, L, 20, det_freq, 1);

  std::vector<PS*> loaded;
  std::vector<std::vector<int32_t>> last_matches(L);
  std::vector<std::vector<history>> h_ref(L), h_gb(L);
  for (int s = 0; s < L; s++) loaded.push_back(new PS(ref.scale(s).domain()));
  host_image2d<gl8u> frame(dom);
  tracking_strategies::gb300::scale_state st;
  int compactions = 0;
  for (int t = 0; t < nframes; t++) {
    for (int r = 0; r < rows; r++)
      std::memcpy(&frame(r, 0), clip.data() + ((size_t)t * rows + r) * cols, cols);
    ref.run(frame);
    oracle_run(o, clip.data() + (size_t)t * rows * cols);
    for (int s = 0; s < L; s++) {
      const PS& want = ref.scale(s).pset();
      const int n = oracle_nparticles(o, s), H = ref.scale(s).domain().nrows(), W = ref.scale(s).domain().ncols();
      // The C ABI's view of this scale.
      std::vector<uint8_t> feat32((size_t)n * 32 + 32);
      std::vector<int32_t> m((size_t)n * 8 + 64);
      int nm = 0;
      st.speed.resize(2 * (size_t)n);
      st.pos.resize(2 * (size_t)n);
      st.age.resize(n);
      oracle_get_particles(o, s, st.speed.data(), st.pos.data(), st.age.data(), feat32.data(), nullptr, &nm);
      m.resize(nm > 0 ? nm : 1);
      oracle_get_particles(o, s, st.speed.data(), st.pos.data(), st.age.data(), feat32.data(), m.data(), &nm);
      st.compacted = oracle_compact_has_run(o, s) != 0;
      if (st.compacted) last_matches[s].assign(m.begin(), m.begin() + nm);
      st.matches = last_matches[s];  // the ABI returns the last compaction's map on every frame
      st.features.resize(16 * (size_t)n);
      for (int i = 0; i < n; i++) std::memcpy(&st.features[16 * (size_t)i], &feat32[32 * (size_t)i], 16);
      st.rows = H;
      st.cols = W;
      st.sparse.resize((size_t)H * W);
      oracle_get_sparse(o, s, st.sparse.data());
      tracking_strategies::gb300::load_pset(st, *loaded[s]);
      compactions += st.compacted;

      const PS& got = *loaded[s];
      if (got.size() != want.size()) return fail(t, s, "size");
      if (got.compact_has_run() != want.compact_has_run()) return fail(t, s, "compact_has_run");
      for (int i = 0; i < got.size(); i++) {
        const particle& a = got.dense_particles()[i];
        const particle& b = want.dense_particles()[i];
        if (std::memcmp(&a.speed, &b.speed, sizeof a.speed) || a.pos != b.pos || a.age != b.age)
          return fail(t, s, "particle");
        const bc2s& fa = got.features()[i];
        const bc2s& fb = want.features()[i];
        if (std::memcmp(fa.distances, fb.distances, 16) || std::memcmp(fa.weights, fb.weights, 16))
          return fail(t, s, "feature");
      }
      if (got.matches().size() != want.matches().size()) return fail(t, s, "matches size");
      for (size_t i = 0; i < got.matches().size(); i++)
        if (got.matches()[i] != want.matches()[i]) return fail(t, s, "matches");
      for (int r = 0; r < H; r++)
        for (int c = 0; c < W; c++)
          if (got.sparse_particles()(r, c) != want.sparse_particles()(r, c)) return fail(t, s, "sparse index");
      if (const_cast<PS&>(got).frame_cpt() != const_cast<PS&>(want).frame_cpt()) return fail(t, s, "frame_cpt");
      step_histories(h_ref[s], want);
      step_histories(h_gb[s], got);
      if (h_ref[s].size() != h_gb[s].size()) return fail(t, s, "history count");
      for (size_t i = 0; i < h_ref[s].size(); i++)
        if (h_ref[s][i].pts != h_gb[s][i].pts) return fail(t, s, "history");
    }
  }
  std::printf("ok frames=%d scales=%d compactions=%d particles=%u\n", nframes, L, compactions, ref.nparticles());
  for (PS* p : loaded) delete p;
  oracle_destroy(o);
  return 0;
}
