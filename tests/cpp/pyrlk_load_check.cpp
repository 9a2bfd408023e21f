// Checks pyrlk_gb300's particle-set loader (gb300::load_pset for particle_f
// particles, include/cuimg_gb300_strategy.hpp) against the reference's own
// pyramidal LK tracker, tracker<pyrlk_cpu<fast_detector<cpu>,
// iterative_lk_match_5x5>> (cuimg/tracking2/pyrlk_tracker.h:16-82).
//
// Built by tests/test_cpp_boundary.py against the reference headers (with the
// oracle/shim stand-ins for Boost / Eigen) and the oracle library.  Every
// frame of a clip with a black margin (so that the reference's LK windows stay
// inside its images), it runs the reference tracker and the oracle's
// restatement, turns the oracle's state into the C ABI's view of each scale
// (gbt_get_particles_f + the sparse stage image; the GPU returns exactly the
// oracle's state, which the GPU tests check), loads it into a particle set of
// pyrlk_gb300's type and compares it with the reference tracker's pset():
// positions, speeds and ages of every slot, matches, compact_has_run(), the
// sparse index, frame_cpt() and a trajectory history kept through
// sync_attributes.  Exit status 0 when every frame and scale agrees.
#include <cassert>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <new>
#include <vector>

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

#include "cuimg_gb300_strategy.hpp"

extern "C" {
void* oracle_pyrlk_create(int rows, int cols, int nscales, int threshold, int det_freq, int filt_freq);
void oracle_pyrlk_destroy(void* h);
int oracle_pyrlk_run(void* h, const uint8_t* frame);
int oracle_pyrlk_nparticles(void* h, int s);
void oracle_pyrlk_get(void* h, int s, float* pos, float* speed, uint16_t* age, int32_t* matches, int* nmatches,
                      int* compact_has_run);
void oracle_pyrlk_get_sparse(void* h, int s, uint32_t* out);
}

using namespace cuimg;

struct history {
  std::deque<i_float2> pts;
};

template <typename PS>
static void step_histories(std::vector<history>& v, const PS& pset) {
  pset.sync_attributes(v, history());
  const auto& parts = pset.dense_particles();
  for (size_t i = 0; i < v.size(); i++) {
    if (parts[i].age > 0) {
      v[i].pts.push_back(parts[i].pos);
      if (v[i].pts.size() > 20) v[i].pts.pop_front();
    } else {
      v[i].pts.clear();
    }
  }
}

static bool same_history(const std::vector<history>& a, const std::vector<history>& b) {
  if (a.size() != b.size()) return false;
  for (size_t i = 0; i < a.size(); i++) {
    if (a[i].pts.size() != b[i].pts.size()) return false;
    for (size_t k = 0; k < a[i].pts.size(); k++)
      if (std::memcmp(&a[i].pts[k], &b[i].pts[k], sizeof(i_float2))) return false;
  }
  return true;
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

  typedef tracking_strategies::pyrlk_cpu<fast_detector<cpu>, tracking_strategies::iterative_lk_match_5x5> S;
  typedef tracker<S> T;
  typedef tracking_strategies::pyrlk_gb300::particles_type PS;
  const obox2d dom(rows, cols);
  T ref(dom, L);
  ref.strategy().set_detector_frequency(det_freq);
  ref.strategy().set_filtering_frequency(1);
  for (int s = 0; s < L; s++) ref.scale(s).strategy().detector().set_n(9).set_fast_threshold(20);
  void* o = oracle_pyrlk_create(rows, cols, L, 20, det_freq, 1);

  std::vector<PS*> loaded;
  std::vector<std::vector<history>> h_ref(L), h_gb(L);
  for (int s = 0; s < L; s++) loaded.push_back(new PS(ref.scale(s).domain()));
  host_image2d<gl8u> frame(dom);
  tracking_strategies::gb300::lk_scale_state st;
  int compactions = 0;
  for (int t = 0; t < nframes; t++) {
    for (int r = 0; r < rows; r++)
      std::memcpy(&frame(r, 0), clip.data() + ((size_t)t * rows + r) * cols, cols);
    ref.run(frame);
    oracle_pyrlk_run(o, clip.data() + (size_t)t * rows * cols);
    for (int s = 0; s < L; s++) {
      const auto& want = ref.scale(s).pset();
      const int n = oracle_pyrlk_nparticles(o, s), H = ref.scale(s).domain().nrows(), W = ref.scale(s).domain().ncols();
      int nm = 0, comp = 0;
      oracle_pyrlk_get(o, s, nullptr, nullptr, nullptr, nullptr, &nm, &comp);
      st.pos.resize(2 * (size_t)n);
      st.speed.resize(2 * (size_t)n);
      st.age.resize(n);
      st.matches.resize(nm);
      oracle_pyrlk_get(o, s, st.pos.data(), st.speed.data(), st.age.data(), st.matches.data(), &nm, &comp);
      st.compacted = comp != 0;
      st.rows = H;
      st.cols = W;
      st.sparse.resize((size_t)H * W);
      oracle_pyrlk_get_sparse(o, s, st.sparse.data());
      tracking_strategies::gb300::load_pset(st, *loaded[s]);
      compactions += st.compacted;

      const PS& got = *loaded[s];
      if (got.size() != want.size()) return fail(t, s, "size");
      if (got.compact_has_run() != want.compact_has_run()) return fail(t, s, "compact_has_run");
      for (int i = 0; i < got.size(); i++) {
        const auto& a = got.dense_particles()[i];
        const auto& b = want.dense_particles()[i];
        if (std::memcmp(&a.speed, &b.speed, sizeof a.speed) || std::memcmp(&a.pos, &b.pos, sizeof a.pos) ||
            a.age != b.age)
          return fail(t, s, "particle");
      }
      if (got.matches().size() != want.matches().size()) return fail(t, s, "matches size");
      for (size_t i = 0; i < got.matches().size(); i++)
        if (got.matches()[i] != want.matches()[i]) return fail(t, s, "matches");
      for (int r = 0; r < H; r++)
        for (int c = 0; c < W; c++)
          if (got.sparse_particles()(r, c) != want.sparse_particles()(r, c)) return fail(t, s, "sparse index");
      if (const_cast<PS&>(got).frame_cpt() != const_cast<S::particles_type&>(want).frame_cpt())
        return fail(t, s, "frame_cpt");
      step_histories(h_ref[s], want);
      step_histories(h_gb[s], got);
      if (!same_history(h_ref[s], h_gb[s])) return fail(t, s, "history");
    }
  }
  std::printf("ok frames=%d scales=%d compactions=%d particles=%u\n", nframes, L, compactions, ref.nparticles());
  for (PS* p : loaded) delete p;
  oracle_pyrlk_destroy(o);
  return 0;
}
