// The reference sample's tracking loop (samples/tracking/main.cc:94-128,
// without its OpenCV capture and display) with the strategy name changed to
// tracking_strategies::bc2s_fast_gradient_gb300 -- the drop-in use of
// include/cuimg_gb300_strategy.hpp.  Built by tests/test_cpp_boundary.py
// against the reference headers, the oracle/shim stand-ins for Boost / Eigen
// and libcuimg_gb300.so.
//
// Reads `nframes` gray rows x cols frames from a raw file, runs
// tracker<bc2s_fast_gradient_gb300>, keeps per-scale trajectories with
// pset().sync_attributes as the sample does, and writes, per frame and scale,
// the particle count and the live particles' positions and ages to the output
// file.  Exits 3 with the strategy's error message when the GPU path cannot run
// (no GPU, or the library reports a failure).
#include <cassert>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <exception>
#include <vector>

#include <cuimg/profiler.h>
#include <cuimg/dsl/all.h>
#include <cuimg/cpu/host_image2d.h>
#include <cuimg/tracking2/tracker.h>

#include "cuimg_gb300_strategy.hpp"

// The GB300 strategy the loop runs (bc2s_fast_gradient_gb300 unless the build
// names another, e.g. -DSAMPLE_STRATEGY=pyrlk_gb300).
#ifndef SAMPLE_STRATEGY
#define SAMPLE_STRATEGY bc2s_fast_gradient_gb300
#endif

using namespace cuimg;

struct trajectory {
  trajectory() : alive(true) {}
  std::deque<i_int2> history;
  bool alive;
};

template <typename TR>
void update_trajectories(std::vector<trajectory>& v, TR& pset) {
  const auto& parts = pset.dense_particles();
  for (unsigned i = 0; i < v.size(); i++) {
    v[i].alive = parts[i].age > 0;
    if (parts[i].age > 0) {
      v[i].history.push_back(i_int2(parts[i].pos));  // i_int2 of a float position truncates, as in the sample
      if (v[i].history.size() > 20) v[i].history.pop_front();
    } else {
      v[i].history.clear();
    }
  }
}

int main(int argc, char** argv) {
  if (argc != 8) {
    std::fprintf(stderr, "usage: %s rows cols nscales threshold nframes frames.raw out.txt\n", argv[0]);
    return 2;
  }
  const int rows = std::atoi(argv[1]), cols = std::atoi(argv[2]), NSCALES = std::atoi(argv[3]);
  const int detector_threshold = std::atoi(argv[4]), nframes = std::atoi(argv[5]);
  std::vector<uint8_t> clip((size_t)rows * cols * nframes);
  FILE* f = std::fopen(argv[6], "rb");
  if (!f || std::fread(clip.data(), 1, clip.size(), f) != clip.size()) return 2;
  std::fclose(f);
  FILE* out = std::fopen(argv[7], "w");
  if (!out) return 2;

  obox2d domain(rows, cols);
  host_image2d<gl8u> frame_gl(domain);
  try {
    // Tracker definition: the only line that differs from the sample.
    typedef tracker<tracking_strategies::SAMPLE_STRATEGY> T1;
    T1 tr1(domain, NSCALES);

    // Tracker settings, as the sample makes them.
    tr1.strategy().set_detector_frequency(10);
    tr1.strategy().set_filtering_frequency(1);
    for (int s = 0; s < NSCALES; s++) tr1.scale(s).strategy().detector().set_n(9).set_fast_threshold(detector_threshold);

    std::vector<std::vector<trajectory> > trajectories(NSCALES);
    for (int t = 0; t < nframes; t++) {
      for (int r = 0; r < rows; r++) std::memcpy(&frame_gl(r, 0), clip.data() + ((size_t)t * rows + r) * cols, cols);
      tr1.run(frame_gl);
      for (int s = 0; s < NSCALES; s++) {
        tr1.scale(s).pset().sync_attributes(trajectories[s], trajectory());
        update_trajectories(trajectories[s], tr1.scale(s).pset());
        const auto& parts = tr1.scale(s).pset().dense_particles();
        size_t longest = 0;
        for (const trajectory& tj : trajectories[s]) longest = tj.history.size() > longest ? tj.history.size() : longest;
        std::fprintf(out, "frame %d scale %d n %d compact %d longest %zu\n", t, s, tr1.scale(s).pset().size(),
                     (int)tr1.scale(s).pset().compact_has_run(), longest);
        for (size_t i = 0; i < parts.size(); i++)
          std::fprintf(out, "%g %g %d\n", (double)parts[i].pos.x, (double)parts[i].pos.y, parts[i].age);
      }
    }
    std::printf("ok frames=%d particles=%u\n", nframes, tr1.nparticles());
  } catch (const std::exception& e) {
    std::printf("error: %s\n", e.what());
    std::fclose(out);
    return 3;
  }
  std::fclose(out);
  return 0;
}
