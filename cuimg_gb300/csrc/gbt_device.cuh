// Device-side data layout and helpers shared by the tracker kernels.
//
// The tracker state of one (stream, scale) pair -- a "unit" -- lives in HBM as:
//   level image   uint8, H x W, pitch ipitch (multiple of 64 B), no border:
//                 the reference's clamp-filled border (cuimg/border.h:128-137)
//                 is reproduced by clamping coordinates on read;
//   s1, s2        uint8 BC2S blurs with a zero border of RB rows / CB columns
//                 (the reference's never-written outer ring and clamp-filled
//                 border are all zero, cuimg/cpu/gaussian_blur.h:9-47);
//   occ, pmask    one 64-bit word per 8x8-pixel bin, bit (r&7)*8 + (c&7):
//                 "a particle moved here this frame" and the detector's
//                 particle mask (tracking_strategies.hpp:202-225);
//   idx           64-bit per pixel: (stamp << 32) | particle index, the
//                 reference's sparse index image (particle_container.h:172)
//                 without per-frame clearing -- an entry is current when its
//                 stamp belongs to the current frame;
//   bins          per 8x8 bin: stats count / last speed, flow, multiscale count;
//   particles     structure of arrays, double-buffered for compaction:
//                 pos (short2 row,col), speed (short2; integral on this path),
//                 age (uint16), feature (16 bytes).
#pragma once
#include <cstdint>
#include <cuda.h>  // CUtensorMap (the type only; the library does not link the driver API)
#include <cuda_runtime.h>

namespace gbt {

constexpr int RB = 8;    // rows of zero border around s1/s2
constexpr int CB = 16;   // columns of zero border around s1/s2
constexpr int CHUNK = 1024;  // particle slots per compaction chunk
// s1/s2 row pitch of every unit whose bordered width fits: a compile-time
// pitch turns the matcher's ring offsets into load immediates.
constexpr int FIXED_FPITCH = 4096;

struct Unit {
  int H, W;
  int stream, scale, nscales;
  int upper;        // unit index of scale + 1 of the same stream, -1 at the top
  int threshold, nfast, k, det_freq, filt_freq, with_merge;
  int det_kind, det_step, det_grad_th;  // GBT_DETECTOR_*, regular_detector step / grad_th
  int max_births;                       // births one detector frame can add
  int birth_items;                      // ordered birth candidates (3 x tiles for FAST, pixels otherwise)
  // images
  uint8_t* img;
  int ipitch;
  uint8_t* s1;
  uint8_t* s2;
  int fpitch;
  // bins
  int BH, BW;
  unsigned long long* occ;
  unsigned long long* pmask;
  unsigned long long* ppos;   // particle slot positions (detector frames, FAST)
  unsigned long long* idx;
  int* st_n;
  int2* st_sp;
  float2* flow;
  unsigned* msc;
  // particles
  short2* pos[2];
  short2* spd[2];
  unsigned short* age[2];
  uint4* feat[2];
  int* matches;
  int cap;
  int max_chunks;
  int* chunk_cnt;     // survivors per 32 slots (cap / 32), then offsets
  // detector
  int TH, TW;
  uint8_t* tilecode;  // TH * TW
  int birth_chunks;   // ceil(3 * TH * TW / CHUNK)
  int* birth_cnt;     // births per 32 items (birth_items / 32), then offsets
  // merge
  int* act_cnt;       // merge actives per 32 slots (cap / 32), then offsets
  uint8_t* cmask;     // cap candidate direction masks
  int4* act_list;     // cap entries: (i, pos packed, ncand, first cand) + cand store
  int* act_cand;      // cap * 8: an active slot's candidate slots, in c8_h order
  // matcher tiles (k_match_tiled)
  int MTR, MTC;       // tiles per column / row
  int mt_base;        // first tile of this unit in the context-wide tile arrays
  // trajectories (k_traj; null until enabled): position k of slot j's history
  // ring at tpos[b][k * cap + j], next write at thead, length tlen
  short2* tpos[2];
  uint8_t* thead[2];
  uint8_t* tlen[2];
};

// Frame ingest of one stream for the next frame: mode 0 = the gray frame is
// already in level 0; 1 = interleaved RGB at `rgb`, track channel 0 (get_x,
// dsl/get_comp.h:105); 2 = the same, BT.601 luma (77 R + 150 G + 29 B + 128) / 256.
// How k_pyramid gets a stream's level 0: mode 0 = already in the unit's image;
// 1 / 2 = from interleaved RGB at `rgb` (channel 0 / BT.601 luma); 3 = from a
// gray frame in device memory at `rgb` (the name covers both sources).
struct Ingest {
  const uint8_t* rgb;
  long long pitch;
  int mode;
  int pad;
};

// Mutable per-unit counters, kept on the device so that captured graphs replay.
struct UState {
  int n;         // particle slots in the current buffer
  int cur;       // current particle buffer (0/1)
  int nmatches;  // slots before the last compaction
  int compact;   // did this frame compact
  int n_old;     // slots before compaction (scratch)
  int S;         // survivors (scratch)
  int B;         // births (scratch)
  int A;         // merge actives (scratch)
};

struct Frame {
  int f;    // frames completed so far (the frame being processed)
  int err;  // error bits
};

constexpr int ERR_CAPACITY = 1;
constexpr int ERR_MERGE_OVERFLOW = 2;
constexpr int ERR_TIMEOUT = 4;  // a bounded wait on an asynchronous copy gave up
// ... and the copies were still in flight after a second bounded wait, when
// the CTA had to return: they may complete into shared memory that another
// CTA owns by then, so the context's results are no longer trustworthy.
constexpr int ERR_COPY_INFLIGHT = 8;

// c8_h in raster order (cuimg/neighb2d_data.h:80-85), (row, col).
__constant__ int8_t c_c8[8][2] = {{-1, 1}, {0, 1}, {1, 1}, {-1, 0}, {1, 0}, {-1, -1}, {0, -1}, {1, -1}};
// c8_it_h (cuimg/neighb2d_data.h:162-180).
__constant__ int8_t c_c8it[9][2] = {{6, 3}, {0, 3}, {0, 5}, {2, 5}, {2, 7}, {4, 7}, {4, 1}, {6, 1}, {0, 0}};
// circle_r3_h (cuimg/neighb2d_data.h:184-189).
__constant__ int8_t c_ring[16][2] = {{-3, 0}, {-3, 1}, {-2, 2}, {-1, 3}, {0, 3},   {1, 3},   {2, 2},   {3, 1},
                                     {3, 0},  {3, -1}, {2, -2}, {1, -3}, {0, -3}, {-1, -3}, {-2, -2}, {-3, -1}};
// The same ring as constant expressions (offsets fold into load immediates
// when the index and the pitch are compile-time constants).
__host__ __device__ constexpr int circle16_r(int i) {
  return i == 0 ? -3 : i == 1 ? -3 : i == 2 ? -2 : i == 3 ? -1 : i == 4 ? 0 : i == 5 ? 1 : i == 6 ? 2 : i == 7 ? 3
       : i == 8 ? 3 : i == 9 ? 3 : i == 10 ? 2 : i == 11 ? 1 : i == 12 ? 0 : i == 13 ? -1 : i == 14 ? -2 : -3;
}
__host__ __device__ constexpr int circle16_c(int i) { return circle16_r((i + 4) & 15); }

// fast::compute_saliency (tracking2/fast_detector.hpp:28-157) without
// branches, from the centre value vp and the 16 ring values (circle16 order).
// A ring pixel is "strong" when it differs from the centre by more than th
// (bright: above, dark: below); the reference scans the ring for the longest
// run of strong pixels of one sign, wrapping around (:95-146), and scores
// max(sum bright, sum dark) over all strong pixels (stored as gl8u).  Here the
// runs are tested on 16-bit masks doubled to 32 bits (so a run may wrap): a
// run of n_ exists iff the AND of the mask shifted by 0..n_-1 is non-zero.
// The reference's pre-test on ring pixels 0, 4, 8, 12 only rejects pixels the
// full test rejects too (a run of n_ >= 9 covers two cyclically adjacent ones
// of them, n_ >= 12 three), so it is left out.  th >= 0.
__device__ __forceinline__ int fast_score(const int (&ring)[16], int vp, int n_, int th) {
  unsigned B = 0, D = 0;
  int sb = 0, sd = 0;
#pragma unroll
  for (int i = 0; i < 16; i++) {
    const int d = ring[i] - vp;
    const bool br = d > th, dk = -d > th;
    B |= (unsigned)br << i;
    D |= (unsigned)dk << i;
    sb += br ? d : 0;
    sd += dk ? -d : 0;
  }
  if (n_ > 16) return 0;
  const unsigned MB = B | (B << 16), MD = D | (D << 16);
  unsigned xb, xd;
  if (n_ == 9) {  // runs of 2, 4, 8, then 9
    xb = MB & (MB >> 1);
    xd = MD & (MD >> 1);
    xb &= xb >> 2;
    xd &= xd >> 2;
    xb &= xb >> 4;
    xd &= xd >> 4;
    xb &= MB >> 8;
    xd &= MD >> 8;
  } else {
    xb = MB;
    xd = MD;
    for (int k = 1; k < n_; k++) {
      xb &= MB >> k;
      xd &= MD >> k;
    }
  }
  return (xb | xd) ? ((sb > sd ? sb : sd) & 255) : 0;
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Level image read with the reference's clamp-to-edge border semantics.
__device__ __forceinline__ int img_at(const Unit& u, int r, int c) {
  r = clampi(r, 0, u.H - 1);
  c = clampi(c, 0, u.W - 1);
  return u.img[(size_t)r * u.ipitch + c];
}

__device__ __forceinline__ const uint8_t* fptr(const uint8_t* base, int pitch, int r, int c) {
  return base + (size_t)(r + RB) * pitch + (c + CB);
}

__device__ __forceinline__ bool in_dom(const Unit& u, int r, int c) {
  return r >= 0 && r < u.H && c >= 0 && c < u.W;
}

__device__ __forceinline__ size_t bin_word(const Unit& u, int r, int c) {
  return (size_t)(r >> 3) * u.BW + (c >> 3);
}
__device__ __forceinline__ unsigned long long bin_bit(int r, int c) {
  return 1ull << (((r & 7) << 3) | (c & 7));
}

// Index-map stamps: frame f writes 2(f+1) during matching and 2(f+1)+1 for
// compaction, so that atomicMax resolves "last writer = highest index" within a
// phase and a later phase always wins; zero-initialised memory is never current.
__device__ __forceinline__ unsigned stamp_match(int f) { return 2u * (unsigned)(f + 1); }
__device__ __forceinline__ unsigned stamp_compact(int f) { return 2u * (unsigned)(f + 1) + 1u; }
__device__ __forceinline__ bool idx_current(unsigned long long e, int f) {
  return (unsigned)(e >> 33) == (unsigned)(f + 1);
}

// Unit lookup in a prefix table (first entry 0, nunits + 1 entries).
__device__ __forceinline__ int find_unit(const int* prefix, int nunits, int t) {
  int lo = 0, hi = nunits - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= t) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

}  // namespace gbt
