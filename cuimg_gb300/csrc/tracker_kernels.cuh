// Tracker kernels: one launch per stage processes every (stream, scale) unit.
// Each kernel cites the reference functor whose semantics it reproduces.
#pragma once
#include <type_traits>

#include "gbt_device.cuh"

namespace gbt {

// ---------------------------------------------------------------------------
// Block-wide exclusive prefix of a 0/1 predicate (blockDim.x a multiple of 32).
__device__ __forceinline__ int block_prefix(bool pred, int* warp_tot, int& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned b = __ballot_sync(0xffffffffu, pred);
  int local = __popc(b & ((1u << lane) - 1u));
  if (lane == 0) warp_tot[wid] = __popc(b);
  __syncthreads();
  if (wid == 0) {
    int v = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    warp_tot[32 + lane] = x - v;  // exclusive
    if (lane == 31) warp_tot[64] = x;
  }
  __syncthreads();
  int r = warp_tot[32 + wid] + local;
  total = warp_tot[64];
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------------------
// Pyramid: mipmap_kernel (cuimg/gpu/mipmap.h:24-49) applied level after level,
// out(p) = (a + b + c + d) / 4 over the 2x2 block at 2p.  One CTA of 256
// threads turns a 64 x 128 tile of level `base` into up to five coarser levels
// held in shared memory, so each frame is read from HBM once.  A thread loads
// two 16-byte chunks of the tile, both issued before either is stored, so that
// twice the bytes are in flight while the CTA waits on memory; eight CTAs fit
// on an SM (32 registers a thread).
constexpr int PYR_TR = 64, PYR_TC = 128, PYR_THREADS = 256;
constexpr int PYR_CPR = PYR_TC / 16, PYR_NCH = PYR_TR * PYR_CPR / PYR_THREADS;  // chunks per row / per thread
static_assert(PYR_TR * PYR_CPR % PYR_THREADS == 0, "whole chunks per thread");

// Four outputs (a + b + c + d) / 4 from 8 pixels of two rows (a, b: the upper
// and lower rows' bytes).  The even and odd bytes of each 32-bit half go to
// 16-bit lanes, where a sum of four bytes (at most 1020) cannot carry into the
// next lane.
__device__ __forceinline__ uint32_t pyr_mean2(uint32_t x, uint32_t y) {
  constexpr uint32_t LO = 0x00FF00FFu;
  return (((x & LO) + ((x >> 8) & LO) + (y & LO) + ((y >> 8) & LO)) >> 2) & LO;  // outputs in bytes 0 and 2
}
__device__ __forceinline__ uint32_t pyr_mean4(uint2 a, uint2 b) {
  return __byte_perm(pyr_mean2(a.x, b.x), pyr_mean2(a.y, b.y), 0x6420);
}

__global__ void __launch_bounds__(PYR_THREADS, 8) k_pyramid(const Unit* __restrict__ units,
                                                 const int* __restrict__ stream_unit0,
                                                 const int* __restrict__ tile_prefix, int nstreams, int base,
                                                 const Ingest* __restrict__ ingest) {
  __shared__ __align__(16) uint8_t sm[2][PYR_TR * PYR_TC];
  const int t = blockIdx.x;
  const int s = find_unit(tile_prefix, nstreams, t);
  const int local = t - tile_prefix[s];
  const int u0 = stream_unit0[s];
  const Unit& B = units[u0 + base];
  const int nlev = min(B.nscales - 1 - base, 5);
  const Ingest in = base == 0 ? ingest[s] : Ingest{nullptr, 0, 0, 0};
  if (nlev <= 0 && in.mode == 0) return;
  const int tw = (B.W + PYR_TC - 1) / PYR_TC;
  const int R0 = (local / tw) * PYR_TR, C0 = (local % tw) * PYR_TC;

  if (in.mode == 3) {
    // Fused ingest of a gray frame in device memory: level 0 copied into the
    // unit's image and the shared tile (16 bytes at a time where the source
    // chunk is aligned).
    uint4 x[PYR_NCH];
    bool vec[PYR_NCH];
#pragma unroll
    for (int k = 0; k < PYR_NCH; k++) {
      const int v = threadIdx.x + PYR_THREADS * k, gr = R0 + v / PYR_CPR, gc = C0 + (v % PYR_CPR) * 16;
      const uint8_t* src = in.rgb + (size_t)gr * in.pitch + gc;
      vec[k] = gr < B.H && gc + 16 <= B.W && ((uintptr_t)src & 15) == 0;
      if (vec[k]) x[k] = *(const uint4*)src;
    }
#pragma unroll
    for (int k = 0; k < PYR_NCH; k++) {
      const int v = threadIdx.x + PYR_THREADS * k;
      const int r = v / PYR_CPR, c16 = (v % PYR_CPR) * 16;
      const int gr = R0 + r, gc = C0 + c16;
      uint8_t* d = &sm[0][r * PYR_TC + c16];
      const uint8_t* src = in.rgb + (size_t)gr * in.pitch + gc;
      uint8_t* dst = B.img + (size_t)gr * B.ipitch + gc;
      if (vec[k]) {
        *(uint4*)d = x[k];
        *(uint4*)dst = x[k];
      } else {
        for (int j = 0; j < 16; j++) {
          const bool in_img = gr < B.H && gc + j < B.W;
          const uint8_t g = in_img ? src[j] : 0;
          d[j] = g;
          if (in_img) dst[j] = g;
        }
      }
    }
    if (nlev <= 0) return;
  } else if (in.mode != 0) {
    // Fused ingest: RGB -> gray into level 0 and the shared tile.
    for (int v = threadIdx.x; v < PYR_TR * PYR_TC; v += blockDim.x) {
      const int r = v / PYR_TC, c = v % PYR_TC, gr = R0 + r, gc = C0 + c;
      uint8_t g = 0;
      if (gr < B.H && gc < B.W) {
        const uint8_t* px = in.rgb + (size_t)gr * in.pitch + 3 * gc;
        g = in.mode == 1 ? px[0] : (uint8_t)((77 * px[0] + 150 * px[1] + 29 * px[2] + 128) >> 8);
        B.img[(size_t)gr * B.ipitch + gc] = g;
      }
      sm[0][r * PYR_TC + c] = g;
    }
    if (nlev <= 0) return;
  } else {
    // Load the level-`base` tile.
    uint4 x[PYR_NCH];
#pragma unroll
    for (int k = 0; k < PYR_NCH; k++) {
      const int v = threadIdx.x + PYR_THREADS * k, gr = R0 + v / PYR_CPR, gc = C0 + (v % PYR_CPR) * 16;
      if (gr < B.H && gc + 16 <= B.W) x[k] = *(const uint4*)(B.img + (size_t)gr * B.ipitch + gc);
    }
#pragma unroll
    for (int k = 0; k < PYR_NCH; k++) {
      const int v = threadIdx.x + PYR_THREADS * k;
      const int r = v / PYR_CPR, c16 = (v % PYR_CPR) * 16;
      const int gr = R0 + r, gc = C0 + c16;
      uint8_t* d = &sm[0][r * PYR_TC + c16];
      if (gr < B.H && gc + 16 <= B.W) {
        *(uint4*)d = x[k];
      } else {
        for (int j = 0; j < 16; j++) d[j] = (gr < B.H && gc + j < B.W) ? B.img[(size_t)gr * B.ipitch + gc + j] : 0;
      }
    }
  }
  __syncthreads();
  int src = 0;
  for (int l = 1; l <= nlev; l++) {
    const Unit& O = units[u0 + base + l];
    const int tr = PYR_TR >> l, tw4 = (PYR_TC >> l) / 4;  // output rows, 4-pixel words per row
    const int r0 = R0 >> l, c0 = C0 >> l;                 // c0 is a multiple of 4 (l <= 5)
    const uint8_t* S = sm[src];
    uint8_t* D = sm[src ^ 1];
    for (int v = threadIdx.x; v < tr * tw4; v += blockDim.x) {
      const int r = v / tw4, c = 4 * (v % tw4);
      const uint2 a = *(const uint2*)&S[(2 * r) * PYR_TC + 2 * c];
      const uint2 b = *(const uint2*)&S[(2 * r + 1) * PYR_TC + 2 * c];
      const uint32_t o = pyr_mean4(a, b);
      *(uint32_t*)&D[r * PYR_TC + c] = o;
      const int gr = r0 + r, gc = c0 + c;
      if (gr < O.H) {
        uint8_t* g = O.img + (size_t)gr * O.ipitch + gc;
        if (gc + 4 <= O.W) *(uint32_t*)g = o;
        else
          for (int j = 0; j < 4 && gc + j < O.W; j++) g[j] = (uint8_t)(o >> (8 * j));
      }
    }
    __syncthreads();
    src ^= 1;
  }
}

// ---------------------------------------------------------------------------
// BC2S blurs: bc2s_feature<cpu>::update (tracking2/bc2s_feature.hpp:372-393)
// = gaussian_blur_sigma1 twice (cuimg/cpu/gaussian_blur.h:9-47).  Row pass
// t(r,c) = (2 x[c] + x[c-1] + x[c+1]) / 4 for c in [1, W-2]; column pass
// s(r,c) = (2 t[r] + t[r-1] + t[r+1]) / 4 for r in [1, H-2]; every other
// pixel (the ring and the border) is zero.
//
// One warp walks down a strip of SR rows, 128 columns wide: every lane owns
// four columns (one 32-bit word per row), takes its horizontal neighbours from
// the adjacent lanes by shuffle, and keeps the last three rows of both row
// passes in registers, so each level pixel is read once and s1 / s2 are each
// written once.  Lanes 0 and 31 only supply the horizontal halo; strips overlap
// by 8 columns.  The arithmetic filters a word's four pixels at once:
// floor((a + 2b + c) / 4) == floor((floor((a + c) / 2) + b) / 2) for all
// integers a, b, c >= 0 (with a + c = 2k + e, e in {0, 1}, both sides are
// floor((k + b) / 2): the extra e / 4 never reaches the next integer), and the
// bytewise floor average (a & b) + ((a ^ b) >> 1 & 0x7F7F7F7F) cannot carry
// from one byte into the next.
constexpr int BL_SR = 64;                 // default rows per strip (tunable: 16, 32, 64)
constexpr int BL_OC = 120;                // output columns per warp (lanes 1..30)
constexpr int BL_WARPS = 8;

// Per-byte floor((a + b) / 2).
__device__ __forceinline__ uint32_t havg4(uint32_t a, uint32_t b) {
  return (a & b) + (((a ^ b) >> 1) & 0x7F7F7F7Fu);
}

// Row pass (2 x[c] + x[c-1] + x[c+1]) / 4 of a lane's word w; wl / wr are the
// words of the lanes to its left and right.  m zeroes the pixels outside
// [1, W-2] (or the whole row).
__device__ __forceinline__ uint32_t row_pass4(uint32_t w, uint32_t wl, uint32_t wr, uint32_t m) {
  const uint32_t L = __funnelshift_l(wl, w, 8);  // byte j: pixel j - 1
  const uint32_t R = __funnelshift_r(w, wr, 8);  // byte j: pixel j + 1
  return havg4(havg4(L, R), w) & m;
}

// Column pass (2 t[r] + t[r-1] + t[r+1]) / 4; m zeroes a row outside [1, H-2].
__device__ __forceinline__ uint32_t col_pass4(uint32_t up, uint32_t mid, uint32_t dn, uint32_t m) {
  return havg4(havg4(up, dn), mid) & m;
}

// A lane's word of s1 or s2 (pixels c0 .. c0 + 3, clipped to the row).
__device__ __forceinline__ void blur_store(uint8_t* p, uint32_t v, bool full_word, int c0, int W) {
  if (full_word) *(uint32_t*)p = v;
  else
    for (int j = 0; j < 4 && c0 + j < W; j++) p[j] = (uint8_t)(v >> (8 * j));
}

// One row step: level row r enters (word w); s1 row r-1 and s2 row r-2 leave,
// stored at d1 / d2 when they belong to the strip [r0, r1).  a1/b1/c1 are the
// row-pass values of rows r-2, r-1 and (written here) r; a2/b2/c2 those of s1
// rows r-3, r-2 and (written here) r-1.  EDGE: the strip reaches the image's
// first or last two rows, so rows outside the image or its [1, H-2] interior
// are zeroed; inside, every row that reaches a stored pixel is interior.
template <bool EDGE>
__device__ __forceinline__ void blur_step(uint32_t w, int r, int r0, int r1, int H, int W, int c0, bool out_lane,
                                          bool full_word, uint32_t mcol, uint32_t a1, uint32_t b1, uint32_t& c1,
                                          uint32_t a2, uint32_t b2, uint32_t& c2, uint8_t* d1, uint8_t* d2) {
  const uint32_t wl = __shfl_up_sync(0xffffffffu, w, 1), wr = __shfl_down_sync(0xffffffffu, w, 1);
  const int rs1 = r - 1, rs2 = r - 2;
  c1 = row_pass4(w, wl, wr, (!EDGE || (r >= 0 && r < H)) ? mcol : 0u);
  const uint32_t s1 = col_pass4(a1, b1, c1, (!EDGE || (rs1 >= 1 && rs1 <= H - 2)) ? ~0u : 0u);
  const uint32_t s1l = __shfl_up_sync(0xffffffffu, s1, 1), s1r = __shfl_down_sync(0xffffffffu, s1, 1);
  c2 = row_pass4(s1, s1l, s1r, (!EDGE || (rs1 >= 0 && rs1 < H)) ? mcol : 0u);
  const uint32_t s2 = col_pass4(a2, b2, c2, (!EDGE || (rs2 >= 1 && rs2 <= H - 2)) ? ~0u : 0u);
  if (out_lane) {
    if (rs1 >= r0 && rs1 < r1) blur_store(d1, s1, full_word, c0, W);
    if (rs2 >= r0 && rs2 < r1) blur_store(d2, s2, full_word, c0, W);
  }
}

// Rows r0 - 2 .. r1 + 1 enter, six per batch: two rounds of three steps in
// which the register windows rotate by renaming; the output row pointers move
// down one row per step.
template <bool EDGE>
__device__ __forceinline__ void blur_strip(const uint8_t* img, int ipitch, uint8_t* s1, uint8_t* s2, int fpitch,
                                           int H, int W, int r0, int r1, int c0, bool word_ok, bool out_lane,
                                           bool full_word, uint32_t mcol) {
  uint32_t t1a = 0, t1b = 0, t1c = 0, t2a = 0, t2b = 0, t2c = 0;
  // The first step (r = r0 - 2) leaves s1 row r0 - 3 and s2 row r0 - 4.
  uint8_t* d1 = s1 + (ptrdiff_t)(r0 - 3 + RB) * fpitch + (c0 + CB);
  uint8_t* d2 = s2 + (ptrdiff_t)(r0 - 4 + RB) * fpitch + (c0 + CB);
  for (int rb = r0 - 2; rb <= r1 + 1; rb += 6) {
    uint32_t w6[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
      const int r = rb + k;
      const bool ok = word_ok && r < H && (!EDGE || r >= 0);
      w6[k] = ok ? *(const uint32_t*)(img + (ptrdiff_t)r * ipitch + c0) : 0u;
    }
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int r = rb + 3 * h;
      blur_step<EDGE>(w6[3 * h], r, r0, r1, H, W, c0, out_lane, full_word, mcol, t1b, t1c, t1a, t2b, t2c, t2a, d1, d2);
      d1 += fpitch;
      d2 += fpitch;
      blur_step<EDGE>(w6[3 * h + 1], r + 1, r0, r1, H, W, c0, out_lane, full_word, mcol, t1c, t1a, t1b, t2c, t2a, t2b,
                      d1, d2);
      d1 += fpitch;
      d2 += fpitch;
      blur_step<EDGE>(w6[3 * h + 2], r + 2, r0, r1, H, W, c0, out_lane, full_word, mcol, t1a, t1b, t1c, t2a, t2b, t2c,
                      d1, d2);
      d1 += fpitch;
      d2 += fpitch;
    }
  }
}

template <int SR>
__global__ void __launch_bounds__(32 * BL_WARPS) k_blur(const Unit* __restrict__ units,
                                                        const int* __restrict__ item_prefix, int nunits) {
  const int lane = threadIdx.x & 31;
  const int item = blockIdx.x * BL_WARPS + (threadIdx.x >> 5);
  if (item >= item_prefix[nunits]) return;
  const int ui = find_unit(item_prefix, nunits, item);
  const Unit& U = units[ui];
  const int local = item - item_prefix[ui];
  const int ncs = (U.W + BL_OC - 1) / BL_OC;
  const int rs = local / ncs, cs = local % ncs;
  const int H = U.H, W = U.W;
  const int c0 = cs * BL_OC - 4 + 4 * lane;  // first column of this lane's word
  const int r0 = rs * SR, r1 = min(r0 + SR, H);
  const bool out_lane = lane >= 1 && lane <= 30 && c0 < W;
  const bool full_word = c0 + 4 <= W;
  // Row-pass column mask: pixel c0 + j is filtered iff 1 <= c0 + j <= W - 2.
  uint32_t mcol = 0;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const int c = c0 + j;
    if (c >= 1 && c <= W - 2) mcol |= 0xFFu << (8 * j);
  }
  const bool word_ok = c0 >= 0 && c0 < U.ipitch;
  if (r0 >= 2 && r1 <= H - 2)  // warp-uniform
    blur_strip<false>(U.img, U.ipitch, U.s1, U.s2, U.fpitch, H, W, r0, r1, c0, word_ok, out_lane, full_word, mcol);
  else
    blur_strip<true>(U.img, U.ipitch, U.s1, U.s2, U.fpitch, H, W, r0, r1, c0, word_ok, out_lane, full_word, mcol);
}

// ---------------------------------------------------------------------------
// Feature access: bc2s_internals::distance / compute_feature
// (tracking2/bc2s_feature.hpp:173-284).  Samples s1 at the even
// circle_r3_h offsets and s2 at twice those; weights are the constant 255, so
// the distance is the plain sum of absolute differences.
struct Feat {
  const uint8_t* s1;
  const uint8_t* s2;
  int o1[8], o2[8];
  __device__ __forceinline__ static constexpr bool safe(int, int) { return true; }  // the whole bordered image
  __device__ __forceinline__ void init(const Unit& u) {
    s1 = fptr(u.s1, u.fpitch, 0, 0);
    s2 = fptr(u.s2, u.fpitch, 0, 0);
#pragma unroll
    for (int i = 0; i < 8; i++) {
      o1[i] = c_ring[2 * i][0] * u.fpitch + c_ring[2 * i][1];
      o2[i] = 2 * c_ring[2 * i][0] * u.fpitch + 2 * c_ring[2 * i][1];
    }
  }
  __device__ __forceinline__ uint4 at(int r, int c, int pitch) const {
    const uint8_t* a = s1 + (ptrdiff_t)r * pitch + c;
    const uint8_t* b = s2 + (ptrdiff_t)r * pitch + c;
    uint4 f;
    f.x = a[o1[0]] | (a[o1[1]] << 8) | (a[o1[2]] << 16) | ((uint32_t)a[o1[3]] << 24);
    f.y = a[o1[4]] | (a[o1[5]] << 8) | (a[o1[6]] << 16) | ((uint32_t)a[o1[7]] << 24);
    f.z = b[o2[0]] | (b[o2[1]] << 8) | (b[o2[2]] << 16) | ((uint32_t)b[o2[3]] << 24);
    f.w = b[o2[4]] | (b[o2[5]] << 8) | (b[o2[6]] << 16) | ((uint32_t)b[o2[7]] << 24);
    return f;
  }
  __device__ __forceinline__ int dist(const uint4& f, int r, int c, int pitch, bool with_s1) const {
    const uint8_t* b = s2 + (ptrdiff_t)r * pitch + c;
    uint32_t z = b[o2[0]] | (b[o2[1]] << 8) | (b[o2[2]] << 16) | ((uint32_t)b[o2[3]] << 24);
    uint32_t w = b[o2[4]] | (b[o2[5]] << 8) | (b[o2[6]] << 16) | ((uint32_t)b[o2[7]] << 24);
    int d = (int)(__vsadu4(z, f.z) + __vsadu4(w, f.w));
    if (with_s1) {
      const uint8_t* a = s1 + (ptrdiff_t)r * pitch + c;
      uint32_t x = a[o1[0]] | (a[o1[1]] << 8) | (a[o1[2]] << 16) | ((uint32_t)a[o1[3]] << 24);
      uint32_t y = a[o1[4]] | (a[o1[5]] << 8) | (a[o1[6]] << 16) | ((uint32_t)a[o1[7]] << 24);
      d += (int)(__vsadu4(x, f.x) + __vsadu4(y, f.y));
    }
    return d;
  }
  __device__ __forceinline__ int s1_part(const uint4& f, int r, int c, int pitch) const {
    const uint8_t* a = s1 + (ptrdiff_t)r * pitch + c;
    uint32_t x = a[o1[0]] | (a[o1[1]] << 8) | (a[o1[2]] << 16) | ((uint32_t)a[o1[3]] << 24);
    uint32_t y = a[o1[4]] | (a[o1[5]] << 8) | (a[o1[6]] << 16) | ((uint32_t)a[o1[7]] << 24);
    return (int)(__vsadu4(x, f.x) + __vsadu4(y, f.y));
  }
};

// The even entries of circle_r3_h (the BC2S feature ring) as constant
// expressions, so that with a compile-time pitch every ring offset folds into
// the load instruction's immediate.
__host__ __device__ constexpr int ring_r(int k) { return circle16_r(2 * k); }
__host__ __device__ constexpr int ring_c(int k) { return circle16_c(2 * k); }
static_assert(ring_r(0) == -3 && ring_c(0) == 0 && ring_r(1) == -2 && ring_c(1) == 2 && ring_r(2) == 0 &&
                  ring_c(2) == 3 && ring_r(5) == 2 && ring_c(5) == -2 && ring_r(7) == -2 && ring_c(7) == -2,
              "even entries of circle_r3_h");

// Feat with the s1/s2 pitch fixed at compile time (every unit's fpitch == P).
template <int P>
struct FeatFP {
  const uint8_t* s1;
  const uint8_t* s2;
  __device__ __forceinline__ void init(const Unit& u) {
    s1 = fptr(u.s1, P, 0, 0);
    s2 = fptr(u.s2, P, 0, 0);
  }
  template <int S, int K>
  __device__ __forceinline__ static uint32_t word(const uint8_t* a) {
    // Four ring samples K..K+3 at S times the ring radius.
    constexpr int o0 = S * (ring_r(K) * P + ring_c(K)), o1 = S * (ring_r(K + 1) * P + ring_c(K + 1));
    constexpr int o2 = S * (ring_r(K + 2) * P + ring_c(K + 2)), o3 = S * (ring_r(K + 3) * P + ring_c(K + 3));
    return (uint32_t)a[o0] | ((uint32_t)a[o1] << 8) | ((uint32_t)a[o2] << 16) | ((uint32_t)a[o3] << 24);
  }
  __device__ __forceinline__ uint4 at(int r, int c, int) const {
    const uint8_t* a = s1 + (r * P + c);
    const uint8_t* b = s2 + (r * P + c);
    return make_uint4(word<1, 0>(a), word<1, 4>(a), word<2, 0>(b), word<2, 4>(b));
  }
  __device__ __forceinline__ int dist(const uint4& f, int r, int c, int, bool with_s1) const {
    const uint8_t* b = s2 + (r * P + c);
    int d = (int)(__vsadu4(word<2, 0>(b), f.z) + __vsadu4(word<2, 4>(b), f.w));
    if (with_s1) {
      const uint8_t* a = s1 + (r * P + c);
      d += (int)(__vsadu4(word<1, 0>(a), f.x) + __vsadu4(word<1, 4>(a), f.y));
    }
    return d;
  }
  __device__ __forceinline__ int s1_part(const uint4& f, int r, int c, int) const {
    const uint8_t* a = s1 + (r * P + c);
    return (int)(__vsadu4(word<1, 0>(a), f.x) + __vsadu4(word<1, 4>(a), f.y));
  }
  // Whether a descent may continue around (r, c): always, since the whole
  // bordered image (or a tile with a full-descent margin) is readable.
  __device__ __forceinline__ static constexpr bool safe(int, int) { return true; }
};

// FeatFP over a staged tile whose margins do not cover the longest descent:
// rows lo_r - 7 .. lo_r - 7 + SR - 1 and columns lo_c - 7 .. lo_c - 7 + SC - 1
// of s1 / s2 are staged at pitch SC.  A descent centred at (r, c) reads its
// candidates (r +- 1, c +- 1) and their ring taps (6 pixels further at most),
// so it may continue there only when (r, c) is at least 7 pixels inside the
// staged rectangle.
template <int SC, int SR>
struct FeatTile : FeatFP<SC> {
  int lo_r, lo_c;
  __device__ __forceinline__ bool safe(int r, int c) const {
    return (unsigned)(r - lo_r) < (unsigned)(SR - 14) && (unsigned)(c - lo_c) < (unsigned)(SC - 14);
  }
};

// gradient_descent_match (tracking2/gradient_descent_matcher.hpp:9-76): greedy
// 8-neighbour descent over c8_h with the c8_it_h partial sweeps; the first
// distance is always the s1+s2 one.  (pr, pc) is inside the domain.
// c8_h and c8_it_h (cuimg/neighb2d_data.h:80-85,162-180) in registers: the
// tables are indexed by per-lane values, which constant memory serialises.
// c8_h entry i = (c8r(i), c8c(i)); the sweep after a move to neighbour mi
// starts at c8_it_h[mi][0] and runs up to (not including) c8_it_h[mi][1],
// wrapping mod 8; mi = 8 (no move yet) sweeps all eight.
__host__ __device__ constexpr int c8r(int i) {
  return i == 0 ? -1 : i == 1 ? 0 : i == 2 ? 1 : i == 3 ? -1 : i == 4 ? 1 : i == 5 ? -1 : i == 6 ? 0 : 1;
}
__host__ __device__ constexpr int c8c(int i) { return i < 3 ? 1 : i < 5 ? 0 : -1; }
__host__ __device__ constexpr unsigned c8_pack(bool col) {
  unsigned v = 0;
  for (int i = 0; i < 8; i++) v |= (unsigned)((col ? c8c(i) : c8r(i)) + 1) << (2 * i);
  return v;
}
__host__ __device__ constexpr int sweep_first(int mi) { return mi == 8 ? 0 : (mi & 1) ? mi - 1 : (mi + 6) & 7; }
__host__ __device__ constexpr int sweep_len(int mi) { return mi == 8 ? 8 : (mi & 1) ? 3 : 5; }
constexpr int k_c8_tab[8][2] = {{-1, 1}, {0, 1}, {1, 1}, {-1, 0}, {1, 0}, {-1, -1}, {0, -1}, {1, -1}};
constexpr int k_c8it_tab[9][2] = {{6, 3}, {0, 3}, {0, 5}, {2, 5}, {2, 7}, {4, 7}, {4, 1}, {6, 1}, {0, 0}};
constexpr bool c8_tables_agree() {
  for (int i = 0; i < 8; i++)
    if (c8r(i) != k_c8_tab[i][0] || c8c(i) != k_c8_tab[i][1]) return false;
  for (int m = 0; m < 9; m++)
    if (sweep_first(m) != k_c8it_tab[m][0] || ((k_c8it_tab[m][1] - k_c8it_tab[m][0] - 1) & 7) + 1 != sweep_len(m))
      return false;
  return true;
}
static_assert(c8_tables_agree(), "register forms of c8_h / c8_it_h");
__device__ __forceinline__ int c8_dr(int i) { return (int)((c8_pack(false) >> (2 * i)) & 3u) - 1; }
__device__ __forceinline__ int c8_dc(int i) { return (int)((c8_pack(true) >> (2 * i)) & 3u) - 1; }

// gradient_descent_match (tracking2/gradient_descent_matcher.hpp:9-76): greedy
// 8-neighbour descent over c8_h with the c8_it_h partial sweeps from (pr, pc),
// inside the domain.  `best` enters as the distance at (pr, pc) -- always the
// s1+s2 one -- and leaves as the distance at the match.  Every candidate's
// distance is computed whole: stopping at a partial sum that already reaches
// the best would give the same descent, but the branches serialise the 8 or 16
// independent gathers, which costs more than the loads saved.  Returns false,
// with nothing written, when the descent moves to a centre where F cannot
// serve the next sweep (F.safe), so the caller can redo the match from the
// images in global memory; true otherwise.  (pr, pc) itself must be safe.
template <bool WITH_S1, class FeatT>
__device__ __forceinline__ bool gd_match(const Unit& u, const FeatT& F, const uint4& f, int pr, int pc, int& best,
                                         int& dr, int& dc) {
  int predr = pr, predc = pc, mr = pr, mc = pc;
  int mi = 8;
  bool ok = true;
  for (int search = 0; search < 10; search++) {
    const int i0 = sweep_first(mi), n = sweep_len(mi);
    for (int j = 0; j < n; j++) {
      const int i = (i0 + j) & 7;
      const int nr = predr + c8_dr(i), nc = predc + c8_dc(i);
      if (in_dom(u, nr, nc)) {
        const int d = F.dist(f, nr, nc, u.fpitch, WITH_S1);
        if (d < best) {
          mr = nr;
          mc = nc;
          mi = i;
          best = d;
        }
      }
    }
    if ((predr == mr && predc == mc) || !in_dom(u, mr, mc)) break;
    if (!F.safe(mr, mc)) {
      ok = false;
      break;
    }
    predr = mr;
    predc = mc;
  }
  dr = mr - pr;
  dc = mc - pc;
  return ok;
}

// Asks L1 for the level-image rows r - 3 .. r + 3 around column c (clamped
// into the image): the contrast test of a match near (r, c) then reads L1
// instead of waiting on L2.  A hint only; it changes no result.
__device__ __forceinline__ void prefetch_contrast(const Unit& u, int r, int c) {
  const int cc = clampi(c, 0, u.W - 1);
#pragma unroll
  for (int d = -3; d <= 3; d++) {
    const uint8_t* a = u.img + (size_t)clampi(r + d, 0, u.H - 1) * u.ipitch + cc;
    asm volatile("prefetch.global.L1 [%0];" ::"l"(a));
  }
}

// contrast_kernel (tracking_strategies.hpp:101-135), clamped level reads.
__device__ __forceinline__ int contrast_at(const Unit& u, int r, int c) {
  const int d = 2;
  return abs(img_at(u, r, c + d) - img_at(u, r, c - d)) + abs(img_at(u, r - d, c) - img_at(u, r + d, c)) +
         abs(img_at(u, r - d, c - d) - img_at(u, r + d, c + d)) + abs(img_at(u, r - d, c + d) - img_at(u, r + d, c - d));
}

// Chunk tables: table[u] = first global chunk of unit u, table[nunits] = total.
struct ChunkCursor {
  int unit, chunk;
};
__device__ __forceinline__ ChunkCursor chunk_of(const int* table, int nunits, int g) {
  ChunkCursor cc;
  cc.unit = find_unit(table, nunits, g);
  cc.chunk = g - table[cc.unit];
  return cc;
}

// ---------------------------------------------------------------------------
// Matcher: match_particles_kernel (tracking_strategies.hpp:274-426) with
// multiscale_prediction == motion_based_prediction (predictions.h:15-33),
// two_step_gradient_descent_match (gradient_descent_matcher.hpp:118-124) and
// kernel_particle_container::move (particle_container.hpp:422-466).  The
// sparse-index write keeps the highest slot per pixel (atomicMax), i.e. the
// single-threaded reference's last writer.
constexpr int MATCH_BLOCK = 256;
constexpr int MATCH_SUB = CHUNK / MATCH_BLOCK;

// Prediction of a live particle (motion_based_prediction, predictions.h:15-33).
__device__ __forceinline__ void predict(unsigned short age, short2 pos, short2 spd, int& pr, int& pc) {
  pr = (short)(pos.x + (age == 1 ? 0 : spd.x));
  pc = (short)(pos.y + (age == 1 ? 0 : spd.y));
}

// Match one live particle whose prediction (pr, pc) is inside the domain, and
// apply the result (kernel_particle_container::move or remove).
template <class FeatT>
__device__ __forceinline__ void match_finish(const Unit& u, const FeatT& F, int f, int b, int i, unsigned short age,
                                             short2 pos, int pr, int pc, const uint4& feat, int dr, int dc);

// Returns false, with nothing written, when a descent left the area F can
// serve (see gd_match).
template <class FeatT>
__device__ __forceinline__ bool match_one(const Unit& u, const FeatT& F, int f, int b, int i, unsigned short age,
                                          short2 pos, int pr, int pc, const uint4& feat) {
  int d1r, d1c, d2r, d2c;
  // Step 1 compares s2-only candidates against the s1+s2 distance at the
  // prediction.  Step 2 starts from step 1's match with its s1+s2 distance:
  // the prediction's own when the match is the prediction (step 1 may also
  // come back to it, ending with its s2 distance), else the s2 distance step 1
  // ended with plus the s1 part there.
  const int init = F.dist(feat, pr, pc, u.fpitch, true);
  int best = init;
  bool ok = gd_match<false>(u, F, feat, pr, pc, best, d1r, d1c);
  if (ok) {
    prefetch_contrast(u, pr + d1r, pc + d1c);  // step 2 rarely moves far from step 1's match
    best = (d1r != 0 || d1c != 0) ? best + F.s1_part(feat, pr + d1r, pc + d1c, u.fpitch) : init;
    ok = gd_match<true>(u, F, feat, pr + d1r, pc + d1c, best, d2r, d2c);
  }
  if (ok) match_finish(u, F, f, b, i, age, pos, pr, pc, feat, d1r + d2r, d1c + d2c);
  return ok;
}

// The match's acceptance and the particle update (kernel_particle_container::
// move or remove) for a total descent (dr, dc) from the prediction.
template <class FeatT>
__device__ __forceinline__ void match_finish(const Unit& u, const FeatT& F, int f, int b, int i, unsigned short age,
                                             short2 pos, int pr, int pc, const uint4& feat, int dr, int dc) {
  const int mr = (short)(pr + dr), mc = (short)(pc + dc);
  bool accept = in_dom(u, mr, mc);
  uint4 mf = make_uint4(0, 0, 0, 0);
  if (accept) {
    mf = F.at(mr, mc, u.fpitch);
    // n_diff over the s2 entries (every weight is 255 > 150, so cpt = 8).
    unsigned n_diff = 0;
    const uint32_t a0 = feat.z, a1 = feat.w, c0 = mf.z, c1 = mf.w;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int x = (a0 >> (8 * j)) & 255, y = (c0 >> (8 * j)) & 255;
      if (abs(x - y) > u.k) n_diff++;
      x = (a1 >> (8 * j)) & 255;
      y = (c1 >> (8 * j)) & 255;
      if (abs(x - y) > u.k) n_diff++;
    }
    accept = n_diff < 4u;
  }
  if (!accept || contrast_at(u, mr, mc) < 3) {
    u.age[b][i] = 0;
    return;
  }
  const int sr = pr - pos.x + dr, sc = pc - pos.y + dc;
  u.age[b][i] = (unsigned short)(age + 1);
  u.spd[b][i] = make_short2((short)sr, (short)sc);
  u.pos[b][i] = make_short2((short)mr, (short)mc);
  if (sr != 0 || sc != 0) u.feat[b][i] = mf;
  atomicOr(&u.occ[bin_word(u, mr, mc)], bin_bit(mr, mc));
  atomicMax(&u.idx[(size_t)mr * u.W + mc], ((unsigned long long)stamp_match(f) << 32) | (unsigned)i);
}

template <class FeatT>
__global__ void __launch_bounds__(MATCH_BLOCK) k_match(const Unit* __restrict__ units, UState* __restrict__ st,
                                                       const Frame* __restrict__ fr, const int* __restrict__ table,
                                                       int nunits) {
  const int f = fr->f;
  const int total = table[nunits] * MATCH_SUB;
  for (int g = blockIdx.x; g < total; g += gridDim.x) {
    ChunkCursor cc = chunk_of(table, nunits, g / MATCH_SUB);
    const Unit& u = units[cc.unit];
    const UState s = st[cc.unit];
    const int i = cc.chunk * CHUNK + (g % MATCH_SUB) * MATCH_BLOCK + threadIdx.x;
    if (i >= s.n) continue;
    const int b = s.cur;
    const unsigned short age = u.age[b][i];
    if (age == 0) continue;
    const short2 pos = u.pos[b][i];
    int pr, pc;
    predict(age, pos, u.spd[b][i], pr, pc);
    if (!in_dom(u, pr, pc)) {
      u.age[b][i] = 0;
      continue;
    }
    FeatT F;
    F.init(u);
    match_one(u, F, f, b, i, age, pos, pr, pc, u.feat[b][i]);
  }
}

// ---------------------------------------------------------------------------
// Tiled matcher.  Live particles are binned by their prediction into tiles of
// MT_R x MT_C pixels (k_mt_list: fixed-capacity tile lists, the rare excess in
// an overflow list matched from global memory); one CTA per non-empty tile stages
// the tile's s1 / s2 neighbourhood in shared memory (TMA, or 16-byte cp.async
// copies) and matches its particles from there.  A descent moves at most 10
// pixels per step in each axis (two steps) and the BC2S taps reach 6 pixels
// further, so with the full margins (26 rows, 32 columns) every sample a
// particle of the tile can touch is staged.  The slim margins (14 rows, 16
// columns) stage 34% fewer bytes, so that more CTAs fit on an SM; a particle
// whose descent would read outside them (about 0.1% of them on 1080p video:
// most descents end within a few pixels, and only particles near a tile edge
// can reach the margin) is matched again from the images in global memory,
// with the same result.  Particles are independent (each writes only its own slot;
// the sparse index keeps the highest slot with atomicMax), so the order inside
// a tile does not change any result.
constexpr int MT_R = 64, MT_C = 128;                // tile
constexpr int MT_MR = 26, MT_MC = 32;              // full staged margins
constexpr int MT_SR = MT_R + 2 * MT_MR;            // staged rows (116)
constexpr int MT_SC = MT_C + 2 * MT_MC;            // staged columns (192), 16-byte chunks
constexpr int MT_MR_SLIM = 14, MT_MC_SLIM = 16;    // slim staged margins: 92 rows x 160 columns
constexpr int MT_THREADS = 256;
// Particles a tile's list holds (k_mt_list); the rest of a fuller tile is
// matched by k_match_overflow.  Steady-state 1080p video puts at most about
// 640 particles in one tile (the oracle over 40 frames, any level).
constexpr int MT_LIST_CAP = 1024;
static_assert(MT_MR >= 2 * 10 + 6 && MT_MC >= 2 * 10 + 6, "full staged margins cover a full descent");
static_assert(MT_MR_SLIM >= 7 && MT_MC_SLIM >= 7, "the prediction's own sweep is always staged");
static_assert(MT_SC % 16 == 0 && MT_MC % 16 == 0 && MT_MC_SLIM % 16 == 0, "16-byte staging");

__device__ __forceinline__ int mt_tile(const Unit& u, int pr, int pc) {
  return u.mt_base + (pr / MT_R) * u.MTC + pc / MT_C;
}

// One pass bins the live particles by the tile of their prediction (and
// removes those predicted outside the domain, as the matcher does): a
// particle's rank in its tile comes from the tile's counter, and the particle
// goes to slot rank of the tile's fixed-capacity list (tile t's list starts at
// t * cap).  A particle ranked at or beyond cap goes to the overflow list
// instead ((unit, slot) pairs, counted in cnt[ntiles]), which k_match_overflow
// matches from global memory.  The order within a tile or the overflow list is
// the order of the atomics; it changes no result (particles are independent).
__global__ void __launch_bounds__(CHUNK) k_mt_list(const Unit* __restrict__ units, const UState* __restrict__ st,
                                                   const int* __restrict__ table, int nunits, int* __restrict__ cnt,
                                                   int ntiles, int cap, int* __restrict__ list,
                                                   int2* __restrict__ ovf) {
  const int total = table[nunits];
  for (int g = blockIdx.x; g < total; g += gridDim.x) {
    ChunkCursor cc = chunk_of(table, nunits, g);
    const Unit& u = units[cc.unit];
    const UState s = st[cc.unit];
    const int i = cc.chunk * CHUNK + threadIdx.x;
    if ((i & ~31) >= s.n) continue;  // whole warp past the slots
    const int b = s.cur;
    int tile = -1;
    if (i < s.n) {
      const unsigned short age = u.age[b][i];
      if (age != 0) {
        int pr, pc;
        predict(age, u.pos[b][i], u.spd[b][i], pr, pc);
        if (!in_dom(u, pr, pc))
          u.age[b][i] = 0;
        else
          tile = mt_tile(u, pr, pc);
      }
    }
    // Slots follow birth order, which is raster order within a detector
    // frame, so a warp's particles mostly share a few tiles: one atomic per
    // distinct tile of the warp.
    const int lane = threadIdx.x & 31;
    const unsigned peers = __match_any_sync(0xffffffffu, tile);
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if (tile >= 0 && lane == leader) base = atomicAdd(&cnt[tile], __popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (tile >= 0) {
      const int rank = base + __popc(peers & ((1u << lane) - 1u));
      if (rank < cap)
        list[(size_t)tile * cap + rank] = i;
      else
        ovf[atomicAdd(&cnt[ntiles], 1)] = make_int2(cc.unit, i);
    }
  }
}

__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gsrc) : "memory");
}

// Stages rows R0s .. R0s + SR - 1 and columns C0s .. C0s + SC - 1 of s1 and
// s2 (mt_stage_issue, below), skipping chunks outside the bordered images
// (never sampled: the taps stay within 6 pixels of the domain, inside the zero
// border).  mt_tma_issue stages the same tile by two TMA copies (one per
// image) that complete on an mbarrier.  The staged region starts at byte
// column C0s + CB of the bordered rows, a multiple of 16 (C0s = 128 k - MC
// with a margin MC of 32 or 16 columns, CB = 16); rows above or below the
// bordered image, and columns right of it, read zeros.  Thread 0 issues;
// mt_tma_wait waits.
template <int SR, int SC>
__device__ __forceinline__ void mt_tma_issue(const CUtensorMap* m1, const CUtensorMap* m2, int R0s, int C0s,
                                             uint8_t* ts1, uint8_t* ts2, unsigned long long* mbar, bool copies) {
  const unsigned bar = (unsigned)__cvta_generic_to_shared(mbar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int x = C0s + CB, y = R0s + RB;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(2 * SR * SC)
                 : "memory");
    if (!copies) return;  // test hook: the barrier is armed but nothing will complete it
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(
            (unsigned)__cvta_generic_to_shared(ts1)),
        "l"(m1), "r"(x), "r"(y), "r"(bar)
        : "memory");
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(
            (unsigned)__cvta_generic_to_shared(ts2)),
        "l"(m2), "r"(x), "r"(y), "r"(bar)
        : "memory");
  }
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits for the tile (phase 0 of the mbarrier); false when it gave up.  The
// budget is MT_WAIT_NS of the GPU's global timer counted only while this CTA
// is resident: the gap between two consecutive polls counts at most
// MT_POLL_GAP_NS, so time the context spends switched out (time-slicing with
// other contexts) does not use the budget up; each poll asks to be suspended
// no longer than MT_SUSPEND_HINT_NS, well inside that cap.  2^24 polls at
// most, whatever the timer says.  Called by one thread.
constexpr unsigned long long MT_WAIT_NS = 500000000ull;
constexpr unsigned long long MT_POLL_GAP_NS = 100000ull;
constexpr unsigned MT_SUSPEND_HINT_NS = 10000u;  // each poll suspends the thread for at most about this long
__device__ __forceinline__ bool mt_tma_wait(unsigned long long* mbar) {
  const unsigned bar = (unsigned)__cvta_generic_to_shared(mbar);
  unsigned long long prev = global_ns(), counted = 0;
  for (int it = 0; it < (1 << 24); it++) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0, %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(MT_SUSPEND_HINT_NS)
        : "memory");
    if (done) return true;
    const unsigned long long now = global_ns(), gap = now - prev;
    prev = now;
    counted += gap < MT_POLL_GAP_NS ? gap : MT_POLL_GAP_NS;
    if (counted > MT_WAIT_NS) break;
  }
  return false;
}

// Thread 0 waits for the tile and every thread of the CTA learns the outcome
// (one branch for the whole CTA).  When the wait gives up after real copies
// were issued, thread 0 waits once more with the same budget for them to
// land, since a CTA cannot return with bulk copies still writing into its
// shared memory without risking the next CTA's; if they still have not
// landed, it flags ERR_COPY_INFLIGHT (the context is unrecoverable: the copies
// may complete into another CTA's tile).  Returns false on a timeout, after
// flagging ERR_TIMEOUT.
__device__ __forceinline__ bool mt_tma_wait_cta(unsigned long long* mbar, bool copies_issued, int* err,
                                                int* verdict) {
  if (threadIdx.x == 0) {
    int ok = mt_tma_wait(mbar) ? 1 : 0;
    if (!ok) {
      int flags = ERR_TIMEOUT;
      if (copies_issued && !mt_tma_wait(mbar)) flags |= ERR_COPY_INFLIGHT;
      atomicOr(err, flags);
    }
    *verdict = ok;
  }
  __syncthreads();
  return *verdict != 0;
}

template <int SR, int SC>
__device__ __forceinline__ void mt_stage_issue(const Unit& u, int R0s, int C0s, uint8_t* ts1, uint8_t* ts2) {
  constexpr int CPR = SC / 16;
  for (int v = threadIdx.x; v < SR * CPR; v += blockDim.x) {
    const int row = v / CPR, ck = v % CPR;
    const int gr = R0s + row;                    // image row
    const int gb = C0s + CB + 16 * ck;           // byte offset inside the bordered row
    if (gr < -RB || gr >= u.H + RB || gb < 0 || gb + 16 > FIXED_FPITCH) continue;
    const size_t go = (size_t)(gr + RB) * FIXED_FPITCH + gb;
    cp_async16(&ts1[row * SC + 16 * ck], u.s1 + go);
    cp_async16(&ts2[row * SC + 16 * ck], u.s2 + go);
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// The tile arrives by TMA when the context encoded tensor maps (tmaps: s1
// and s2 of every unit, for the frame's parity), by cp.async otherwise.
// THREADS per CTA; with DYN the threads take the tile's particles one at a
// time from a shared counter (a thread that finishes a short descent takes the
// next particle) instead of every THREADS-th one.  A tile whose wait gives up
// sets ERR_TIMEOUT in *err and leaves its particles unmatched (and
// ERR_COPY_INFLIGHT if its copies never landed); `withhold` (a test hook) arms
// the barrier without issuing the copies, so that the wait gives up.  MR x MC
// are the staged margins: the full ones, or the slim ones, with which a
// particle whose descent leaves the staged area is matched again by its thread
// from the bordered images in global memory (counted in *fallbacks).
template <int THREADS, bool DYN, int MINB, int MR, int MC>
__global__ void __launch_bounds__(THREADS, MINB) k_match_tiled(const Unit* __restrict__ units,
                                                               const UState* __restrict__ st,
                                                               const Frame* __restrict__ fr,
                                                               const int* __restrict__ tile_prefix, int nunits,
                                                               const int* __restrict__ cnt, int cap,
                                                               const int* __restrict__ list,
                                                               const CUtensorMap* __restrict__ tmaps,
                                                               int* __restrict__ err, int withhold,
                                                               unsigned long long* __restrict__ fallbacks) {
  constexpr int SR = MT_R + 2 * MR, SC = MT_C + 2 * MC;
  constexpr bool FULL = MR >= MT_MR && MC >= MT_MC;  // every sample of every descent is staged
  __shared__ __align__(128) uint8_t ts1[SR * SC];
  __shared__ __align__(128) uint8_t ts2[SR * SC];
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ int next;
  __shared__ int tile_ok;
  const int t = blockIdx.x;
  const int n0 = t * cap, n1 = n0 + min(cnt[t], cap);  // the tile's list (k_mt_list)
  if (n0 == n1) return;
  const int ui = find_unit(tile_prefix, nunits, t);
  const Unit& u = units[ui];
  const int local = t - tile_prefix[ui];
  const int R0s = (local / u.MTC) * MT_R - MR, C0s = (local % u.MTC) * MT_C - MC;
  if (DYN && threadIdx.x == 0) next = n0 + THREADS;
  if (tmaps)
    mt_tma_issue<SR, SC>(tmaps + 2 * ui, tmaps + 2 * ui + 1, R0s, C0s, ts1, ts2, &mbar, !withhold);
  else
    mt_stage_issue<SR, SC>(u, R0s, C0s, ts1, ts2);
  // The thread's first particle is read while the tile arrives.
  const int f = fr->f;
  const int b = st[ui].cur;
  int k = n0 + threadIdx.x;
  int i = 0;
  unsigned short age = 0;
  short2 pos = make_short2(0, 0), spd = make_short2(0, 0);
  uint4 feat = make_uint4(0, 0, 0, 0);
  if (k < n1) {
    i = list[k];
    age = u.age[b][i];
    pos = u.pos[b][i];
    spd = u.spd[b][i];
    feat = u.feat[b][i];
  }
  if (tmaps) {
    if (!mt_tma_wait_cta(&mbar, !withhold, err, &tile_ok)) return;  // the whole CTA returns together
  } else {
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();
  }
  typename std::conditional<FULL, FeatFP<SC>, FeatTile<SC, SR>>::type F;
  F.s1 = ts1 - (R0s * SC + C0s);  // F.s1 + (r * SC + c) is staged pixel (r, c)
  F.s2 = ts2 - (R0s * SC + C0s);
  if constexpr (!FULL) {
    F.lo_r = R0s + 7;
    F.lo_c = C0s + 7;
  }
  while (k < n1) {
    int pr, pc;
    predict(age, pos, spd, pr, pc);
    if (!match_one(u, F, f, b, i, age, pos, pr, pc, feat)) {
      // The descent left the staged area (slim margins only): the same match
      // from the bordered images in global memory.
      FeatFP<FIXED_FPITCH> G;
      G.init(u);
      match_one(u, G, f, b, i, age, pos, pr, pc, feat);
      atomicAdd(fallbacks, 1ull);
    }
    k = DYN ? atomicAdd(&next, 1) : k + THREADS;
    if (k < n1) {
      i = list[k];
      age = u.age[b][i];
      pos = u.pos[b][i];
      spd = u.spd[b][i];
      feat = u.feat[b][i];
    }
  }
}

// The particles k_mt_list could not place in their tile's list (more than
// `cap` in one tile), matched from the bordered images in global memory like
// k_match; a thread per entry, any order (particles are independent).  The
// list is usually empty and the CTAs return at once.
__global__ void __launch_bounds__(256) k_match_overflow(const Unit* __restrict__ units, const UState* __restrict__ st,
                                                        const Frame* __restrict__ fr, const int* __restrict__ nov,
                                                        const int2* __restrict__ ovf) {
  const int f = fr->f, n = *nov;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int2 e = ovf[k];
    const Unit& u = units[e.x];
    const int b = st[e.x].cur, i = e.y;
    const unsigned short age = u.age[b][i];
    const short2 pos = u.pos[b][i];
    int pr, pc;
    predict(age, pos, u.spd[b][i], pr, pc);  // inside the domain: k_mt_list removed the others
    FeatFP<FIXED_FPITCH> G;
    G.init(u);
    match_one(u, G, f, b, i, age, pos, pr, pc, u.feat[b][i]);
  }
}

// Warp-per-particle matcher variant (same results as k_match).  Four lanes
// evaluate one sweep candidate (each gathers two s1 and two s2 ring samples),
// so a whole sweep -- up to 8 candidates -- is one round of gathers whose lanes
// share rows and therefore L1 sectors, and the warp never waits on another
// particle's longer descent.  The order of the sweep and the strict "<" keep
// gradient_descent_match's first-best-in-sweep-order semantics.
constexpr int MW_WARPS = 8;

struct LaneRing {  // the lane's two s1 and two s2 ring offsets (ring index q and q + 4)
  int s1a, s1b, s2a, s2b;
};

__device__ __forceinline__ int warp_eval(const Unit& u, const uint8_t* s1, const uint8_t* s2, const LaneRing& o,
                                         const uint4& f, int q, int r, int c, bool with_s1, bool active) {
  int d = 0;
  if (active) {
    const ptrdiff_t off = (ptrdiff_t)r * u.fpitch + c;
    const int fa2 = (q < 4 ? (f.z >> (8 * q)) : (f.w >> (8 * (q - 4)))) & 255;  // s2 ring q
    const int fb2 = (f.w >> (8 * q)) & 255;                                      // s2 ring q + 4
    d = abs((int)__ldg(s2 + off + o.s2a) - fa2) + abs((int)__ldg(s2 + off + o.s2b) - fb2);
    if (with_s1) {
      const int fa1 = (f.x >> (8 * q)) & 255, fb1 = (f.y >> (8 * q)) & 255;
      d += abs((int)__ldg(s1 + off + o.s1a) - fa1) + abs((int)__ldg(s1 + off + o.s1b) - fb1);
    }
  }
  d += __shfl_xor_sync(0xffffffffu, d, 1);
  d += __shfl_xor_sync(0xffffffffu, d, 2);
  return d;  // every lane of the 4-lane group holds its candidate's distance
}

__global__ void __launch_bounds__(32 * MW_WARPS) k_match_warp(const Unit* __restrict__ units, UState* __restrict__ st,
                                                              const Frame* __restrict__ fr,
                                                              const int* __restrict__ table, int nunits) {
  const int f = fr->f;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int cand = lane >> 2, q = lane & 3;
  const int total = table[nunits];
  for (int g = blockIdx.x; g < total; g += gridDim.x) {
    ChunkCursor cc = chunk_of(table, nunits, g);
    const Unit& u = units[cc.unit];
    const UState s = st[cc.unit];
    const int b = s.cur;
    const uint8_t* s1 = fptr(u.s1, u.fpitch, 0, 0);
    const uint8_t* s2 = fptr(u.s2, u.fpitch, 0, 0);
    LaneRing o;
    o.s1a = c_ring[2 * q][0] * u.fpitch + c_ring[2 * q][1];
    o.s1b = c_ring[2 * (q + 4)][0] * u.fpitch + c_ring[2 * (q + 4)][1];
    o.s2a = 2 * o.s1a;
    o.s2b = 2 * o.s1b;
    for (int k = warp; k < CHUNK; k += MW_WARPS) {
      const int i = cc.chunk * CHUNK + k;
      if (i >= s.n) break;
      const unsigned short age = u.age[b][i];
      if (age == 0) continue;
      const short2 pos = u.pos[b][i];
      const short2 spd = u.spd[b][i];
      const int pr = (short)(pos.x + (age == 1 ? 0 : spd.x)), pc = (short)(pos.y + (age == 1 ? 0 : spd.y));
      if (!in_dom(u, pr, pc)) {
        if (lane == 0) u.age[b][i] = 0;
        continue;
      }
      const uint4 feat = u.feat[b][i];
      int mr = pr, mc = pc;
      for (int desc = 0; desc < 2; desc++) {
        const bool with_s1 = desc == 1;
        int predr = mr, predc = mc;
        // First distance: always s1 + s2 (lanes 0..3).
        int best = __shfl_sync(0xffffffffu, warp_eval(u, s1, s2, o, feat, q, predr, predc, true, cand == 0), 0);
        int mi = 8;
        for (int search = 0; search < 10; search++) {
          const int start = c_c8it[mi][0], end = c_c8it[mi][1];
          const int m = ((end - start + 7) & 7) + 1;  // sweep length: 8 when start == end
          const int pos_in_sweep = (cand - start + 8) & 7;
          const bool in_sweep = pos_in_sweep < m;
          const int nr = predr + c_c8[cand][0], nc = predc + c_c8[cand][1];
          const bool ok = in_sweep && in_dom(u, nr, nc);
          const int d = warp_eval(u, s1, s2, o, feat, q, nr, nc, with_s1, ok);
          // Sequential compare in sweep order (identical on every lane).
          int nmr = mr, nmc = mc, nmi = mi, nbest = best;
          for (int t = 0; t < m; t++) {
            const int cidx = (start + t) & 7;
            const int dc = __shfl_sync(0xffffffffu, d, 4 * cidx);
            const bool okc = __shfl_sync(0xffffffffu, ok, 4 * cidx);
            if (okc && dc < nbest) {
              nbest = dc;
              nmr = predr + c_c8[cidx][0];
              nmc = predc + c_c8[cidx][1];
              nmi = cidx;
            }
          }
          mr = nmr;
          mc = nmc;
          mi = nmi;
          best = nbest;
          if ((predr == mr && predc == mc) || !in_dom(u, mr, mc)) break;
          predr = mr;
          predc = mc;
        }
      }
      // Feature at the match (lanes 0..3 hold it), acceptance and move.
      uint32_t x = 0, y = 0, z = 0, w = 0;
      if (cand == 0) {
        const ptrdiff_t off = (ptrdiff_t)mr * u.fpitch + mc;
        x = (uint32_t)__ldg(s1 + off + o.s1a) << (8 * q);
        y = (uint32_t)__ldg(s1 + off + o.s1b) << (8 * q);
        z = (uint32_t)__ldg(s2 + off + o.s2a) << (8 * q);
        w = (uint32_t)__ldg(s2 + off + o.s2b) << (8 * q);
      }
      x |= __shfl_xor_sync(0xffffffffu, x, 1);
      y |= __shfl_xor_sync(0xffffffffu, y, 1);
      z |= __shfl_xor_sync(0xffffffffu, z, 1);
      w |= __shfl_xor_sync(0xffffffffu, w, 1);
      x |= __shfl_xor_sync(0xffffffffu, x, 2);
      y |= __shfl_xor_sync(0xffffffffu, y, 2);
      z |= __shfl_xor_sync(0xffffffffu, z, 2);
      w |= __shfl_xor_sync(0xffffffffu, w, 2);
      if (lane == 0) {
        const uint4 mf = make_uint4(x, y, z, w);
        unsigned n_diff = 0;
#pragma unroll
        for (int j = 0; j < 4; j++) {
          int a = (feat.z >> (8 * j)) & 255, c = (mf.z >> (8 * j)) & 255;
          if (abs(a - c) > u.k) n_diff++;
          a = (feat.w >> (8 * j)) & 255;
          c = (mf.w >> (8 * j)) & 255;
          if (abs(a - c) > u.k) n_diff++;
        }
        if (n_diff >= 4u || contrast_at(u, mr, mc) < 3) {
          u.age[b][i] = 0;
        } else {
          const int sr = mr - pos.x, sc = mc - pos.y;  // = pred - pos + delta
          u.age[b][i] = (unsigned short)(age + 1);
          u.spd[b][i] = make_short2((short)sr, (short)sc);
          u.pos[b][i] = make_short2((short)mr, (short)mc);
          if (sr != 0 || sc != 0) u.feat[b][i] = mf;
          atomicOr(&u.occ[bin_word(u, mr, mc)], bin_bit(mr, mc));
          atomicMax(&u.idx[(size_t)mr * u.W + mc], ((unsigned long long)stamp_match(f) << 32) | (unsigned)i);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Flow statistics and fusion for every 8x8 bin of every unit:
// compute_flow_stats_kernel (tracking_strategies.hpp:525-574: count of
// occupied pixels whose particle has age >= 1, and the speed of the last one
// in raster order), then flow_fusion_kernel / flow_fusion_kernel_root
// (:576-639).  The fused flow of a bin follows its chain of parent bins up to
// the first scale with more than one particle (the root divides the speed by
// the count), doubling per scale, so all scales are computed in one launch.
//
// The statistics run right after the matcher, when the occupancy bits are
// exactly the pixels the matcher wrote this frame (births come later in the
// frame) and the index entry of each is a particle it just moved, whose age
// is at least 2.  So a bin's count is the population of its occupancy word and
// its last particle is the one at the word's highest bit: one index and one
// speed load per bin, which lets every thread read its parent bins directly.
struct BinStat {
  int n;
  int2 sp;
};
__device__ __forceinline__ BinStat bin_stat(const Unit& u, int b, size_t bin, int br, int bc) {
  const unsigned long long w = u.occ[bin];
  BinStat o{__popcll(w), make_int2(0, 0)};
  if (w) {
    const int bit = 63 - __clzll((long long)w);
    const unsigned j = (unsigned)(u.idx[(size_t)(br * 8 + (bit >> 3)) * u.W + bc * 8 + (bit & 7)] & 0xffffffffu);
    const short2 v = u.spd[b][j];
    o.sp = make_int2(v.x, v.y);
  }
  return o;
}

__global__ void __launch_bounds__(256) k_stats(const Unit* __restrict__ units, UState* __restrict__ st,
                                               const int* __restrict__ bin_prefix, int nunits) {
  if (blockIdx.x == 0)
    for (int k = threadIdx.x; k < nunits; k += blockDim.x) st[k].compact = 0;
  const int total = bin_prefix[nunits];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  const int ui = find_unit(bin_prefix, nunits, t);
  const Unit& u = units[ui];
  const int local = t - bin_prefix[ui];
  const int br = local / u.BW, bc = local % u.BW;
  const BinStat own = bin_stat(u, st[ui].cur, local, br, bc);
  u.st_n[local] = own.n;
  u.st_sp[local] = own.sp;
  unsigned msc = (unsigned)own.n;
  if (u.upper >= 0) {
    const Unit& up = units[u.upper];
    msc += (unsigned)__popcll(up.occ[(size_t)(br >> 1) * up.BW + (bc >> 1)]);
  }
  u.msc[local] = msc;
  float2 flow = make_float2(-500.f, -500.f);
  int vi = ui, vbr = br, vbc = bc;
  BinStat v = own;
  float scale = 1.f;
  while (true) {
    const Unit& x = units[vi];
    if (x.upper < 0) {
      if (v.n > 1) flow = make_float2((float)(v.sp.x / v.n) * scale, (float)(v.sp.y / v.n) * scale);
      break;
    }
    if (v.n > 1) {
      flow = make_float2((float)v.sp.x * scale, (float)v.sp.y * scale);
      break;
    }
    vi = x.upper;
    vbr >>= 1;
    vbc >>= 1;
    scale *= 2.f;
    const Unit& y = units[vi];
    v = bin_stat(y, st[vi].cur, (size_t)vbr * y.BW + vbc, vbr, vbc);
  }
  u.flow[local] = flow;
}

// ---------------------------------------------------------------------------
// Detector mask, part 1: particle_mask_kernel (tracking_strategies.hpp:201-225)
// zeroes the mask at every particle slot's position and its 8 neighbours
// (dead slots included).  Here those pixels get a bit in `pmask`: k_pmask marks
// every slot's position in `ppos` (one atomic per slot) and k_pmask_dilate
// dilates that bitmap by the 3x3 box, one 64-bit bin word per thread.
__device__ __forceinline__ bool det_frame(const Unit& u, int f) { return (f % u.det_freq) == 0; }
__device__ __forceinline__ bool filt_frame(const Unit& u, int f) { return (f % u.filt_freq) == 0; }

__global__ void __launch_bounds__(CHUNK) k_pmask(const Unit* __restrict__ units, const UState* __restrict__ st,
                                                 const Frame* __restrict__ fr, const int* __restrict__ table,
                                                 int nunits) {
  const int f = fr->f;
  const int total = table[nunits];
  for (int g = blockIdx.x; g < total; g += gridDim.x) {
    ChunkCursor cc = chunk_of(table, nunits, g);
    const Unit& u = units[cc.unit];
    if (!det_frame(u, f) || u.det_kind != GBT_DETECTOR_FAST) continue;
    const UState s = st[cc.unit];
    const int i = cc.chunk * CHUNK + threadIdx.x;
    if (i >= s.n) continue;
    const short2 p = u.pos[s.cur][i];
    atomicOr(&u.ppos[bin_word(u, p.x, p.y)], bin_bit(p.x, p.y));
  }
}

// Row-wise 3-pixel dilation of a bin word (bit (r&7)*8 + (c&7)) with the
// edge columns of its left and right neighbour words.
__device__ __forceinline__ unsigned long long dilate_row(unsigned long long w, unsigned long long wl,
                                                         unsigned long long wr) {
  const unsigned long long C0 = 0x0101010101010101ull, C7 = 0x8080808080808080ull;
  return w | ((w << 1) & ~C0) | ((w >> 1) & ~C7) | ((wl >> 7) & C0) | ((wr << 7) & C7);
}

__global__ void __launch_bounds__(256) k_pmask_dilate(const Unit* __restrict__ units, const Frame* __restrict__ fr,
                                                      const int* __restrict__ bin_prefix, int nunits) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= bin_prefix[nunits]) return;
  const int ui = find_unit(bin_prefix, nunits, t);
  const Unit& u = units[ui];
  if (!det_frame(u, fr->f) || u.det_kind != GBT_DETECTOR_FAST) return;
  const int local = t - bin_prefix[ui];
  const int br = local / u.BW, bc = local % u.BW;
  auto word = [&](int r, int c) -> unsigned long long {
    return (r >= 0 && r < u.BH && c >= 0 && c < u.BW) ? u.ppos[(size_t)r * u.BW + c] : 0ull;
  };
  auto hrow = [&](int r) -> unsigned long long { return dilate_row(word(r, bc), word(r, bc - 1), word(r, bc + 1)); };
  const unsigned long long h = hrow(br), hu = hrow(br - 1), hd = hrow(br + 1);
  u.pmask[local] = h | (h << 8) | (h >> 8) | (hu >> 56) | (hd << 56);
}

// fast::compute_saliency for a pixel P of a shared tile with compile-time row
// length LD (the score itself: fast_score in gbt_device.cuh).
template <int LD>
__device__ __forceinline__ int fast_saliency_bf(const uint8_t* P, int n_, int th) {
  int ring[16];
#pragma unroll
  for (int i = 0; i < 16; i++) ring[i] = P[circle16_r(i) * LD + circle16_c(i)];
  return fast_score(ring, P[0], n_, th);
}

// A necessary condition of the FAST run test for n_ >= 8: any 8 cyclically
// consecutive ring positions hold two cyclically adjacent ones of the four
// cardinal positions 0, 4, 8, 12, so a run of n_ >= 8 strong pixels of one
// sign makes two adjacent cardinals strong with that sign.  Pixels that fail
// it score 0 in fast_saliency_bf.
template <int LD>
__device__ __forceinline__ bool fast_pretest(const uint8_t* P, int th) {
  const int vp = P[0];
  unsigned B = 0, D = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int d = (int)P[circle16_r(4 * k) * LD + circle16_c(4 * k)] - vp;
    B |= (unsigned)(d > th) << k;
    D |= (unsigned)(-d > th) << k;
  }
  const unsigned rb = ((B >> 1) | (B << 3)) & 15u, rd = ((D >> 1) | (D << 3)) & 15u;
  return ((B & rb) | (D & rd)) != 0;
}

// Saliency + 3x3 tile non-maximum selection: fast_detector::update and
// new_particles(cpu) (tracking2/fast_detector.hpp:217-262,296-313) fused.  A
// tile q owns pixels 3q + (1,1) + [0,2]^2; it is skipped when any of them holds
// a particle, otherwise its first strict maximum (raster order) becomes a birth
// if the saliency reaches the threshold and the point lies in the
// domain - border(3).  Result per tile: dr * 3 + dc, or 0xFF.  A pixel's
// saliency is 0 where the detector mask is cleared (next to a particle,
// particle_mask_kernel) or the contrast is below 5 (flow_mask_kernel,
// tracking_strategies.hpp:202-252).
//
// A CTA covers 8 x 32 tiles: it stages their pixels (with the ring's 3-pixel
// halo) and the occupancy / mask words of the bins they touch in shared
// memory.  Each thread screens the nine pixels of its tile (unoccupied tile,
// unmasked pixel, fast_pretest) and lists the survivors -- about a quarter of
// the pixels -- so that the full test (contrast and fast_saliency_bf) runs
// packed over the CTA's threads; then each thread takes the first strict
// maximum of its tile.
constexpr int DT_R = 8, DT_C = 32;  // tiles per CTA
constexpr int DT_PR = DT_R * 3 + 6, DT_PC = DT_C * 3 + 6;
constexpr int DT_BR = (DT_R * 3 + 7) / 8 + 1, DT_BC = (DT_C * 3 + 7) / 8 + 1;  // bins touched

__global__ void __launch_bounds__(256) k_detect(const Unit* __restrict__ units, const Frame* __restrict__ fr,
                                                const int* __restrict__ blk_prefix, int nunits) {
  __shared__ uint8_t tile[DT_PR][DT_PC];
  __shared__ unsigned long long s_occ[DT_BR][DT_BC], s_pm[DT_BR][DT_BC];
  __shared__ uint8_t sal[DT_R * DT_C][9];
  __shared__ unsigned short cand[DT_R * DT_C * 9];  // tile * 9 + pixel
  __shared__ int ncand;
  const int f = fr->f;
  const int t = blockIdx.x;
  const int ui = find_unit(blk_prefix, nunits, t);
  const Unit& u = units[ui];
  if (!det_frame(u, f) || u.det_kind != GBT_DETECTOR_FAST) return;
  const int local = t - blk_prefix[ui];
  const int bw = (u.TW + DT_C - 1) / DT_C;
  const int TR0 = (local / bw) * DT_R, TC0 = (local % bw) * DT_C;
  const int pr0 = 3 * TR0 + 1 - 3, pc0 = 3 * TC0 + 1 - 3;  // staged origin
  const int br0 = (3 * TR0 + 1) >> 3, bc0 = (3 * TC0 + 1) >> 3;
  for (int v = threadIdx.x; v < DT_PR * DT_PC; v += blockDim.x) {
    const int r = v / DT_PC, c = v % DT_PC;
    tile[r][c] = (uint8_t)img_at(u, pr0 + r, pc0 + c);
  }
  for (int v = threadIdx.x; v < DT_BR * DT_BC; v += blockDim.x) {
    const int r = v / DT_BC, c = v % DT_BC;
    const int br = br0 + r, bc = bc0 + c;
    const bool ok = br < u.BH && bc < u.BW;
    s_occ[r][c] = ok ? u.occ[(size_t)br * u.BW + bc] : 0ull;
    s_pm[r][c] = ok ? u.pmask[(size_t)br * u.BW + bc] : 0ull;
  }
  if (threadIdx.x == 0) ncand = 0;
  __syncthreads();
  auto bit = [&](const unsigned long long (*w)[DT_BC], int r, int c) -> bool {
    return (w[(r >> 3) - br0][(c >> 3) - bc0] >> (((r & 7) << 3) | (c & 7))) & 1ull;
  };
  // Screening: the thread's own tile.
  const int lt = threadIdx.x;
  const int tr = TR0 + lt / DT_C, tc = TC0 + lt % DT_C;
  const int pr = 3 * tr + 1, pc = 3 * tc + 1;
  const bool valid = tr < u.TH && tc < u.TW;
  bool open = false;
  if (valid) {
    bool occupied = false;
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
      for (int c = 0; c < 3; c++)
        if (in_dom(u, pr + r, pc + c) && bit(s_occ, pr + r, pc + c)) occupied = true;
    open = !occupied;
    if (occupied) u.tilecode[(size_t)tr * u.TW + tc] = 0xFF;
  }
  const bool pre = u.nfast >= 8;
  const uint8_t* P0 = &tile[pr - pr0][pc - pc0];
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const int r = q / 3, c = q % 3;
    sal[lt][q] = 0;
    const bool keep = open && in_dom(u, pr + r, pc + c) && !bit(s_pm, pr + r, pc + c) &&
                      (!pre || fast_pretest<DT_PC>(P0 + r * DT_PC + c, u.threshold));
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    int base = 0;
    if ((threadIdx.x & 31) == 0 && m) base = atomicAdd(&ncand, __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (keep) cand[base + __popc(m & ((1u << (threadIdx.x & 31)) - 1u))] = (unsigned short)(lt * 9 + q);
  }
  __syncthreads();
  // Full test of the listed pixels, packed over the CTA.
  for (int k = threadIdx.x; k < ncand; k += blockDim.x) {
    const int e = cand[k], ct = e / 9, q = e % 9;
    const int cpr = 3 * (TR0 + ct / DT_C) + 1 + q / 3, cpc = 3 * (TC0 + ct % DT_C) + 1 + q % 3;
    const uint8_t* P = &tile[cpr - pr0][cpc - pc0];
    const int d = 2;
    const int con = abs((int)P[d] - (int)P[-d]) + abs((int)P[-d * DT_PC] - (int)P[d * DT_PC]) +
                    abs((int)P[-d * DT_PC - d] - (int)P[d * DT_PC + d]) +
                    abs((int)P[-d * DT_PC + d] - (int)P[d * DT_PC - d]);
    if (con >= 5) sal[ct][q] = (uint8_t)fast_saliency_bf<DT_PC>(P, u.nfast, u.threshold);
  }
  __syncthreads();
  if (!open) return;
  // The first strict maximum of the tile (pixels outside the domain do not
  // take part; every other pixel does, with saliency 0 where it was screened out).
  int vmax = -1, mr = 0, mc = 0;
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const int r = q / 3, c = q % 3;
    if (!in_dom(u, pr + r, pc + c)) continue;
    const int v = sal[lt][q];
    if (vmax < v) {
      vmax = v;
      mr = r;
      mc = c;
    }
  }
  uint8_t code = 0xFF;
  if (vmax >= u.threshold) {
    const int gr = pr + mr, gc = pc + mc;
    if (gr >= 3 && gr <= u.H - 4 && gc >= 3 && gc <= u.W - 4) code = (uint8_t)(mr * 3 + mc);
  }
  u.tilecode[(size_t)tr * u.TW + tc] = code;
}

// The regular and dense detectors (regular_detector.hpp:62-103,
// dense_detector.hpp:19-31): one thread per 8x8 bin writes the bin's birth
// bits into `pmask` (which the FAST mask does not use for these units).
// Regular: pixels whose row and column are multiples of `step` and whose
// contrast -- the mean of |I(p + 2 c8_h[i]) - I(p)| over the 8 neighbours, on
// domain - border(1), 0 on the outer ring -- reaches grad_th (existing
// particles are not checked).  Dense: every pixel no particle matched to.
__global__ void __launch_bounds__(256) k_detect_alt(const Unit* __restrict__ units, const Frame* __restrict__ fr,
                                                    const int* __restrict__ bin_prefix, int nunits) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= bin_prefix[nunits]) return;
  const int ui = find_unit(bin_prefix, nunits, t);
  const Unit& u = units[ui];
  if (u.det_kind == GBT_DETECTOR_FAST || !det_frame(u, fr->f)) return;
  const int local = t - bin_prefix[ui];
  const int br = local / u.BW, bc = local % u.BW;
  unsigned long long w = 0;
  if (u.det_kind == GBT_DETECTOR_DENSE) {
    w = ~u.occ[local];
  } else {
    for (int k = 0; k < 64; k++) {
      const int r = br * 8 + (k >> 3), c = bc * 8 + (k & 7);
      if (r % u.det_step || c % u.det_step) continue;
      int rc = 0;
      if (r >= 1 && r <= u.H - 2 && c >= 1 && c <= u.W - 2) {
        const int vp = img_at(u, r, c);
        int res = 0;
#pragma unroll
        for (int i = 0; i < 8; i++) res += abs(img_at(u, r + 2 * c8r(i), c + 2 * c8c(i)) - vp);
        rc = res / 8;
      }
      if (rc >= u.det_grad_th) w |= 1ull << k;
    }
  }
  // Pixels outside the domain (last bin row / column) never give birth.
  const int vr = min(8, u.H - br * 8), vc = min(8, u.W - bc * 8);
  unsigned long long valid = 0;
  for (int k = 0; k < 64; k++)
    if ((k >> 3) < vr && (k & 7) < vc) valid |= 1ull << k;
  u.pmask[local] = w & valid;
}

// Birth items.  FAST: ordered (tile row, row inside the tile, tile column),
// which is the raster order of the birth pixels (st_apply2d over
// domain - border(3), fast_detector.hpp:256-260).  Regular / dense: the
// pixels of the domain in raster order (domain - border(0)), births where
// k_detect_alt set a bit.
__device__ __forceinline__ bool birth_item(const Unit& u, int v, int& r, int& c) {
  if (u.det_kind != GBT_DETECTOR_FAST) {
    r = v / u.W;
    c = v % u.W;
    return (u.pmask[bin_word(u, r, c)] & bin_bit(r, c)) != 0;
  }
  const int per = u.TW;
  int row3 = v / per, tc = v % per;
  int tr = row3 / 3, dr = row3 % 3;
  if (tr >= u.TH) return false;
  uint8_t code = u.tilecode[(size_t)tr * u.TW + tc];
  if (code == 0xFF || code / 3 != dr) return false;
  r = 3 * tr + 1 + dr;
  c = 3 * tc + 1 + code % 3;
  return true;
}

// Counts per chunk: survivors (age != 0) over the pre-compaction slots of each
// detector-frame unit, and births over its birth items.
// Survivors and births are counted per warp of 32 slots / items
// (chunk_cnt[i / 32], birth_cnt[i / 32]); the unit scan turns the counts into
// offsets, so neither pass needs a block-wide prefix.
__global__ void __launch_bounds__(CHUNK) k_det_count(const Unit* __restrict__ units, const UState* __restrict__ st,
                                                     const Frame* __restrict__ fr, const int* __restrict__ table,
                                                     const int* __restrict__ btable, int nunits) {
  const int f = fr->f;
  const int ts = table[nunits], tb = btable[nunits];
  for (int g = blockIdx.x; g < ts + tb; g += gridDim.x) {
    bool births = g >= ts;
    ChunkCursor cc = births ? chunk_of(btable, nunits, g - ts) : chunk_of(table, nunits, g);
    const Unit& u = units[cc.unit];
    if (!det_frame(u, f)) continue;  // uniform per block
    const int i = cc.chunk * CHUNK + threadIdx.x;
    bool pred;
    int lim;
    if (births) {
      int r, c;
      lim = u.birth_items;
      pred = i < lim && birth_item(u, i, r, c);
    } else {
      const UState s = st[cc.unit];
      lim = s.n;
      pred = i < lim && u.age[s.cur][i] != 0;
    }
    const unsigned b = __ballot_sync(0xffffffffu, pred);
    if ((threadIdx.x & 31) == 0 && i < lim) (births ? u.birth_cnt : u.chunk_cnt)[i >> 5] = __popc(b);
  }
}

// Per-unit exclusive scans of chunk counts.  which: 0 = detector (survivors
// and births), 1 = merge actives.
__global__ void __launch_bounds__(1024) k_unit_scan(const Unit* __restrict__ units, UState* __restrict__ st,
                                                    const Frame* __restrict__ fr) {
  __shared__ int wt[65];
  const int ui = blockIdx.x;
  const Unit& u = units[ui];
  const int f = fr->f;
  if (!det_frame(u, f)) return;
  UState& s = st[ui];
  auto scan = [&](int* cnt, int nch) -> int {
    int carry = 0;
    for (int base = 0; base < nch; base += 1024) {
      int k = base + threadIdx.x;
      int v = k < nch ? cnt[k] : 0;
      // inclusive block scan of v
      const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
      int x = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      if (lane == 31) wt[wid] = x;
      __syncthreads();
      if (wid == 0) {
        int w = wt[lane];
        int z = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          int y = __shfl_up_sync(0xffffffffu, z, o);
          if (lane >= o) z += y;
        }
        wt[32 + lane] = z - w;
        if (lane == 31) wt[64] = z;
      }
      __syncthreads();
      int excl = carry + wt[32 + wid] + x - v;
      if (k < nch) cnt[k] = excl;
      carry += wt[64];
      __syncthreads();
    }
    return carry;
  };
  // per-warp counts of k_det_count
  int S = scan(u.chunk_cnt, (s.n + 31) / 32);
  int B = scan(u.birth_cnt, (u.birth_items + 31) / 32);
  if (threadIdx.x == 0) {
    s.n_old = s.n;
    s.S = S;
    s.B = B;
  }
}

// Stable compaction (particle_container::compact(cpu),
// particle_container.hpp:215-252) and births (fast_detector.hpp:256-260 +
// particle_container::add, :370-387): survivors keep their order, births follow
// in raster order; matches[old] = new slot (-1 for dead slots).
__global__ void __launch_bounds__(CHUNK) k_det_scatter(const Unit* __restrict__ units, const UState* __restrict__ st,
                                                       Frame* __restrict__ fr, const int* __restrict__ table,
                                                       const int* __restrict__ btable, int nunits) {
  const int f = fr->f;
  const int ts = table[nunits], tb = btable[nunits];
  const unsigned lt = (1u << (threadIdx.x & 31)) - 1u;
  for (int g = blockIdx.x; g < ts + tb; g += gridDim.x) {
    bool births = g >= ts;
    ChunkCursor cc = births ? chunk_of(btable, nunits, g - ts) : chunk_of(table, nunits, g);
    const Unit& u = units[cc.unit];
    if (!det_frame(u, f)) continue;
    const UState s = st[cc.unit];
    const int i = cc.chunk * CHUNK + threadIdx.x;
    const int ob = s.cur, nb = s.cur ^ 1;
    const unsigned long long stamp = (unsigned long long)stamp_compact(f) << 32;
    if (!births) {
      if ((i & ~31) >= s.n_old) continue;  // whole warp past the slots
      bool alive = i < s.n_old && u.age[ob][i] != 0;
      int o = u.chunk_cnt[i >> 5] + __popc(__ballot_sync(0xffffffffu, alive) & lt);
      if (i < s.n_old) u.matches[i] = alive ? o : -1;
      if (alive) {
        short2 p = u.pos[ob][i];
        u.pos[nb][o] = p;
        u.spd[nb][o] = u.spd[ob][i];
        u.age[nb][o] = u.age[ob][i];
        u.feat[nb][o] = u.feat[ob][i];
        atomicMax(&u.idx[(size_t)p.x * u.W + p.y], stamp | (unsigned)o);
      }
    } else {
      if ((i & ~31) >= u.birth_items) continue;  // whole warp past the items
      int r = 0, c = 0;
      bool born = i < u.birth_items && birth_item(u, i, r, c);
      int k = u.birth_cnt[i >> 5] + __popc(__ballot_sync(0xffffffffu, born) & lt);
      if (born) {
        int o = s.S + k;
        if (o >= u.cap) {
          atomicOr(&fr->err, ERR_CAPACITY);
        } else {
          Feat F;
          F.init(u);
          u.pos[nb][o] = make_short2((short)r, (short)c);
          u.spd[nb][o] = make_short2(0, 0);
          u.age[nb][o] = 1;
          u.feat[nb][o] = F.at(r, c, u.fpitch);
          u.matches[s.n_old + k] = o;
          atomicMax(&u.idx[(size_t)r * u.W + c], stamp | (unsigned)o);
          atomicOr(&u.occ[bin_word(u, r, c)], bin_bit(r, c));  // occ <=> a current index entry
        }
      }
    }
  }
}

// Commits detector-frame counters and rebuilds a chunk table over the
// current slot counts (one CTA).
__device__ void build_table(const Unit* units, const UState* st, int nunits, int* table) {
  __shared__ int wt[65];
  int carry = 0;
  for (int base = 0; base < nunits; base += blockDim.x) {
    int k = base + threadIdx.x;
    int v = k < nunits ? (st[k].n + CHUNK - 1) / CHUNK : 0;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wt[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int nw = blockDim.x / 32;
      int w = lane < nw ? wt[lane] : 0;
      int z = w;
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, z, o);
        if (lane >= o) z += y;
      }
      wt[32 + lane] = z - w;
      if (lane == 31) wt[64] = z;
    }
    __syncthreads();
    if (k < nunits) table[k] = carry + wt[32 + wid] + x - v;
    carry += wt[64];
    __syncthreads();
  }
  if (threadIdx.x == 0) table[nunits] = carry;
}

__global__ void __launch_bounds__(1024) k_commit(const Unit* __restrict__ units, UState* __restrict__ st,
                                                 const Frame* __restrict__ fr, int* __restrict__ post_table,
                                                 int nunits) {
  const int f = fr->f;
  for (int k = threadIdx.x; k < nunits; k += blockDim.x) {
    const Unit& u = units[k];
    if (!det_frame(u, f)) continue;
    UState& s = st[k];
    int n = s.S + s.B;
    s.n = n < u.cap ? n : u.cap;
    s.nmatches = s.n_old + s.B;
    s.compact = 1;
    s.cur ^= 1;
  }
  __syncthreads();
  build_table(units, st, nunits, post_table);
}

// ---------------------------------------------------------------------------
// filter_bad_particles_kernel (tracking_strategies.hpp:482-523): whether live
// particle i at p survives.  It is removed when older than 2 frames and more
// than 10 px from its bin's fused flow, or when its bin's multiscale count is
// 1 and no c8 bin has a nonzero count.
// The decision from the bin's count m, its flow fl and the particle's speed v.
__device__ __forceinline__ bool filter_decide(const Unit& u, unsigned short age, unsigned m, float2 fl, short2 v,
                                              int br, int bc) {
  if (age > 2 && m > 0) {
    float dx = __fsub_rn((float)v.x, fl.x), dy = __fsub_rn((float)v.y, fl.y);
    float nrm = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
    if (nrm > 10.f) return false;
  }
  if (m != 1) return true;
  for (int k = 0; k < 8; k++) {
    int nr = br + c_c8[k][0], nc = bc + c_c8[k][1];
    if (nr >= 0 && nr < u.BH && nc >= 0 && nc < u.BW && u.msc[(size_t)nr * u.BW + nc] != 0) return true;
  }
  return false;
}

__device__ __forceinline__ bool filter_keeps(const Unit& u, int b, int i, unsigned short age, short2 p) {
  const int br = p.x / 8, bc = p.y / 8;
  const size_t w = (size_t)br * u.BW + bc;
  const unsigned m = u.msc[w];
  if (age > 2 && m > 0) {
    short2 v = u.spd[b][i];
    float2 fl = u.flow[w];
    float dx = __fsub_rn((float)v.x, fl.x), dy = __fsub_rn((float)v.y, fl.y);
    float nrm = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
    if (nrm > 10.f) return false;
  }
  if (m != 1) return true;
  for (int k = 0; k < 8; k++) {
    int nr = br + c_c8[k][0], nc = bc + c_c8[k][1];
    if (nr >= 0 && nr < u.BH && nc >= 0 && nc < u.BW && u.msc[(size_t)nr * u.BW + nc] != 0) return true;
  }
  return false;
}

// ---------------------------------------------------------------------------
// merge_trajectories (tracking2/merge_trajectories.h:10-35) over the slots in
// index order.  Kills only go from a particle to an older neighbour, and only
// particles with at least one qualifying neighbour ("actives", a few hundred
// per frame) can kill.  Step 1 (parallel): the qualifying c8 directions of each
// live particle, using pre-merge ages.  Step 2: ordered list of actives.
// Step 3: one warp per unit replays the sequential order; groups of 32 actives
// whose positions are more than 2 pixels apart cannot interact and are
// resolved in parallel, other groups lane by lane.
// With FILTERED false the ages of the filter's victims are still in place
// (the filter runs in the same launch), so a neighbour also has to pass
// filter_keeps; the filter's decision is a function of the bin statistics
// alone, so both passes see the same candidates.
// occ marks exactly the pixels whose index entry is current (matched
// particles, and births on detector frames): most neighbours are empty.  The
// 3x3 box around p touches at most four bin words (rows ra / rb, columns ca /
// cb), loaded by box_words.
struct BoxWords {
  unsigned long long a, b, c, d;
};
__device__ __forceinline__ BoxWords box_words(const Unit& u, short2 p) {
  const int ra = max(p.x - 1, 0), rb = min(p.x + 1, u.H - 1), ca = max(p.y - 1, 0), cb = min(p.y + 1, u.W - 1);
  return BoxWords{u.occ[bin_word(u, ra, ca)], u.occ[bin_word(u, ra, cb)], u.occ[bin_word(u, rb, ca)],
                  u.occ[bin_word(u, rb, cb)]};
}

template <bool FILTERED>
__device__ __forceinline__ unsigned merge_dirs_w(const Unit& u, const UState& s, int f, short2 p, short2 v,
                                                 unsigned short age, const BoxWords& bw, int* cand, int& ncand) {
  unsigned m = 0;
  ncand = 0;
  const int ra = max(p.x - 1, 0), ca = max(p.y - 1, 0);
  const unsigned long long wa = bw.a, wb = bw.b, wc = bw.c, wd = bw.d;
  unsigned nb = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int r = p.x + c8r(k), c = p.y + c8c(k);
    const bool top = (r >> 3) == (ra >> 3), left = (c >> 3) == (ca >> 3);
    const unsigned long long w = top ? (left ? wa : wb) : (left ? wc : wd);
    if (in_dom(u, r, c) && (w & bin_bit(r, c))) nb |= 1u << k;
  }
  if (!nb) return 0;
  while (nb) {  // occupied neighbours in c8_h order
    const int k = __ffs(nb) - 1;
    nb &= nb - 1;
    const int r = p.x + c8_dr(k), c = p.y + c8_dc(k);
    unsigned long long e = u.idx[(size_t)r * u.W + c];
    if (!idx_current(e, f)) continue;
    unsigned j = (unsigned)(e & 0xffffffffu);
    unsigned short aj = u.age[s.cur][j];
    if ((int)aj > (int)age + 2) {
      short2 w = u.spd[s.cur][j];
      int dx = v.x - w.x, dy = v.y - w.y;
      if (dx * dx + dy * dy < 4 &&  // sqrt(dx^2 + dy^2) < 2 with integral speeds
          (FILTERED || filter_keeps(u, s.cur, (int)j, aj, make_short2((short)r, (short)c)))) {
        m |= 1u << k;
        if (cand) cand[ncand] = (int)j;
        ncand++;
      }
    }
  }
  return m;
}

template <bool FILTERED>
__device__ __forceinline__ unsigned merge_dirs(const Unit& u, const UState& s, int f, int i, short2 p,
                                               unsigned short age, int* cand, int& ncand) {
  return merge_dirs_w<FILTERED>(u, s, f, p, u.spd[s.cur][i], age, box_words(u, p), cand, ncand);
}

// filter_bad_particles_kernel (tracking_strategies.hpp:482-523) and step 1 of
// the merge in one pass: each live particle applies the filter to itself and,
// when it survives, finds its qualifying directions.  Actives are counted per
// warp of 32 slots (act_cnt[i / 32]) and their candidates stored at their slot
// (act_cand[8 i ..]) for k_merge_unit.
// Quarter-chunk CTAs (256 threads) for the merge passes, compiled for five
// CTAs per SM (at most 48 registers a thread; with no bound the kernel takes
// 60 and four fit): the pass waits on dependent global loads, so more
// resident threads keep more of them in flight.
constexpr int FM_THREADS = 256;
constexpr int FM_SUB = CHUNK / FM_THREADS;

__global__ void __launch_bounds__(FM_THREADS, 5) k_filter_merge(const Unit* __restrict__ units,
                                                             const UState* __restrict__ st,
                                                             const Frame* __restrict__ fr,
                                                             const int* __restrict__ table, int nunits) {
  const int f = fr->f;
  const int total = table[nunits] * FM_SUB;
  for (int g = blockIdx.x; g < total; g += gridDim.x) {
    ChunkCursor cc = chunk_of(table, nunits, g / FM_SUB);
    const Unit& u = units[cc.unit];
    if (!filt_frame(u, f)) continue;
    const UState s = st[cc.unit];
    const int i = cc.chunk * CHUNK + (g % FM_SUB) * FM_THREADS + threadIdx.x;
    unsigned m = 0;
    if (i < s.n) {
      const unsigned short age = u.age[s.cur][i];
      if (age != 0) {
        // Everything that depends only on the slot and its position, loaded
        // together: the bin's count and flow, the speed, the box's occupancy.
        const short2 p = u.pos[s.cur][i];
        const int br = p.x / 8, bc = p.y / 8;
        const size_t w = (size_t)br * u.BW + bc;
        const unsigned mc = u.msc[w];
        const float2 fl = u.flow[w];
        const short2 v = u.spd[s.cur][i];
        const BoxWords bw = box_words(u, p);
        if (!filter_decide(u, age, mc, fl, v, br, bc)) {
          u.age[s.cur][i] = 0;
        } else if (u.with_merge) {
          // An active's candidates (c8_h order) go to act_cand at its slot.
          int cand[8], nc;
          m = merge_dirs_w<false>(u, s, f, p, v, age, bw, cand, nc);
          for (int q = 0; q < nc; q++) u.act_cand[(size_t)i * 8 + q] = cand[q];
        }
      }
      if (u.with_merge) u.cmask[i] = (uint8_t)m;
    }
    const unsigned b = __ballot_sync(0xffffffffu, m != 0);
    if (u.with_merge && (threadIdx.x & 31) == 0 && i < s.n) u.act_cnt[i >> 5] = __popc(b);
  }
}

// Liveness of the particles a batch of actives touches, in a shared-memory
// open-addressing table (key = slot + 1, top bit = killed).  Falls back to the
// global age array when the table would overflow.
constexpr int MR_NB = 512;      // actives per batch
constexpr int MR_HASH = 4096;   // table slots (power of two)

__device__ __forceinline__ int mr_find(unsigned* tab, unsigned key) {
  unsigned h = (key * 2654435761u) & (MR_HASH - 1);
  for (int probe = 0; probe < MR_HASH; probe++) {
    unsigned k = tab[h] & 0x7fffffffu;
    if (k == key || k == 0) return (int)h;
    h = (h + 1) & (MR_HASH - 1);
  }
  return -1;
}

// Block-wide exclusive prefix sum of one int per thread (blockDim.x a multiple
// of 32, at most 1024); `total` gets the sum.
__device__ __forceinline__ int block_scan(int v, int* warp_tot, int& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  if (wid == 0) {
    const int w = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
    int z = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, z, o);
      if (lane >= o) z += y;
    }
    warp_tot[32 + lane] = z - w;
    if (lane == 31) warp_tot[64] = z;
  }
  __syncthreads();
  const int r = warp_tot[32 + wid] + x - v;
  total = warp_tot[64];
  __syncthreads();
  return r;
}

// Steps 2 and 3 of the merge for one unit per CTA.  Step 2: the actives in
// slot order -- warps of 32 slots taken 1024 at a time, their active counts
// (act_cnt, from k_filter_merge) scanned across the CTA, and each warp with
// actives expanded by a warp of threads into act_list (slot, position, number
// of candidates; the candidates themselves are at the slot in act_cand).
// Step 3: the ordered replay described above.
constexpr int MU_THREADS = 1024;
static_assert(MR_HASH >= 2 * MU_THREADS, "the active-warp lists fit in the liveness table");

__global__ void __launch_bounds__(MU_THREADS) k_merge_unit(const Unit* __restrict__ units, UState* __restrict__ st,
                                                          const Frame* __restrict__ fr) {
  __shared__ int4 ent[MR_NB];
  __shared__ int cnd[MR_NB][8];
  __shared__ unsigned tab[MR_HASH];
  __shared__ int tab_fill, tab_over;
  __shared__ int wt[65];
  const int ui = blockIdx.x;
  const Unit& u = units[ui];
  const int f = fr->f;
  if (!filt_frame(u, f) || !u.with_merge) return;
  const UState s = st[ui];
  int A = 0;
  const int nw = (s.n + 31) >> 5;
  const int lane0 = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int* wl = (int*)tab;             // slot warps with actives (the table is free until step 3)
  int* wo = (int*)tab + MU_THREADS;  // and their first position in the ordered list
  for (int w0 = 0; w0 < nw; w0 += blockDim.x) {
    const int w = w0 + threadIdx.x;
    const int c = w < nw ? u.act_cnt[w] : 0;
    int tot, nact;
    const int off = A + block_scan(c, wt, tot);
    const int k = block_prefix(c > 0, wt, nact);
    if (c > 0) {
      wl[k] = w;
      wo[k] = off;
    }
    __syncthreads();
    // One warp of threads per listed slot warp: a lane per slot.
    for (int q = wid; q < nact; q += (int)(blockDim.x >> 5)) {
      const int i = 32 * wl[q] + lane0;
      const bool act = i < s.n && u.cmask[i] != 0;
      const unsigned bal = __ballot_sync(0xffffffffu, act);
      if (act) {
        // One candidate per direction bit, stored at the slot by k_filter_merge.
        const int o = wo[q] + __popc(bal & ((1u << lane0) - 1u));
        const short2 p = u.pos[s.cur][i];
        u.act_list[o] = make_int4(i, (int)(((unsigned)(unsigned short)p.x << 16) | (unsigned short)p.y),
                                  __popc((unsigned)u.cmask[i]), 0);
      }
    }
    A += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) st[ui].A = A;
  __threadfence_block();
  __syncthreads();
  unsigned short* age = u.age[s.cur];
  const int lane = threadIdx.x & 31;
  for (int base = 0; base < A; base += MR_NB) {
    const int nb = min(MR_NB, A - base);
    for (int k = threadIdx.x; k < MR_HASH; k += blockDim.x) tab[k] = 0;
    if (threadIdx.x == 0) {
      tab_fill = 0;
      tab_over = 0;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nb; k += blockDim.x) {
      int4 e = u.act_list[base + k];
      ent[k] = e;
      for (int q = 0; q < e.z; q++) cnd[k][q] = u.act_cand[(size_t)e.x * 8 + q];
    }
    __syncthreads();
    // Register every touched slot with its current liveness (killed bit set
    // when an earlier batch already killed it).
    for (int k = threadIdx.x; k < nb; k += blockDim.x) {
      const int4 e = ent[k];
      for (int q = -1; q < e.z; q++) {
        const unsigned slot = (unsigned)(q < 0 ? e.x : cnd[k][q]);
        const unsigned key = slot + 1u;
        if (atomicAdd(&tab_fill, 1) >= MR_HASH / 2) {
          tab_over = 1;
          continue;
        }
        unsigned h = (key * 2654435761u) & (MR_HASH - 1);
        for (int probe = 0; probe < MR_HASH; probe++) {
          unsigned prev = atomicCAS(&tab[h], 0u, key | (age[slot] == 0 ? 0x80000000u : 0u));
          if (prev == 0 || (prev & 0x7fffffffu) == key) break;
          h = (h + 1) & (MR_HASH - 1);
        }
      }
    }
    __syncthreads();
    const bool smem = !tab_over;
    if (threadIdx.x < 32) {
      for (int g0 = 0; g0 < nb; g0 += 32) {
        const int k = g0 + lane;
        const bool valid = k < nb;
        const int4 e = valid ? ent[k] : make_int4(-1, 0, 0, 0);
        const int pr = (short)((unsigned)e.y >> 16), pc = (short)((unsigned)e.y & 0xffffu);
        // Earlier lanes whose candidate sets may meet this lane's (within 2 px).
        unsigned before = 0;
        for (int o = 0; o < 32; o++) {
          int qr = __shfl_sync(0xffffffffu, pr, o), qc = __shfl_sync(0xffffffffu, pc, o);
          bool ov = __shfl_sync(0xffffffffu, valid, o);
          if (o < lane && ov && valid && abs(qr - pr) <= 2 && abs(qc - pc) <= 2) before |= 1u << o;
        }
        // Wavefronts: a lane decides once no earlier unresolved lane conflicts.
        unsigned pending = __ballot_sync(0xffffffffu, valid);
        while (pending) {
          const bool mine = (pending >> lane) & 1u;
          const bool ready = mine && !(before & pending);
          if (ready) {
            bool alive;
            int hs = -1;
            if (smem) {
              hs = mr_find(tab, (unsigned)e.x + 1u);
              alive = !(tab[hs] & 0x80000000u);
            } else {
              alive = *(volatile unsigned short*)&age[e.x] != 0;
            }
            if (alive) {
              for (int q = 0; q < e.z; q++) {
                const int j = cnd[k][q];
                bool jalive;
                int hj = -1;
                if (smem) {
                  hj = mr_find(tab, (unsigned)j + 1u);
                  jalive = !(tab[hj] & 0x80000000u);
                } else {
                  jalive = *(volatile unsigned short*)&age[j] != 0;
                }
                if (jalive) {
                  if (smem) tab[hj] |= 0x80000000u;
                  age[j] = 0;
                  break;
                }
              }
            }
          }
          __syncwarp();
          pending &= ~__ballot_sync(0xffffffffu, ready);
        }
      }
    }
    __syncthreads();
  }
}

// End of frame: frame counter and the chunk table of the next frame.
// ---------------------------------------------------------------------------
// Device-side trajectories: the sample's per-particle position history
// (samples/tracking/main.cc:39-57,125-127, at most T positions) kept in step
// with the particle slots the way particle_container::sync_attributes does
// (particle_container.hpp:514-553): after a compaction the history of old slot
// i moves to slot matches[i] (and is dropped when matches[i] < 0) and births
// start empty; then every live particle appends its position, dropping the
// oldest beyond T, and every dead slot's history is cleared
// (update_trajectories).  Runs after the frame's last kill.
__device__ __forceinline__ void traj_append(const Unit& u, int b, int j, int T, uint8_t head, uint8_t len) {
  if (u.age[b][j] > 0) {
    u.tpos[b][(size_t)head * u.cap + j] = u.pos[b][j];
    u.thead[b][j] = (uint8_t)(head + 1 == T ? 0 : head + 1);
    u.tlen[b][j] = (uint8_t)(len < T ? len + 1 : T);
  } else {
    u.thead[b][j] = 0;
    u.tlen[b][j] = 0;
  }
}

__global__ void __launch_bounds__(CHUNK) k_traj(const Unit* __restrict__ units, const UState* __restrict__ st,
                                                const int* __restrict__ cap_table, int nunits, int T) {
  const int total = cap_table[nunits];
  for (int g = blockIdx.x; g < total; g += gridDim.x) {
    ChunkCursor cc = chunk_of(cap_table, nunits, g);
    const Unit& u = units[cc.unit];
    const UState s = st[cc.unit];
    const int i = cc.chunk * CHUNK + threadIdx.x;
    const int b = s.cur;
    if (s.compact) {
      const int ob = b ^ 1;
      if (i < s.n_old) {
        const int ni = u.matches[i];
        if (ni >= 0) {
          const uint8_t len = u.tlen[ob][i], head = u.thead[ob][i];
          for (int k = 0; k < T; k++) u.tpos[b][(size_t)k * u.cap + ni] = u.tpos[ob][(size_t)k * u.cap + i];
          traj_append(u, b, ni, T, head, len);
        }
      }
      if (i >= s.S && i < s.n) traj_append(u, b, i, T, 0, 0);  // birth
    } else if (i < s.n) {
      traj_append(u, b, i, T, u.thead[b][i], u.tlen[b][i]);
    }
  }
}

// Rebuilds the per-frame chunk table from the current counters (after a
// checkpoint load).
// Every unit's particle slot count, gathered for one host read.
__global__ void k_counts(const UState* __restrict__ st, int nunits, int* __restrict__ out) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nunits; k += gridDim.x * blockDim.x) out[k] = st[k].n;
}

__global__ void __launch_bounds__(1024) k_tick_table(const Unit* __restrict__ units, const UState* __restrict__ st,
                                                     int nunits, int* __restrict__ pre_table) {
  build_table(units, st, nunits, pre_table);
}

__global__ void __launch_bounds__(1024) k_tick(const Unit* __restrict__ units, const UState* __restrict__ st,
                                               Frame* __restrict__ fr, int* __restrict__ pre_table, int nunits) {
  build_table(units, st, nunits, pre_table);
  if (threadIdx.x == 0) fr->f += 1;
}

}  // namespace gbt
