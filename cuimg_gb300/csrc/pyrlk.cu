// Pyramidal LK tracker strategy for sm_103a.
//
// Runs the reference's tracker<pyrlk_cpu<fast_detector<cpu>,
// iterative_lk_match_5x5>> (cuimg/tracking2/pyrlk_tracker.h:16-82,
// pyrlk_tracker.hpp:772-1063) for many streams at once: per frame, for every
// (stream, scale) unit,
//   - the level image and the strategy's input_ image: input_ is a fresh
//     bordered copy of the level made by copy(in, input_), which for equal
//     borders copies nrows * pitch bytes from the start of the allocation
//     (cuimg/copy.h:30-40, cuimg/cpu/host_image2d.hpp:76-110), so the top,
//     left and right borders hold the level's clamped values and the bottom
//     B rows of the domain and the bottom border stay zero (B = 3, the FAST
//     detector's border, pyrlk_tracker.hpp:822-827);
//   - frames > 0: the Sobel/8 gradient of the previous frame's input_ and the
//     LK match of every particle (pyrlk_match_particles_kernel, :677-769):
//     the prediction through the upper scales' get_flow_at (:1027-1063;
//     predictions.h:61-74), iterative_lk_match_5x5::match (:165-334) and
//     kernel_particle_container::move (particle_container.hpp:422-466);
//   - detector frames: the particle mask (every slot's position and its 8
//     neighbours, dead slots included, pyrlk_tracker.hpp:878-887), the FAST
//     saliency (fast_detector.hpp:296-313), 3x3 tile maxima and births in
//     raster order (:217-262), then the stable compaction
//     (particle_container.hpp:215-252);
//   - filtering frames: filter_bad_particles_kernel reads the strategy's
//     multiscale_count_ image, which pyrlk_cpu only ever memsets to zero, so
//     it removes nothing; then merge_trajectories (merge_trajectories.h:10-35)
//     in slot order.
// Window samples outside a level are clamped to its edge (the reference reads
// outside its images there).
//
// Every floating-point step is the reference's, in its order: bilinear
// samples with separate multiply and add roundings (this file is compiled
// with --fmad=false), the normal matrix and right-hand side summed over the
// masked pixels in window order, and the 25-pixel mask chosen as
// std::nth_element chooses it (nth_select.cuh).  One warp matches one
// particle: lanes sample the window in parallel, and the ordered sums are
// read back from shared memory by every lane, so all lanes hold the same
// iterate and take the same branches.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cuimg_gb300.h"
#include "gbt_device.cuh"
#include "nth_select.cuh"
#include "pyrlk.h"

namespace gbt_pk {

constexpr int BB = 3;    // input_ border (fast_detector::border_needed)
constexpr int MB = 4;    // detector mask border
constexpr int WS = 11, HWS = WS / 2, NW = WS * WS;  // iterative_lk_match_5x5's window
constexpr int NMASK = 25, MAXIT = 30;
constexpr float EPS = 0.1f;
constexpr int PPL = (NW + 31) / 32;  // window pixels per lane
constexpr int MW = 8;                // warps per matcher CTA
constexpr int SCAN_T = 1024;         // threads of the per-unit births / compaction CTA
constexpr int ERR_CAPACITY = 1;

struct PUnit {
  int H, W, stream, scale, nscales, base;  // base: unit index of scale 0 of the stream
  int threshold, nfast, det_freq, filt_freq, k, with_merge;
  int ipitch, mpitch;
  uint8_t* img[2];  // input_ by frame parity: (H + 2 BB) rows of ipitch bytes
  uint8_t* lvl;     // the tracker's level, H x W
  float2* grad;     // Sobel/8 of the previous input_, H x W (.x d/drow, .y d/dcol)
  uint8_t* mask;    // (H + 2 MB) rows of mpitch bytes
  uint8_t* sal;     // H x W
  uint32_t* sparse; // H x W: slot + 1, 0 = none
  float2* pos[2];
  float2* spd[2];
  uint16_t* age[2];
  int32_t* matches;
  uint8_t* cmask;   // merge candidate directions per slot
  uint8_t* items;   // 3 * TH * TW: births by (tile row * 3 + row in tile, tile column): column in tile + 1
  int cap, TH, TW;
};

struct PState {
  int n, cur, nmatches, compact;
};

__device__ __forceinline__ bool det_frame(const PUnit& u, int f) { return f % u.det_freq == 0; }
__device__ __forceinline__ bool merge_frame(const PUnit& u, int f) { return f % u.filt_freq == 0 && u.with_merge; }

__device__ __forceinline__ const uint8_t* img_at(const PUnit& u, int par, int r, int c) {
  return u.img[par] + (size_t)(r + BB) * u.ipitch + (c + BB);
}

__device__ __forceinline__ int find_unit(const int* prefix, int nunits, int g) {
  int lo = 0, hi = nunits - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= g)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// (domain - border(b)).has(i_int2(p)): truncation towards zero.
__device__ __forceinline__ bool box_has(int H, int W, int b, float y, float x) {
  const int r = (int)y, c = (int)x;
  return r >= b && r <= H - b - 1 && c >= b && c <= W - b - 1;
}

// li() (pyrlk_tracker.hpp:130-146) on input_ (domain coordinates clamped).
__device__ __forceinline__ float li_u8(const PUnit& u, int par, float y, float x) {
  int y0 = (int)y, x0 = (int)x;
  const float a0 = __fsub_rn(y, (float)y0), a1 = __fsub_rn(x, (float)x0);
  const int y1 = min(max(y0 + 1, 0), u.H - 1), x1 = min(max(x0 + 1, 0), u.W - 1);
  y0 = min(max(y0, 0), u.H - 1);
  x0 = min(max(x0, 0), u.W - 1);
  const float v00 = *img_at(u, par, y0, x0), v10 = *img_at(u, par, y1, x0);
  const float v01 = *img_at(u, par, y0, x1), v11 = *img_at(u, par, y1, x1);
  const float b0 = __fsub_rn(1.f, a0), b1 = __fsub_rn(1.f, a1);
  return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(b0, b1), v00), __fmul_rn(__fmul_rn(a0, b1), v10)),
                             __fmul_rn(__fmul_rn(b0, a1), v01)),
                   __fmul_rn(__fmul_rn(a0, a1), v11));
}

__device__ __forceinline__ float2 li_grad(const PUnit& u, float y, float x) {
  int y0 = (int)y, x0 = (int)x;
  const float a0 = __fsub_rn(y, (float)y0), a1 = __fsub_rn(x, (float)x0);
  const int y1 = min(max(y0 + 1, 0), u.H - 1), x1 = min(max(x0 + 1, 0), u.W - 1);
  y0 = min(max(y0, 0), u.H - 1);
  x0 = min(max(x0, 0), u.W - 1);
  const float2 v00 = u.grad[(size_t)y0 * u.W + x0], v10 = u.grad[(size_t)y1 * u.W + x0];
  const float2 v01 = u.grad[(size_t)y0 * u.W + x1], v11 = u.grad[(size_t)y1 * u.W + x1];
  const float b0 = __fsub_rn(1.f, a0), b1 = __fsub_rn(1.f, a1);
  const float w00 = __fmul_rn(b0, b1), w10 = __fmul_rn(a0, b1), w01 = __fmul_rn(b0, a1), w11 = __fmul_rn(a0, a1);
  float2 o;
  o.x = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(w00, v00.x), __fmul_rn(w10, v10.x)), __fmul_rn(w01, v01.x)),
                  __fmul_rn(w11, v11.x));
  o.y = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(w00, v00.y), __fmul_rn(w10, v10.y)), __fmul_rn(w01, v01.y)),
                  __fmul_rn(w11, v11.y));
  return o;
}

struct __align__(8) WarpSmem {
  unsigned long long ord[NW];  // (norm bits << 32 | window index) while selecting
  float as[NW];                // template, truncated to uint8 (i_uchar1 as[], :187)
  float tt[NW];                // residual terms of the final error
  float mgr[NMASK], mgc[NMASK], mas[NMASK];
  float p0[32], p1[32];
  short mr[NW], mc[NW];        // masked pixels' offsets; mr doubles as the selection flags
};

// iterative_lk_match_5x5::match (pyrlk_tracker.hpp:165-334) at level u of the
// point p with prediction transform ptr, by the whole warp.  Returns false
// when the matcher rejects (tr = (-1, -1), err = 1000 as the reference).  The
// final error is computed only when `want_err` (get_flow_at ignores it).  Not
// inlined: k_pk_match calls it for the upper scales and for the particle's
// own, and one copy of its long exact-order body keeps the kernel's code small.
__device__ __noinline__ bool lk_match(const PUnit& u, int par, WarpSmem& S, float py, float px, float ptr_y, float ptr_x,
                         bool want_err, float& tr_y, float& tr_x, float& err) {
  const int lane = threadIdx.x & 31;
  const int prev = par ^ 1;
  float gr[PPL], gc[PPL];
  unsigned nb[PPL];
  bool valid[PPL];
#pragma unroll
  for (int k = 0; k < PPL; k++) {
    const int i = lane + 32 * k;
    gr[k] = gc[k] = 0.f;
    nb[k] = 0;
    valid[k] = i < NW;
    if (valid[k]) {
      const int r = i / WS - HWS, c = i % WS - HWS;
      const float y = __fadd_rn(py, (float)r), x = __fadd_rn(px, (float)c);
      const float2 g = li_grad(u, y, x);
      gr[k] = g.x;
      gc[k] = g.y;
      S.as[i] = (float)(unsigned char)li_u8(u, prev, y, x);
      nb[k] = __float_as_uint(__fsqrt_rn(__fadd_rn(__fmul_rn(g.x, g.x), __fmul_rn(g.y, g.y))));
    }
  }
  // The NMASK strongest gradients as std::nth_element leaves them
  // (:207-228): a bitwise search for the NMASK-th largest norm t; when the
  // norms equal to t do not all fit, one lane replays nth_element's steps.
  bool sel[PPL];
  {
    unsigned t = 0;
    for (int bit = 30; bit >= 0; bit--) {
      const unsigned cand = t | (1u << bit);
      int cnt = 0;
#pragma unroll
      for (int k = 0; k < PPL; k++) cnt += __popc(__ballot_sync(0xffffffffu, valid[k] && nb[k] >= cand));
      if (cnt >= NMASK) t = cand;
    }
    int atleast = 0;
#pragma unroll
    for (int k = 0; k < PPL; k++) atleast += __popc(__ballot_sync(0xffffffffu, valid[k] && nb[k] >= t));
    if (atleast == NMASK) {
#pragma unroll
      for (int k = 0; k < PPL; k++) sel[k] = valid[k] && nb[k] >= t;
    } else {
#pragma unroll
      for (int k = 0; k < PPL; k++) {
        const int i = lane + 32 * k;
        if (valid[k]) {
          S.ord[i] = ((unsigned long long)nb[k] << 32) | (unsigned)i;
          S.mr[i] = 0;
        }
      }
      __syncwarp();
      if (lane == 0) gbt_sel::nth_select(S.ord, NW, NMASK);
      __syncwarp();
      if (lane < NMASK) S.mr[(int)(S.ord[lane] & 0xffffffffu)] = 1;
      __syncwarp();
#pragma unroll
      for (int k = 0; k < PPL; k++) sel[k] = valid[k] && S.mr[lane + 32 * k] != 0;
      __syncwarp();
    }
  }
  // Masked pixels in window order.
  {
    const unsigned lt = (1u << lane) - 1u;
    int base = 0;
#pragma unroll
    for (int k = 0; k < PPL; k++) {
      const unsigned bs = __ballot_sync(0xffffffffu, sel[k]);
      if (sel[k]) {
        const int m = base + __popc(bs & lt), i = lane + 32 * k;
        S.mgr[m] = gr[k];
        S.mgc[m] = gc[k];
        S.mas[m] = S.as[i];
        S.mr[m] = (short)(i / WS - HWS);
        S.mc[m] = (short)(i % WS - HWS);
      }
      base += __popc(bs);
    }
  }
  __syncwarp();
  // Normal matrix, summed in window order (every lane the same sums).
  float g00 = 0.f, g01 = 0.f, g11 = 0.f;
  for (int m = 0; m < NMASK; m++) {
    const float a = S.mgr[m], b = S.mgc[m];
    g00 = __fadd_rn(g00, __fmul_rn(a, a));
    g01 = __fadd_rn(g01, __fmul_rn(a, b));
    g11 = __fadd_rn(g11, __fmul_rn(b, b));
  }
  // Eigenvalues of the symmetric 2x2 G and its inverse (the 2x2 forms the
  // reference's Eigen calls reduce to).
  const float tr2 = __fmul_rn(__fadd_rn(g00, g11), 0.5f);
  const float det = __fsub_rn(__fmul_rn(g00, g11), __fmul_rn(g01, g01));
  const float disc = __fsqrt_rn(fmaxf(__fsub_rn(__fmul_rn(tr2, tr2), det), 0.f));
  const float e1 = fabsf(__fadd_rn(tr2, disc)), e2 = fabsf(__fsub_rn(tr2, disc));
  bool ok = !((e1 < e2 ? e1 : e2) < 0.0001f);
  const float pred_y = __fadd_rn(py, ptr_y), pred_x = __fadd_rn(px, ptr_x);
  float vy = pred_y, vx = pred_x;
  if (ok) {
    const float i00 = __fdiv_rn(g11, det), i01 = __fdiv_rn(-g01, det), i11 = __fdiv_rn(g00, det);
    float nk0 = 1.f, nk1 = 1.f;
    for (int it = 0; it < MAXIT && __fsqrt_rn(__fadd_rn(__fmul_rn(nk0, nk0), __fmul_rn(nk1, nk1))) >= EPS; it++) {
      if (lane < NMASK) {
        const float dt = __fsub_rn(S.mas[lane], li_u8(u, par, __fadd_rn(vy, (float)S.mr[lane]),
                                                      __fadd_rn(vx, (float)S.mc[lane])));
        S.p0[lane] = __fmul_rn(S.mgr[lane], dt);
        S.p1[lane] = __fmul_rn(S.mgc[lane], dt);
      }
      __syncwarp();
      float b0 = 0.f, b1 = 0.f;
      for (int m = 0; m < NMASK; m++) {
        b0 = __fadd_rn(b0, S.p0[m]);
        b1 = __fadd_rn(b1, S.p1[m]);
      }
      __syncwarp();
      nk0 = __fadd_rn(__fmul_rn(i00, b0), __fmul_rn(i01, b1));
      nk1 = __fadd_rn(__fmul_rn(i01, b0), __fmul_rn(i11, b1));
      vy = __fadd_rn(vy, nk0);
      vx = __fadd_rn(vx, nk1);
      const float d0 = __fsub_rn(pred_y, vy), d1 = __fsub_rn(pred_x, vx);
      if (__fsqrt_rn(__fadd_rn(__fmul_rn(d0, d0), __fmul_rn(d1, d1))) > (float)(WS * 4) ||
          !box_has(u.H, u.W, 3, vy, vx)) {
        ok = false;
        break;
      }
    }
  }
  __syncwarp();  // every lane is done with this call's masked-pixel arrays
  if (!ok) {
    tr_y = tr_x = -1.f;
    err = 1000.f;
    return false;
  }
  tr_y = __fsub_rn(vy, py);
  tr_x = __fsub_rn(vx, px);
  err = 0.f;
  if (want_err) {
    // Mean absolute residual with the reference's template index
    // (r + hws) * hws + (c + hws) and its running counter (:320-331), summed
    // in window order.
#pragma unroll
    for (int k = 0; k < PPL; k++) {
      const int i = lane + 32 * k;
      if (i < NW) {
        const int r = i / WS - HWS, c = i % WS - HWS;
        const int j = (r + HWS) * HWS + (c + HWS);
        S.tt[i] = fabsf(__fsub_rn(S.as[j], li_u8(u, par, __fadd_rn(vy, (float)r), __fadd_rn(vx, (float)c))));
      }
    }
    __syncwarp();
    float e = 0.f;
    for (int i = 0; i < NW; i++) e = __fadd_rn(e, S.tt[i]);
    err = __fdiv_rn(e, (float)(NMASK + NW));
  }
  __syncwarp();
  return true;
}

// ---------------------------------------------------------------------------
// Kernels.  Units of a stream are contiguous (scale 0 first); `par` is the
// current frame's parity (input_ = img[par], the previous frame's = img[par ^ 1]).

// Level `scale` of every stream: the tracker's level (2x2 floor means of the
// level below, tracker.hpp:53-69 and mipmap.h:24-49; level 0 is the frame,
// already in lvl) and input_ (see the file header).
__global__ void k_pk_level(PUnit* __restrict__ units, const int* __restrict__ scale_units, int nstreams, int par) {
  const int s = blockIdx.y;
  if (s >= nstreams) return;
  const int ui = scale_units[s];
  if (ui < 0) return;
  PUnit& u = units[ui];
  const PUnit* lo = u.scale > 0 ? &units[ui - 1] : nullptr;
  const int BH = u.H + 2 * BB, BW = u.W + 2 * BB;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < BH * BW; t += gridDim.x * blockDim.x) {
    const int r = t / BW - BB, c = t % BW - BB;
    const int rr = min(max(r, 0), u.H - 1), cc = min(max(c, 0), u.W - 1);
    int v;
    if (lo) {
      const uint8_t* a = lo->lvl + (size_t)(2 * rr) * lo->W + 2 * cc;
      v = ((int)a[0] + (int)a[1] + (int)a[lo->W] + (int)a[lo->W + 1]) / 4;
      if (r == rr && c == cc) u.lvl[(size_t)r * u.W + c] = (uint8_t)v;
    } else {
      v = u.lvl[(size_t)rr * u.W + cc];
    }
    u.img[par][(size_t)(r + BB) * u.ipitch + (c + BB)] = r < u.H - BB ? (uint8_t)v : 0;
  }
}

// Per unit: on frames > 0 the gradient of the previous input_ (Sobel/8 over
// domain - border(1), zero on the outer ring, pyrlk_tracker.hpp:910-938) and
// the emptied sparse index (before_matching); on detector frames the mask
// set to 255 (create_detector_mask's memset).
__global__ void k_pk_prep(PUnit* __restrict__ units, int nunits, int f, int par) {
  const int ui = blockIdx.y;
  if (ui >= nunits) return;
  PUnit& u = units[ui];
  const int prev = par ^ 1;
  const int np = u.H * u.W;
  const int stride = gridDim.x * blockDim.x;
  if (f > 0)
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < np; t += stride) {
      const int r = t / u.W, c = t % u.W;
      float2 g = make_float2(0.f, 0.f);
      if (r >= 1 && r < u.H - 1 && c >= 1 && c < u.W - 1) {
#define P(dr, dc) ((int)*img_at(u, prev, r + (dr), c + (dc)))
        g.x = (float)(P(1, -1) + 2 * P(1, 0) + P(1, 1) - P(-1, -1) - 2 * P(-1, 0) - P(-1, 1)) / 8.f;
        g.y = (float)(P(-1, 1) + 2 * P(0, 1) + P(1, 1) - P(-1, -1) - 2 * P(0, -1) - P(1, -1)) / 8.f;
#undef P
      }
      u.grad[t] = g;
      u.sparse[t] = 0u;
    }
  if (det_frame(u, f)) {
    const int nm = (u.H + 2 * MB) * u.mpitch / 4;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nm; t += stride) ((uint32_t*)u.mask)[t] = 0xFFFFFFFFu;
  }
}

// Per-unit slot counts -> prefix (slot-walking kernels index all units' slots).
__global__ void k_pk_prefix(const PState* __restrict__ st, int nunits, int* __restrict__ prefix) {
  if (threadIdx.x == 0) {
    int s = 0;
    for (int u = 0; u < nunits; u++) {
      prefix[u] = s;
      s += st[u].n;
    }
    prefix[nunits] = s;
  }
}

// pyrlk_match_particles_kernel (:677-769) for every slot, a warp per slot.
// Two CTAs per SM: 128 registers a thread hold the match without spilling
// (three CTAs at 80 registers spilled and measured 2% slower).
__global__ void __launch_bounds__(32 * MW, 2) k_pk_match(PUnit* __restrict__ units, PState* __restrict__ st, int nunits,
                                                     const int* __restrict__ prefix, int par) {
  __shared__ WarpSmem smem[MW];
  WarpSmem& S = smem[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int total = prefix[nunits];
  for (int g = blockIdx.x * MW + (threadIdx.x >> 5); g < total; g += gridDim.x * MW) {
    const int ui = find_unit(prefix, nunits, g);
    const PUnit& u = units[ui];
    const int i = g - prefix[ui], b = st[ui].cur;
    const unsigned short age = u.age[b][i];
    if (age == 0) continue;
    const float2 p = u.pos[b][i];
    if (!box_has(u.H, u.W, 3, p.x, p.y)) {
      if (lane == 0) u.age[b][i] = 0;
      continue;
    }
    // Prediction: the upper scales' get_flow_at, coarsest first, or the
    // motion at the top scale (recursive_prediction, predictions.h:61-74).
    float pty, ptx;
    if (u.scale + 1 < u.nscales) {
      float fy = 0.f, fx = 0.f;
      for (int l = u.nscales - 1; l > u.scale; l--) {
        const PUnit& L = units[u.base + l];
        float qy = p.x, qx = p.y;
        for (int k = u.scale; k < l; k++) {
          qy = __fdiv_rn(qy, 2.f);
          qx = __fdiv_rn(qx, 2.f);
        }
        const float uy = l + 1 < u.nscales ? __fmul_rn(2.f, fy) : 0.f;
        const float ux = l + 1 < u.nscales ? __fmul_rn(2.f, fx) : 0.f;
        float ny = 0.f, nx = 0.f;
        if (box_has(L.H, L.W, 3, __fadd_rn(qy, uy), __fadd_rn(qx, ux))) {
          float ty, tx, e;
          lk_match(L, par, S, qy, qx, uy, ux, false, ty, tx, e);
          if (box_has(L.H, L.W, 0, __fadd_rn(qy, ty), __fadd_rn(qx, tx))) {
            ny = ty;
            nx = tx;
          }
        }
        fy = ny;
        fx = nx;
      }
      pty = __fmul_rn(2.f, fy);
      ptx = __fmul_rn(2.f, fx);
    } else if (age != 1) {
      const float2 v = u.spd[b][i];
      pty = v.x;
      ptx = v.y;
    } else {
      pty = ptx = 0.f;
    }
    const float pred_y = __fadd_rn(p.x, pty), pred_x = __fadd_rn(p.y, ptx);
    bool keep = false;
    float ty = 0.f, tx = 0.f;
    if (box_has(u.H, u.W, 3, pred_y, pred_x)) {
      float e;
      lk_match(u, par, S, p.x, p.y, pty, ptx, true, ty, tx, e);
      const float my = (float)(int)__fadd_rn(p.x, ty), mx = (float)(int)__fadd_rn(p.y, tx);
      const float d0 = __fsub_rn(my, pred_y), d1 = __fsub_rn(mx, pred_x);
      keep = box_has(u.H, u.W, 3, __fadd_rn(p.x, ty), __fadd_rn(p.y, tx)) && e < (float)u.k &&
             __fsqrt_rn(__fadd_rn(__fmul_rn(d0, d0), __fmul_rn(d1, d1))) < 160.f;
    }
    if (lane == 0) {
      if (keep) {
        const float2 np = make_float2(__fadd_rn(p.x, ty), __fadd_rn(p.y, tx));
        u.age[b][i] = (unsigned short)(age + 1);
        u.spd[b][i] = make_float2(ty, tx);
        u.pos[b][i] = np;
        atomicMax(&u.sparse[(size_t)(int)np.x * u.W + (int)np.y], (unsigned)i + 1u);
      } else {
        u.age[b][i] = 0;
      }
    }
  }
}

// particle_mask_kernel (tracking_strategies.hpp:202-225) for every slot of the
// detector units (dead slots included, as the reference).
__global__ void k_pk_mask(PUnit* __restrict__ units, const PState* __restrict__ st, int nunits,
                          const int* __restrict__ prefix, int f) {
  const int total = prefix[nunits];
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
    const int ui = find_unit(prefix, nunits, g);
    const PUnit& u = units[ui];
    if (!det_frame(u, f)) continue;
    const float2 p = u.pos[st[ui].cur][g - prefix[ui]];
    const int r = (int)p.x, c = (int)p.y;
    for (int dr = -1; dr <= 1; dr++)
      for (int dc = -1; dc <= 1; dc++) u.mask[(size_t)(r + dr + MB) * u.mpitch + (c + dc + MB)] = 0;
  }
}

// FAST saliency (fast_detector::update, fast_detector.hpp:296-313) on input_
// where the mask is set.
__global__ void k_pk_saliency(PUnit* __restrict__ units, int nunits, int f, int par) {
  const int ui = blockIdx.y;
  if (ui >= nunits) return;
  const PUnit& u = units[ui];
  if (!det_frame(u, f)) return;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < u.H * u.W; t += gridDim.x * blockDim.x) {
    const int r = t / u.W, c = t % u.W;
    int v = 0;
    if (u.mask[(size_t)(r + MB) * u.mpitch + (c + MB)] != 0) {
      const uint8_t* P = img_at(u, par, r, c);
      int ring[16];
#pragma unroll
      for (int i = 0; i < 16; i++) ring[i] = P[gbt::circle16_r(i) * u.ipitch + gbt::circle16_c(i)];
      v = gbt::fast_score(ring, P[0], u.nfast, u.threshold);
    }
    u.sal[t] = (uint8_t)v;
  }
}

// new_particles(cpu)'s tile pass (fast_detector.hpp:217-253): a 3x3 tile
// holding a particle (sparse index) is skipped; otherwise its first strict
// maximum becomes a birth when it reaches the threshold and lies in
// domain - border(3), the raster pass's domain (:255-260).
__global__ void k_pk_nms(PUnit* __restrict__ units, int nunits, int f) {
  const int ui = blockIdx.y;
  if (ui >= nunits) return;
  const PUnit& u = units[ui];
  if (!det_frame(u, f)) return;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < u.TH * u.TW; t += gridDim.x * blockDim.x) {
    const int tr = t / u.TW, tc = t % u.TW;
    const int pr = 3 * tr + 1, pc = 3 * tc + 1;
    int code = -1;  // row in tile * 3 + column in tile
    bool skip = false;
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++)
        if (pr + r < u.H && pc + c < u.W && u.sparse[(size_t)(pr + r) * u.W + pc + c] != 0u) skip = true;
    if (!skip) {
      int vmax = u.sal[(size_t)pr * u.W + pc], mr = 0, mc = 0;
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
          if (pr + r < u.H && pc + c < u.W) {
            const int v = u.sal[(size_t)(pr + r) * u.W + pc + c];
            if (vmax < v) {
              vmax = v;
              mr = r;
              mc = c;
            }
          }
      const int R = pr + mr, C = pc + mc;
      if (vmax >= u.threshold && R >= 3 && R <= u.H - 4 && C >= 3 && C <= u.W - 4) code = mr * 3 + mc;
    }
    for (int dr = 0; dr < 3; dr++)
      u.items[(size_t)(3 * tr + dr) * u.TW + tc] = (code >= 0 && code / 3 == dr) ? (uint8_t)(code % 3 + 1) : 0;
  }
}

// Exclusive scan of one value per thread over a SCAN_T-thread CTA; returns
// the thread's offset and sets *total.
__device__ __forceinline__ int block_scan(int v, int* wsum, int* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (w == 0) {
    int s = lane < SCAN_T / 32 ? wsum[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    wsum[lane] = s;  // inclusive per warp
  }
  __syncthreads();
  const int off = (w ? wsum[w - 1] : 0) + x - v;
  *total = wsum[SCAN_T / 32 - 1];
  __syncthreads();
  return off;
}

// Births in raster order (particle_container::add, particle_container.hpp:
// 370-387) and the stable compaction (compact(cpu), :215-252), then the
// sparse index of the survivors (the last survivor at a pixel wins).  One CTA
// per unit; the CTAs of units that do not detect in frame f return at once.
__global__ void __launch_bounds__(SCAN_T) k_pk_births_compact(PUnit* __restrict__ units, PState* __restrict__ st,
                                                               int f, int* __restrict__ err) {
  __shared__ int wsum[32];
  const int ui = blockIdx.x;
  const PUnit& u = units[ui];
  if (!det_frame(u, f)) return;  // uniform per CTA
  PState s = st[ui];
  const int b = s.cur, nitems = 3 * u.TH * u.TW;
  int nb = 0, total;
  for (int c0 = 0; c0 < nitems; c0 += SCAN_T) {
    const int it = c0 + threadIdx.x;
    const int code = it < nitems ? u.items[it] : 0;
    const int off = block_scan(code != 0, wsum, &total);
    if (code) {
      const int slot = s.n + nb + off;
      if (slot < u.cap) {
        const int row = it / u.TW + 1, col = 3 * (it % u.TW) + code;  // 3 tr + dr + 1, 3 tc + 1 + dc
        u.pos[b][slot] = make_float2((float)row, (float)col);
        u.spd[b][slot] = make_float2(0.f, 0.f);
        u.age[b][slot] = 1;
      } else {
        atomicOr(err, ERR_CAPACITY);
      }
    }
    nb += total;
  }
  const int n1 = min(s.n + nb, u.cap);
  __syncthreads();
  int o = 0;
  for (int c0 = 0; c0 < n1; c0 += SCAN_T) {
    const int i = c0 + threadIdx.x;
    const bool alive = i < n1 && u.age[b][i] != 0;
    const int off = block_scan(alive, wsum, &total);
    if (i < n1) {
      u.matches[i] = alive ? o + off : -1;
      if (alive) {
        u.pos[b ^ 1][o + off] = u.pos[b][i];
        u.spd[b ^ 1][o + off] = u.spd[b][i];
        u.age[b ^ 1][o + off] = u.age[b][i];
      }
    }
    o += total;
  }
  __syncthreads();
  const int np = u.H * u.W;
  for (int t = threadIdx.x; t < np; t += SCAN_T) u.sparse[t] = 0u;
  __syncthreads();
  for (int j = threadIdx.x; j < o; j += SCAN_T) {
    const float2 p = u.pos[b ^ 1][j];
    atomicMax(&u.sparse[(size_t)(int)p.x * u.W + (int)p.y], (unsigned)j + 1u);
  }
  if (threadIdx.x == 0) {
    s.n = o;
    s.cur = b ^ 1;
    s.nmatches = n1;
    s.compact = 1;
    st[ui] = s;
  }
}

// merge_trajectories (merge_trajectories.h:10-35), step 1: for every live
// slot, the c8_h directions whose neighbour qualifies with the ages before the
// merge (ages only fall to 0 during the merge, so no other neighbour can).
__global__ void k_pk_merge_cand(PUnit* __restrict__ units, const PState* __restrict__ st, int nunits,
                                const int* __restrict__ prefix, int f) {
  constexpr int C8R[8] = {-1, 0, 1, -1, 1, -1, 0, 1}, C8C[8] = {1, 1, 1, 0, 0, -1, -1, -1};
  const int total = prefix[nunits];
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
    const int ui = find_unit(prefix, nunits, g);
    const PUnit& u = units[ui];
    if (!merge_frame(u, f)) continue;
    const int i = g - prefix[ui], b = st[ui].cur;
    const int a = u.age[b][i];
    unsigned m = 0;
    if (a != 0) {
      const float2 p = u.pos[b][i], v = u.spd[b][i];
      const int r = (int)p.x, c = (int)p.y;
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const unsigned j1 = u.sparse[(size_t)(r + C8R[k]) * u.W + (c + C8C[k])];
        if (j1 == 0u) continue;
        const int j = (int)j1 - 1;
        const float2 w = u.spd[b][j];
        const float dx = __fsub_rn(v.x, w.x), dy = __fsub_rn(v.y, w.y);
        if ((int)u.age[b][j] > a + 2 && __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy))) < 2.f)
          m |= 1u << k;
      }
    }
    u.cmask[i] = (uint8_t)m;
  }
}

// Step 2: one warp per unit replays the slots with candidates in slot order
// with the current ages, as the reference's loop does (the warps of units that
// do not merge in frame f return at once).
__global__ void k_pk_merge_replay(PUnit* __restrict__ units, const PState* __restrict__ st, int f) {
  constexpr int C8R[8] = {-1, 0, 1, -1, 1, -1, 0, 1}, C8C[8] = {1, 1, 1, 0, 0, -1, -1, -1};
  const int ui = blockIdx.x;
  const PUnit& u = units[ui];
  if (!merge_frame(u, f)) return;
  const PState s = st[ui];
  const int b = s.cur, lane = threadIdx.x & 31;
  for (int base = 0; base < s.n; base += 32) {
    const int i0 = base + lane;
    unsigned act = __ballot_sync(0xffffffffu, i0 < s.n && u.cmask[i0] != 0);
    while (act) {
      const int bit = __ffs(act) - 1;
      act &= act - 1;
      if (lane == 0) {
        const int i = base + bit;
        const int a = u.age[b][i];
        if (a != 0) {
          const unsigned m = u.cmask[i];
          const float2 p = u.pos[b][i], v = u.spd[b][i];
          const int r = (int)p.x, c = (int)p.y;
          for (int k = 0; k < 8; k++) {
            if (!((m >> k) & 1u)) continue;
            const int j = (int)u.sparse[(size_t)(r + C8R[k]) * u.W + (c + C8C[k])] - 1;
            const float2 w = u.spd[b][j];
            const float dx = __fsub_rn(v.x, w.x), dy = __fsub_rn(v.y, w.y);
            if ((int)u.age[b][j] > a + 2 && __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy))) < 2.f) {
              u.age[b][j] = 0;
              break;
            }
          }
        }
      }
      __syncwarp();
    }
  }
}

// Matching resets compact_has_run (before_matching).
__global__ void k_pk_begin_match(PState* __restrict__ st, int nunits) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u < nunits) st[u].compact = 0;
}

}  // namespace gbt_pk

using namespace gbt_pk;

// ---------------------------------------------------------------------------
// Host side.

struct PkStream {
  gbt_config cfg;
  int unit0;
  uint8_t* pinned = nullptr;  // staging of pageable host frames
};

struct PkTracker {
  int device = 0, nsm = 0;
  cudaStream_t stream = nullptr;
  std::vector<PkStream> streams;
  std::vector<PUnit> units;
  PUnit* d_units = nullptr;
  PState* d_state = nullptr;
  int* d_prefix = nullptr;
  int* d_err = nullptr;
  int* d_scale_units = nullptr;  // per scale: the unit of every stream (-1 when the stream has fewer scales)
  int maxL = 0;
  int frame = 0;
  int64_t launches = 0;
  int last_launches = 0;
  std::vector<void*> allocs;
  std::string err;
};

static int pk_fail(PkTracker* t, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  t->err = buf;
  return code;
}

#define PCK(call)                                                                                  \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return pk_fail(t, GBT_E_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

template <class T>
static int pk_alloc(PkTracker* t, T** p, size_t n) {
  void* q = nullptr;
  if (cudaMalloc(&q, n * sizeof(T) + 16) != cudaSuccess) return pk_fail(t, GBT_E_OOM, "device allocation failed");
  t->allocs.push_back(q);
  if (cudaMemset(q, 0, n * sizeof(T) + 16) != cudaSuccess) return pk_fail(t, GBT_E_CUDA, "cudaMemset failed");
  *p = (T*)q;
  return GBT_OK;
}

static int pk_upload_units(PkTracker* t) {
  PCK(cudaMemcpyAsync(t->d_units, t->units.data(), t->units.size() * sizeof(PUnit), cudaMemcpyHostToDevice,
                      t->stream));
  PCK(cudaStreamSynchronize(t->stream));
  return GBT_OK;
}

static void pk_free(PkTracker* t) {
  if (!t) return;
  cudaSetDevice(t->device);
  if (t->stream) cudaStreamSynchronize(t->stream);
  for (void* p : t->allocs) cudaFree(p);
  for (auto& s : t->streams)
    if (s.pinned) cudaFreeHost(s.pinned);
  if (t->stream) cudaStreamDestroy(t->stream);
  delete t;
}

int pk_create(const gbt_config* cfgs, int nstreams, int device, PkTracker** out, std::string& err) {
  *out = nullptr;
  PkTracker* t = new PkTracker;
  t->device = device;
  auto fail = [&](int r) {
    err = t->err;
    pk_free(t);
    return r;
  };
  if (cudaSetDevice(device) != cudaSuccess) {
    t->err = "cudaSetDevice failed";
    return fail(GBT_E_CUDA);
  }
  cudaDeviceGetAttribute(&t->nsm, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking) != cudaSuccess) {
    t->err = "cudaStreamCreate failed";
    return fail(GBT_E_CUDA);
  }
  int r;
  for (int s = 0; s < nstreams; s++) {
    PkStream ps;
    ps.cfg = cfgs[s];
    ps.unit0 = (int)t->units.size();
    const gbt_config& c = cfgs[s];
    t->maxL = std::max(t->maxL, c.nscales);
    if (cudaMallocHost(&ps.pinned, (size_t)c.rows * c.cols) != cudaSuccess) {
      t->err = "pinned allocation failed";
      return fail(GBT_E_OOM);
    }
    int H = c.rows, W = c.cols;
    for (int l = 0; l < c.nscales; l++) {
      PUnit u{};
      u.H = H;
      u.W = W;
      u.stream = s;
      u.scale = l;
      u.nscales = c.nscales;
      u.base = ps.unit0;
      u.threshold = c.detector_threshold;
      u.nfast = c.detector_n;
      u.det_freq = c.detector_frequency;
      u.filt_freq = c.filtering_frequency;
      u.k = c.k;
      u.with_merge = c.with_merge;
      u.ipitch = (W + 2 * BB + 15) / 16 * 16;
      u.mpitch = (W + 2 * MB + 15) / 16 * 16;
      u.TH = H / 3;
      u.TW = W / 3;
      u.cap = H * W / 4 + 4096;
      const size_t np = (size_t)H * W;
      if ((r = pk_alloc(t, &u.img[0], (size_t)(H + 2 * BB) * u.ipitch)) || (r = pk_alloc(t, &u.img[1], (size_t)(H + 2 * BB) * u.ipitch)) ||
          (r = pk_alloc(t, &u.lvl, np)) || (r = pk_alloc(t, &u.grad, np)) ||
          (r = pk_alloc(t, &u.mask, (size_t)(H + 2 * MB) * u.mpitch)) || (r = pk_alloc(t, &u.sal, np)) ||
          (r = pk_alloc(t, &u.sparse, np)) || (r = pk_alloc(t, &u.matches, (size_t)u.cap)) ||
          (r = pk_alloc(t, &u.cmask, (size_t)u.cap)) || (r = pk_alloc(t, &u.items, (size_t)3 * u.TH * u.TW)))
        return fail(r);
      for (int k = 0; k < 2; k++)
        if ((r = pk_alloc(t, &u.pos[k], (size_t)u.cap)) || (r = pk_alloc(t, &u.spd[k], (size_t)u.cap)) ||
            (r = pk_alloc(t, &u.age[k], (size_t)u.cap)))
          return fail(r);
      t->units.push_back(u);
      H /= 2;
      W /= 2;
    }
    t->streams.push_back(ps);
  }
  const int nu = (int)t->units.size();
  std::vector<int> su((size_t)t->maxL * nstreams, -1);
  for (int s = 0; s < nstreams; s++)
    for (int l = 0; l < t->streams[s].cfg.nscales; l++) su[(size_t)l * nstreams + s] = t->streams[s].unit0 + l;
  if ((r = pk_alloc(t, &t->d_units, (size_t)nu)) || (r = pk_alloc(t, &t->d_state, (size_t)nu)) ||
      (r = pk_alloc(t, &t->d_prefix, (size_t)nu + 1)) || (r = pk_alloc(t, &t->d_err, 1)) ||
      (r = pk_alloc(t, &t->d_scale_units, su.size())))
    return fail(r);
  if (cudaMemcpy(t->d_scale_units, su.data(), su.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
      (r = pk_upload_units(t)))
    return fail(r ? r : GBT_E_CUDA);
  if (cudaDeviceSynchronize() != cudaSuccess) {
    t->err = "device synchronisation failed";
    return fail(GBT_E_CUDA);
  }
  *out = t;
  return GBT_OK;
}

void pk_destroy(PkTracker* t) { pk_free(t); }
const std::string& pk_error(const PkTracker* t) { return t->err; }
cudaStream_t pk_stream(const PkTracker* t) { return t->stream; }

int pk_run(PkTracker* t, const uint8_t* const* frames, const int64_t* pitches, int location) {
  if (!frames || !pitches) return GBT_E_INVALID;
  if (location != GBT_FRAMES_HOST && location != GBT_FRAMES_DEVICE)
    return pk_fail(t, GBT_E_INVALID, "the LK tracker takes gray frames (GBT_FRAMES_HOST or GBT_FRAMES_DEVICE)");
  PCK(cudaSetDevice(t->device));
  const int nstreams = (int)t->streams.size(), nu = (int)t->units.size();
  const int f = t->frame, par = f & 1;
  int launches = 0;
  // Level 0 of every stream: the frame.
  for (int s = 0; s < nstreams; s++) {
    PkStream& ps = t->streams[s];
    const PUnit& u = t->units[ps.unit0];
    if (!frames[s] || pitches[s] < u.W) return pk_fail(t, GBT_E_INVALID, "stream %d: bad frame or pitch", s);
    if (location == GBT_FRAMES_HOST) {
      PCK(cudaStreamSynchronize(t->stream));  // the staging buffer is free again
      for (int r = 0; r < u.H; r++) memcpy(ps.pinned + (size_t)r * u.W, frames[s] + (size_t)r * pitches[s], u.W);
      PCK(cudaMemcpyAsync(u.lvl, ps.pinned, (size_t)u.H * u.W, cudaMemcpyHostToDevice, t->stream));
    } else {
      PCK(cudaMemcpy2DAsync(u.lvl, u.W, frames[s], pitches[s], u.W, u.H, cudaMemcpyDeviceToDevice, t->stream));
    }
  }
  // Whether any unit detects / merges this frame (each kernel's CTAs check
  // their own unit, so no per-frame list goes to the device and the host
  // queues frames without waiting for the GPU).
  bool any_det = false, any_mer = false;
  for (int i = 0; i < nu; i++) {
    const PUnit& u = t->units[i];
    any_det |= f % u.det_freq == 0;
    any_mer |= f % u.filt_freq == 0 && u.with_merge;
  }
  int maxpx = 0;
  for (const PUnit& u : t->units) maxpx = std::max(maxpx, (u.H + 2 * MB) * u.mpitch);
  const int pxblocks = std::min(1024, std::max(1, (maxpx + 255) / 256));
  for (int l = 0; l < t->maxL; l++) {
    k_pk_level<<<dim3(pxblocks, nstreams), 256, 0, t->stream>>>(t->d_units, t->d_scale_units + (size_t)l * nstreams,
                                                                nstreams, par);
    launches++;
  }
  k_pk_prep<<<dim3(pxblocks, nu), 256, 0, t->stream>>>(t->d_units, nu, f, par);
  k_pk_prefix<<<1, 32, 0, t->stream>>>(t->d_state, nu, t->d_prefix);
  launches += 2;
  const int slot_grid = t->nsm * 8;
  if (f > 0) {
    k_pk_begin_match<<<(nu + 127) / 128, 128, 0, t->stream>>>(t->d_state, nu);
    k_pk_match<<<t->nsm * 6, 32 * MW, 0, t->stream>>>(t->d_units, t->d_state, nu, t->d_prefix, par);
    launches += 2;
  }
  if (any_det) {
    k_pk_mask<<<slot_grid, 256, 0, t->stream>>>(t->d_units, t->d_state, nu, t->d_prefix, f);
    k_pk_saliency<<<dim3(pxblocks, nu), 256, 0, t->stream>>>(t->d_units, nu, f, par);
    k_pk_nms<<<dim3(pxblocks, nu), 256, 0, t->stream>>>(t->d_units, nu, f);
    k_pk_births_compact<<<nu, SCAN_T, 0, t->stream>>>(t->d_units, t->d_state, f, t->d_err);
    k_pk_prefix<<<1, 32, 0, t->stream>>>(t->d_state, nu, t->d_prefix);
    launches += 5;
  }
  if (any_mer) {
    k_pk_merge_cand<<<slot_grid, 256, 0, t->stream>>>(t->d_units, t->d_state, nu, t->d_prefix, f);
    k_pk_merge_replay<<<nu, 32, 0, t->stream>>>(t->d_units, t->d_state, f);
    launches += 2;
  }
  PCK(cudaGetLastError());
  t->frame++;
  t->launches += launches;
  t->last_launches = launches;
  return GBT_OK;
}

int pk_sync(PkTracker* t) {
  PCK(cudaSetDevice(t->device));
  PCK(cudaStreamSynchronize(t->stream));
  int e = 0;
  PCK(cudaMemcpy(&e, t->d_err, sizeof e, cudaMemcpyDeviceToHost));
  if (e & ERR_CAPACITY) return pk_fail(t, GBT_E_CAPACITY, "particle capacity exceeded");
  return GBT_OK;
}

static int pk_unit(PkTracker* t, int stream, int scale) {
  if (stream < 0 || stream >= (int)t->streams.size()) return -1;
  if (scale < 0 || scale >= t->streams[stream].cfg.nscales) return -1;
  return t->streams[stream].unit0 + scale;
}

static int* pk_param(PUnit& u, int key, int& lo, int& hi) {
  lo = 0;
  hi = 1 << 30;
  switch (key) {
    case GBT_PARAM_DETECTOR_THRESHOLD: return &u.threshold;
    case GBT_PARAM_DETECTOR_N: lo = 1; hi = 16; return &u.nfast;
    case GBT_PARAM_DETECTOR_FREQUENCY: lo = 1; return &u.det_freq;
    case GBT_PARAM_FILTERING_FREQUENCY: lo = 1; return &u.filt_freq;
    case GBT_PARAM_K: return &u.k;
    case GBT_PARAM_WITH_MERGE: hi = 1; return &u.with_merge;
    default: return nullptr;
  }
}

int pk_set_param(PkTracker* t, int stream, int scale, int key, int value) {
  if (stream < 0 || stream >= (int)t->streams.size()) return GBT_E_INVALID;
  const int L = t->streams[stream].cfg.nscales;
  if (scale < -1 || scale >= L) return GBT_E_INVALID;
  int lo, hi;
  if (!pk_param(t->units[t->streams[stream].unit0], key, lo, hi))
    return pk_fail(t, GBT_E_INVALID, "parameter %d is not a setting of the LK tracker", key);
  if (value < lo || value > hi) return pk_fail(t, GBT_E_INVALID, "parameter %d out of range: %d", key, value);
  PCK(cudaSetDevice(t->device));
  PCK(cudaStreamSynchronize(t->stream));
  for (int l = scale < 0 ? 0 : scale; l < (scale < 0 ? L : scale + 1); l++)
    *pk_param(t->units[t->streams[stream].unit0 + l], key, lo, hi) = value;
  return pk_upload_units(t);
}

int pk_get_param(PkTracker* t, int stream, int scale, int key, int32_t* value) {
  const int ui = pk_unit(t, stream, scale);
  int lo, hi;
  if (ui < 0 || !value) return GBT_E_INVALID;
  const int* p = pk_param(t->units[ui], key, lo, hi);
  if (!p) return GBT_E_INVALID;
  *value = *p;
  return GBT_OK;
}

static int pk_state(PkTracker* t, int ui, PState* s) {
  PCK(cudaSetDevice(t->device));
  PCK(cudaStreamSynchronize(t->stream));
  PCK(cudaMemcpy(s, t->d_state + ui, sizeof *s, cudaMemcpyDeviceToHost));
  return GBT_OK;
}

int pk_nparticles(PkTracker* t, int stream, int scale, int32_t* n) {
  const int ui = pk_unit(t, stream, scale);
  if (ui < 0 || !n) return GBT_E_INVALID;
  PState s;
  int r = pk_state(t, ui, &s);
  if (r) return r;
  *n = s.n;
  return GBT_OK;
}

int pk_frame_count(PkTracker* t, int stream, int scale, int32_t* n) {
  if (pk_unit(t, stream, scale) < 0 || !n) return GBT_E_INVALID;
  *n = t->frame;
  return GBT_OK;
}

int pk_get_particles(PkTracker* t, int stream, int scale, float* pos, float* speed, uint16_t* age, int32_t* matches,
                     int32_t* nmatches, int32_t* compact_has_run) {
  const int ui = pk_unit(t, stream, scale);
  if (ui < 0) return GBT_E_INVALID;
  PState s;
  int r = pk_state(t, ui, &s);
  if (r) return r;
  const PUnit& u = t->units[ui];
  if (pos && s.n) PCK(cudaMemcpy(pos, u.pos[s.cur], (size_t)s.n * sizeof(float2), cudaMemcpyDeviceToHost));
  if (speed && s.n) PCK(cudaMemcpy(speed, u.spd[s.cur], (size_t)s.n * sizeof(float2), cudaMemcpyDeviceToHost));
  if (age && s.n) PCK(cudaMemcpy(age, u.age[s.cur], (size_t)s.n * sizeof(uint16_t), cudaMemcpyDeviceToHost));
  if (nmatches) *nmatches = s.nmatches;
  if (matches && s.nmatches)
    PCK(cudaMemcpy(matches, u.matches, (size_t)s.nmatches * sizeof(int32_t), cudaMemcpyDeviceToHost));
  if (compact_has_run) *compact_has_run = s.compact;
  return GBT_OK;
}

int pk_get_stage(PkTracker* t, int stream, int scale, int stage, int border, void* out) {
  const int ui = pk_unit(t, stream, scale);
  if (ui < 0 || !out) return GBT_E_INVALID;
  PCK(cudaSetDevice(t->device));
  PCK(cudaStreamSynchronize(t->stream));
  const PUnit& u = t->units[ui];
  const size_t np = (size_t)u.H * u.W;
  if (stage == GBT_STAGE_SPARSE) {
    std::vector<uint32_t> v(np);
    PCK(cudaMemcpy(v.data(), u.sparse, np * 4, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < np; i++) ((uint32_t*)out)[i] = v[i] ? v[i] - 1u : 0xFFFFFFFFu;
    return GBT_OK;
  }
  if (stage == GBT_STAGE_SALIENCY) {
    PCK(cudaMemcpy(out, u.sal, np, cudaMemcpyDeviceToHost));
    return GBT_OK;
  }
  if (stage == GBT_STAGE_MASK) {
    PCK(cudaMemcpy2D(out, u.W, u.mask + (size_t)MB * u.mpitch + MB, u.mpitch, u.W, u.H, cudaMemcpyDeviceToHost));
    return GBT_OK;
  }
  if (stage == GBT_STAGE_INPUT) {  // the strategy's input_ of the last frame, with up to BB border pixels
    if (border < 0 || border > BB) return pk_fail(t, GBT_E_INVALID, "border %d: the LK tracker keeps %d", border, BB);
    const int par = (t->frame - 1) & 1;
    const uint8_t* src = u.img[par] + (size_t)(BB - border) * u.ipitch + (BB - border);
    PCK(cudaMemcpy2D(out, u.W + 2 * border, src, u.ipitch, u.W + 2 * border, u.H + 2 * border,
                     cudaMemcpyDeviceToHost));
    return GBT_OK;
  }
  return pk_fail(t, GBT_E_INVALID, "stage %d is not kept by the LK tracker", stage);
}

int pk_read_counts(PkTracker* t, int32_t* counts, int n, bool async) {
  if (!counts || n < (int)t->units.size()) return GBT_E_INVALID;
  PCK(cudaSetDevice(t->device));
  for (size_t i = 0; i < t->units.size(); i++)
    PCK(cudaMemcpyAsync(counts + i, &t->d_state[i].n, sizeof(int32_t), cudaMemcpyDeviceToHost, t->stream));
  if (!async) PCK(cudaStreamSynchronize(t->stream));
  return GBT_OK;
}

int pk_kernel_launches(PkTracker* t, int64_t* total) {
  if (!total) return GBT_E_INVALID;
  *total = t->launches;
  return GBT_OK;
}

int pk_kernels_per_frame(PkTracker* t, int32_t* n) {
  if (!n) return GBT_E_INVALID;
  *n = t->last_launches;
  return GBT_OK;
}
