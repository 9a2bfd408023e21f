// Differentiable pyramidal LK residual and its hand-written adjoint (sm_103a).
//
// Forward (per point): the translational LK of iterative_lk_match_5x5
// (cuimg/tracking2/pyrlk_tracker.hpp:165-334) with its discrete parts removed so
// that it is differentiable: sigma-1 Gaussian pyramids of both frames
// (cuimg/gpu/mipmap.h:94-108 form), Sobel/8 gradients of the previous level
// (pyrlk_tracker.hpp:910-938), every window pixel used, exactly `iters`
// Gauss-Newton steps per level, coarse-to-fine start from twice the coarser
// displacement (predictions.h:61-74) and from u0 / 2^(L-1) at the top,
// floor-based bilinear sampling with clamped taps (window pixel (r, c) of a
// window centred at v is sampled at floor(v) + (r, c) with the weights of
// frac(v), which is the sample at v + (r, c) in exact arithmetic).  Loss per point = sum over
// the level-0 window of (A0(p + o) - B0(v + o))^2 at the final position v.
//
// Adjoint: gradients of sum_i dloss_i * loss_i with respect to both frames and
// u0.  The backward pass recomputes the pyramid levels (nothing from the
// forward call is kept), replays each point's forward in a warp, then sweeps
// back through the iterations: step v += M b with M = G^-1 gives
// dM += dv b^T, db = M dv; b = sum g r gives dg += r db and dr = g . db; r =
// T - B(v + o) scatters into dA, dB and dv; finally dG = -M dM M and
// dg += (dG + dG^T) g.  Level images are then pulled back through the Sobel
// transpose and the transpose of blur-and-decimate, top level first.
#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "cuimg_gb300.h"

extern "C" int gbt_gaussian_pyramid_f32(const float* in, int64_t in_pitch, int32_t rows, int32_t cols, int32_t nlevels,
                                        float* out, void* stream);

namespace gbt_lkd {

constexpr int MAXW = 15;
constexpr int MAXL = 9;
constexpr int MAXK = 32;
constexpr int WARPS = 4;

struct Lvl {
  int H, W;
  const float* A;
  const float* B;
  const float2* S;  // Sobel/8 of A: (d/drow, d/dcol)
  float* dA;
  float* dB;
  float2* dS;
};

struct Bil {
  int i00, i10, i01, i11;
  float w00, w10, w01, w11;
  float a, b;       // fractional parts (row, col)
  int y0, x0;       // clamped top-left tap (the others are y0 or y0 + 1, x0 or x0 + 1 clamped)
  int dy, dx;       // 1 where the second tap row / column differs from the first, 0 at the clamp
};

// All pixels of a window centred at (y, x) share the fractional part of the
// centre: their bilinear weights are computed once (the taps of window pixel
// (r, c) are floor(y) + r .. + 1 and floor(x) + c .. + 1, exactly the taps of
// (y + r, x + c) in exact arithmetic), and when the whole window lies inside
// the image no tap needs clamping.
struct Win {
  int y0, x0;
  float a, b, w00, w10, w01, w11;
  bool inner;
};

__device__ __forceinline__ Win win_at(int H, int W, float y, float x, int h) {
  Win s;
  s.y0 = __float2int_rd(y);
  s.x0 = __float2int_rd(x);
  s.a = y - (float)s.y0;
  s.b = x - (float)s.x0;
  s.w00 = (1.f - s.a) * (1.f - s.b);
  s.w10 = s.a * (1.f - s.b);
  s.w01 = (1.f - s.a) * s.b;
  s.w11 = s.a * s.b;
  s.inner = s.y0 - h >= 0 && s.y0 + h + 1 <= H - 1 && s.x0 - h >= 0 && s.x0 + h + 1 <= W - 1;
  return s;
}

// The sample of window pixel (r, c).
__device__ __forceinline__ Bil bil_win(int H, int W, const Win& s, int r, int c) {
  Bil o;
  o.a = s.a;
  o.b = s.b;
  o.w00 = s.w00;
  o.w10 = s.w10;
  o.w01 = s.w01;
  o.w11 = s.w11;
  int y0 = s.y0 + r, x0 = s.x0 + c, y1, x1;
  if (s.inner) {
    y1 = y0 + 1;
    x1 = x0 + 1;
  } else {
    y1 = min(max(y0 + 1, 0), H - 1);
    x1 = min(max(x0 + 1, 0), W - 1);
    y0 = min(max(y0, 0), H - 1);
    x0 = min(max(x0, 0), W - 1);
  }
  o.i00 = y0 * W + x0;
  o.i10 = y1 * W + x0;
  o.i01 = y0 * W + x1;
  o.i11 = y1 * W + x1;
  o.y0 = y0;
  o.x0 = x0;
  o.dy = y1 - y0;
  o.dx = x1 - x0;
  return o;
}

__device__ __forceinline__ float bil_val(const float* img, const Bil& s) {
  return s.w00 * img[s.i00] + s.w10 * img[s.i10] + s.w01 * img[s.i01] + s.w11 * img[s.i11];
}
__device__ __forceinline__ float2 bil_val2(const float2* img, const Bil& s) {
  float2 a = img[s.i00], b = img[s.i10], c = img[s.i01], d = img[s.i11];
  return make_float2(s.w00 * a.x + s.w10 * b.x + s.w01 * c.x + s.w11 * d.x,
                     s.w00 * a.y + s.w10 * b.y + s.w01 * c.y + s.w11 * d.y);
}
// d/d(position) of the bilinear interpolant.
__device__ __forceinline__ float2 bil_grad(const float* img, const Bil& s) {
  float v00 = img[s.i00], v10 = img[s.i10], v01 = img[s.i01], v11 = img[s.i11];
  return make_float2((1.f - s.b) * (v10 - v00) + s.b * (v11 - v01), (1.f - s.a) * (v01 - v00) + s.a * (v11 - v10));
}
// The taps of a whole window: tap (i, j) = img(clamp(y0 - h + i),
// clamp(x0 - h + j)) for i, j in [0, ws], staged once per window in the
// warp's shared buffer tg (row-major, ws + 1 per row) by row loads.  Window
// pixel (r, c) (0-based) then reads its four taps at tg[r (ws + 1) + c ..]:
// they are the taps bil_win gives it, since bil_win clamps each tap
// coordinate on its own.  A window of ws x ws samples needs (ws + 1)^2
// distinct taps, not 4 ws^2 scattered loads.
template <int WS>
__device__ __forceinline__ void stage_taps(const float* img, int H, int W, const Win& w, float* tg) {
  constexpr int TW = WS + 1, NT = TW * TW, h = WS / 2;
  __syncwarp();  // every lane is done with the previous window's taps
#pragma unroll
  for (int k = 0; k < (NT + 31) / 32; k++) {
    const int t = (threadIdx.x & 31) + 32 * k;
    if (t < NT) {
      int y = w.y0 - h + t / TW, x = w.x0 - h + t % TW;
      if (!w.inner) {
        y = min(max(y, 0), H - 1);
        x = min(max(x, 0), W - 1);
      }
      tg[t] = img[(size_t)y * W + x];
    }
  }
  __syncwarp();
}
// bil_val of the sample whose four taps start at p (row pitch TW).
template <int TW>
__device__ __forceinline__ float tap_val(const float* p, const Win& s) {
  return s.w00 * p[0] + s.w10 * p[TW] + s.w01 * p[1] + s.w11 * p[TW + 1];
}

__device__ __forceinline__ void bil_scatter(float* img, const Bil& s, float v) {
  atomicAdd(img + s.i00, s.w00 * v);
  atomicAdd(img + s.i10, s.w10 * v);
  atomicAdd(img + s.i01, s.w01 * v);
  atomicAdd(img + s.i11, s.w11 * v);
}

__device__ __forceinline__ float wsum(float v) {  // every lane gets the same sum (butterfly)
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

struct Setup {  // per level of one point
  float q0, q1, M00, M01, M11;
};

__device__ __forceinline__ float level_scale(int l) {
  float s = 1.f;
  for (int k = 0; k < l; k++) s *= 2.f;
  return s;
}

__host__ __device__ constexpr int ppl_of(int ws) { return (ws * ws + 31) / 32; }  // window pixels per lane

// The level's template at q + o for the lane's window pixels: Sobel gradient
// and A value, fixed through the level's Gauss-Newton steps.
template <int PPL>
struct Tmpl {
  float2 g[PPL];
  float a[PPL];
};

template <int WS>
__device__ __forceinline__ void load_template(const Lvl& e, int /*window: WS*/, float q0, float q1, Tmpl<ppl_of(WS)>& T) {
  constexpr int ws = WS, PPL = (WS * WS + 31) / 32;
  const int lane = threadIdx.x & 31, hws = ws / 2, n = ws * ws;
  const Win wq = win_at(e.H, e.W, q0, q1, hws);
#pragma unroll
  for (int k = 0; k < PPL; k++) {
    const int i = lane + 32 * k;
    T.g[k] = make_float2(0.f, 0.f);
    T.a[k] = 0.f;
    if (i < n) {
      Bil st = bil_win(e.H, e.W, wq, i / ws - hws, i % ws - hws);
      T.g[k] = bil_val2(e.S, st);
      T.a[k] = bil_val(e.A, st);
    }
  }
}

// Normal matrix inverse at one level (all lanes get identical values).
template <int PPL>
__device__ __forceinline__ void level_setup(const Tmpl<PPL>& T, int n, float& M00, float& M01, float& M11) {
  const int lane = threadIdx.x & 31;
  float g00 = 0.f, g01 = 0.f, g11 = 0.f;
#pragma unroll
  for (int k = 0; k < PPL; k++)
    if (lane + 32 * k < n) {
      const float2 g = T.g[k];
      g00 += g.x * g.x;
      g01 += g.x * g.y;
      g11 += g.y * g.y;
    }
  g00 = wsum(g00);
  g01 = wsum(g01);
  g11 = wsum(g11);
  const float det = g00 * g11 - g01 * g01;
  M00 = g11 / det;
  M01 = -g01 / det;
  M11 = g00 / det;
}

// One Gauss-Newton right-hand side b = sum g (T - B(v + o)).
// tg: the warp's tap buffer ((ws + 1)^2 floats, stage_taps).
template <int WS>
__device__ __forceinline__ void rhs(const Lvl& e, int /*window: WS*/, const Tmpl<ppl_of(WS)>& T, float v0, float v1, float& b0,
                                    float& b1, float* tg) {
  constexpr int ws = WS, PPL = (WS * WS + 31) / 32;
  const int lane = threadIdx.x & 31, hws = ws / 2, n = ws * ws;
  b0 = 0.f;
  b1 = 0.f;
  const Win wv = win_at(e.H, e.W, v0, v1, hws);
  stage_taps<WS>(e.B, e.H, e.W, wv, tg);
#pragma unroll
  for (int k = 0; k < PPL; k++) {
    const int i = lane + 32 * k;
    if (i < n) {
      const float res = T.a[k] - tap_val<WS + 1>(tg + (i / ws) * (ws + 1) + i % ws, wv);
      b0 += T.g[k].x * res;
      b1 += T.g[k].y * res;
    }
  }
  b0 = wsum(b0);
  b1 = wsum(b1);
}

// Forward of one point; fills the per-level setup and the iterate history.
template <int WS>
__device__ float point_forward(const Lvl* lv, int L, int /*window: WS*/, int K, float p0, float p1, float u0, float u1,
                               Setup* su, float4* hist, int hs, float& vf0, float& vf1, float* tg) {
  constexpr int ws = WS, PPL = (WS * WS + 31) / 32;
  const int n = ws * ws;
  const float top = level_scale(L - 1);
  float d0 = u0 / top, d1 = u1 / top, v0 = 0.f, v1 = 0.f;
  for (int l = L - 1; l >= 0; l--) {
    const Lvl& e = lv[l];
    const float s = level_scale(l);
    const float q0 = p0 / s, q1 = p1 / s;
    Tmpl<PPL> T;
    load_template<WS>(e, ws, q0, q1, T);
    float M00, M01, M11;
    level_setup<PPL>(T, n, M00, M01, M11);
    if (su) su[l] = Setup{q0, q1, M00, M01, M11};
    v0 = q0 + d0;
    v1 = q1 + d1;
    for (int k = 0; k < K; k++) {
      float b0, b1;
      rhs<WS>(e, ws, T, v0, v1, b0, b1, tg);
      if (hist) hist[l * hs + k] = make_float4(v0, v1, b0, b1);  // iterate and its right-hand side
      v0 += M00 * b0 + M01 * b1;
      v1 += M01 * b0 + M11 * b1;
    }
    if (hist) hist[l * hs + K] = make_float4(v0, v1, 0.f, 0.f);
    d0 = 2.f * (v0 - q0);
    d1 = 2.f * (v1 - q1);
  }
  vf0 = v0;
  vf1 = v1;
  const Lvl& e = lv[0];
  const int lane = threadIdx.x & 31, hws = ws / 2;
  float loss = 0.f;
  const Win wp = win_at(e.H, e.W, p0, p1, hws), wv = win_at(e.H, e.W, v0, v1, hws);
#pragma unroll
  for (int k = 0; k < PPL; k++) {
    const int i = lane + 32 * k;
    if (i < n) {
      const int r = i / ws - hws, c = i % ws - hws;
      float res = bil_val(e.A, bil_win(e.H, e.W, wp, r, c)) - bil_val(e.B, bil_win(e.H, e.W, wv, r, c));
      loss += res * res;
    }
  }
  return wsum(loss);
}

// Tape of one point (gbt_lkd_forward_tape / gbt_lkd_backward_tape): the
// iterate history hist[L][K + 1] (float4: v, then the step's right-hand side
// b), the per-level setup su[L], the final position; stride tape_stride.
__host__ __device__ inline long long tape_stride(int L, int K) {
  return ((long long)16 * L * (K + 1) + (long long)sizeof(Setup) * L + 8 + 15) / 16 * 16;
}
struct TapeView {
  float4* hist;
  Setup* su;
  float* vf;
};
__device__ __forceinline__ TapeView tape_at(void* tape, long long g, int L, int K) {
  char* b = (char*)tape + g * tape_stride(L, K);
  TapeView t;
  t.hist = (float4*)b;
  t.su = (Setup*)(b + 16 * L * (K + 1));
  t.vf = (float*)(b + 16 * L * (K + 1) + sizeof(Setup) * L);
  return t;
}

template <int WS>
__global__ void __launch_bounds__(32 * WARPS) k_lkd_forward(const Lvl* __restrict__ levels, int L, int /*window: WS*/, int K,
                                                            int npairs, int npts, const float* __restrict__ pts,
                                                            const float* __restrict__ u0, float* __restrict__ loss,
                                                            float* __restrict__ vfinal, void* __restrict__ tape) {
  constexpr int ws = WS;
  __shared__ float tg_all[WARPS][(WS + 1) * (WS + 1)];  // each warp's window taps (stage_taps)
  const long long g = (long long)blockIdx.x * WARPS + (threadIdx.x >> 5);
  if (g >= (long long)npairs * npts) return;
  const int pair = (int)(g / npts);
  float vf0, vf1;
  // Every lane holds the same values; the tape stores of the 32 lanes go to
  // one address each.
  TapeView t{nullptr, nullptr, nullptr};
  if (tape) t = tape_at(tape, g, L, K);
  float l = point_forward<WS>(levels + (size_t)pair * L, L, ws, K, pts[2 * g], pts[2 * g + 1], u0[2 * g],
                               u0[2 * g + 1], t.su, t.hist, K + 1, vf0, vf1, tg_all[threadIdx.x >> 5]);
  if ((threadIdx.x & 31) == 0) {
    loss[g] = l;
    vfinal[2 * g] = vf0;
    vfinal[2 * g + 1] = vf1;
    if (tape) {
      t.vf[0] = vf0;
      t.vf[1] = vf1;
    }
  }
}

// Scatter accumulator of one warp: a box of image pixels in shared memory
// (atomics there), added to the level image once at the end; samples whose
// taps fall outside the box go to the image directly.
constexpr int GRID_CELLS = 1024;
// Backward CTAs per SM the registers are sized for: five (96 registers) for
// small windows, four (128) from 9 x 9 up, where 96 registers spill the
// per-pixel accumulators of the window's three pixels per lane.
constexpr int bw_minb(int ws) { return ws >= 9 ? 4 : 5; }
struct Grid {
  float* c;        // cells, row-major GW per row
  int y0, x0, GH, GW;
  int stride;      // image element stride in floats (2 for one component of a float2 image)
  __device__ __forceinline__ bool holds(const Bil& s) const {
    return s.y0 >= y0 && s.y0 + s.dy < y0 + GH && s.x0 >= x0 && s.x0 + s.dx < x0 + GW;
  }
  // Adds v00 .. v11 at the sample's four taps.
  __device__ __forceinline__ void add4(float* img, const Bil& s, float v00, float v10, float v01, float v11) const {
    if (holds(s)) {
      float* b = c + (s.y0 - y0) * GW + (s.x0 - x0);
      atomicAdd(b, v00);
      atomicAdd(b + s.dy * GW, v10);
      atomicAdd(b + s.dx, v01);
      atomicAdd(b + s.dy * GW + s.dx, v11);
    } else {
      atomicAdd(img + stride * s.i00, v00);
      atomicAdd(img + stride * s.i10, v10);
      atomicAdd(img + stride * s.i01, v01);
      atomicAdd(img + stride * s.i11, v11);
    }
  }
  __device__ __forceinline__ void add(float* img, const Bil& s, float v) const {
    if (holds(s)) {
      float* b = c + (s.y0 - y0) * GW + (s.x0 - x0);
      atomicAdd(b, s.w00 * v);
      atomicAdd(b + s.dy * GW, s.w10 * v);
      atomicAdd(b + s.dx, s.w01 * v);
      atomicAdd(b + s.dy * GW + s.dx, s.w11 * v);
    } else {
      atomicAdd(img + stride * s.i00, s.w00 * v);
      atomicAdd(img + stride * s.i10, s.w10 * v);
      atomicAdd(img + stride * s.i01, s.w01 * v);
      atomicAdd(img + stride * s.i11, s.w11 * v);
    }
  }
};

// Box of the clamped taps of samples at rows [ylo, yhi] + [-h, h] and columns
// [xlo, xhi] + [-h, h]; GH = 0 when it does not fit in `cells`.
__device__ __forceinline__ void grid_box(int H, int W, float ylo, float yhi, float xlo, float xhi, int h, int cells,
                                         Grid& g) {
  const int r0 = min(max((int)floorf(ylo) - h, 0), H - 1), r1 = min(max((int)floorf(yhi) + h + 1, 0), H - 1);
  const int c0 = min(max((int)floorf(xlo) - h, 0), W - 1), c1 = min(max((int)floorf(xhi) + h + 1, 0), W - 1);
  g.y0 = r0;
  g.x0 = c0;
  g.GH = r1 - r0 + 1;
  g.GW = c1 - c0 + 1;
  if (g.GH * g.GW > cells) g.GH = g.GW = 0;
}

__device__ __forceinline__ void grid_clear(Grid& g, int ncells) {
  for (int k = threadIdx.x & 31; k < ncells; k += 32) g.c[k] = 0.f;
  __syncwarp();
}

__device__ __forceinline__ void grid_flush(const Grid& g, float* img, int W) {
  __syncwarp();
  for (int k = threadIdx.x & 31; k < g.GH * g.GW; k += 32) {
    const float v = g.c[k];
    if (v != 0.f) atomicAdd(img + ((g.y0 + k / g.GW) * W + g.x0 + k % g.GW) * g.stride, v);
  }
  __syncwarp();
}

// Vector reductions (sm_90 and later): four or two consecutive floats in one
// L2 operation; the address must be 16- / 8-byte aligned.
__device__ __forceinline__ void red_add_v4(float* p, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(a), "f"(b), "f"(c), "f"(d) : "memory");
}
__device__ __forceinline__ void red_add_v2(float* p, float a, float b) {
  asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(a), "f"(b) : "memory");
}

// The box's cell (row, col), zero outside the box.
__device__ __forceinline__ float grid_cell(const Grid& g, int row, int col) {
  return (col >= 0 && col < g.GW) ? g.c[row * g.GW + col] : 0.f;
}

// grid_flush of a one-float-per-pixel image (stride 1) with one red.v4 per
// 16-byte-aligned run of four pixels of a box row (cells outside the box add
// zero; runs of four zeros are skipped): about a third of the reductions of
// one per cell.  Images whose rows or base are not 16-byte aligned take
// grid_flush.
__device__ __forceinline__ void grid_flush_v4(const Grid& g, float* img, int W) {
  if ((W & 3) != 0 || (((unsigned long long)img) & 15) != 0) {
    grid_flush(g, img, W);
    return;
  }
  __syncwarp();
  const int q0 = g.x0 >> 2, nq = ((g.x0 + g.GW - 1) >> 2) - q0 + 1;
  for (int it = threadIdx.x & 31; it < g.GH * nq; it += 32) {
    const int row = it / nq, x = 4 * (q0 + it % nq), col = x - g.x0;
    const float a = grid_cell(g, row, col), b = grid_cell(g, row, col + 1);
    const float c = grid_cell(g, row, col + 2), d = grid_cell(g, row, col + 3);
    if (a != 0.f || b != 0.f || c != 0.f || d != 0.f) red_add_v4(img + (size_t)(g.y0 + row) * W + x, a, b, c, d);
  }
  __syncwarp();
}

// Both components of a float2 image (gx: .x, gy: .y, the same box) in one
// pass: one red.v4 per 16-byte-aligned pair of pixels, or one red.v2 per
// pixel where the image's rows or base allow only 8-byte alignment.
__device__ __forceinline__ void grid_flush_pair(const Grid& gx, const Grid& gy, float2* img, int W) {
  const unsigned long long a = (unsigned long long)img;
  if ((a & 7) != 0) {
    grid_flush(gx, (float*)img, W);
    grid_flush(gy, (float*)img + 1, W);
    return;
  }
  __syncwarp();
  if ((W & 1) == 0 && (a & 15) == 0) {
    const int p0 = gx.x0 >> 1, np = ((gx.x0 + gx.GW - 1) >> 1) - p0 + 1;
    for (int it = threadIdx.x & 31; it < gx.GH * np; it += 32) {
      const int row = it / np, x = 2 * (p0 + it % np), col = x - gx.x0;
      const float u0 = grid_cell(gx, row, col), v0 = grid_cell(gy, row, col);
      const float u1 = grid_cell(gx, row, col + 1), v1 = grid_cell(gy, row, col + 1);
      if (u0 != 0.f || v0 != 0.f || u1 != 0.f || v1 != 0.f)
        red_add_v4((float*)(img + (size_t)(gx.y0 + row) * W + x), u0, v0, u1, v1);
    }
  } else {
    for (int k = threadIdx.x & 31; k < gx.GH * gx.GW; k += 32) {
      const float u = gx.c[k], v = gy.c[k];
      if (u != 0.f || v != 0.f) red_add_v2((float*)(img + (size_t)(gx.y0 + k / gx.GW) * W + gx.x0 + k % gx.GW), u, v);
    }
  }
  __syncwarp();
}

template <int WS, bool TAPE>
__global__ void __launch_bounds__(32 * WARPS, bw_minb(WS)) k_lkd_backward(const Lvl* __restrict__ levels, int L, int /*window: WS*/, int K,
                                                             int npairs, int npts, const float* __restrict__ pts,
                                                             const float* __restrict__ u0,
                                                             const float* __restrict__ dloss, float* __restrict__ du0,
                                                             const void* __restrict__ tape) {
  constexpr int ws = WS, PPL = (WS * WS + 31) / 32;
  __shared__ Setup su_all[WARPS][MAXL];
  extern __shared__ float4 hist_dyn[];  // WARPS x L x (K + 1): the iterate history
  __shared__ float gB_all[WARPS][GRID_CELLS];                       // dB over the level's residual samples
  __shared__ float gT_all[WARPS][3][(MAXW + 1) * (MAXW + 1)];      // dA, dS.x, dS.y over the template
  __shared__ float tg_all[WARPS][(WS + 1) * (WS + 1)];              // window taps of the replayed forward
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* tg = tg_all[warp];
  const long long gidx = (long long)blockIdx.x * WARPS + warp;
  if (gidx >= (long long)npairs * npts) return;
  const int pair = (int)(gidx / npts);
  const Lvl* lv = levels + (size_t)pair * L;
  Setup* su = su_all[warp];
  const int HS = K + 1;
  float4* hist = hist_dyn + (size_t)warp * L * HS;
  const float p0 = pts[2 * gidx], p1 = pts[2 * gidx + 1];
  float vf0, vf1;
  if (TAPE) {
    // The forward's record of this point instead of a replay.
    const TapeView t = tape_at(const_cast<void*>(tape), gidx, L, K);
    for (int q = lane; q < L * HS; q += 32) hist[q] = t.hist[q];
    if (lane < L) su[lane] = t.su[lane];
    vf0 = t.vf[0];
    vf1 = t.vf[1];
  } else {
    point_forward<WS>(lv, L, ws, K, p0, p1, u0[2 * gidx], u0[2 * gidx + 1], su, hist, HS, vf0, vf1, tg);
  }
  __syncwarp();
  const float w = dloss[gidx];
  const int hws = ws / 2, n = ws * ws;
  constexpr int TC = (MAXW + 1) * (MAXW + 1);
  float dv0 = 0.f, dv1 = 0.f;
  for (int l = 0; l < L; l++) {
    const Lvl& e = lv[l];
    const Setup S = su[l];
    // Scatter boxes: the template footprint, and every residual sample of the
    // level's steps (and, at level 0, of the loss).
    Grid gA{gT_all[warp][0], 0, 0, 0, 0, 1}, gS0{gT_all[warp][1], 0, 0, 0, 0, 2};
    Grid gS1{gT_all[warp][2], 0, 0, 0, 0, 2}, gB{gB_all[warp], 0, 0, 0, 0, 1};
    grid_box(e.H, e.W, S.q0, S.q0, S.q1, S.q1, hws, TC, gA);
    gS0.y0 = gS1.y0 = gA.y0;
    gS0.x0 = gS1.x0 = gA.x0;
    gS0.GH = gS1.GH = gA.GH;
    gS0.GW = gS1.GW = gA.GW;
    {
      float ylo = 1e30f, yhi = -1e30f, xlo = 1e30f, xhi = -1e30f;
      for (int k = 0; k <= K; k++) {
        if (k == K && l != 0) break;
        const float4 v = hist[l * HS + k];
        ylo = fminf(ylo, v.x);
        yhi = fmaxf(yhi, v.x);
        xlo = fminf(xlo, v.y);
        xhi = fmaxf(xhi, v.y);
      }
      grid_box(e.H, e.W, ylo, yhi, xlo, xhi, hws, GRID_CELLS, gB);
    }
    grid_clear(gA, gA.GH * gA.GW);
    grid_clear(gS0, gS0.GH * gS0.GW);
    grid_clear(gS1, gS1.GH * gS1.GW);
    grid_clear(gB, gB.GH * gB.GW);
    Tmpl<PPL> T;
    load_template<WS>(e, ws, S.q0, S.q1, T);
    if (l == 0) {
      // Loss at level 0: r = A0(p + o) - B0(v + o), dL/dr = 2 r w.
      const Win wp = win_at(e.H, e.W, p0, p1, hws), wf = win_at(e.H, e.W, vf0, vf1, hws);
#pragma unroll
      for (int kk = 0; kk < PPL; kk++) {
        const int i = lane + 32 * kk;
        if (i < n) {
          const int r = i / ws - hws, c = i % ws - hws;
          Bil sa = bil_win(e.H, e.W, wp, r, c), sb = bil_win(e.H, e.W, wf, r, c);
          const float res = bil_val(e.A, sa) - bil_val(e.B, sb);
          const float dr = 2.f * res * w;
          gA.add(e.dA, sa, dr);
          gB.add(e.dB, sb, -dr);
          float2 gb = bil_grad(e.B, sb);
          dv0 -= dr * gb.x;
          dv1 -= dr * gb.y;
        }
      }
      dv0 = wsum(dv0);
      dv1 = wsum(dv1);
    }
    float dM00 = 0.f, dM01 = 0.f, dM10 = 0.f, dM11 = 0.f;
    float dg0[PPL], dg1[PPL], dT[PPL];
#pragma unroll
    for (int k = 0; k < PPL; k++) dg0[k] = dg1[k] = dT[k] = 0.f;
    // The residual samples' adjoint goes to dB at each step's window taps.
    // Every window pixel of a step shares the centre's integer position, and
    // the iterates converge, so consecutive steps mostly share their taps:
    // the four tap contributions of each window pixel are summed in registers
    // (acc) while the window's integer position stays (wacc), and scattered
    // once when it changes and after the last step.
    Win wacc;
    wacc.y0 = INT_MIN;
    float acc00[PPL], acc10[PPL], acc01[PPL], acc11[PPL];
    auto scatter_acc = [&]() {
#pragma unroll
      for (int kk = 0; kk < PPL; kk++) {
        const int i = lane + 32 * kk;
        if (i < n) {
          const Bil sb = bil_win(e.H, e.W, wacc, i / ws - hws, i % ws - hws);
          gB.add4(e.dB, sb, acc00[kk], acc10[kk], acc01[kk], acc11[kk]);
        }
      }
    };
    for (int k = K - 1; k >= 0; k--) {
      const float4 vk = hist[l * HS + k];  // v_k and b_k of the forward
      const float d0 = dv0, d1 = dv1;                       // adjoint of v_{k+1}
      const float db0 = S.M00 * d0 + S.M01 * d1, db1 = S.M01 * d0 + S.M11 * d1;
      const float b0 = vk.z, b1 = vk.w;
      float pv0 = 0.f, pv1 = 0.f;
      const Win wk = win_at(e.H, e.W, vk.x, vk.y, hws);
      if (wk.y0 != wacc.y0 || wk.x0 != wacc.x0) {  // warp-uniform
        if (wacc.y0 != INT_MIN) scatter_acc();
        wacc = wk;
#pragma unroll
        for (int kk = 0; kk < PPL; kk++) acc00[kk] = acc10[kk] = acc01[kk] = acc11[kk] = 0.f;
      }
#pragma unroll
      for (int kk = 0; kk < PPL; kk++) {
        const int i = lane + 32 * kk;
        if (i < n) {
          const Bil sb = bil_win(e.H, e.W, wk, i / ws - hws, i % ws - hws);
          const float bv = bil_val(e.B, sb);
          const float2 gb = bil_grad(e.B, sb);
          const float2 g = T.g[kk];
          const float res = T.a[kk] - bv;
          const float dres = g.x * db0 + g.y * db1;
          dg0[kk] += res * db0;
          dg1[kk] += res * db1;
          dT[kk] += dres;
          acc00[kk] -= wk.w00 * dres;
          acc10[kk] -= wk.w10 * dres;
          acc01[kk] -= wk.w01 * dres;
          acc11[kk] -= wk.w11 * dres;
          pv0 -= dres * gb.x;
          pv1 -= dres * gb.y;
        }
      }
      dv0 = d0 + wsum(pv0);
      dv1 = d1 + wsum(pv1);
      dM00 += d0 * b0;
      dM01 += d0 * b1;
      dM10 += d1 * b0;
      dM11 += d1 * b1;
    }
    if (wacc.y0 != INT_MIN) scatter_acc();
    // dG = -M dM M (M symmetric); then dg += (dG + dG^T) g.
    const float t00 = dM00 * S.M00 + dM01 * S.M01, t01 = dM00 * S.M01 + dM01 * S.M11;
    const float t10 = dM10 * S.M00 + dM11 * S.M01, t11 = dM10 * S.M01 + dM11 * S.M11;
    const float G00 = -(S.M00 * t00 + S.M01 * t10), G01 = -(S.M00 * t01 + S.M01 * t11);
    const float G10 = -(S.M01 * t00 + S.M11 * t10), G11 = -(S.M01 * t01 + S.M11 * t11);
    const float H00 = 2.f * G00, H01 = G01 + G10, H11 = 2.f * G11;
    const Win wq = win_at(e.H, e.W, S.q0, S.q1, hws);
#pragma unroll
    for (int kk = 0; kk < PPL; kk++) {
      const int i = lane + 32 * kk;
      if (i < n) {
        Bil st = bil_win(e.H, e.W, wq, i / ws - hws, i % ws - hws);
        const float2 g = T.g[kk];
        gS0.add((float*)e.dS, st, dg0[kk] + H00 * g.x + H01 * g.y);
        gS1.add((float*)e.dS + 1, st, dg1[kk] + H01 * g.x + H11 * g.y);
        gA.add(e.dA, st, dT[kk]);
      }
    }
    grid_flush_v4(gA, e.dA, e.W);
    grid_flush_pair(gS0, gS1, e.dS, e.W);
    grid_flush_v4(gB, e.dB, e.W);
    // v_0 = q + d_init: the adjoint of d_init is dv.
    if (l + 1 < L) {
      dv0 *= 2.f;  // d_init(l) = 2 (v_K(l+1) - q(l+1))
      dv1 *= 2.f;
    }
  }
  const float top = level_scale(L - 1);
  if (lane == 0) {
    du0[2 * gidx] = dv0 / top;
    du0[2 * gidx + 1] = dv1 / top;
  }
}

__global__ void k_to_dense(const float* __restrict__ in, long long pitch, long long img_bytes, int H, int W,
                           float* __restrict__ out) {
  const int pair = blockIdx.y;
  const float* s = (const float*)((const char*)in + pair * img_bytes);
  float* d = out + (size_t)pair * H * W;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < H * W; t += gridDim.x * blockDim.x)
    d[t] = ((const float*)((const char*)s + (size_t)(t / W) * pitch))[t % W];
}

__global__ void k_sobel(const float* __restrict__ a, int H, int W, long long stride, float2* __restrict__ g) {
  const int pair = blockIdx.y;
  const float* A = a + pair * stride;
  float2* G = g + pair * stride;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < H * W; t += gridDim.x * blockDim.x) {
    int r = t / W, c = t % W;
    float2 v = make_float2(0.f, 0.f);
    if (r >= 1 && r < H - 1 && c >= 1 && c < W - 1) {
#define P(dr, dc) A[(size_t)(r + (dr)) * W + (c + (dc))]
      v.x = (P(1, -1) + 2 * P(1, 0) + P(1, 1) - P(-1, -1) - 2 * P(-1, 0) - P(-1, 1)) / 8.f;
      v.y = (P(-1, 1) + 2 * P(0, 1) + P(1, 1) - P(-1, -1) - 2 * P(0, -1) - P(1, -1)) / 8.f;
#undef P
    }
    G[t] = v;
  }
}

// dA += Sobel^T(dS): each interior source pixel's weights, gathered.
__global__ void k_sobel_t(const float2* __restrict__ dS, int H, int W, long long stride, float* __restrict__ dA) {
  const int pair = blockIdx.y;
  const float2* G = dS + pair * stride;
  float* A = dA + pair * stride;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < H * W; t += gridDim.x * blockDim.x) {
    const int y = t / W, x = t % W;
    float acc = 0.f;
    for (int dr = -1; dr <= 1; dr++)
      for (int dc = -1; dc <= 1; dc++) {
        const int r = y - dr, c = x - dc;  // source pixel that reads A(y, x) at offset (dr, dc)
        if (r < 1 || r >= H - 1 || c < 1 || c >= W - 1) continue;
        const float wr = (dr == 0) ? 0.f : (float)dr * (dc == 0 ? 2.f : 1.f) / 8.f;
        const float wc = (dc == 0) ? 0.f : (float)dc * (dr == 0 ? 2.f : 1.f) / 8.f;
        const float2 gv = G[(size_t)r * W + c];
        acc += wr * gv.x + wc * gv.y;
      }
    A[t] += acc;
  }
}

struct Taps7 {
  float w[7];
};

// Transpose of "blur columns at even positions, keep row 2r": fills tmp
// (H x W) from the level above (H2 x W2).
__global__ void k_decimate_t_rows(const float* __restrict__ up, int H2, int W2, long long ustride,
                                  float* __restrict__ tmp, int H, int W, long long tstride, Taps7 t) {
  const int pair = blockIdx.y;
  const float* U = up + pair * ustride;
  float* T = tmp + pair * tstride;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < H * W; i += gridDim.x * blockDim.x) {
    const int y = i / W, x = i % W;
    float acc = 0.f;
    if ((x & 1) == 0 && x / 2 < W2) {
      const int c = x / 2;
      const int rlo = max(0, (y - 4) / 2 - 1), rhi = min(H2 - 1, (y + 4) / 2 + 1);
      for (int r = rlo; r <= rhi; r++)
        for (int k = -3; k <= 3; k++) {
          const int yy = min(max(2 * r + k, 0), H - 1);
          if (yy == y) acc += t.w[k + 3] * U[(size_t)r * W2 + c];
        }
      // Rows beyond the small window can only reach y through clamping.
      if (y == 0 || y == H - 1)
        for (int r = 0; r < H2; r++) {
          if (r >= rlo && r <= rhi) continue;
          for (int k = -3; k <= 3; k++) {
            const int yy = min(max(2 * r + k, 0), H - 1);
            if (yy == y) acc += t.w[k + 3] * U[(size_t)r * W2 + c];
          }
        }
    }
    T[i] = acc;
  }
}

// Transpose of the row blur (clamped): dA(y, x) += sum_{c, k: clamp(c + k) == x} w_k tmp(y, c).
__global__ void k_blur_t_cols(const float* __restrict__ tmp, int H, int W, long long stride, float* __restrict__ dA,
                              Taps7 t) {
  const int pair = blockIdx.y;
  const float* T = tmp + pair * stride;
  float* A = dA + pair * stride;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < H * W; i += gridDim.x * blockDim.x) {
    const int y = i / W, x = i % W;
    float acc = 0.f;
    const int clo = (x == 0) ? 0 : max(0, x - 3), chi = (x == W - 1) ? W - 1 : min(W - 1, x + 3);
    for (int c = clo; c <= chi; c++)
      for (int k = -3; k <= 3; k++) {
        const int xx = min(max(c + k, 0), W - 1);
        if (xx == x) acc += t.w[k + 3] * T[(size_t)y * W + c];
      }
    A[i] += acc;
  }
}

}  // namespace gbt_lkd

using namespace gbt_lkd;

extern "C" int64_t gbt_lkd_scratch_bytes(int32_t rows, int32_t cols, int32_t nlevels, int32_t npairs) {
  if (rows < 16 || cols < 16 || nlevels < 1 || nlevels > MAXL || npairs < 1) return -1;
  int64_t px = 0;
  for (int l = 0, h = rows, w = cols; l < nlevels; l++, h /= 2, w /= 2) px += (int64_t)h * w;
  // A, B, S (2), dA, dB, dS (2), tmp: 9 floats per pixel; plus the level table.
  return px * npairs * 36 + (int64_t)npairs * nlevels * sizeof(Lvl) + 4096;
}

namespace {

std::mutex g_mu;
std::vector<std::pair<void*, int64_t>> g_arena;

void* arena_for(int64_t need, cudaStream_t st) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(g_mu);
  if ((int)g_arena.size() <= dev) g_arena.resize(dev + 1, {nullptr, 0});
  if (g_arena[dev].second < need) {
    if (g_arena[dev].first) {
      cudaStreamSynchronize(st);
      cudaFree(g_arena[dev].first);
    }
    g_arena[dev] = {nullptr, 0};
    if (cudaMalloc(&g_arena[dev].first, need) != cudaSuccess) return nullptr;
    g_arena[dev].second = need;
  }
  return g_arena[dev].first;
}

struct Plan {
  int L, H[MAXL], W[MAXL];
  int64_t off[MAXL], px;
  float *A, *B, *dA, *dB, *tmp;
  float2 *S, *dS;
  Lvl* table;
};

// Lays out the arena and builds both pyramids and the Sobel images.
int prepare(const float* I0, const float* I1, int64_t pitch, int64_t img_bytes, int rows, int cols, int L, int npairs,
            bool adjoint, Plan& P, cudaStream_t st) {
  const int64_t need = gbt_lkd_scratch_bytes(rows, cols, L, npairs);
  if (need < 0) return GBT_E_INVALID;
  char* base = (char*)arena_for(need, st);
  if (!base) return GBT_E_OOM;
  P.L = L;
  P.px = 0;
  for (int l = 0, h = rows, w = cols; l < L; l++, h /= 2, w /= 2) {
    P.H[l] = h;
    P.W[l] = w;
    P.off[l] = P.px;
    P.px += (int64_t)h * w * npairs;
  }
  float* f = (float*)base;
  P.A = f;
  P.B = f + P.px;
  P.dA = f + 2 * P.px;
  P.dB = f + 3 * P.px;
  P.tmp = f + 4 * P.px;
  P.S = (float2*)(f + 5 * P.px);
  P.dS = (float2*)(f + 7 * P.px);
  P.table = (Lvl*)(f + 9 * P.px);
  dim3 blk(256);
  for (int which = 0; which < 2; which++) {
    float* dst = which ? P.B : P.A;
    k_to_dense<<<dim3(128, npairs), blk, 0, st>>>(which ? I1 : I0, pitch, img_bytes, rows, cols, dst);
    for (int p = 0; p < npairs; p++) {
      const float* src = dst + (int64_t)p * rows * cols;
      int64_t sp = (int64_t)cols * 4;
      for (int l = 1; l < L; l++) {
        float* lvl = dst + P.off[l] + (int64_t)p * P.H[l] * P.W[l];
        int r = gbt_gaussian_pyramid_f32(src, sp, P.H[l - 1], P.W[l - 1], 2, lvl, st);
        if (r) return r;
        src = lvl;
        sp = (int64_t)P.W[l] * 4;
      }
    }
  }
  for (int l = 0; l < L; l++)
    k_sobel<<<dim3(64, npairs), blk, 0, st>>>(P.A + P.off[l], P.H[l], P.W[l], (long long)P.H[l] * P.W[l],
                                              P.S + P.off[l]);
  if (adjoint) {
    cudaMemsetAsync(P.dA, 0, P.px * 8, st);           // dA and dB
    cudaMemsetAsync(P.dS, 0, P.px * 8, st);
  }
  std::vector<Lvl> h((size_t)npairs * L);
  for (int p = 0; p < npairs; p++)
    for (int l = 0; l < L; l++) {
      int64_t o = P.off[l] + (int64_t)p * P.H[l] * P.W[l];
      h[(size_t)p * L + l] = Lvl{P.H[l], P.W[l], P.A + o, P.B + o, P.S + o, P.dA + o, P.dB + o, P.dS + o};
    }
  cudaMemcpyAsync(P.table, h.data(), h.size() * sizeof(Lvl), cudaMemcpyHostToDevice, st);
  cudaStreamSynchronize(st);  // the host table must outlive the copy
  return cudaGetLastError() == cudaSuccess ? GBT_OK : GBT_E_CUDA;
}

int check_args(const float* I0, const float* I1, int rows, int cols, int L, int ws, int K, int npairs, int npts) {
  if (!I0 || !I1 || rows < 16 || cols < 16 || L < 1 || L > MAXL || npairs < 1 || npts < 0) return GBT_E_INVALID;
  if (ws < 3 || ws > MAXW || !(ws & 1) || K < 0 || K > MAXK) return GBT_E_INVALID;
  if ((rows >> (L - 1)) < 4 || (cols >> (L - 1)) < 4) return GBT_E_INVALID;
  return GBT_OK;
}

}  // namespace

extern "C" int64_t gbt_lkd_tape_bytes(int32_t nlevels, int32_t iters, int32_t npairs, int32_t npts) {
  if (nlevels < 1 || nlevels > MAXL || iters < 0 || iters > MAXK || npairs < 1 || npts < 0) return -1;
  return tape_stride(nlevels, iters) * npairs * npts;
}

extern "C" int gbt_lkd_forward_tape(const float* I0, const float* I1, int64_t pitch, int64_t img_bytes, int32_t rows,
                                    int32_t cols, int32_t nlevels, int32_t window, int32_t iters, int32_t npairs,
                                    const float* pts, const float* u0, int32_t npts, float* loss, float* vfinal,
                                    void* tape, void* stream) {
  int r = check_args(I0, I1, rows, cols, nlevels, window, iters, npairs, npts);
  if (r) return r;
  if (npts > 0 && (!pts || !u0 || !loss || !vfinal)) return GBT_E_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  Plan P;
  if ((r = prepare(I0, I1, pitch, img_bytes, rows, cols, nlevels, npairs, false, P, st))) return r;
  long long total = (long long)npairs * npts;
  if (total > 0)
    switch (window) {
#define GO(WS) k_lkd_forward<WS><<<(unsigned)((total + WARPS - 1) / WARPS), 32 * WARPS, 0, st>>>( \
      P.table, nlevels, window, iters, npairs, npts, pts, u0, loss, vfinal, tape)
      case 3: GO(3); break;
      case 5: GO(5); break;
      case 7: GO(7); break;
      case 9: GO(9); break;
      case 11: GO(11); break;
      case 13: GO(13); break;
      default: GO(15); break;
#undef GO
    }
  return cudaGetLastError() == cudaSuccess ? GBT_OK : GBT_E_CUDA;
}

extern "C" int gbt_lkd_forward(const float* I0, const float* I1, int64_t pitch, int64_t img_bytes, int32_t rows,
                               int32_t cols, int32_t nlevels, int32_t window, int32_t iters, int32_t npairs,
                               const float* pts, const float* u0, int32_t npts, float* loss, float* vfinal,
                               void* stream) {
  return gbt_lkd_forward_tape(I0, I1, pitch, img_bytes, rows, cols, nlevels, window, iters, npairs, pts, u0, npts,
                              loss, vfinal, nullptr, stream);
}

extern "C" int gbt_lkd_backward_tape(const float* I0, const float* I1, int64_t pitch, int64_t img_bytes, int32_t rows,
                                     int32_t cols, int32_t nlevels, int32_t window, int32_t iters, int32_t npairs,
                                     const float* pts, const float* u0, int32_t npts, const float* dloss, float* dI0,
                                     float* dI1, float* du0, const void* tape, void* stream) {
  int r = check_args(I0, I1, rows, cols, nlevels, window, iters, npairs, npts);
  if (r) return r;
  if (!dI0 || !dI1) return GBT_E_INVALID;
  if (npts > 0 && (!pts || !u0 || !dloss || !du0)) return GBT_E_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  Plan P;
  if ((r = prepare(I0, I1, pitch, img_bytes, rows, cols, nlevels, npairs, true, P, st))) return r;
  long long total = (long long)npairs * npts;
  const size_t hbytes = (size_t)WARPS * nlevels * (iters + 1) * sizeof(float4);
  if (total > 0)
    switch (window) {
#define GO(WS)                                                                                            \
  if (tape)                                                                                               \
    k_lkd_backward<WS, true><<<(unsigned)((total + WARPS - 1) / WARPS), 32 * WARPS, hbytes, st>>>(       \
        P.table, nlevels, window, iters, npairs, npts, pts, u0, dloss, du0, tape);                        \
  else                                                                                                    \
    k_lkd_backward<WS, false><<<(unsigned)((total + WARPS - 1) / WARPS), 32 * WARPS, hbytes, st>>>(      \
        P.table, nlevels, window, iters, npairs, npts, pts, u0, dloss, du0, tape)
      case 3: GO(3); break;
      case 5: GO(5); break;
      case 7: GO(7); break;
      case 9: GO(9); break;
      case 11: GO(11); break;
      case 13: GO(13); break;
      default: GO(15); break;
#undef GO
    }
  float taps_f[16];
  int32_t R;
  gbt_gaussian_taps(1.f, taps_f, &R);
  Taps7 t;
  for (int k = 0; k < 7; k++) t.w[k] = taps_f[k];
  dim3 blk(256);
  // Sobel transpose on every level, then pull each level down the pyramid.
  for (int l = 0; l < nlevels; l++)
    k_sobel_t<<<dim3(64, npairs), blk, 0, st>>>(P.dS + P.off[l], P.H[l], P.W[l], (long long)P.H[l] * P.W[l],
                                                P.dA + P.off[l]);
  for (int which = 0; which < 2; which++) {
    float* d = which ? P.dB : P.dA;
    for (int l = nlevels - 1; l >= 1; l--) {
      k_decimate_t_rows<<<dim3(64, npairs), blk, 0, st>>>(d + P.off[l], P.H[l], P.W[l], (long long)P.H[l] * P.W[l],
                                                          P.tmp, P.H[l - 1], P.W[l - 1],
                                                          (long long)P.H[l - 1] * P.W[l - 1], t);
      k_blur_t_cols<<<dim3(64, npairs), blk, 0, st>>>(P.tmp, P.H[l - 1], P.W[l - 1],
                                                      (long long)P.H[l - 1] * P.W[l - 1], d + P.off[l - 1], t);
    }
  }
  cudaMemcpyAsync(dI0, P.dA, (size_t)npairs * rows * cols * 4, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(dI1, P.dB, (size_t)npairs * rows * cols * 4, cudaMemcpyDeviceToDevice, st);
  return cudaGetLastError() == cudaSuccess ? GBT_OK : GBT_E_CUDA;
}

extern "C" int gbt_lkd_backward(const float* I0, const float* I1, int64_t pitch, int64_t img_bytes, int32_t rows,
                                int32_t cols, int32_t nlevels, int32_t window, int32_t iters, int32_t npairs,
                                const float* pts, const float* u0, int32_t npts, const float* dloss, float* dI0,
                                float* dI1, float* du0, void* stream) {
  return gbt_lkd_backward_tape(I0, I1, pitch, img_bytes, rows, cols, nlevels, window, iters, npairs, pts, u0, npts,
                               dloss, dI0, dI1, du0, nullptr, stream);
}
