// Pyramidal Lucas-Kanade for sm_103a.
//
// Reproduces iterative_lk_match_5x5::match (cuimg/tracking2/pyrlk_tracker.hpp:165-334)
// with the coarse-to-fine recursion of get_flow_at / recursive_prediction
// (:1027-1063, cuimg/tracking2/predictions.h:61-74) and the acceptance rule of
// pyrlk_match_particles_kernel (:677-769), for batches of frame pairs and
// points.  Window size, mask size and iteration count are parameters (the
// reference hard-codes 11, 25 and 30).  Undefined reference cases are defined
// as in the oracle: clamp-to-edge sampling, identity flow when an upper match
// leaves its level.  Equal gradient norms at the edge of the strongest-gradient
// selection are resolved as the reference's std::nth_element (GNU libstdc++)
// resolves them.
//
// Layout: per pair and level, the previous and current levels (fp32, dense
// rows) and the Sobel/8 gradient of the previous level (float2), all in one
// scratch arena.  One warp tracks one point through all levels: window pixels
// are spread over the lanes, the masked pixels are compacted by rank, and the
// 2x2 normal matrix and right-hand side are warp reductions whose lane-0
// result is broadcast, so every lane takes identical decisions.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <vector>

#include "cuimg_gb300.h"
#include "nth_select.cuh"

namespace gbt_lk {

constexpr int MAXW = 15;             // largest window
constexpr int MAXPIX = MAXW * MAXW;  // 225

struct Level {
  int H, W;
  const float* prev;
  const float* cur;
  const float2* grad;  // (d/drow, d/dcol)
};

struct Params {
  int ws, npix, max_iter, L;
  float eps, max_err;
  int u8;
};

__device__ __forceinline__ float li(const float* img, int H, int W, float y, float x) {
  int y0 = (int)y, x0 = (int)x;
  float a0 = y - (float)y0, a1 = x - (float)x0;
  int y1 = min(max(y0 + 1, 0), H - 1), x1 = min(max(x0 + 1, 0), W - 1);
  y0 = min(max(y0, 0), H - 1);
  x0 = min(max(x0, 0), W - 1);
  float v00 = __ldg(img + (size_t)y0 * W + x0), v10 = __ldg(img + (size_t)y1 * W + x0);
  float v01 = __ldg(img + (size_t)y0 * W + x1), v11 = __ldg(img + (size_t)y1 * W + x1);
  return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(1.f - a0, 1.f - a1), v00), __fmul_rn(__fmul_rn(a0, 1.f - a1), v10)),
                             __fmul_rn(__fmul_rn(1.f - a0, a1), v01)),
                   __fmul_rn(__fmul_rn(a0, a1), v11));
}

__device__ __forceinline__ float2 li2(const float2* img, int H, int W, float y, float x) {
  int y0 = (int)y, x0 = (int)x;
  float a0 = y - (float)y0, a1 = x - (float)x0;
  int y1 = min(max(y0 + 1, 0), H - 1), x1 = min(max(x0 + 1, 0), W - 1);
  y0 = min(max(y0, 0), H - 1);
  x0 = min(max(x0, 0), W - 1);
  float2 v00 = img[(size_t)y0 * W + x0], v10 = img[(size_t)y1 * W + x0];
  float2 v01 = img[(size_t)y0 * W + x1], v11 = img[(size_t)y1 * W + x1];
  float w00 = __fmul_rn(1.f - a0, 1.f - a1), w10 = __fmul_rn(a0, 1.f - a1), w01 = __fmul_rn(1.f - a0, a1),
        w11 = __fmul_rn(a0, a1);
  float2 o;
  o.x = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(w00, v00.x), __fmul_rn(w10, v10.x)), __fmul_rn(w01, v01.x)),
                  __fmul_rn(w11, v11.x));
  o.y = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(w00, v00.y), __fmul_rn(w10, v10.y)), __fmul_rn(w01, v01.y)),
                  __fmul_rn(w11, v11.y));
  return o;
}

__device__ __forceinline__ bool box_has(int H, int W, int b, float y, float x) {
  int r = (int)y, c = (int)x;
  return r >= b && r <= H - b - 1 && c >= b && c <= W - b - 1;
}

// Sum over the warp, reduced to lane 0 and broadcast.
__device__ __forceinline__ float warp_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return __shfl_sync(0xffffffffu, v, 0);
}

struct __align__(8) WarpSmem {
  union {
    struct {
      float r[MAXPIX], c[MAXPIX];  // gradients of the masked pixels by rank
    } mg;
    unsigned long long ord[MAXPIX];  // (norm bits << 32 | window index) while selecting
  };
  float as[MAXPIX], mas[MAXPIX];
  short mr[MAXPIX], mc[MAXPIX];
};

// iterative_lk_match_5x5::match for one point (all lanes of the warp); PPL
// window pixels per lane (ceil(window^2 / 32)).
// Returns true when accepted by the matcher itself; tr / err as the reference.
template <int PPL>
__device__ bool lk_match(const Level& lv, const Params& P, WarpSmem& S, float py, float px, float ptr_y, float ptr_x,
                         float& tr_y, float& tr_x, float& err) {
  const int lane = threadIdx.x & 31;
  const int ws = P.ws, hws = ws / 2, n = ws * ws;
  const int N = P.npix < n ? P.npix : n;
  float gr[PPL], gc[PPL];
  unsigned nb[PPL];  // gradient norm bits (norms are >= 0, so they order like the floats)
  bool valid[PPL];
#pragma unroll
  for (int k = 0; k < PPL; k++) {
    int i = lane + 32 * k;
    gr[k] = gc[k] = 0.f;
    nb[k] = 0;
    valid[k] = i < n;
    if (valid[k]) {
      int r = i / ws - hws, c = i % ws - hws;
      float y = py + (float)r, x = px + (float)c;
      float2 g = li2(lv.grad, lv.H, lv.W, y, x);
      gr[k] = g.x;
      gc[k] = g.y;
      float a = li(lv.prev, lv.H, lv.W, y, x);
      S.as[i] = P.u8 ? (float)(unsigned char)a : a;
      nb[k] = __float_as_uint(__fsqrt_rn(__fadd_rn(__fmul_rn(g.x, g.x), __fmul_rn(g.y, g.y))));
    }
  }
  // The N strongest gradients, the reference's nth_element selection
  // (pyrlk_tracker.hpp:207-228): a bitwise search for the N-th largest norm t;
  // every norm above t is selected.  When the norms equal to t all fit
  // (#above + #equal == N) they are selected too; otherwise which of them the
  // reference keeps depends on nth_element's steps, replayed by one lane.
  bool sel[PPL];
  if (N >= n) {
#pragma unroll
    for (int k = 0; k < PPL; k++) sel[k] = valid[k];
  } else {
    unsigned t = 0;
    for (int bit = 30; bit >= 0; bit--) {
      const unsigned cand = t | (1u << bit);
      int cnt = 0;
#pragma unroll
      for (int k = 0; k < PPL; k++) cnt += __popc(__ballot_sync(0xffffffffu, valid[k] && nb[k] >= cand));
      if (cnt >= N) t = cand;
    }
    int atleast = 0;
#pragma unroll
    for (int k = 0; k < PPL; k++) atleast += __popc(__ballot_sync(0xffffffffu, valid[k] && nb[k] >= t));
    if (atleast == N) {
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
      if (lane == 0) gbt_sel::nth_select(S.ord, n, N);
      __syncwarp();
      for (int j = lane; j < N; j += 32) S.mr[(int)(S.ord[j] & 0xffffffffu)] = 1;
      __syncwarp();
#pragma unroll
      for (int k = 0; k < PPL; k++) sel[k] = valid[k] && S.mr[lane + 32 * k] != 0;
      __syncwarp();
    }
  }
  // Selected pixels, compacted in window order.
  {
    const unsigned lt = (1u << lane) - 1u;
    int base = 0;
#pragma unroll
    for (int k = 0; k < PPL; k++) {
      const unsigned bs = __ballot_sync(0xffffffffu, sel[k]);
      if (sel[k]) {
        const int m = base + __popc(bs & lt), i = lane + 32 * k;
        S.mg.r[m] = gr[k];
        S.mg.c[m] = gc[k];
        S.mas[m] = S.as[i];
        S.mr[m] = (short)(i / ws - hws);
        S.mc[m] = (short)(i % ws - hws);
      }
      base += __popc(bs);
    }
  }
  __syncwarp();
  // Normal matrix over the masked pixels.
  float g00 = 0.f, g01 = 0.f, g11 = 0.f;
  for (int m = lane; m < N; m += 32) {
    float a = S.mg.r[m], b = S.mg.c[m];
    g00 += a * a;
    g01 += a * b;
    g11 += b * b;
  }
  g00 = warp_sum(g00);
  g01 = warp_sum(g01);
  g11 = warp_sum(g11);
  const float tr2 = (g00 + g11) * 0.5f, det = g00 * g11 - g01 * g01;
  const float disc = sqrtf(fmaxf(tr2 * tr2 - det, 0.f));
  const float e1 = fabsf(tr2 + disc), e2 = fabsf(tr2 - disc);
  bool ok = fminf(e1, e2) >= 0.0001f;
  float vy = py + ptr_y, vx = px + ptr_x;
  const float pred_y = vy, pred_x = vx;
  if (ok) {
    const float i00 = g11 / det, i01 = -g01 / det, i11 = g00 / det;
    float nk0 = 1.f, nk1 = 1.f;
    for (int it = 0; it < P.max_iter && sqrtf(nk0 * nk0 + nk1 * nk1) >= P.eps; it++) {
      float b0 = 0.f, b1 = 0.f;
      for (int m = lane; m < N; m += 32) {
        float dt = S.mas[m] - li(lv.cur, lv.H, lv.W, vy + (float)S.mr[m], vx + (float)S.mc[m]);
        b0 += S.mg.r[m] * dt;
        b1 += S.mg.c[m] * dt;
      }
      b0 = warp_sum(b0);
      b1 = warp_sum(b1);
      nk0 = i00 * b0 + i01 * b1;
      nk1 = i01 * b0 + i11 * b1;
      vy += nk0;
      vx += nk1;
      float d0 = pred_y - vy, d1 = pred_x - vx;
      if (sqrtf(d0 * d0 + d1 * d1) > (float)(ws * 4) || !box_has(lv.H, lv.W, 3, vy, vx)) {
        ok = false;
        break;
      }
    }
  }
  if (ok) {
    // Mean absolute residual with the reference's window index
    // (r + hws) * hws + (c + hws) and running counter (pyrlk_tracker.hpp:320-331).
    float e = 0.f;
    for (int i = lane; i < n; i += 32) {
      int r = i / ws - hws, c = i % ws - hws;
      int j = (r + hws) * hws + (c + hws);
      e += fabsf(S.as[j] - li(lv.cur, lv.H, lv.W, vy + (float)r, vx + (float)c));
    }
    e = warp_sum(e);
    tr_y = vy - py;
    tr_x = vx - px;
    err = e / (float)(N + n);
  } else {
    tr_y = tr_x = -1.f;
    err = 1000.f;
  }
  __syncwarp();
  return ok;
}

template <int PPL, int NW>
__global__ void __launch_bounds__(32 * NW) k_lk_track(const Level* __restrict__ levels, Params P, int npairs,
                                                         int npts, const float* __restrict__ pts,
                                                         float* __restrict__ out, int* __restrict__ status,
                                                         float* __restrict__ err) {
  __shared__ WarpSmem smem[NW];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long g = (long long)blockIdx.x * NW + warp;
  if (g >= (long long)npairs * npts) return;
  const int pair = (int)(g / npts);
  const Level* lv = levels + (size_t)pair * P.L;
  WarpSmem& S = smem[warp];
  const float p_y = pts[2 * g], p_x = pts[2 * g + 1];
  // Coarse-to-fine: flow of the upper levels (get_flow_at), top first.
  float fy = 0.f, fx = 0.f;  // flow returned by level l + 1
  for (int l = P.L - 1; l >= 1; l--) {
    float qy = p_y, qx = p_x;
    for (int k = 0; k < l; k++) {
      qy = qy / 2.f;
      qx = qx / 2.f;
    }
    const Level& L = lv[l];
    float ptr_y = (l + 1 < P.L) ? 2.f * fy : 0.f, ptr_x = (l + 1 < P.L) ? 2.f * fx : 0.f;
    float ny = 0.f, nx = 0.f;
    if (box_has(L.H, L.W, 3, qy + ptr_y, qx + ptr_x)) {
      float ty, tx, e;
      lk_match<PPL>(L, P, S, qy, qx, ptr_y, ptr_x, ty, tx, e);
      if (box_has(L.H, L.W, 0, qy + ty, qx + tx)) {
        ny = ty;
        nx = tx;
      }
    }
    fy = ny;
    fx = nx;
  }
  // Level 0: pyrlk_match_particles_kernel's prediction and acceptance.
  const Level& L0 = lv[0];
  int st = 0;
  float oy = p_y, ox = p_x, oe = 1000.f;
  if (box_has(L0.H, L0.W, 3, p_y, p_x)) {
    float ptr_y = P.L > 1 ? 2.f * fy : 0.f, ptr_x = P.L > 1 ? 2.f * fx : 0.f;
    float pred_y = p_y + ptr_y, pred_x = p_x + ptr_x;
    if (box_has(L0.H, L0.W, 3, pred_y, pred_x)) {
      float ty, tx, e;
      lk_match<PPL>(L0, P, S, p_y, p_x, ptr_y, ptr_x, ty, tx, e);
      float m0 = (float)(int)(p_y + ty), m1 = (float)(int)(p_x + tx);
      float d0 = m0 - pred_y, d1 = m1 - pred_x;
      oe = e;
      if (box_has(L0.H, L0.W, 3, p_y + ty, p_x + tx) && e < P.max_err && sqrtf(d0 * d0 + d1 * d1) < 160.f) {
        st = 1;
        oy = p_y + ty;
        ox = p_x + tx;
      }
    }
  }
  if (lane == 0) {
    out[2 * g] = oy;
    out[2 * g + 1] = ox;
    status[g] = st;
    err[g] = oe;
  }
}

// One warp per point; the window pixels per lane (PPL) and the warps per CTA
// (NW, a tuning choice) are compile-time.
template <int NW>
void launch_lk_nw(const Level* table, const Params& P, int ppl, int npairs, int npts, const float* pts, float* out,
                  int* status, float* err, cudaStream_t st) {
  const long long blocks = ((long long)npairs * npts + NW - 1) / NW;
  auto go = [&](auto kern) { kern<<<(unsigned)blocks, 32 * NW, 0, st>>>(table, P, npairs, npts, pts, out, status, err); };
  switch (ppl) {
    case 1: go(k_lk_track<1, NW>); break;
    case 2: go(k_lk_track<2, NW>); break;
    case 3: go(k_lk_track<3, NW>); break;
    case 4: go(k_lk_track<4, NW>); break;
    case 5: case 6: go(k_lk_track<6, NW>); break;
    default: go(k_lk_track<8, NW>); break;
  }
}

inline void launch_lk(const Level* table, const Params& P, const gbt_lk_params* prm, int npairs, int npts,
                      const float* pts, float* out, int* status, float* err, cudaStream_t st) {
  const int ppl = (prm->window * prm->window + 31) / 32;
  if (prm->warps_per_block == 2)
    launch_lk_nw<2>(table, P, ppl, npairs, npts, pts, out, status, err, st);
  else if (prm->warps_per_block == 4)
    launch_lk_nw<4>(table, P, ppl, npairs, npts, pts, out, status, err, st);
  else
    launch_lk_nw<8>(table, P, ppl, npairs, npts, pts, out, status, err, st);
}

// Level images (fp32) of a uint8 frame: level 0 converted, then 2x2 floor means.
__global__ void k_u8_to_f32(const uint8_t* __restrict__ in, long long pitch, long long img_bytes, int H, int W,
                            float* __restrict__ out, long long out_img) {
  const int pair = blockIdx.y;
  const uint8_t* src = in + pair * img_bytes;
  float* dst = out + pair * out_img;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < H * W; t += gridDim.x * blockDim.x)
    dst[t] = (float)src[(size_t)(t / W) * pitch + t % W];
}

__global__ void k_box_f32(const float* __restrict__ in, int H, int W, long long in_img, float* __restrict__ out,
                          long long out_img) {
  const int pair = blockIdx.y;
  const int H2 = H / 2, W2 = W / 2;
  const float* a = in + pair * in_img;
  float* o = out + pair * out_img;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < H2 * W2; t += gridDim.x * blockDim.x) {
    int r = t / W2, c = t % W2;
    int s = (int)a[(size_t)(2 * r) * W + 2 * c] + (int)a[(size_t)(2 * r) * W + 2 * c + 1] +
            (int)a[(size_t)(2 * r + 1) * W + 2 * c] + (int)a[(size_t)(2 * r + 1) * W + 2 * c + 1];
    o[t] = (float)(s / 4);
  }
}

// Sobel/8 of the previous level over domain - border(1), zero on the ring
// (pyrlk_cpu::match_particles, pyrlk_tracker.hpp:910-938).
__global__ void k_sobel8(const float* __restrict__ in, int H, int W, long long in_img, float2* __restrict__ out,
                         long long out_img) {
  const int pair = blockIdx.y;
  const float* a = in + pair * in_img;
  float2* o = out + pair * out_img;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < H * W; t += gridDim.x * blockDim.x) {
    int r = t / W, c = t % W;
    float2 g = make_float2(0.f, 0.f);
    if (r >= 1 && r < H - 1 && c >= 1 && c < W - 1) {
#define P(dr, dc) a[(size_t)(r + (dr)) * W + (c + (dc))]
      g.x = (P(1, -1) + 2 * P(1, 0) + P(1, 1) - P(-1, -1) - 2 * P(-1, 0) - P(-1, 1)) / 8.f;
      g.y = (P(-1, 1) + 2 * P(0, 1) + P(1, 1) - P(-1, -1) - 2 * P(0, -1) - P(1, -1)) / 8.f;
#undef P
    }
    o[t] = g;
  }
}

}  // namespace gbt_lk

using namespace gbt_lk;

extern "C" int gbt_gaussian_pyramid_f32(const float* in, int64_t in_pitch, int32_t rows, int32_t cols, int32_t nlevels,
                                        float* out, void* stream);

extern "C" void gbt_lk_params_default(gbt_lk_params* p) {
  p->window = 11;
  p->npix = 25;
  p->max_iter = 30;
  p->eps = 0.1f;
  p->max_err = 300.f;
  p->warps_per_block = 0;
}

// Bytes of scratch gbt_lk_track_batch needs for `npairs` pairs.
extern "C" int64_t gbt_lk_scratch_bytes(int32_t rows, int32_t cols, int32_t nlevels, int32_t npairs) {
  if (rows < 1 || cols < 1 || nlevels < 1 || npairs < 1) return -1;
  int64_t px = 0;
  int h = rows, w = cols;
  for (int l = 0; l < nlevels; l++) {
    px += (int64_t)h * w;
    h /= 2;
    w /= 2;
  }
  // prev + cur (fp32) + gradient (float2) per pixel, plus the level table.
  return px * npairs * 16 + (int64_t)npairs * nlevels * sizeof(Level) + 1024;
}

static int lk_run(const void* prev, const void* cur, int64_t pitch, int64_t img_bytes, int rows, int cols, int is_u8,
                  int nlevels, const gbt_lk_params* prm, int npairs, const float* pts, int npts, float* out,
                  int* status, float* err, void* scratch, int64_t scratch_bytes, cudaStream_t st) {
  if (!prev || !cur || !prm || !scratch) return GBT_E_INVALID;
  if (npts > 0 && (!pts || !out || !status || !err)) return GBT_E_INVALID;
  if (rows < 16 || cols < 16 || nlevels < 1 || npairs < 1 || npts < 0) return GBT_E_INVALID;
  if (prm->window < 3 || prm->window > MAXW || !(prm->window & 1) || prm->npix < 1 || prm->max_iter < 0 ||
      (prm->warps_per_block != 0 && prm->warps_per_block != 2 && prm->warps_per_block != 4 && prm->warps_per_block != 8))
    return GBT_E_INVALID;
  if ((rows >> (nlevels - 1)) < 8 || (cols >> (nlevels - 1)) < 8) return GBT_E_INVALID;
  if (scratch_bytes < gbt_lk_scratch_bytes(rows, cols, nlevels, npairs)) return GBT_E_INVALID;
  // Arena: [prev levels][cur levels][grad levels][level table]; each level
  // block holds all pairs back to back.
  std::vector<int> H(nlevels), W(nlevels);
  std::vector<int64_t> off(nlevels);
  int64_t px = 0;
  for (int l = 0, h = rows, w = cols; l < nlevels; l++, h /= 2, w /= 2) {
    H[l] = h;
    W[l] = w;
    off[l] = px;
    px += (int64_t)h * w * npairs;
  }
  char* base = (char*)scratch;
  float* P0 = (float*)base;
  float* C0 = P0 + px;
  float2* G0 = (float2*)(C0 + px);
  Level* table = (Level*)(G0 + px);
  std::vector<Level> h_table((size_t)npairs * nlevels);
  dim3 blk(256);
  for (int which = 0; which < 2; which++) {
    float* dst = which ? C0 : P0;
    const void* src = which ? cur : prev;
    if (is_u8) {
      k_u8_to_f32<<<dim3(64, npairs), blk, 0, st>>>((const uint8_t*)src, pitch, img_bytes, rows, cols, dst,
                                                     (long long)rows * cols);
      for (int l = 1; l < nlevels; l++)
        k_box_f32<<<dim3(64, npairs), blk, 0, st>>>(dst + off[l - 1], H[l - 1], W[l - 1],
                                                    (long long)H[l - 1] * W[l - 1], dst + off[l],
                                                    (long long)H[l] * W[l]);
    } else {
      for (int p = 0; p < npairs; p++) {
        const float* s = (const float*)((const char*)src + p * img_bytes);
        cudaMemcpy2DAsync(dst + (int64_t)p * rows * cols, (size_t)cols * 4, s, pitch, (size_t)cols * 4, rows,
                          cudaMemcpyDeviceToDevice, st);
      }
      if (nlevels > 1) {
        // Gaussian pyramid per pair, one level at a time into its level block.
        for (int p = 0; p < npairs; p++) {
          const float* s = dst + (int64_t)p * rows * cols;
          std::vector<float*> lvl(nlevels);
          for (int l = 1; l < nlevels; l++) lvl[l] = dst + off[l] + (int64_t)p * H[l] * W[l];
          // gbt_gaussian_pyramid_f32 writes dense levels back to back; run it
          // level by level so each lands in its own block.
          const float* src_l = s;
          int64_t sp = (int64_t)cols * 4;
          for (int l = 1; l < nlevels; l++) {
            int r = gbt_gaussian_pyramid_f32(src_l, sp, H[l - 1], W[l - 1], 2, lvl[l], st);
            if (r) return r;
            src_l = lvl[l];
            sp = (int64_t)W[l] * 4;
          }
        }
      }
    }
  }
  for (int l = 0; l < nlevels; l++)
    gbt_lk::k_sobel8<<<dim3(64, npairs), blk, 0, st>>>(P0 + off[l], H[l], W[l], (long long)H[l] * W[l], G0 + off[l],
                                                       (long long)H[l] * W[l]);
  for (int p = 0; p < npairs; p++)
    for (int l = 0; l < nlevels; l++) {
      Level& L = h_table[(size_t)p * nlevels + l];
      L.H = H[l];
      L.W = W[l];
      L.prev = P0 + off[l] + (int64_t)p * H[l] * W[l];
      L.cur = C0 + off[l] + (int64_t)p * H[l] * W[l];
      L.grad = G0 + off[l] + (int64_t)p * H[l] * W[l];
    }
  cudaMemcpyAsync(table, h_table.data(), h_table.size() * sizeof(Level), cudaMemcpyHostToDevice, st);
  Params P{prm->window, prm->npix, prm->max_iter, nlevels, prm->eps, prm->max_err, is_u8};
  long long total = (long long)npairs * npts;
  if (total > 0) {
    launch_lk(table, P, prm, npairs, npts, pts, out, status, err, st);
  }
  // The host table must outlive the asynchronous copy.
  cudaStreamSynchronize(st);
  return cudaGetLastError() == cudaSuccess ? GBT_OK : GBT_E_CUDA;
}

// Scratch cache of the allocating entry point (one arena per device, grown on
// demand, released at exit).
static std::mutex g_scratch_mu;
static std::vector<std::pair<void*, int64_t>> g_scratch;

extern "C" int gbt_lk_track_batch(const void* prev, const void* cur, int64_t pitch, int64_t img_bytes, int32_t rows,
                                  int32_t cols, int32_t is_u8, int32_t nlevels, const gbt_lk_params* params,
                                  int32_t npairs, const float* pts, int32_t npts, float* out, int32_t* status,
                                  float* err, void* stream) {
  int64_t need = gbt_lk_scratch_bytes(rows, cols, nlevels, npairs);
  if (need < 0) return GBT_E_INVALID;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GBT_E_CUDA;
  void* arena = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if ((int)g_scratch.size() <= dev) g_scratch.resize(dev + 1, {nullptr, 0});
    if (g_scratch[dev].second < need) {
      if (g_scratch[dev].first) {
        cudaStreamSynchronize((cudaStream_t)stream);
        cudaFree(g_scratch[dev].first);
      }
      g_scratch[dev] = {nullptr, 0};
      if (cudaMalloc(&g_scratch[dev].first, need) != cudaSuccess) return GBT_E_OOM;
      g_scratch[dev].second = need;
    }
    arena = g_scratch[dev].first;
  }
  return lk_run(prev, cur, pitch, img_bytes, rows, cols, is_u8, nlevels, params, npairs, pts, npts, out, status, err,
                arena, need, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// Allocation-free variant of gbt_lk_track_batch.
//
// For callers that cannot allocate device memory themselves -- code running
// under an allocator they do not own (a host application with its own device
// pool or a strict memory budget, a plugin that must not touch the CUDA heap,
// a context where cudaMalloc would synchronise or fail) -- this entry point
// uses a fixed scratch arena that lives in this file as a static device
// array.  The array is part of the library's device image: every GPU that
// loads this library holds NOALLOC_SCRATCH_BYTES of it until the process
// exits, whether or not the entry point is called.  The caller still passes
// frames, points and outputs.
//
// Set-up: the first call on a device, with that device current, looks up the
// array's device address once (cudaGetSymbolAddress) and caches it for that
// device's context; a context re-created after cudaDeviceReset gets its own
// lookup on its first call.  Make those first calls before capturing any
// stream into a CUDA graph.  Every call shares
// the one arena and overwrites it completely (levels, gradients, level table),
// so nothing needs clearing between calls -- but calls whose GPU work overlaps
// (different streams or host threads without ordering) race on it.
constexpr int64_t NOALLOC_SCRATCH_BYTES = 48ll << 20;  // 48 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

namespace gbt_lk {

constexpr int NOALLOC_MAX_LEVELS = 9;
constexpr int NOALLOC_MAX_DEVICES = 64;

struct TableArgs {
  int H[NOALLOC_MAX_LEVELS], W[NOALLOC_MAX_LEVELS];
  long long off[NOALLOC_MAX_LEVELS];
};

// Fills the per-(pair, level) table on the device (no host staging buffer).
__global__ void k_fill_table(Level* table, int npairs, int nlevels, const float* P0, const float* C0,
                             const float2* G0, TableArgs a) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npairs * nlevels) return;
  int p = t / nlevels, l = t % nlevels;
  long long o = a.off[l] + (long long)p * a.H[l] * a.W[l];
  Level L;
  L.H = a.H[l];
  L.W = a.W[l];
  L.prev = P0 + o;
  L.cur = C0 + o;
  L.grad = G0 + o;
  table[t] = L;
}

}  // namespace gbt_lk

// The array's address is valid for one CUDA context: a device whose context
// is destroyed and re-created (cudaDeviceReset) loads the library's device
// image again, so the cache is keyed on the context's unique id, read through
// the runtime's driver entry points (the library does not link the driver
// API).  0 when no context is current or the entry points are unavailable.
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

static unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (CtxGetCurrentFn)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (CtxGetIdFn)f;
    cudaGetLastError();
  });
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[NOALLOC_MAX_DEVICES];
static unsigned long long g_noalloc_ctx[NOALLOC_MAX_DEVICES];

extern "C" int64_t gbt_lk_noalloc_max_bytes(void) { return NOALLOC_SCRATCH_BYTES; }

extern "C" int gbt_lk_track_batch_noalloc(const void* prev, const void* cur, int64_t pitch, int64_t img_bytes,
                                          int32_t rows, int32_t cols, int32_t is_u8, int32_t nlevels,
                                          const gbt_lk_params* prm, int32_t npairs, const float* pts, int32_t npts,
                                          float* out, int32_t* status, float* err, void* stream) {
  if (!prev || !cur || !prm) return GBT_E_INVALID;
  if (npts > 0 && (!pts || !out || !status || !err)) return GBT_E_INVALID;
  if (rows < 16 || cols < 16 || nlevels < 1 || nlevels > NOALLOC_MAX_LEVELS || npairs < 1 || npts < 0)
    return GBT_E_INVALID;
  if (prm->window < 3 || prm->window > MAXW || !(prm->window & 1) || prm->npix < 1 || prm->max_iter < 0 ||
      (prm->warps_per_block != 0 && prm->warps_per_block != 2 && prm->warps_per_block != 4 && prm->warps_per_block != 8))
    return GBT_E_INVALID;
  if ((rows >> (nlevels - 1)) < 8 || (cols >> (nlevels - 1)) < 8) return GBT_E_INVALID;
  const int64_t need = gbt_lk_scratch_bytes(rows, cols, nlevels, npairs);
  if (need < 0) return GBT_E_INVALID;
  if (need > NOALLOC_SCRATCH_BYTES) return GBT_E_TOO_LARGE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES) return GBT_E_CUDA;
  void* arena = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    const unsigned long long ctx_id = current_context_id();
    if (!g_noalloc_ptr[dev] || ctx_id == 0 || ctx_id != g_noalloc_ctx[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
        g_noalloc_ptr[dev] = nullptr;
        return GBT_E_CUDA;
      }
      g_noalloc_ptr[dev] = p;
      g_noalloc_ctx[dev] = current_context_id();  // the lookup made the context current if none was
    }
    arena = g_noalloc_ptr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  TableArgs a{};
  int64_t px = 0;
  for (int l = 0, h = rows, w = cols; l < nlevels; l++, h /= 2, w /= 2) {
    a.H[l] = h;
    a.W[l] = w;
    a.off[l] = px;
    px += (int64_t)h * w * npairs;
  }
  float* P0 = (float*)arena;
  float* C0 = P0 + px;
  float2* G0 = (float2*)(C0 + px);
  Level* table = (Level*)(G0 + px);
  dim3 blk(256);
  for (int which = 0; which < 2; which++) {
    float* dst = which ? C0 : P0;
    const void* src = which ? cur : prev;
    if (is_u8) {
      k_u8_to_f32<<<dim3(64, npairs), blk, 0, st>>>((const uint8_t*)src, pitch, img_bytes, rows, cols, dst,
                                                     (long long)rows * cols);
      for (int l = 1; l < nlevels; l++)
        k_box_f32<<<dim3(64, npairs), blk, 0, st>>>(dst + a.off[l - 1], a.H[l - 1], a.W[l - 1],
                                                    (long long)a.H[l - 1] * a.W[l - 1], dst + a.off[l],
                                                    (long long)a.H[l] * a.W[l]);
    } else {
      for (int p = 0; p < npairs; p++) {
        const float* s = (const float*)((const char*)src + p * img_bytes);
        if (cudaMemcpy2DAsync(dst + (int64_t)p * rows * cols, (size_t)cols * 4, s, pitch, (size_t)cols * 4, rows,
                              cudaMemcpyDeviceToDevice, st) != cudaSuccess)
          return GBT_E_CUDA;
        const float* src_l = dst + (int64_t)p * rows * cols;
        int64_t sp = (int64_t)cols * 4;
        for (int l = 1; l < nlevels; l++) {
          float* lvl = dst + a.off[l] + (int64_t)p * a.H[l] * a.W[l];
          int r = gbt_gaussian_pyramid_f32(src_l, sp, a.H[l - 1], a.W[l - 1], 2, lvl, st);
          if (r) return r;
          src_l = lvl;
          sp = (int64_t)a.W[l] * 4;
        }
      }
    }
  }
  for (int l = 0; l < nlevels; l++)
    k_sobel8<<<dim3(64, npairs), blk, 0, st>>>(P0 + a.off[l], a.H[l], a.W[l], (long long)a.H[l] * a.W[l],
                                               G0 + a.off[l], (long long)a.H[l] * a.W[l]);
  k_fill_table<<<(npairs * nlevels + 255) / 256, 256, 0, st>>>(table, npairs, nlevels, P0, C0, G0, a);
  Params P{prm->window, prm->npix, prm->max_iter, nlevels, prm->eps, prm->max_err, is_u8};
  long long total = (long long)npairs * npts;
  if (total > 0) {
    launch_lk(table, P, prm, npairs, npts, pts, out, status, err, st);
  }
  return cudaGetLastError() == cudaSuccess ? GBT_OK : GBT_E_CUDA;
}
