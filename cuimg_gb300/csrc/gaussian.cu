// Separable fp32 Gaussian, Gaussian pyramid and uint8 box pyramid for sm_103a.
//
// Taps (host): for integer sigma in 1..50 the values of the reference's
// generated meta_kernel<meta_gaussian<0, sigma>, x>::coef() tables
// (tools/make_meta_gaussian/make_meta_gaussian.cpp:11-16,63-105: the normal
// density evaluated in double precision, returned as float and printed with
// six significant digits), reproduced here by evaluating the same density and
// rounding it to six significant digits; for any other sigma the float
// gaussian_derivative<0> of cuimg/gaussian_kernel.h:13-18.  Radius
// R = ceil(3 sigma); taps are not normalised (the reference never normalises).
//
// Filter: row pass then column pass (meta_convolve_row2d / col2d,
// cuimg/gpu/meta_convolve.h:131-161,288-314) with clamp-to-edge sampling,
// fused in one kernel so each image is read from and written to HBM once
// (8 B/pixel).  k_gauss_strip (radius 2, 3, 6, 9, 12): a CTA walks down a
// 128-column strip, 16 input rows at a time; cp.async stages the next rows in
// shared memory while the row pass computes four adjacent outputs per thread
// from 16-byte shared loads, and each thread runs the column pass of its own
// column from a register window of the last 2R + 1 row-pass values, so the
// column pass reads no shared memory at all.  k_gauss (any other radius) is
// the plain tile version: (32 + 2R) x (64 + 2R) input tile, row pass into a
// second shared tile, column pass from it.  Both accumulate the taps in the
// same order (x, then y, ascending from -R) and give the same bits.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "cuimg_gb300.h"

namespace gbt_gauss {

constexpr int TR = 32, TC = 64, MAXR = 24;

struct Taps {
  float w[2 * MAXR + 1];
};

// Shared tile: rows x cols floats with cols padded to avoid bank conflicts.
template <int R>
__global__ void __launch_bounds__(256) k_gauss(const float* __restrict__ in, long long in_pitch, long long in_img,
                                               float* __restrict__ out, long long out_pitch, long long out_img, int H,
                                               int W, int rt, Taps taps, int Rrt) {
  const int RR = R > 0 ? R : Rrt;
  extern __shared__ float smem[];
  const int LW = TC + 2 * RR + 1;          // input tile row length (padded)
  float* tin = smem;                       // (TR + 2R) x LW
  float* trow = smem + (TR + 2 * RR) * LW; // (TR + 2R) x (TC + 1)
  const int img = blockIdx.y;
  const float* src = (const float*)((const char*)in + img * in_img);
  float* dst = (float*)((char*)out + img * out_img);
  const int tcols = (W + TC - 1) / TC;
  const int R0 = (blockIdx.x / tcols) * TR, C0 = (blockIdx.x % tcols) * TC;
  if (R0 >= H) return;
  // Stage the clamped input tile.
  const int nrow = TR + 2 * RR, ncol = TC + 2 * RR;
  for (int v = threadIdx.x; v < nrow * ncol; v += blockDim.x) {
    int r = v / ncol, c = v % ncol;
    int gr = min(max(R0 - RR + r, 0), H - 1), gc = min(max(C0 - RR + c, 0), W - 1);
    tin[r * LW + c] = __ldg((const float*)((const char*)src + gr * in_pitch) + gc);
  }
  __syncthreads();
  // Row pass: taps from -R to R.
  for (int v = threadIdx.x; v < nrow * TC; v += blockDim.x) {
    int r = v / TC, c = v % TC;
    const float* p = tin + r * LW + c;
    float acc = 0.f;
    if (R > 0) {
#pragma unroll
      for (int x = 0; x <= 2 * R; x++) acc = fmaf(p[x], taps.w[x], acc);
    } else {
      for (int x = 0; x <= 2 * RR; x++) acc = fmaf(p[x], taps.w[x], acc);
    }
    trow[r * (TC + 1) + c] = acc;
  }
  __syncthreads();
  // Column pass and store.
  for (int v = threadIdx.x; v < TR * TC; v += blockDim.x) {
    int r = v / TC, c = v % TC;
    int gr = R0 + r, gc = C0 + c;
    if (gr >= H || gc >= W) continue;
    const float* p = trow + r * (TC + 1) + c;
    float acc = 0.f;
    if (R > 0) {
#pragma unroll
      for (int y = 0; y <= 2 * R; y++) acc = fmaf(p[y * (TC + 1)], taps.w[y], acc);
    } else {
      for (int y = 0; y <= 2 * RR; y++) acc = fmaf(p[y * (TC + 1)], taps.w[y], acc);
    }
    ((float*)((char*)dst + gr * out_pitch))[gc] = acc;
  }
}

__device__ __forceinline__ void cp_async4(void* sdst, const void* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

constexpr int SC = 128;  // strip width = threads per CTA
constexpr int RB = 16;   // input rows per batch

// Grid (strips, row segments, images); a segment is `SR` output rows, which
// need SR + 2R input rows (clamped at the image edges).  The staged row holds
// image columns C0 - RA .. C0 + SC + RA - 1 with RA = R rounded up to a
// multiple of 4, so interior strips of a 16-byte aligned image are staged with
// 16-byte copies; edge strips (and unaligned images) copy clamped floats.
template <int R>
__global__ void __launch_bounds__(SC) k_gauss_strip(const float* __restrict__ in, long long in_pitch, long long in_img,
                                                    float* __restrict__ out, long long out_pitch, long long out_img,
                                                    int H, int W, int SR, Taps taps) {
  constexpr int NW = 2 * R + 1;              // taps
  constexpr int RA = (R + 3) / 4 * 4;        // staged halo
  constexpr int OFF = RA - R;                // staged index of column C0 - R
  constexpr int LW = SC + 2 * RA;            // staged row length (16-byte multiple)
  constexpr int CH = LW / 4;                 // 16-byte chunks per staged row
  constexpr int NV = (OFF + 3 + 2 * R) / 4 + 1;  // float4 reads per quad of row-pass outputs
  static_assert(4 * (SC / 4 - 1) + 4 * NV <= LW, "row pass reads stay inside the staged row");
  __shared__ __align__(16) float tin[2][RB][LW];
  __shared__ __align__(16) float th[RB][SC];
  const float* src = (const float*)((const char*)in + blockIdx.z * in_img);
  float* dst = (float*)((char*)out + blockIdx.z * out_img);
  const int t = threadIdx.x;
  const int C0 = blockIdx.x * SC, R0 = blockIdx.y * SR;
  const int nout = min(SR, H - R0);
  const int nin = nout + 2 * R;  // segment input row k is image row R0 - R + k
  const int nb = (nin + RB - 1) / RB;
  const bool vec = ((((unsigned long long)src) | (unsigned long long)in_pitch) & 15) == 0 && C0 - RA >= 0 &&
                   C0 + SC + RA <= W;

  auto issue = [&](int b) {
    float(*buf)[LW] = tin[b & 1];
    if (vec) {
      for (int v = t; v < RB * CH; v += SC) {
        const int i = v / CH, ch = v % CH;
        const int gr = min(max(R0 - R + b * RB + i, 0), H - 1);
        cp_async16(&buf[i][4 * ch], (const float*)((const char*)src + gr * in_pitch) + C0 - RA + 4 * ch);
      }
    } else {
#pragma unroll 4
      for (int i = 0; i < RB; i++) {
        const int gr = min(max(R0 - R + b * RB + i, 0), H - 1);
        const float* row = (const float*)((const char*)src + gr * in_pitch);
        for (int c = t; c < LW; c += SC) cp_async4(&buf[i][c], row + min(max(C0 - RA + c, 0), W - 1));
      }
    }
    cp_async_commit();
  };

  float win[NW];  // win[NW - 1] is the newest row-pass value of this thread's column
#pragma unroll
  for (int y = 0; y < NW; y++) win[y] = 0.f;
  issue(0);
  for (int b = 0; b < nb; b++) {
    if (b + 1 < nb) {
      issue(b + 1);  // into the buffer whose row pass finished before the last barrier
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    // Row pass: RB rows x 32 quads, four outputs per quad.
#pragma unroll
    for (int it = 0; it < RB * (SC / 4) / SC; it++) {
      const int item = t + it * SC, i = item / (SC / 4), q = item % (SC / 4);
      const float4* p4 = reinterpret_cast<const float4*>(&tin[b & 1][i][4 * q]);
      float v[4 * NV];
#pragma unroll
      for (int k = 0; k < NV; k++) {
        const float4 f = p4[k];
        v[4 * k] = f.x;
        v[4 * k + 1] = f.y;
        v[4 * k + 2] = f.z;
        v[4 * k + 3] = f.w;
      }
      float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll
      for (int x = 0; x < NW; x++) {
        a0 = fmaf(v[OFF + x], taps.w[x], a0);
        a1 = fmaf(v[OFF + x + 1], taps.w[x], a1);
        a2 = fmaf(v[OFF + x + 2], taps.w[x], a2);
        a3 = fmaf(v[OFF + x + 3], taps.w[x], a3);
      }
      *reinterpret_cast<float4*>(&th[i][4 * q]) = make_float4(a0, a1, a2, a3);
    }
    __syncthreads();
    // Column pass from the register window.  The shift is unconditional (rows
    // past the segment are clamped copies and only skip their store), so the
    // unrolled batch renames registers instead of moving them.
    // Rows i in [lo, hi) of this batch complete an output row.
    const int lo = max(0, 2 * R - b * RB), hi = C0 + t < W ? min(RB, nin - b * RB) : 0;
    char* orow = (char*)(dst + C0 + t) + (long long)(R0 - 2 * R + b * RB) * out_pitch;
#pragma unroll
    for (int i = 0; i < RB; i++) {
#pragma unroll
      for (int y = 0; y < NW - 1; y++) win[y] = win[y + 1];
      win[NW - 1] = th[i][t];
      if (i >= lo) {
        float acc = 0.f;
#pragma unroll
        for (int y = 0; y < NW; y++) acc = fmaf(win[y], taps.w[y], acc);
        if (i < hi) *(float*)orow = acc;
      }
      orow += out_pitch;
    }
  }
}

// Gaussian pyramid level: out(r, c) = blur_sigma1(in)(2r, 2c), clamped.
__global__ void __launch_bounds__(256) k_gauss_decimate(const float* __restrict__ in, long long in_pitch, int H, int W,
                                                        float* __restrict__ out, int H2, int W2, Taps taps) {
  const int R = 3;
  __shared__ float tin[2 * 16 + 2 * R + 1][2 * 32 + 2 * R + 1];
  __shared__ float trow[2 * 16 + 2 * R + 1][32 + 1];
  const int tcols = (W2 + 31) / 32;
  const int r0 = (blockIdx.x / tcols) * 16, c0 = (blockIdx.x % tcols) * 32;
  const int gr0 = 2 * r0 - R, gc0 = 2 * c0 - R;
  const int nrow = 2 * 16 + 2 * R, ncol = 2 * 32 + 2 * R;
  for (int v = threadIdx.x; v < nrow * ncol; v += blockDim.x) {
    int r = v / ncol, c = v % ncol;
    int gr = min(max(gr0 + r, 0), H - 1), gc = min(max(gc0 + c, 0), W - 1);
    tin[r][c] = ((const float*)((const char*)in + gr * in_pitch))[gc];
  }
  __syncthreads();
  for (int v = threadIdx.x; v < nrow * 32; v += blockDim.x) {
    int r = v / 32, c = v % 32;
    float acc = 0.f;
#pragma unroll
    for (int x = 0; x <= 2 * R; x++) acc = fmaf(tin[r][2 * c + x], taps.w[x], acc);
    trow[r][c] = acc;
  }
  __syncthreads();
  for (int v = threadIdx.x; v < 16 * 32; v += blockDim.x) {
    int r = v / 32, c = v % 32;
    if (r0 + r >= H2 || c0 + c >= W2) continue;
    float acc = 0.f;
#pragma unroll
    for (int y = 0; y <= 2 * R; y++) acc = fmaf(trow[2 * r + y][c], taps.w[y], acc);
    out[(size_t)(r0 + r) * W2 + c0 + c] = acc;
  }
}

// 2x2 floor-mean level (mipmap_kernel, cuimg/gpu/mipmap.h:24-49).
__global__ void k_box_u8(const uint8_t* __restrict__ in, long long in_pitch, uint8_t* __restrict__ out, int H2,
                         int W2) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= H2 * W2) return;
  int r = t / W2, c = t % W2;
  const uint8_t* a = in + (size_t)(2 * r) * in_pitch + 2 * c;
  int v = a[0] + a[1] + a[in_pitch] + a[in_pitch + 1];
  out[t] = (uint8_t)(v >> 2);
}

}  // namespace gbt_gauss

using namespace gbt_gauss;

extern "C" int gbt_gaussian_taps(float sigma, float* taps, int32_t* radius) {
  if (!(sigma > 0.f) || !taps || !radius) return GBT_E_INVALID;
  const int R = (int)ceilf(3.f * sigma);
  if (R > MAXR) return GBT_E_INVALID;
  const bool is_int = sigma >= 1.f && sigma <= 50.f && floorf(sigma) == sigma;
  const float pi_f = 3.14159265f;  // CUIMG_PI
  for (int x = -R; x <= R; x++) {
    float v;
    if (is_int) {
      double s = sigma, pi = pi_f;
      // -(x*x) / (2*sigma*sigma) is an int / float division: float precision.
      float e = (float)(-(x * x)) / (2.f * sigma * sigma);
      float res = (float)((1.0 / (sqrt(2.0 * pi) * s)) * exp((double)e));
      char buf[32];
      snprintf(buf, sizeof buf, "%.6g", (double)res);
      v = strtof(buf, nullptr);
    } else {
      v = (1.f / (sqrtf(2.f * pi_f) * sigma)) * expf(-(float)(x * x) / (2.f * sigma * sigma));
    }
    taps[x + R] = v;
  }
  *radius = R;
  return GBT_OK;
}

static int launch_gauss(const float* in, long long in_pitch, long long in_img, float* out, long long out_pitch,
                        long long out_img, int rows, int cols, int nimg, float sigma, cudaStream_t st) {
  Taps t{};
  int R;
  int r = gbt_gaussian_taps(sigma, t.w, &R);
  if (r) return r;
  auto strip = [&](auto kern) {
    // Segments per strip: minimise (waves of CTAs) x (rows a CTA stages), so
    // that the last wave is not a sliver and the halo rows stay a small share.
    static int sms = 0, per_sm[32] = {};
    if (!sms) {
      int dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    if (!per_sm[R]) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[R], kern, SC, 0);
    const long long slots = (long long)(sms > 0 ? sms : 152) * (per_sm[R] > 0 ? per_sm[R] : 1);
    const long long M = (long long)((cols + SC - 1) / SC) * nimg;
    int best_s = 1;
    long long best = -1;
    for (int sg = 1; sg <= (rows + 15) / 16; sg++) {
      const int SR = (rows + sg - 1) / sg;
      if (sg > 1 && (rows + SR - 1) / SR != sg) continue;
      const long long cost = ((M * sg + slots - 1) / slots) * (long long)(SR + 2 * R);
      if (best < 0 || cost < best) best = cost, best_s = sg;
    }
    const int SR = (rows + best_s - 1) / best_s;
    dim3 g((cols + SC - 1) / SC, (rows + SR - 1) / SR, nimg);
    kern<<<g, SC, 0, st>>>(in, in_pitch, in_img, out, out_pitch, out_img, rows, cols, SR, t);
    return cudaGetLastError() == cudaSuccess ? GBT_OK : GBT_E_CUDA;
  };
  switch (R) {
    case 2: return strip(k_gauss_strip<2>);
    case 3: return strip(k_gauss_strip<3>);
    case 6: return strip(k_gauss_strip<6>);
    case 9: return strip(k_gauss_strip<9>);
    case 12: return strip(k_gauss_strip<12>);
    default: break;
  }
  const int tiles = ((rows + TR - 1) / TR) * ((cols + TC - 1) / TC);
  dim3 grid(tiles, nimg);
  size_t sm = (size_t)((TR + 2 * R) * (TC + 2 * R + 1) + (TR + 2 * R) * (TC + 1)) * sizeof(float);
  auto go = [&](auto kern) {
    if (sm > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kern<<<grid, 256, sm, st>>>(in, in_pitch, in_img, out, out_pitch, out_img, rows, cols, tiles, t, R);
  };
  go(k_gauss<0>);
  return cudaGetLastError() == cudaSuccess ? GBT_OK : GBT_E_CUDA;
}

extern "C" int gbt_gaussian_f32(const float* in, int64_t in_pitch, float* out, int64_t out_pitch, int32_t rows,
                                int32_t cols, float sigma, void* stream) {
  if (!in || !out || rows < 1 || cols < 1 || in_pitch < cols * 4 || out_pitch < cols * 4) return GBT_E_INVALID;
  return launch_gauss(in, in_pitch, 0, out, out_pitch, 0, rows, cols, 1, sigma, (cudaStream_t)stream);
}

// Batched variant: `nimg` images, image i at in + i * in_img_bytes.
extern "C" int gbt_gaussian_f32_batch(const float* in, int64_t in_pitch, int64_t in_img_bytes, float* out,
                                      int64_t out_pitch, int64_t out_img_bytes, int32_t rows, int32_t cols,
                                      int32_t nimg, float sigma, void* stream) {
  if (!in || !out || rows < 1 || cols < 1 || nimg < 1 || nimg > 65535 || in_pitch < cols * 4 || out_pitch < cols * 4)
    return GBT_E_INVALID;
  return launch_gauss(in, in_pitch, in_img_bytes, out, out_pitch, out_img_bytes, rows, cols, nimg, sigma,
                      (cudaStream_t)stream);
}

extern "C" int gbt_gaussian_pyramid_f32(const float* in, int64_t in_pitch, int32_t rows, int32_t cols,
                                        int32_t nlevels, float* out, void* stream) {
  if (!in || !out || rows < 2 || cols < 2 || nlevels < 2 || in_pitch < cols * 4) return GBT_E_INVALID;
  Taps t{};
  int R;
  gbt_gaussian_taps(1.f, t.w, &R);
  const float* src = in;
  long long sp = in_pitch;
  int h = rows, w = cols;
  float* dst = out;
  for (int l = 1; l < nlevels; l++) {
    int h2 = h / 2, w2 = w / 2;
    if (h2 < 1 || w2 < 1) return GBT_E_INVALID;
    int tiles = ((h2 + 15) / 16) * ((w2 + 31) / 32);
    k_gauss_decimate<<<tiles, 256, 0, (cudaStream_t)stream>>>(src, sp, h, w, dst, h2, w2, t);
    src = dst;
    sp = (long long)w2 * 4;
    dst += (size_t)h2 * w2;
    h = h2;
    w = w2;
  }
  return cudaGetLastError() == cudaSuccess ? GBT_OK : GBT_E_CUDA;
}

extern "C" int gbt_pyramid_u8(const uint8_t* in, int64_t in_pitch, int32_t rows, int32_t cols, int32_t nlevels,
                              uint8_t* out, void* stream) {
  if (!in || !out || rows < 2 || cols < 2 || nlevels < 2 || in_pitch < cols) return GBT_E_INVALID;
  const uint8_t* src = in;
  long long sp = in_pitch;
  int h = rows, w = cols;
  uint8_t* dst = out;
  for (int l = 1; l < nlevels; l++) {
    int h2 = h / 2, w2 = w / 2;
    if (h2 < 1 || w2 < 1) return GBT_E_INVALID;
    k_box_u8<<<(h2 * w2 + 255) / 256, 256, 0, (cudaStream_t)stream>>>(src, sp, dst, h2, w2);
    src = dst;
    sp = w2;
    dst += (size_t)h2 * w2;
    h = h2;
    w = w2;
  }
  return cudaGetLastError() == cudaSuccess ? GBT_OK : GBT_E_CUDA;
}
