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
// fused in one kernel: a CTA stages a (32 + 2R) x (64 + 2R) input tile in shared
// memory, runs the row pass into a second shared tile and the column pass into
// registers, so each image is read from and written to HBM once (8 B/pixel).
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
  const int tiles = ((rows + TR - 1) / TR) * ((cols + TC - 1) / TC);
  dim3 grid(tiles, nimg);
  size_t sm = (size_t)((TR + 2 * R) * (TC + 2 * R + 1) + (TR + 2 * R) * (TC + 1)) * sizeof(float);
  auto go = [&](auto kern) {
    if (sm > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kern<<<grid, 256, sm, st>>>(in, in_pitch, in_img, out, out_pitch, out_img, rows, cols, tiles, t, R);
  };
  switch (R) {
    case 2: go(k_gauss<2>); break;
    case 3: go(k_gauss<3>); break;
    case 6: go(k_gauss<6>); break;
    case 12: go(k_gauss<12>); break;
    default: go(k_gauss<0>); break;
  }
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
