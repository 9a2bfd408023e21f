/*
 * CPU restatement of cuimg's separable Gaussian -- TEST INFRASTRUCTURE ONLY.
 *
 * Taps: meta_kernel<meta_gaussian<0, sigma>, x>::coef() values as written by
 * the reference's tap generator (tools/make_meta_gaussian/make_meta_gaussian.cpp:
 * gaussian_derivative<0> :11-16 evaluated through double-precision libm and
 * returned as float, printed with the stream's default 6 significant digits
 * :86-97, then read back as a float literal) for integer sigma in 1..50, and
 * gaussian_derivative<0>(float sigma, int x) from cuimg/gaussian_kernel.h:13-18
 * (single-precision sqrtf/expf) for any other sigma.  Taps are unnormalised,
 * as in the reference.  Radius R = ceil(3 sigma).
 *
 * Filter: meta_convolve_row2d then meta_convolve_col2d
 * (cuimg/gpu/meta_convolve.h:25-161,288-314), each output the right-recursive
 * sum term(-R) + (term(-R+1) + (... + term(R))) of the unrolled template, in
 * fp32, with clamp-to-edge sampling.  (The reference's host fallback skips a
 * border of R pixels and drops one tap, meta_convolve.h:183-206; the clamped
 * GPU form is the one restated here.)
 *
 * Gaussian pyramid option: blur with sigma = 1 (R = 3) and keep every second
 * pixel, out(p) = blur(2p), the form of the disabled pyramid code in
 * cuimg/gpu/mipmap.h:94-108,229-246.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#define ORACLE_PI_F 3.14159265f /* CUIMG_PI, cuimg/util.h */

int oracle_gauss_radius(float sigma) { return (int)ceilf(3.f * sigma); }

/* Writes 2R+1 taps for x = -R..R; returns R. */
int oracle_gauss_taps(float sigma, float* taps) {
  int R = oracle_gauss_radius(sigma);
  int is_int = sigma >= 1.f && sigma <= 50.f && floorf(sigma) == sigma;
  for (int x = -R; x <= R; x++) {
    float v;
    if (is_int) {
      double pi = (double)ORACLE_PI_F;
      double s = (double)sigma;
      /* -(x*x) / (2*sigma*sigma) is an int / float division: float precision. */
      float e = (float)(-(x * x)) / (2.f * sigma * sigma);
      float res = (float)((1.0 / (sqrt(2.0 * pi) * s)) * exp((double)e));
      char buf[64];
      snprintf(buf, sizeof buf, "%.6g", (double)res);
      v = strtof(buf, NULL);
    } else {
      v = (1.f / (sqrtf(2.f * ORACLE_PI_F) * sigma)) * expf(-(float)(x * x) / (2.f * sigma * sigma));
    }
    taps[x + R] = v;
  }
  return R;
}

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* Row pass then column pass, clamp-to-edge; `tmp` holds H*W floats. */
void oracle_gauss_sep_f32(const float* in, int H, int W, const float* taps, int R, float* tmp, float* out) {
  for (int r = 0; r < H; r++)
    for (int c = 0; c < W; c++) {
      float acc = in[(size_t)r * W + clampi(c + R, 0, W - 1)] * taps[2 * R];
      for (int x = R - 1; x >= -R; x--) acc = in[(size_t)r * W + clampi(c + x, 0, W - 1)] * taps[x + R] + acc;
      tmp[(size_t)r * W + c] = acc;
    }
  for (int r = 0; r < H; r++)
    for (int c = 0; c < W; c++) {
      float acc = tmp[(size_t)clampi(r + R, 0, H - 1) * W + c] * taps[2 * R];
      for (int y = R - 1; y >= -R; y--) acc = tmp[(size_t)clampi(r + y, 0, H - 1) * W + c] * taps[y + R] + acc;
      out[(size_t)r * W + c] = acc;
    }
}

/* Gaussian pyramid (sigma 1, then keep every second pixel): writes levels
 * 1..L-1 back to back into `out` (level l has (H>>l) x (W>>l) pixels, the
 * tracker's truncating halving).  `tmp` and `blur` hold H*W floats each. */
void oracle_gauss_pyramid_f32(const float* in, int H, int W, int L, float* tmp, float* blur, float* work,
                              float* out) {
  float taps[7];
  int R = oracle_gauss_taps(1.f, taps);
  const float* src = in;
  int h = H, w = W;
  float* dst = out;
  for (int l = 1; l < L; l++) {
    oracle_gauss_sep_f32(src, h, w, taps, R, tmp, blur);
    int h2 = h / 2, w2 = w / 2;
    for (int r = 0; r < h2; r++)
      for (int c = 0; c < w2; c++) work[(size_t)r * w2 + c] = blur[(size_t)(2 * r) * w + 2 * c];
    for (size_t i = 0; i < (size_t)h2 * w2; i++) dst[i] = work[i];
    src = dst;
    dst += (size_t)h2 * w2;
    h = h2;
    w = w2;
  }
}
