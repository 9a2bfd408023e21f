/*
 * FP64 oracle for the differentiable pyramidal LK residual -- TEST INFRASTRUCTURE ONLY.
 *
 * The differentiable forward is the translational LK of
 * cuimg/tracking2/pyrlk_tracker.hpp:165-334 with its discrete parts removed:
 *   - both frames go through the sigma-1 Gaussian pyramid (blur with the
 *     generator's sigma-1 taps, clamp-to-edge, keep every second pixel: the
 *     disabled pyramid of cuimg/gpu/mipmap.h:94-108);
 *   - gradients are the Sobel/8 of the previous level (pyrlk_tracker.hpp:910-938),
 *     zero on the one-pixel ring;
 *   - every window pixel is used (no strongest-gradient mask), every level runs
 *     exactly `iters` Gauss-Newton steps (no early stop, no rejection);
 *   - coarse to fine: the top level starts from the initial flow u0 / 2^(L-1),
 *     every finer level from twice the coarser level's displacement
 *     (recursive_prediction, cuimg/tracking2/predictions.h:61-74);
 *   - bilinear sampling uses floor and clamps the four taps to the image.
 * Loss per point = sum over the level-0 window of
 * (A0(p + o) - B0(v + o))^2 at the final position v.
 *
 * The FP64 reference gradient is the central difference of this forward with
 * respect to every pixel of both frames and both components of u0.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

int oracle_gauss_taps(float sigma, float* taps);

typedef struct {
  int H, W;
  double *A, *B, *Sr, *Sc;
} dlev;

static double bil(const double* img, int H, int W, double y, double x) {
  double fy = floor(y), fx = floor(x);
  int y0 = (int)fy, x0 = (int)fx;
  double a = y - fy, b = x - fx;
  int y1 = y0 + 1, x1 = x0 + 1;
  y0 = y0 < 0 ? 0 : (y0 > H - 1 ? H - 1 : y0);
  y1 = y1 < 0 ? 0 : (y1 > H - 1 ? H - 1 : y1);
  x0 = x0 < 0 ? 0 : (x0 > W - 1 ? W - 1 : x0);
  x1 = x1 < 0 ? 0 : (x1 > W - 1 ? W - 1 : x1);
  return (1 - a) * (1 - b) * img[(size_t)y0 * W + x0] + a * (1 - b) * img[(size_t)y1 * W + x0] +
         (1 - a) * b * img[(size_t)y0 * W + x1] + a * b * img[(size_t)y1 * W + x1];
}

static void blur_decimate(const double* in, int H, int W, const double* w, int R, double* out, double* tmp) {
  for (int r = 0; r < H; r++)
    for (int c = 0; c < W; c++) {
      double acc = 0;
      for (int t = -R; t <= R; t++) {
        int cc = c + t;
        cc = cc < 0 ? 0 : (cc > W - 1 ? W - 1 : cc);
        acc += w[t + R] * in[(size_t)r * W + cc];
      }
      tmp[(size_t)r * W + c] = acc;
    }
  int H2 = H / 2, W2 = W / 2;
  for (int r = 0; r < H2; r++)
    for (int c = 0; c < W2; c++) {
      double acc = 0;
      for (int t = -R; t <= R; t++) {
        int rr = 2 * r + t;
        rr = rr < 0 ? 0 : (rr > H - 1 ? H - 1 : rr);
        acc += w[t + R] * tmp[(size_t)rr * W + 2 * c];
      }
      out[(size_t)r * W2 + c] = acc;
    }
}

static void sobel8(const double* a, int H, int W, double* gr, double* gc) {
  memset(gr, 0, sizeof(double) * H * W);
  memset(gc, 0, sizeof(double) * H * W);
  for (int r = 1; r < H - 1; r++)
    for (int c = 1; c < W - 1; c++) {
#define P(dr, dc) a[(size_t)(r + (dr)) * W + (c + (dc))]
      gr[(size_t)r * W + c] = (P(1, -1) + 2 * P(1, 0) + P(1, 1) - P(-1, -1) - 2 * P(-1, 0) - P(-1, 1)) / 8.0;
      gc[(size_t)r * W + c] = (P(-1, 1) + 2 * P(0, 1) + P(1, 1) - P(-1, -1) - 2 * P(0, -1) - P(1, -1)) / 8.0;
#undef P
    }
}

static dlev* build_levels(const double* I0, const double* I1, int H, int W, int L) {
  float tf[7];
  int R = oracle_gauss_taps(1.f, tf);
  double w[7];
  for (int i = 0; i <= 2 * R; i++) w[i] = tf[i];
  dlev* lv = (dlev*)calloc(L, sizeof(dlev));
  int h = H, wd = W;
  for (int l = 0; l < L; l++) {
    lv[l].H = h;
    lv[l].W = wd;
    size_t np = (size_t)h * wd;
    lv[l].A = (double*)malloc(np * 8);
    lv[l].B = (double*)malloc(np * 8);
    lv[l].Sr = (double*)malloc(np * 8);
    lv[l].Sc = (double*)malloc(np * 8);
    h /= 2;
    wd /= 2;
  }
  memcpy(lv[0].A, I0, (size_t)H * W * 8);
  memcpy(lv[0].B, I1, (size_t)H * W * 8);
  double* tmp = (double*)malloc((size_t)H * W * 8);
  for (int l = 1; l < L; l++) {
    blur_decimate(lv[l - 1].A, lv[l - 1].H, lv[l - 1].W, w, R, lv[l].A, tmp);
    blur_decimate(lv[l - 1].B, lv[l - 1].H, lv[l - 1].W, w, R, lv[l].B, tmp);
  }
  free(tmp);
  for (int l = 0; l < L; l++) sobel8(lv[l].A, lv[l].H, lv[l].W, lv[l].Sr, lv[l].Sc);
  return lv;
}

static void free_levels(dlev* lv, int L) {
  for (int l = 0; l < L; l++) {
    free(lv[l].A);
    free(lv[l].B);
    free(lv[l].Sr);
    free(lv[l].Sc);
  }
  free(lv);
}

/* One point through all levels; returns the loss and the final position. */
static double point_forward(const dlev* lv, int L, int ws, int iters, const double p[2], const double u0[2],
                            double vout[2]) {
  const int hws = ws / 2;
  double scale = 1.0;
  for (int l = 1; l < L; l++) scale *= 2.0;
  double d0 = u0[0] / scale, d1 = u0[1] / scale;
  double v0 = 0, v1 = 0;
  for (int l = L - 1; l >= 0; l--) {
    const dlev* e = &lv[l];
    double s = 1.0;
    for (int k = 0; k < l; k++) s *= 2.0;
    const double q0 = p[0] / s, q1 = p[1] / s;
    double G00 = 0, G01 = 0, G11 = 0;
    for (int r = -hws; r <= hws; r++)
      for (int c = -hws; c <= hws; c++) {
        double g0 = bil(e->Sr, e->H, e->W, q0 + r, q1 + c), g1 = bil(e->Sc, e->H, e->W, q0 + r, q1 + c);
        G00 += g0 * g0;
        G01 += g0 * g1;
        G11 += g1 * g1;
      }
    double det = G00 * G11 - G01 * G01;
    double M00 = G11 / det, M01 = -G01 / det, M11 = G00 / det;
    v0 = q0 + d0;
    v1 = q1 + d1;
    for (int k = 0; k < iters; k++) {
      double b0 = 0, b1 = 0;
      for (int r = -hws; r <= hws; r++)
        for (int c = -hws; c <= hws; c++) {
          double g0 = bil(e->Sr, e->H, e->W, q0 + r, q1 + c), g1 = bil(e->Sc, e->H, e->W, q0 + r, q1 + c);
          double rr = bil(e->A, e->H, e->W, q0 + r, q1 + c) - bil(e->B, e->H, e->W, v0 + r, v1 + c);
          b0 += g0 * rr;
          b1 += g1 * rr;
        }
      v0 += M00 * b0 + M01 * b1;
      v1 += M01 * b0 + M11 * b1;
    }
    d0 = 2.0 * (v0 - q0);
    d1 = 2.0 * (v1 - q1);
  }
  vout[0] = v0;
  vout[1] = v1;
  const dlev* e = &lv[0];
  double loss = 0;
  for (int r = -hws; r <= hws; r++)
    for (int c = -hws; c <= hws; c++) {
      double rr = bil(e->A, e->H, e->W, p[0] + r, p[1] + c) - bil(e->B, e->H, e->W, v0 + r, v1 + c);
      loss += rr * rr;
    }
  return loss;
}

/* Forward: per-point loss and final level-0 position. */
int oracle_lkd_forward(const double* I0, const double* I1, int H, int W, int L, int ws, int iters, const double* pts,
                       const double* u0, int n, double* loss, double* vfinal) {
  dlev* lv = build_levels(I0, I1, H, W, L);
  for (int i = 0; i < n; i++) loss[i] = point_forward(lv, L, ws, iters, pts + 2 * i, u0 + 2 * i, vfinal + 2 * i);
  free_levels(lv, L);
  return 0;
}

static double total_loss(const double* I0, const double* I1, int H, int W, int L, int ws, int iters,
                         const double* pts, const double* u0, int n, const double* wts) {
  dlev* lv = build_levels(I0, I1, H, W, L);
  double t = 0, v[2];
  for (int i = 0; i < n; i++) t += wts[i] * point_forward(lv, L, ws, iters, pts + 2 * i, u0 + 2 * i, v);
  free_levels(lv, L);
  return t;
}

/* Central differences of sum_i wts[i] * loss_i with step h. */
int oracle_lkd_grad_fd(const double* I0, const double* I1, int H, int W, int L, int ws, int iters, const double* pts,
                       const double* u0, int n, const double* wts, double h, double* g0, double* g1, double* gu) {
  size_t np = (size_t)H * W;
  double* a = (double*)malloc(np * 8);
  double* b = (double*)malloc(np * 8);
  double* u = (double*)malloc((size_t)n * 16);
  memcpy(a, I0, np * 8);
  memcpy(b, I1, np * 8);
  memcpy(u, u0, (size_t)n * 16);
  for (size_t k = 0; k < np; k++) {
    double keep = a[k];
    a[k] = keep + h;
    double lp = total_loss(a, b, H, W, L, ws, iters, pts, u, n, wts);
    a[k] = keep - h;
    double lm = total_loss(a, b, H, W, L, ws, iters, pts, u, n, wts);
    a[k] = keep;
    g0[k] = (lp - lm) / (2 * h);
    keep = b[k];
    b[k] = keep + h;
    lp = total_loss(a, b, H, W, L, ws, iters, pts, u, n, wts);
    b[k] = keep - h;
    lm = total_loss(a, b, H, W, L, ws, iters, pts, u, n, wts);
    b[k] = keep;
    g1[k] = (lp - lm) / (2 * h);
  }
  for (int k = 0; k < 2 * n; k++) {
    double keep = u[k];
    u[k] = keep + h;
    double lp = total_loss(a, b, H, W, L, ws, iters, pts, u, n, wts);
    u[k] = keep - h;
    double lm = total_loss(a, b, H, W, L, ws, iters, pts, u, n, wts);
    u[k] = keep;
    gu[k] = (lp - lm) / (2 * h);
  }
  free(a);
  free(b);
  free(u);
  return 0;
}
