/*
 * Seeded synthetic video generator (host C).
 *
 * Produces the moving-texture frames every workload of this library is
 * measured and checked on:
 *   texture = 128 + sum of 200 Gaussian blobs (sigma U[2,20] px, amplitude
 *             U[-60,60]) + 4-octave value noise,
 *   frame t = texture warped by the composition of t per-frame affine motions
 *             (translation U[-3,3] px, rotation U[-1,1] deg, scale
 *             U[0.99,1.01]) with bilinear sampling, plus Gaussian noise
 *             sigma = 2, rounded and clipped to uint8.
 * Everything derives from one 64-bit seed (one seed per video stream) through
 * a splitmix64 generator, so a stream is reproducible on any host.  The
 * texture lives on a canvas with a margin around the frame so that drift
 * keeps sampling real texture; samples beyond the canvas clamp to its edge.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  uint64_t s;
} rng_t;

static uint64_t rng_next(rng_t* r) {
  uint64_t z = (r->s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static double rng_unit(rng_t* r) { /* [0, 1) */
  return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0);
}

static double rng_uniform(rng_t* r, double a, double b) {
  return a + (b - a) * rng_unit(r);
}

static double rng_gauss(rng_t* r) { /* Box-Muller */
  double u1 = rng_unit(r), u2 = rng_unit(r);
  if (u1 < 1e-300) u1 = 1e-300;
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

typedef struct {
  uint64_t seed;
  int rows, cols;      /* frame size */
  int margin;          /* canvas margin on each side */
  int crow, ccol;      /* canvas size */
  float* canvas;       /* crow * ccol texture values */
} synth_stream;

/* Affine map: x' = A x + b, with x = (row, col) relative to the frame centre. */
typedef struct {
  double a00, a01, a10, a11, b0, b1;
} affine2;

static affine2 affine_identity(void) {
  affine2 m = {1, 0, 0, 1, 0, 0};
  return m;
}

static affine2 affine_compose(affine2 m, affine2 n) { /* m after n */
  affine2 r;
  r.a00 = m.a00 * n.a00 + m.a01 * n.a10;
  r.a01 = m.a00 * n.a01 + m.a01 * n.a11;
  r.a10 = m.a10 * n.a00 + m.a11 * n.a10;
  r.a11 = m.a10 * n.a01 + m.a11 * n.a11;
  r.b0 = m.a00 * n.b0 + m.a01 * n.b1 + m.b0;
  r.b1 = m.a10 * n.b0 + m.a11 * n.b1 + m.b1;
  return r;
}

static affine2 frame_motion(uint64_t seed, int t) {
  rng_t r = {seed * 0x100000001B3ull + 0x51ED270Bull + (uint64_t)t * 0x2545F4914F6CDD1Dull};
  double ty = rng_uniform(&r, -3, 3), tx = rng_uniform(&r, -3, 3);
  double th = rng_uniform(&r, -1, 1) * 3.141592653589793 / 180.0;
  double sc = rng_uniform(&r, 0.99, 1.01);
  affine2 m;
  m.a00 = sc * cos(th);
  m.a01 = -sc * sin(th);
  m.a10 = sc * sin(th);
  m.a11 = sc * cos(th);
  m.b0 = ty;
  m.b1 = tx;
  return m;
}

/* Map from frame-t coordinates back to texture coordinates (frame 0 frame). */
static affine2 cumulative_inverse(uint64_t seed, int t) {
  affine2 acc = affine_identity();
  for (int k = 1; k <= t; k++) {
    affine2 m = frame_motion(seed, k);
    /* invert m */
    double det = m.a00 * m.a11 - m.a01 * m.a10;
    affine2 inv;
    inv.a00 = m.a11 / det;
    inv.a01 = -m.a01 / det;
    inv.a10 = -m.a10 / det;
    inv.a11 = m.a00 / det;
    inv.b0 = -(inv.a00 * m.b0 + inv.a01 * m.b1);
    inv.b1 = -(inv.a10 * m.b0 + inv.a11 * m.b1);
    acc = affine_compose(acc, inv);
  }
  return acc;
}

static float value_noise(const float* lat, int lr, int lc, double y, double x) {
  int y0 = (int)floor(y), x0 = (int)floor(x);
  double fy = y - y0, fx = x - x0;
  fy = fy * fy * (3 - 2 * fy);
  fx = fx * fx * (3 - 2 * fx);
  if (y0 < 0) y0 = 0;
  if (x0 < 0) x0 = 0;
  if (y0 > lr - 2) y0 = lr - 2;
  if (x0 > lc - 2) x0 = lc - 2;
  const float* p = lat + (size_t)y0 * lc + x0;
  double a = p[0] + (p[1] - p[0]) * fx;
  double b = p[lc] + (p[lc + 1] - p[lc]) * fx;
  return (float)(a + (b - a) * fy);
}

void* synth_create(uint64_t seed, int rows, int cols) {
  if (rows <= 0 || cols <= 0) return NULL;
  synth_stream* s = (synth_stream*)calloc(1, sizeof(synth_stream));
  if (!s) return NULL;
  s->seed = seed;
  s->rows = rows;
  s->cols = cols;
  s->margin = (rows > cols ? rows : cols) / 4 + 32;
  s->crow = rows + 2 * s->margin;
  s->ccol = cols + 2 * s->margin;
  size_t n = (size_t)s->crow * s->ccol;
  s->canvas = (float*)malloc(n * sizeof(float));
  if (!s->canvas) {
    free(s);
    return NULL;
  }
  rng_t r = {seed ^ 0xC0FFEE1234567ull};
  for (size_t i = 0; i < n; i++) s->canvas[i] = 128.0f;

  /* 4-octave value noise. */
  static const int spacing[4] = {8, 4, 2, 1};
  static const float amp[4] = {32.f, 24.f, 18.f, 14.f};
  for (int o = 0; o < 4; o++) {
    int lr = s->crow / spacing[o] + 3, lc = s->ccol / spacing[o] + 3;
    float* lat = (float*)malloc((size_t)lr * lc * sizeof(float));
    if (!lat) continue;
    for (int i = 0; i < lr * lc; i++) lat[i] = (float)rng_uniform(&r, -1, 1);
    for (int y = 0; y < s->crow; y++)
      for (int x = 0; x < s->ccol; x++)
        s->canvas[(size_t)y * s->ccol + x] +=
            amp[o] * value_noise(lat, lr, lc, (double)y / spacing[o], (double)x / spacing[o]);
    free(lat);
  }

  /* 200 Gaussian blobs, scaled by area so large frames keep the density of a
   * 640x480 canvas. */
  double area_scale = (double)n / (double)((480 + 2 * 192) * (640 + 2 * 192));
  int nblobs = (int)(200 * (area_scale < 1 ? 1 : area_scale));
  for (int b = 0; b < nblobs; b++) {
    double cy = rng_uniform(&r, 0, s->crow), cx = rng_uniform(&r, 0, s->ccol);
    double sg = rng_uniform(&r, 2, 20), a = rng_uniform(&r, -60, 60);
    int rad = (int)ceil(3 * sg);
    int y0 = (int)cy - rad, y1 = (int)cy + rad, x0 = (int)cx - rad, x1 = (int)cx + rad;
    if (y0 < 0) y0 = 0;
    if (x0 < 0) x0 = 0;
    if (y1 > s->crow - 1) y1 = s->crow - 1;
    if (x1 > s->ccol - 1) x1 = s->ccol - 1;
    double inv = -0.5 / (sg * sg);
    for (int y = y0; y <= y1; y++)
      for (int x = x0; x <= x1; x++) {
        double d2 = (y - cy) * (y - cy) + (x - cx) * (x - cx);
        s->canvas[(size_t)y * s->ccol + x] += (float)(a * exp(d2 * inv));
      }
  }
  return s;
}

void synth_destroy(void* h) {
  synth_stream* s = (synth_stream*)h;
  if (!s) return;
  free(s->canvas);
  free(s);
}

static float canvas_at(const synth_stream* s, int y, int x) {
  if (y < 0) y = 0;
  if (x < 0) x = 0;
  if (y > s->crow - 1) y = s->crow - 1;
  if (x > s->ccol - 1) x = s->ccol - 1;
  return s->canvas[(size_t)y * s->ccol + x];
}

static float bilinear(const synth_stream* s, double y, double x) {
  int y0 = (int)floor(y), x0 = (int)floor(x);
  double fy = y - y0, fx = x - x0;
  double a = canvas_at(s, y0, x0) * (1 - fx) + canvas_at(s, y0, x0 + 1) * fx;
  double b = canvas_at(s, y0 + 1, x0) * (1 - fx) + canvas_at(s, y0 + 1, x0 + 1) * fx;
  return (float)(a * (1 - fy) + b * fy);
}

/* Frame t as floats (noise included when noise_sigma > 0). */
int synth_frame_f32(void* h, int t, float noise_sigma, float* out) {
  synth_stream* s = (synth_stream*)h;
  if (!s || !out || t < 0) return -1;
  affine2 m = cumulative_inverse(s->seed, t);
  double cy = 0.5 * (s->rows - 1), cx = 0.5 * (s->cols - 1);
  rng_t r = {s->seed * 0x9E3779B97F4A7C15ull + 0xABCDEFull + (uint64_t)t * 0xD1B54A32D192ED03ull};
  for (int y = 0; y < s->rows; y++)
    for (int x = 0; x < s->cols; x++) {
      double py = y - cy, px = x - cx;
      double ty = m.a00 * py + m.a01 * px + m.b0 + cy + s->margin;
      double tx = m.a10 * py + m.a11 * px + m.b1 + cx + s->margin;
      float v = bilinear(s, ty, tx);
      if (noise_sigma > 0) v += (float)(noise_sigma * rng_gauss(&r));
      out[(size_t)y * s->cols + x] = v;
    }
  return 0;
}

/* Frame t as uint8 gray (noise sigma 2, rounded, clipped). */
int synth_frame_u8(void* h, int t, uint8_t* out) {
  synth_stream* s = (synth_stream*)h;
  if (!s || !out || t < 0) return -1;
  size_t n = (size_t)s->rows * s->cols;
  float* tmp = (float*)malloc(n * sizeof(float));
  if (!tmp) return -2;
  synth_frame_f32(h, t, 2.0f, tmp);
  for (size_t i = 0; i < n; i++) {
    float v = floorf(tmp[i] + 0.5f);
    out[i] = (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v));
  }
  free(tmp);
  return 0;
}

/* Frame t as interleaved RGB uint8: channel 0 is the gray frame; channels 1
 * and 2 are tinted copies (the tracker reads channel 0 only). */
int synth_frame_rgb(void* h, int t, uint8_t* out) {
  synth_stream* s = (synth_stream*)h;
  if (!s || !out || t < 0) return -1;
  size_t n = (size_t)s->rows * s->cols;
  uint8_t* g = (uint8_t*)malloc(n);
  if (!g) return -2;
  synth_frame_u8(h, t, g);
  for (size_t i = 0; i < n; i++) {
    int v = g[i];
    out[3 * i] = (uint8_t)v;
    out[3 * i + 1] = (uint8_t)(v * 3 / 4 + 32);
    out[3 * i + 2] = (uint8_t)(255 - v);
  }
  free(g);
  return 0;
}

/* Ground-truth displacement of frame-(t-1) pixel (y, x) into frame t:
 * writes (dy, dx).  Used by the Lucas-Kanade workloads. */
int synth_true_flow(void* h, int t, double y, double x, double* dy, double* dx) {
  synth_stream* s = (synth_stream*)h;
  if (!s || t < 1) return -1;
  affine2 m = frame_motion(s->seed, t);
  double cy = 0.5 * (s->rows - 1), cx = 0.5 * (s->cols - 1);
  double py = y - cy, px = x - cx;
  double ny = m.a00 * py + m.a01 * px + m.b0, nx = m.a10 * py + m.a11 * px + m.b1;
  *dy = ny - py;
  *dx = nx - px;
  return 0;
}
