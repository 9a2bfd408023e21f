/*
 * CPU restatement of cuimg's semi-dense tracker -- TEST INFRASTRUCTURE ONLY.
 *
 * This is the oracle: a plain C restatement of
 *   tracker<tracking_strategies::bc2s_fast_gradient_cpu>::run(frame)
 * (cuimg/tracking2/tracker.hpp:53-91, cuimg/tracking2/tracking_strategies.hpp:155-198)
 * with the single-threaded semantics of the reference CPU build
 * (-DNO_CUDA, no WITH_OPENCV, zero-filled allocations).  It is checked
 * bit-exactly against the reference itself (oracle/_ref, built from the
 * reference sources by oracle/Makefile) and against the committed golden
 * fixtures under tests/golden/.  Only tests/, the smoke check and the CPU
 * baseline leg of bench.py load it; the CUDA product path never does.
 *
 * Layout: every level keeps bordered byte images with the reference's border
 * widths (input 6, s1 3, s2 6, mask 4, saliency 1, sparse index 7), a
 * structure-of-arrays particle set, and the 8x8-pixel flow bins.
 *
 * Parallelism: loops whose iterations are independent in the reference
 * (per pixel, per particle with disjoint writes) may run under OpenMP; every
 * order-dependent step (sparse-index last writer, raster-ordered births,
 * stable compaction, the merge pass) runs sequentially, so the result is the
 * same for any thread count.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define NO_FLOW_V (-500.f) /* cuimg/tracking2/tracker_defines.h:4 */
#define SPARSE_NONE 0xFFFFFFFFu

/* c8_h, raster order (cuimg/neighb2d_data.h:80-85), as (row, col). */
static const int C8[8][2] = {{-1, 1}, {0, 1}, {1, 1}, {-1, 0}, {1, 0}, {-1, -1}, {0, -1}, {1, -1}};
/* c8_it_h: first index and exclusive end of the partial sweep after an
 * improvement in direction k (cuimg/neighb2d_data.h:162-180). */
static const int C8_IT[9][2] = {{6, 3}, {0, 3}, {0, 5}, {2, 5}, {2, 7}, {4, 7}, {4, 1}, {6, 1}, {0, 0}};
/* circle_r3_h (cuimg/neighb2d_data.h:184-189). */
static const int RING[16][2] = {{-3, 0}, {-3, 1}, {-2, 2}, {-1, 3}, {0, 3}, {1, 3}, {2, 2}, {3, 1},
                                {3, 0},  {3, -1}, {2, -2}, {1, -3}, {0, -3}, {-1, -3}, {-2, -2}, {-3, -1}};

typedef struct {
  int H, W;
  int pin, ps1, ps2, pmask, psal, psp; /* pitches (elements) */
  uint8_t* in;      /* border 6 */
  uint8_t* s1;      /* border 3 */
  uint8_t* s2;      /* border 6 */
  uint8_t* tmp;     /* no border */
  uint16_t* contrast;
  uint8_t* mask;    /* border 4 */
  uint8_t* sal;     /* border 1 */
  uint32_t* sparse; /* border 7 */
  uint8_t* newpts;  /* no border */
  int BH, BW;       /* flow bins: ceil(H/8) x ceil(W/8) */
  int32_t* st_n;
  int32_t* st_sp;   /* 2 per bin */
  float* flow;      /* 2 per bin */
  uint32_t* msc;
  /* particle set */
  int n, cap;
  float* speed;     /* 2 per particle */
  int16_t* pos;     /* 2 per particle: row, col */
  uint16_t* age;
  uint8_t* feat;    /* 16 per particle (weights are constant 255) */
  int32_t* matches;
  int nmatches;
  int compact_has_run;
  uint8_t* moved;   /* per particle, scratch */
  int frame_cpt;
  /* This scale's strategy and detector settings (the reference keeps them per
   * scale: generic_strategy and its detector, tracking_strategies.h:99-106). */
  int threshold, det_freq, filt_freq, k, with_merge, n_fast, grad_th;
} olevel;

typedef struct {
  int L;
  olevel* lv;
  int detector, step; /* 0 FAST, 1 regular, 2 dense */
} otracker;

#define AT(img, pitch, b, r, c) ((img)[(size_t)((r) + (b)) * (pitch) + ((c) + (b))])

static int level_alloc(olevel* l, int H, int W) {
  memset(l, 0, sizeof(*l));
  l->H = H;
  l->W = W;
  l->pin = W + 12;
  l->ps1 = W + 6;
  l->ps2 = W + 12;
  l->pmask = W + 8;
  l->psal = W + 2;
  l->psp = W + 14;
  l->in = (uint8_t*)calloc((size_t)(H + 12) * l->pin, 1);
  l->s1 = (uint8_t*)calloc((size_t)(H + 6) * l->ps1, 1);
  l->s2 = (uint8_t*)calloc((size_t)(H + 12) * l->ps2, 1);
  l->tmp = (uint8_t*)calloc((size_t)H * W, 1);
  l->contrast = (uint16_t*)calloc((size_t)H * W, 2);
  l->mask = (uint8_t*)calloc((size_t)(H + 8) * l->pmask, 1);
  l->sal = (uint8_t*)calloc((size_t)(H + 2) * l->psal, 1);
  l->sparse = (uint32_t*)malloc((size_t)(H + 14) * l->psp * 4);
  l->newpts = (uint8_t*)calloc((size_t)H * W, 1);
  l->BH = (H + 7) / 8;
  l->BW = (W + 7) / 8;
  size_t nb = (size_t)l->BH * l->BW;
  l->st_n = (int32_t*)calloc(nb, 4);
  l->st_sp = (int32_t*)calloc(2 * nb, 4);
  l->flow = (float*)calloc(2 * nb, 4);
  l->msc = (uint32_t*)calloc(nb, 4);
  if (!l->in || !l->s1 || !l->s2 || !l->tmp || !l->contrast || !l->mask || !l->sal || !l->sparse ||
      !l->newpts || !l->st_n || !l->st_sp || !l->flow || !l->msc)
    return -1;
  /* particle_container ctor: memset -1 then clamp-fill the border
   * (cuimg/tracking2/particle_container.hpp:23-31). */
  memset(l->sparse, 0xFF, (size_t)(H + 14) * l->psp * 4);
  return 0;
}

static void level_free(olevel* l) {
  free(l->in); free(l->s1); free(l->s2); free(l->tmp); free(l->contrast); free(l->mask);
  free(l->sal); free(l->sparse); free(l->newpts); free(l->st_n); free(l->st_sp); free(l->flow);
  free(l->msc); free(l->speed); free(l->pos); free(l->age); free(l->feat); free(l->matches);
  free(l->moved);
}

static int particles_reserve(olevel* l, int n) {
  if (n <= l->cap) return 0;
  int cap = l->cap ? l->cap : 1024;
  while (cap < n) cap *= 2;
  float* sp = (float*)realloc(l->speed, (size_t)cap * 8);
  if (!sp) return -1;
  l->speed = sp;
  int16_t* po = (int16_t*)realloc(l->pos, (size_t)cap * 4);
  if (!po) return -1;
  l->pos = po;
  uint16_t* ag = (uint16_t*)realloc(l->age, (size_t)cap * 2);
  if (!ag) return -1;
  l->age = ag;
  uint8_t* fe = (uint8_t*)realloc(l->feat, (size_t)cap * 16);
  if (!fe) return -1;
  l->feat = fe;
  int32_t* ma = (int32_t*)realloc(l->matches, (size_t)cap * 4);
  if (!ma) return -1;
  l->matches = ma;
  uint8_t* mv = (uint8_t*)realloc(l->moved, (size_t)cap);
  if (!mv) return -1;
  l->moved = mv;
  l->cap = cap;
  return 0;
}

/* fill_border_clamp (cuimg/border.h:128-137) on a bordered byte image. */
static void clamp_border_u8(uint8_t* img, int pitch, int b, int H, int W) {
  for (int r = -b; r < H + b; r++) {
    int rr = r < 0 ? 0 : (r >= H ? H - 1 : r);
    for (int c = -b; c < W + b; c++) {
      if (r >= 0 && r < H && c >= 0 && c < W) continue;
      int cc = c < 0 ? 0 : (c >= W ? W - 1 : c);
      AT(img, pitch, b, r, c) = AT(img, pitch, b, rr, cc);
    }
  }
}

/* ---------------------------------------------------------------------------
 * Pyramid: tracker::update_input / subsample_input (tracker.hpp:53-69),
 * subsample -> mipmap_kernel (cuimg/gpu/mipmap.h:24-49,206-227): 2x2 mean with
 * integer (floor) division.
 * ------------------------------------------------------------------------- */
static void build_pyramid(otracker* t, const uint8_t* frame) {
  olevel* l0 = &t->lv[0];
  for (int r = 0; r < l0->H; r++) memcpy(&AT(l0->in, l0->pin, 6, r, 0), frame + (size_t)r * l0->W, l0->W);
  clamp_border_u8(l0->in, l0->pin, 6, l0->H, l0->W);
  for (int s = 1; s < t->L; s++) {
    olevel* a = &t->lv[s - 1];
    olevel* o = &t->lv[s];
    for (int r = 0; r < o->H; r++)
      for (int c = 0; c < o->W; c++) {
        int v = AT(a->in, a->pin, 6, 2 * r, 2 * c) + AT(a->in, a->pin, 6, 2 * r, 2 * c + 1) +
                AT(a->in, a->pin, 6, 2 * r + 1, 2 * c) + AT(a->in, a->pin, 6, 2 * r + 1, 2 * c + 1);
        AT(o->in, o->pin, 6, r, c) = (uint8_t)(v / 4);
      }
    clamp_border_u8(o->in, o->pin, 6, o->H, o->W);
  }
}

/* contrast_kernel (tracking_strategies.hpp:101-135). */
static void compute_contrast(olevel* l) {
  const int d = 2;
#pragma omp parallel for schedule(static)
  for (int r = 0; r < l->H; r++)
    for (int c = 0; c < l->W; c++) {
#define I(dr, dc) ((int)AT(l->in, l->pin, 6, r + (dr), c + (dc)))
      int v = abs(I(0, d) - I(0, -d)) + abs(I(-d, 0) - I(d, 0)) + abs(I(-d, -d) - I(d, d)) +
              abs(I(-d, d) - I(d, -d));
#undef I
      l->contrast[(size_t)r * l->W + c] = (uint16_t)v;
    }
}

/* gaussian_blur_sigma1 (cuimg/cpu/gaussian_blur.h:9-47): rows pass writes
 * tmp columns 1..W-2 of every row, columns pass writes out rows 1..H-2 of
 * every column; the untouched ring keeps its (zero) initial value. */
static void blur_sigma1(const uint8_t* in, int pin, int bin, uint8_t* out, int pout, int bout,
                        uint8_t* tmp, int H, int W) {
#pragma omp parallel for schedule(static)
  for (int r = 0; r < H; r++)
    for (int c = 1; c < W - 1; c++) {
      int v = 2 * AT(in, pin, bin, r, c) + AT(in, pin, bin, r, c - 1) + AT(in, pin, bin, r, c + 1);
      tmp[(size_t)r * W + c] = (uint8_t)(v / 4);
    }
#pragma omp parallel for schedule(static)
  for (int r = 1; r < H - 1; r++)
    for (int c = 0; c < W; c++) {
      int v = 2 * tmp[(size_t)r * W + c] + tmp[(size_t)(r - 1) * W + c] + tmp[(size_t)(r + 1) * W + c];
      AT(out, pout, bout, r, c) = (uint8_t)(v / 4);
    }
}

/* bc2s_feature<cpu>::update (bc2s_feature.hpp:372-393, non-OpenCV branch). */
static void update_feature(olevel* l) {
  blur_sigma1(l->in, l->pin, 6, l->s1, l->ps1, 3, l->tmp, l->H, l->W);
  blur_sigma1(l->s1, l->ps1, 3, l->s2, l->ps2, 6, l->tmp, l->H, l->W);
  clamp_border_u8(l->s1, l->ps1, 3, l->H, l->W);
  clamp_border_u8(l->s2, l->ps2, 6, l->H, l->W);
}

/* compute_feature (bc2s_feature.hpp:260-284): s1 at even ring offsets, s2 at
 * twice those. */
static void compute_feature(const olevel* l, int r, int c, uint8_t* f) {
  for (int i = 0; i < 8; i++) {
    f[i] = AT(l->s1, l->ps1, 3, r + RING[2 * i][0], c + RING[2 * i][1]);
    f[8 + i] = AT(l->s2, l->ps2, 6, r + 2 * RING[2 * i][0], c + 2 * RING[2 * i][1]);
  }
}

/* bc2s_internals::distance (bc2s_feature.hpp:173-231).  Weights are always
 * 255 on this path (bc2s() sets them, nothing rewrites them), so
 * (sum |v-a|*255) / 255 == sum |v-a|. */
static int feat_distance(const olevel* l, const uint8_t* f, int r, int c, int scale) {
  int d = 0;
  if (scale == 1)
    for (int i = 0; i < 8; i++)
      d += abs((int)AT(l->s1, l->ps1, 3, r + RING[2 * i][0], c + RING[2 * i][1]) - f[i]);
  for (int i = 0; i < 8; i++)
    d += abs((int)AT(l->s2, l->ps2, 6, r + 2 * RING[2 * i][0], c + 2 * RING[2 * i][1]) - f[8 + i]);
  return d;
}

static int in_dom(const olevel* l, int r, int c) { return r >= 0 && r < l->H && c >= 0 && c < l->W; }

/* gradient_descent_match (gradient_descent_matcher.hpp:9-76).  Returns the
 * offset of the match from `pr,pc`.  The initial distance always uses the
 * scale-1 (s1+s2) distance, whatever `scale` the sweep uses. */
static void gd_match(const olevel* l, int pr, int pc, const uint8_t* f, int scale, int* dr, int* dc) {
  int pred_r = pr, pred_c = pc;
  int mr = pr, mc = pc;
  int best = feat_distance(l, f, pr, pc, 1);
  int mi = 8;
  if (!in_dom(l, pr, pc)) {
    *dr = pr; /* the reference returns the prediction itself here */
    *dc = pc;
    return;
  }
  for (int search = 0; search < 10; search++) {
    int i = C8_IT[mi][0], end = C8_IT[mi][1];
    int first = 1;
    while (first || i != end) {
      first = 0;
      int nr = pred_r + C8[i][0], nc = pred_c + C8[i][1];
      if (in_dom(l, nr, nc)) {
        int d = feat_distance(l, f, nr, nc, scale);
        if (d < best) {
          mr = nr;
          mc = nc;
          mi = i;
          best = d;
        }
      }
      i = (i + 1) & 7;
    }
    if ((pred_r == mr && pred_c == mc) || !in_dom(l, mr, mc)) break;
    pred_r = mr;
    pred_c = mc;
  }
  *dr = mr - pr;
  *dc = mc - pc;
}

/* match_particles (tracking_strategies.hpp:641-696) with
 * match_particles_kernel (:275-426), kernel_particle_container::move
 * (particle_container.hpp:422-466), compute_flow_stats_kernel (:525-574),
 * flow_fusion_kernel(_root) (:576-639). */
static void match_particles(otracker* t, int s) {
  olevel* l = &t->lv[s];
  /* before_matching: sparse = -1 over the whole buffer. */
  memset(l->sparse, 0xFF, (size_t)(l->H + 14) * l->psp * 4);
  l->compact_has_run = 0;

#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < l->n; i++) {
    l->moved[i] = 0;
    if (l->age[i] == 0) continue;
    /* motion_based_prediction (predictions.h:15-24): truncating float->int. */
    int pdr = 0, pdc = 0;
    if (l->age[i] != 1) {
      pdr = (int)l->speed[2 * i];
      pdc = (int)l->speed[2 * i + 1];
    }
    int pr = (int16_t)(l->pos[2 * i] + pdr), pc = (int16_t)(l->pos[2 * i + 1] + pdc);
    if (!in_dom(l, pr, pc)) {
      l->age[i] = 0;
      continue;
    }
    const uint8_t* f = l->feat + 16 * (size_t)i;
    int d1r, d1c, d2r, d2c;
    gd_match(l, pr, pc, f, 2, &d1r, &d1c);
    gd_match(l, pr + d1r, pc + d1c, f, 1, &d2r, &d2c);
    int dr = d1r + d2r, dc = d1c + d2c;
    int mr = (int16_t)(pr + dr), mc = (int16_t)(pc + dc);
    /* Acceptance: n_diff over s2 entries (weights 255 > 150 -> cpt = 8). */
    uint8_t mf[16];
    int accept = in_dom(l, mr, mc);
    if (accept) {
      compute_feature(l, mr, mc, mf);
      unsigned n_diff = 0, cpt = 0;
      for (int j = 8; j < 16; j++) {
        cpt++;
        if (abs((int)f[j] - (int)mf[j]) > l->k) n_diff++;
      }
      accept = n_diff < cpt / 2;
    }
    if (!accept) {
      l->age[i] = 0;
      continue;
    }
    if (l->contrast[(size_t)mr * l->W + mc] < 3) {
      l->age[i] = 0;
      continue;
    }
    /* move(i, pred - pos + delta, feature(match)) */
    int sr = pr - l->pos[2 * i] + dr, sc = pc - l->pos[2 * i + 1] + dc;
    l->age[i]++;
    l->speed[2 * i] = (float)sr;
    l->speed[2 * i + 1] = (float)sc;
    l->pos[2 * i] = (int16_t)mr;
    l->pos[2 * i + 1] = (int16_t)mc;
    if (sr != 0 || sc != 0) memcpy(l->feat + 16 * (size_t)i, mf, 16);
    l->moved[i] = 1;
  }
  /* sparse(pos) = i in index order: the highest index wins. */
  for (int i = 0; i < l->n; i++)
    if (l->moved[i]) AT(l->sparse, l->psp, 7, l->pos[2 * i], l->pos[2 * i + 1]) = (uint32_t)i;

  /* flow statistics per 8x8 bin: live count and the last (raster) speed. */
  size_t nb = (size_t)l->BH * l->BW;
  for (size_t b = 0; b < nb; b++) {
    l->flow[2 * b] = NO_FLOW_V;
    l->flow[2 * b + 1] = NO_FLOW_V;
    l->msc[b] = 0;
  }
  for (int br = 0; br < l->BH; br++)
    for (int bc = 0; bc < l->BW; bc++) {
      int count = 0, lr = 0, lc = 0;
      for (int r = 0; r < 8; r++)
        for (int c = 0; c < 8; c++) {
          int nr = br * 8 + r, nc = bc * 8 + c;
          if (!in_dom(l, nr, nc)) continue;
          uint32_t j = AT(l->sparse, l->psp, 7, nr, nc);
          if (j != SPARSE_NONE && l->age[j] >= 1) {
            count++;
            lr = (int)l->speed[2 * j];
            lc = (int)l->speed[2 * j + 1];
          }
        }
      size_t b = (size_t)br * l->BW + bc;
      l->st_n[b] = count;
      l->st_sp[2 * b] = lr;
      l->st_sp[2 * b + 1] = lc;
    }
  if (s + 1 < t->L) {
    const olevel* u = &t->lv[s + 1];
    for (int br = 0; br < l->BH; br++)
      for (int bc = 0; bc < l->BW; bc++) {
        size_t b = (size_t)br * l->BW + bc;
        int ubr = br / 2, ubc = bc / 2;
        /* Upper bins always cover bin/2 for the sizes the C ABI accepts. */
        size_t ub = (size_t)ubr * u->BW + ubc;
        l->msc[b] = (uint32_t)(l->st_n[b] + u->st_n[ub]);
        if (l->st_n[b] > 1) {
          l->flow[2 * b] = (float)l->st_sp[2 * b];
          l->flow[2 * b + 1] = (float)l->st_sp[2 * b + 1];
        } else if (!(u->flow[2 * ub] == NO_FLOW_V && u->flow[2 * ub + 1] == NO_FLOW_V)) {
          l->flow[2 * b] = u->flow[2 * ub] * 2;
          l->flow[2 * b + 1] = u->flow[2 * ub + 1] * 2;
        }
      }
  } else {
    for (size_t b = 0; b < nb; b++) {
      l->msc[b] = (uint32_t)l->st_n[b];
      if (l->st_n[b] > 1) {
        l->flow[2 * b] = (float)(l->st_sp[2 * b] / l->st_n[b]);
        l->flow[2 * b + 1] = (float)(l->st_sp[2 * b + 1] / l->st_n[b]);
      } else {
        l->flow[2 * b] = NO_FLOW_V;
        l->flow[2 * b + 1] = NO_FLOW_V;
      }
    }
  }
}

/* fast::compute_saliency (fast_detector.hpp:26-157) at pixel (r, c) of an
 * image whose pixel (0, 0) is at `p00`, rows `pitch` bytes apart, with at
 * least 3 pixels of border on every side. */
uint8_t oracle_fast_saliency_at(const uint8_t* p00, int pitch, int r, int c, int n_, int th) {
  unsigned max_n = 0, n = 0;
  int status = 2;
  int vp = p00[(ptrdiff_t)r * pitch + c];
  unsigned sum_bright = 0, sum_dark = 0;
#define RV(i) ((int)p00[(ptrdiff_t)(r + RING[i][0]) * pitch + (c + RING[i][1])])
  if (n_ >= 9) {
    static const int to_test[6] = {0, 4, 8, 12, 0, 4};
    int equals = 0;
    for (int i = 0; i < 6; i++) {
      int vn = RV(to_test[i]);
      int sign = vn > vp;
      unsigned char dist = (unsigned char)abs(vn - vp);
      if (dist > th) {
        if (sign == status) {
          n++;
        } else {
          if (n > max_n) max_n = n;
          status = sign;
          n = 1;
        }
      } else {
        if (n > max_n) max_n = n;
        status = 2;
        equals++;
        if (i < 4 && n_ >= 12 && equals >= 2) return 0;
      }
    }
    if (n > max_n) max_n = n;
    if (n_ >= 12 && max_n < 3) return 0;
    else if (n_ >= 8 && max_n < 2) return 0;
  }
  n = 0;
  status = 2;
  max_n = 0;
  for (int i = 0; i < 16; i++) {
    int vn = RV(i);
    int sign = vn > vp;
    unsigned char dist = (unsigned char)abs(vn - vp);
    if (dist > th) {
      if (sign == status) {
        n++;
      } else {
        if (n > max_n) max_n = n;
        status = sign;
        n = 1;
      }
      if (vn < vp) sum_dark += dist;
      else sum_bright += dist;
    } else {
      if (n > max_n) max_n = n;
      status = 2;
    }
  }
  if (n != 16 && status != 2) {
    int i = 0;
    while (i < 16) {
      int vn = RV(i);
      int sign = vn > vp;
      unsigned char dist = (unsigned char)abs(vn - vp);
      if (dist <= th || sign != status) break;
      n++;
      i++;
    }
  }
#undef RV
  if (n > max_n) max_n = n;
  if (max_n < (unsigned)n_) return 0;
  return (uint8_t)(sum_bright > sum_dark ? sum_bright : sum_dark);
}

static uint8_t fast_saliency(const olevel* l, int r, int c, int n_, int th) {
  return oracle_fast_saliency_at(&AT(l->in, l->pin, 6, 0, 0), l->pin, r, c, n_, th);
}

/* create_detector_mask (tracking_strategies.hpp:254-272), detector update
 * (fast_detector.hpp:296-313), new_particles(cpu) (:217-262),
 * particle_container::add (particle_container.hpp:370-387) and compact(cpu)
 * (:215-252). */
static int add_particle(olevel* l, int r, int c) {
  if (particles_reserve(l, l->n + 1)) return -1;
  int i = l->n++;
  l->age[i] = 1;
  l->speed[2 * i] = 0.f;
  l->speed[2 * i + 1] = 0.f;
  l->pos[2 * i] = (int16_t)r;
  l->pos[2 * i + 1] = (int16_t)c;
  compute_feature(l, r, c, l->feat + 16 * (size_t)i);
  AT(l->sparse, l->psp, 7, r, c) = (uint32_t)i;
  return 0;
}

/* regular_detector::update + new_particles (regular_detector.hpp:62-103):
 * contrast = mean over the 8 neighbours at distance 2 of |I(q) - I(p)| on
 * domain - border(1) (the outer ring is never written: 0); a particle at every
 * pixel whose row and column are multiples of step and whose contrast reaches
 * grad_th, in raster order over the whole domain.  dense_detector
 * (dense_detector.hpp:19-31): a particle at every pixel without one. */
static int alt_births(otracker* t, olevel* l) {
  int H = l->H, W = l->W;
  for (int r = 0; r < H; r++)
    for (int c = 0; c < W; c++) {
      if (t->detector == 2) {
        if (AT(l->sparse, l->psp, 7, r, c) != SPARSE_NONE) continue;
      } else {
        if (r % t->step || c % t->step) continue;
        int rc = 0;
        if (r >= 1 && r <= H - 2 && c >= 1 && c <= W - 2) {
          int vp = AT(l->in, l->pin, 6, r, c), res = 0;
          for (int i = 0; i < 8; i++) res += abs((int)AT(l->in, l->pin, 6, r + 2 * C8[i][0], c + 2 * C8[i][1]) - vp);
          rc = res / 8;
        }
        if (rc < l->grad_th) continue;
      }
      if (add_particle(l, r, c)) return -1;
    }
  return 0;
}

static int detect_and_compact(otracker* t, int s) {
  olevel* l = &t->lv[s];
  int H = l->H, W = l->W;
  if (t->detector != 0) {
    if (alt_births(t, l)) return -1;
    goto compact;
  }
  memset(l->mask, 255, (size_t)(H + 8) * l->pmask);
  for (int i = 0; i < l->n; i++) { /* every slot, dead ones included */
    int pr = l->pos[2 * i], pc = l->pos[2 * i + 1];
    AT(l->mask, l->pmask, 4, pr, pc) = 0;
    for (int k = 0; k < 8; k++) AT(l->mask, l->pmask, 4, pr + C8[k][0], pc + C8[k][1]) = 0;
  }
  for (int r = 0; r < H; r++)
    for (int c = 0; c < W; c++)
      if (l->contrast[(size_t)r * W + c] < 5) AT(l->mask, l->pmask, 4, r, c) = 0;

  memset(l->sal, 0, (size_t)(H + 2) * l->psal);
#pragma omp parallel for schedule(static)
  for (int r = 0; r < H; r++)
    for (int c = 0; c < W; c++)
      if (AT(l->mask, l->pmask, 4, r, c) != 0)
        AT(l->sal, l->psal, 1, r, c) = fast_saliency(l, r, c, l->n_fast, l->threshold);

  memset(l->newpts, 0, (size_t)H * W);
  int TH = H / 3, TW = W / 3;
#pragma omp parallel for schedule(static)
  for (int tr = 0; tr < TH; tr++)
    for (int tc = 0; tc < TW; tc++) {
      int pr = tr * 3 + 1, pc = tc * 3 + 1;
      int skip = 0;
      for (int r = 0; r < 3 && !skip; r++)
        for (int c = 0; c < 3; c++)
          if (in_dom(l, pr + r, pc + c) && AT(l->sparse, l->psp, 7, pr + r, pc + c) != SPARSE_NONE) {
            skip = 1;
            break;
          }
      if (skip) continue;
      float vmax = AT(l->sal, l->psal, 1, pr, pc);
      int mr = pr, mc = pc;
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
          if (in_dom(l, pr + r, pc + c)) {
            float v = AT(l->sal, l->psal, 1, pr + r, pc + c);
            if (vmax < v) {
              vmax = v;
              mr = pr + r;
              mc = pc + c;
            }
          }
      if (vmax < (float)l->threshold) continue;
      l->newpts[(size_t)mr * W + mc] = 1;
    }
  /* Births in raster order over domain - border(3). */
  for (int r = 3; r <= H - 4; r++)
    for (int c = 3; c <= W - 4; c++)
      if (l->newpts[(size_t)r * W + c])
        if (add_particle(l, r, c)) return -1;
compact:
  /* Stable compaction. */
  l->compact_has_run = 1;
  l->nmatches = l->n;
  int o = 0;
  for (int i = 0; i < l->n; i++) {
    l->matches[i] = -1;
    if (l->age[i] == 0) continue;
    l->age[o] = l->age[i];
    l->speed[2 * o] = l->speed[2 * i];
    l->speed[2 * o + 1] = l->speed[2 * i + 1];
    l->pos[2 * o] = l->pos[2 * i];
    l->pos[2 * o + 1] = l->pos[2 * i + 1];
    memmove(l->feat + 16 * (size_t)o, l->feat + 16 * (size_t)i, 16);
    AT(l->sparse, l->psp, 7, l->pos[2 * o], l->pos[2 * o + 1]) = (uint32_t)o;
    l->matches[i] = o;
    o++;
  }
  l->n = o;
  return 0;
}

/* filter_bad_particles_kernel (tracking_strategies.hpp:482-523). */
static void filter_particles(olevel* l) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < l->n; i++) {
    int br = l->pos[2 * i] / 8, bc = l->pos[2 * i + 1] / 8;
    size_t b = (size_t)br * l->BW + bc;
    if (l->age[i] > 2 && l->msc[b] > 0) {
      float dx = l->speed[2 * i] - l->flow[2 * b], dy = l->speed[2 * i + 1] - l->flow[2 * b + 1];
      float nrm = sqrtf(dx * dx + dy * dy);
      if (nrm > 10.f) {
        l->age[i] = 0;
        continue;
      }
    }
    int alone = 1;
    for (int k = 0; k < 8; k++) {
      int nr = br + C8[k][0], nc = bc + C8[k][1];
      if (nr >= 0 && nr < l->BH && nc >= 0 && nc < l->BW && l->msc[(size_t)nr * l->BW + nc] != 0) alone = 0;
    }
    if (alone && l->msc[b] == 1) l->age[i] = 0;
  }
}

/* merge_trajectories (cuimg/tracking2/merge_trajectories.h:10-35), run over
 * the particle index in order. */
static void merge_particles(olevel* l) {
  for (int i = 0; i < l->n; i++) {
    if (l->age[i] == 0) continue;
    int pr = l->pos[2 * i], pc = l->pos[2 * i + 1];
    for (int k = 0; k < 8; k++) {
      uint32_t j = AT(l->sparse, l->psp, 7, pr + C8[k][0], pc + C8[k][1]);
      if (j == SPARSE_NONE) continue;
      float dx = l->speed[2 * i] - l->speed[2 * j], dy = l->speed[2 * i + 1] - l->speed[2 * j + 1];
      if ((int)l->age[j] > (int)l->age[i] + 2 && sqrtf(dx * dx + dy * dy) < 2.f) {
        l->age[j] = 0;
        break;
      }
    }
  }
}

/* generic_strategy::update (tracking_strategies.hpp:155-198). */
static int strategy_update(otracker* t, int s) {
  olevel* l = &t->lv[s];
  compute_contrast(l);
  update_feature(l);
  match_particles(t, s);
  if (!(l->frame_cpt % l->det_freq))
    if (detect_and_compact(t, s)) return -1;
  if (!(l->frame_cpt % l->filt_freq)) {
    filter_particles(l);
    if (l->with_merge) merge_particles(l);
  }
  l->frame_cpt++;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* C ABI (mirrors the reference harness so the same test code drives both).  */

/* Sizes the tracker accepts: every level at least 16x16, and every flow bin
 * of a level has its bin/2 parent inside the upper level's bins (the
 * reference reads past the upper bin image otherwise, flow_fusion_kernel,
 * tracking_strategies.hpp:596-599). */
int oracle_sizes_ok(int rows, int cols, int nscales) {
  if (nscales < 1 || nscales > 9) return 0;
  int H = rows, W = cols;
  for (int s = 0; s < nscales; s++) {
    if (H < 16 || W < 16) return 0;
    if (s + 1 < nscales) {
      int bh = (H + 7) / 8, bw = (W + 7) / 8, ubh = (H / 2 + 7) / 8, ubw = (W / 2 + 7) / 8;
      if ((bh - 1) / 2 >= ubh || (bw - 1) / 2 >= ubw) return 0;
    }
    H /= 2;
    W /= 2;
  }
  return 1;
}

void* oracle_create(int rows, int cols, int nscales, int threshold, int det_freq, int filt_freq) {
  if (!oracle_sizes_ok(rows, cols, nscales) || det_freq < 1 || filt_freq < 1) return NULL;
  otracker* t = (otracker*)calloc(1, sizeof(otracker));
  if (!t) return NULL;
  t->L = nscales;
  t->lv = (olevel*)calloc(nscales, sizeof(olevel));
  int H = rows, W = cols;
  for (int s = 0; s < nscales; s++) {
    olevel* l = &t->lv[s];
    if (level_alloc(l, H, W)) return NULL;
    l->threshold = threshold;
    l->det_freq = det_freq;
    l->filt_freq = filt_freq;
    l->k = 300;
    l->with_merge = 1;
    l->n_fast = 9;
    l->grad_th = 1;
    H /= 2;
    W /= 2;
  }
  return t;
}

void oracle_destroy(void* h) {
  otracker* t = (otracker*)h;
  if (!t) return;
  for (int s = 0; s < t->L; s++) level_free(&t->lv[s]);
  free(t->lv);
  free(t);
}

/* One setting of scale `s` (every scale when s < 0), the keys of
 * gbt_set_param: 0 threshold, 1 n, 2 detector frequency, 3 filtering
 * frequency, 4 k, 5 with_merge, 6 grad_th.  Callable between frames, as the
 * reference's setters are. */
int oracle_set_param(void* h, int s, int key, int value) {
  otracker* t = (otracker*)h;
  int s0 = s < 0 ? 0 : s, s1 = s < 0 ? t->L : s + 1;
  if (s >= t->L) return -1;
  for (int i = s0; i < s1; i++) {
    olevel* l = &t->lv[i];
    switch (key) {
      case 0: l->threshold = value; break;
      case 1: l->n_fast = value; break;
      case 2: l->det_freq = value; break;
      case 3: l->filt_freq = value; break;
      case 4: l->k = value; break;
      case 5: l->with_merge = value; break;
      case 6: l->grad_th = value; break;
      default: return -1;
    }
  }
  return 0;
}
void oracle_set_k(void* h, int k) { oracle_set_param(h, -1, 4, k); }
void oracle_set_with_merge(void* h, int m) { oracle_set_param(h, -1, 5, m); }
void oracle_set_n(void* h, int n) { oracle_set_param(h, -1, 1, n); }
void oracle_set_detector(void* h, int kind, int step, int grad_th) {
  otracker* t = (otracker*)h;
  t->detector = kind;
  t->step = step;
  oracle_set_param(h, -1, 6, grad_th);
}

int oracle_run(void* h, const uint8_t* frame) {
  otracker* t = (otracker*)h;
  build_pyramid(t, frame);
  for (int s = t->L - 1; s >= 0; s--)
    if (strategy_update(t, s)) return -1;
  return 0;
}

void oracle_dims(void* h, int s, int* rows, int* cols) {
  otracker* t = (otracker*)h;
  *rows = t->lv[s].H;
  *cols = t->lv[s].W;
}

static void dump_u8(const uint8_t* img, int pitch, int bimg, int H, int W, int b, uint8_t* out) {
  size_t k = 0;
  for (int r = -b; r < H + b; r++)
    for (int c = -b; c < W + b; c++) out[k++] = AT(img, pitch, bimg, r, c);
}

void oracle_get_input(void* h, int s, int b, uint8_t* out) {
  olevel* l = &((otracker*)h)->lv[s];
  dump_u8(l->in, l->pin, 6, l->H, l->W, b, out);
}
void oracle_get_s1(void* h, int s, int b, uint8_t* out) {
  olevel* l = &((otracker*)h)->lv[s];
  dump_u8(l->s1, l->ps1, 3, l->H, l->W, b, out);
}
void oracle_get_s2(void* h, int s, int b, uint8_t* out) {
  olevel* l = &((otracker*)h)->lv[s];
  dump_u8(l->s2, l->ps2, 6, l->H, l->W, b, out);
}
void oracle_get_saliency(void* h, int s, uint8_t* out) {
  olevel* l = &((otracker*)h)->lv[s];
  dump_u8(l->sal, l->psal, 1, l->H, l->W, 0, out);
}
void oracle_get_mask(void* h, int s, uint8_t* out) {
  olevel* l = &((otracker*)h)->lv[s];
  dump_u8(l->mask, l->pmask, 4, l->H, l->W, 0, out);
}
void oracle_get_contrast(void* h, int s, uint32_t* out) {
  olevel* l = &((otracker*)h)->lv[s];
  for (size_t i = 0; i < (size_t)l->H * l->W; i++) out[i] = l->contrast[i];
}
void oracle_bins(void* h, int s, int* rows, int* cols) {
  olevel* l = &((otracker*)h)->lv[s];
  *rows = l->BH;
  *cols = l->BW;
}
void oracle_get_bins(void* h, int s, float* flow, uint32_t* count, int32_t* stat_n, int32_t* stat_speed) {
  olevel* l = &((otracker*)h)->lv[s];
  size_t nb = (size_t)l->BH * l->BW;
  memcpy(flow, l->flow, nb * 8);
  memcpy(count, l->msc, nb * 4);
  memcpy(stat_n, l->st_n, nb * 4);
  memcpy(stat_speed, l->st_sp, nb * 8);
}
int oracle_frame_count(void* h, int s) { return ((otracker*)h)->lv[s].frame_cpt; }
int oracle_nparticles(void* h, int s) { return ((otracker*)h)->lv[s].n; }
int oracle_total_particles(void* h) {
  otracker* t = (otracker*)h;
  int n = 0;
  for (int s = 0; s < t->L; s++) n += t->lv[s].n;
  return n;
}
int oracle_compact_has_run(void* h, int s) { return ((otracker*)h)->lv[s].compact_has_run; }
void oracle_get_particles(void* h, int s, float* speed, int16_t* pos, uint16_t* age, uint8_t* feat,
                          int32_t* matches, int* nmatches) {
  olevel* l = &((otracker*)h)->lv[s];
  memcpy(speed, l->speed, (size_t)l->n * 8);
  memcpy(pos, l->pos, (size_t)l->n * 4);
  memcpy(age, l->age, (size_t)l->n * 2);
  for (int i = 0; i < l->n; i++) {
    memcpy(feat + 32 * (size_t)i, l->feat + 16 * (size_t)i, 16);
    memset(feat + 32 * (size_t)i + 16, 255, 16);
  }
  *nmatches = l->compact_has_run ? l->nmatches : 0;
  if (matches && l->compact_has_run) memcpy(matches, l->matches, (size_t)l->nmatches * 4);
}
void oracle_get_sparse(void* h, int s, uint32_t* out) {
  olevel* l = &((otracker*)h)->lv[s];
  for (int r = 0; r < l->H; r++)
    for (int c = 0; c < l->W; c++) out[(size_t)r * l->W + c] = AT(l->sparse, l->psp, 7, r, c);
}
