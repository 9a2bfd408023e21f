/*
 * CPU restatement of cuimg's pyramidal Lucas-Kanade -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates iterative_lk_match_5x5::match (cuimg/tracking2/pyrlk_tracker.hpp:165-334),
 * the bilinear sampler li() (:130-146), the Sobel/8 gradient of the previous
 * level (:910-938), pyrlk_match_particles_kernel's prediction and acceptance
 * (:677-769), get_flow_at (:1027-1063) and recursive_prediction
 * (cuimg/tracking2/predictions.h:61-74), for a pair of frames and a set of
 * fresh points (age 1).  The reference hard-codes window 11, a mask of the 25
 * strongest gradients and 30 iterations; they are parameters here.
 *
 * The reference leaves three cases undefined; this restatement defines them:
 *   - window pixels outside the image are sampled with clamp-to-edge
 *     (the reference leaves gs/as uninitialised there, :189-205);
 *   - get_flow_at returns the identity when the match leaves the level
 *     (the reference falls off the end of the function, :1048-1058);
 *   - ties in the strongest-gradient selection (std::nth_element, :212-228)
 *     are left to the library by the C++ standard; this restatement follows
 *     the selection algorithm of GNU libstdc++ (the library the reference's
 *     CPU build links with g++), so equal norms land on the same side of the
 *     N-th position as in the reference (nth_select below).
 * Pyramids: pyr 0 = the tracker's 2x2 floor-mean pyramid of uint8 levels with
 * the template truncated to uint8 (the reference's gl8u path); pyr 1 = the
 * sigma-1 Gaussian fp32 pyramid with an fp32 template.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

void oracle_gauss_pyramid_f32(const float* in, int H, int W, int L, float* tmp, float* blur, float* work, float* out);

typedef struct {
  int H, W;
  float *prev, *cur, *gr, *gc;
} lk_level;

typedef struct {
  int L, ws, npix, max_iter, u8;
  float eps, kerr;
  lk_level* lv;
} lk_ctx;

static float li(const float* img, int H, int W, float y, float x) {
  int y0 = (int)y, x0 = (int)x; /* truncation, as i_int2(p) */
  float a0 = y - (float)y0, a1 = x - (float)x0;
  int y1 = y0 + 1, x1 = x0 + 1;
  if (y0 < 0) y0 = 0;
  if (y0 > H - 1) y0 = H - 1;
  if (y1 < 0) y1 = 0;
  if (y1 > H - 1) y1 = H - 1;
  if (x0 < 0) x0 = 0;
  if (x0 > W - 1) x0 = W - 1;
  if (x1 < 0) x1 = 0;
  if (x1 > W - 1) x1 = W - 1;
  float v00 = img[(size_t)y0 * W + x0], v10 = img[(size_t)y1 * W + x0];
  float v01 = img[(size_t)y0 * W + x1], v11 = img[(size_t)y1 * W + x1];
  return (1 - a0) * (1 - a1) * v00 + a0 * (1 - a1) * v10 + (1 - a0) * a1 * v01 + a0 * a1 * v11;
}

/* ---------------------------------------------------------------------------
 * nth_select: std::nth_element(idx, idx + nth, idx + n, comp) with
 * comp(a, b) = key[a] > key[b], restated from the introselect algorithm
 * (Musser 1997) as GNU libstdc++ implements it: while more than 3 elements
 * remain, pick the median of (second, middle, last) elements, move it to the
 * front, partition the rest around it with two inward scans that stop on
 * elements not strictly on their side (so equal elements are swapped), and
 * keep the side holding nth; after 2 * floor(log2 n) partitions fall back to a
 * heap selection; finish the last <= 3 elements with an insertion sort.  Only
 * the order of elements that compare equal depends on these steps, and the
 * mask the reference takes (the first N positions) depends on it exactly when
 * equal norms straddle position N.  Counts how often each path ran.
 */
long long oracle_nth_heap_paths = 0;
/* Mask selections, and those where equal norms straddle position N (the
 * case in which the order among equal norms changes the mask). */
long long oracle_lk_selections = 0, oracle_lk_straddles = 0;

static int cmp_gt(const float* key, int a, int b) { return key[a] > key[b]; }

/* Moves `val` up from `hole` towards `top` while its parent compares lower. */
static void heap_up(int* h, int hole, int top, int val, const float* key) {
  int parent = (hole - 1) / 2;
  while (hole > top && cmp_gt(key, h[parent], val)) {
    h[hole] = h[parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  h[hole] = val;
}

/* Sinks the hole at `hole` to a leaf along the preferred children, then
 * places `val` by moving it back up. */
static void heap_down(int* h, int hole, int len, int val, const float* key) {
  const int top = hole;
  int child = hole;
  while (child < (len - 1) / 2) {
    child = 2 * (child + 1);
    if (cmp_gt(key, h[child], h[child - 1])) child--;
    h[hole] = h[child];
    hole = child;
  }
  if ((len & 1) == 0 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    h[hole] = h[child - 1];
    hole = child - 1;
  }
  heap_up(h, hole, top, val, key);
}

static void heap_select(int* a, int middle, int len, const float* key) {
  if (middle > 1)
    for (int parent = (middle - 2) / 2;; parent--) {
      heap_down(a, parent, middle, a[parent], key);
      if (parent == 0) break;
    }
  for (int i = middle; i < len; i++)
    if (cmp_gt(key, a[i], a[0])) {
      int v = a[i];
      a[i] = a[0];
      heap_down(a, 0, middle, v, key);
    }
}

static void swap_int(int* a, int* b) {
  int t = *a;
  *a = *b;
  *b = t;
}

static void nth_select(int* a, int n, int nth, const float* key) {
  if (n == 0 || nth == n) return;
  int first = 0, last = n, depth = 0;
  for (int m = n; m > 1; m >>= 1) depth++;
  depth *= 2;
  while (last - first > 3) {
    if (depth == 0) {
      oracle_nth_heap_paths++;
      heap_select(a + first, nth + 1 - first, last - first, key);
      swap_int(&a[first], &a[nth]);
      return;
    }
    depth--;
    /* median of a[first+1], a[mid], a[last-1] to a[first] */
    int x = first + 1, y = first + (last - first) / 2, z = last - 1, m;
    if (cmp_gt(key, a[x], a[y]))
      m = cmp_gt(key, a[y], a[z]) ? y : (cmp_gt(key, a[x], a[z]) ? z : x);
    else
      m = cmp_gt(key, a[x], a[z]) ? x : (cmp_gt(key, a[y], a[z]) ? z : y);
    swap_int(&a[first], &a[m]);
    /* partition [first+1, last) around the pivot a[first] */
    const int piv = a[first];
    int lo = first + 1, hi = last;
    for (;;) {
      while (cmp_gt(key, a[lo], piv)) lo++;
      hi--;
      while (cmp_gt(key, piv, a[hi])) hi--;
      if (!(lo < hi)) break;
      swap_int(&a[lo], &a[hi]);
      lo++;
    }
    if (lo <= nth)
      first = lo;
    else
      last = lo;
  }
  /* insertion sort of [first, last) */
  for (int i = first + 1; i < last; i++) {
    int v = a[i];
    if (cmp_gt(key, v, a[first])) {
      for (int j = i; j > first; j--) a[j] = a[j - 1];
      a[first] = v;
    } else {
      int j = i;
      while (cmp_gt(key, v, a[j - 1])) {
        a[j] = a[j - 1];
        j--;
      }
      a[j] = v;
    }
  }
}

/* Exported for the tests: runs nth_select on idx[0..n) (initially any
 * permutation) with `key`. */
void oracle_nth_select(int* idx, int n, int nth, const float* key) { nth_select(idx, n, nth, key); }

static int box_has(int H, int W, int b, float y, float x) { /* (domain - border(b)).has(i_int2(p)) */
  int r = (int)y, c = (int)x;
  return r >= b && r <= H - b - 1 && c >= b && c <= W - b - 1;
}

/* iterative_lk_match_5x5::match.  Returns 0 on rejection (tr = (-1,-1),
 * err = 1000 as in the reference). */
static int lk_match(const lk_ctx* k, const lk_level* l, const float p[2], const float pred_tr[2], float tr[2],
                    float* err_out) {
  const int ws = k->ws, hws = ws / 2, n = ws * ws;
  float* gsr = (float*)malloc(sizeof(float) * n);
  float* gsc = (float*)malloc(sizeof(float) * n);
  float* as = (float*)malloc(sizeof(float) * n);
  float* nrm = (float*)malloc(sizeof(float) * n);
  char* mask = (char*)calloc(n, 1);
  float pred[2] = {p[0] + pred_tr[0], p[1] + pred_tr[1]};
  float v[2] = {pred[0], pred[1]};
  int ok = 1;
  for (int i = 0, r = -hws; r <= hws; r++)
    for (int c = -hws; c <= hws; c++, i++) {
      float y = p[0] + (float)r, x = p[1] + (float)c;
      gsr[i] = li(l->gr, l->H, l->W, y, x);
      gsc[i] = li(l->gc, l->H, l->W, y, x);
      float a = li(l->prev, l->H, l->W, y, x);
      as[i] = k->u8 ? (float)(unsigned char)a : a;
      nrm[i] = sqrtf(gsr[i] * gsr[i] + gsc[i] * gsc[i]);
    }
  /* The npix strongest gradients: the first N window indexes after
   * nth_element (:207-228). */
  int N = k->npix < n ? k->npix : n;
  int* idx = (int*)malloc(sizeof(int) * n);
  for (int i = 0; i < n; i++) idx[i] = i;
  nth_select(idx, n, N, nrm);
  for (int i = 0; i < N; i++) mask[idx[i]] = 1;
  if (N > 0 && N < n) {
    float t = nrm[idx[0]];
    for (int i = 1; i < N; i++) t = nrm[idx[i]] < t ? nrm[idx[i]] : t;
    int straddle = 0;
    for (int i = N; i < n; i++) straddle |= nrm[idx[i]] == t;
    oracle_lk_selections++;
    oracle_lk_straddles += straddle;
  }
  free(idx);
  float G00 = 0, G01 = 0, G11 = 0;
  for (int i = 0; i < n; i++)
    if (mask[i]) {
      G00 += gsr[i] * gsr[i];
      G01 += gsr[i] * gsc[i];
      G11 += gsc[i] * gsc[i];
    }
  /* eigenvalues of the symmetric 2x2 G */
  float tr2 = (G00 + G11) * 0.5f, det = G00 * G11 - G01 * G01;
  float disc = sqrtf(fmaxf(tr2 * tr2 - det, 0.f));
  float e1 = fabsf(tr2 + disc), e2 = fabsf(tr2 - disc);
  float min_ev = e1 < e2 ? e1 : e2;
  if (min_ev < 0.0001f) ok = 0;
  float i00 = 0, i01 = 0, i11 = 0;
  if (ok) {
    i00 = G11 / det;
    i01 = -G01 / det;
    i11 = G00 / det;
  }
  int cpt = 0;
  if (ok) {
    float nk0 = 1.f, nk1 = 1.f;
    for (int it = 0; it < k->max_iter && sqrtf(nk0 * nk0 + nk1 * nk1) >= k->eps; it++) {
      float b0 = 0, b1 = 0;
      cpt = 0;
      for (int i = 0, r = -hws; r <= hws; r++)
        for (int c = -hws; c <= hws; c++, i++)
          if (mask[i]) {
            float dt = as[i] - li(l->cur, l->H, l->W, v[0] + (float)r, v[1] + (float)c);
            b0 += gsr[i] * dt;
            b1 += gsc[i] * dt;
            cpt++;
          }
      nk0 = i00 * b0 + i01 * b1;
      nk1 = i01 * b0 + i11 * b1;
      v[0] += nk0;
      v[1] += nk1;
      float d0 = pred[0] - v[0], d1 = pred[1] - v[1];
      if (sqrtf(d0 * d0 + d1 * d1) > (float)(ws * 4)) {
        ok = 0;
        break;
      }
      if (!box_has(l->H, l->W, 3, v[0], v[1])) {
        ok = 0;
        break;
      }
    }
  }
  if (ok) {
    /* Mean absolute residual with the reference's window index
     * (r+hws)*hws + (c+hws) and its running counter (:320-331). */
    float e = 0;
    for (int r = -hws; r <= hws; r++)
      for (int c = -hws; c <= hws; c++) {
        int i = (r + hws) * hws + (c + hws);
        e += fabsf(as[i] - li(l->cur, l->H, l->W, v[0] + (float)r, v[1] + (float)c));
        cpt++;
      }
    tr[0] = v[0] - p[0];
    tr[1] = v[1] - p[1];
    *err_out = e / (float)cpt;
  } else {
    tr[0] = -1.f;
    tr[1] = -1.f;
    *err_out = 1000.f;
  }
  free(gsr);
  free(gsc);
  free(as);
  free(nrm);
  free(mask);
  return ok;
}

/* get_flow_at of level l at point q (level coordinates). */
static void flow_at(const lk_ctx* k, int l, const float q[2], float out[2]) {
  const lk_level* lv = &k->lv[l];
  float pred_tr[2] = {0.f, 0.f};
  if (l + 1 < k->L) {
    float q2[2] = {q[0] / 2.f, q[1] / 2.f}, u[2];
    flow_at(k, l + 1, q2, u);
    pred_tr[0] = 2.f * u[0];
    pred_tr[1] = 2.f * u[1];
  }
  float pred[2] = {q[0] + pred_tr[0], q[1] + pred_tr[1]};
  out[0] = out[1] = 0.f;
  if (!box_has(lv->H, lv->W, 3, pred[0], pred[1])) return;
  float tr[2], err;
  lk_match(k, lv, q, pred_tr, tr, &err);
  if (box_has(lv->H, lv->W, 0, q[0] + tr[0], q[1] + tr[1])) {
    out[0] = tr[0];
    out[1] = tr[1];
  }
}

static void sobel8(const float* img, int H, int W, float* gr, float* gc) {
  memset(gr, 0, sizeof(float) * H * W);
  memset(gc, 0, sizeof(float) * H * W);
  for (int r = 1; r < H - 1; r++)
    for (int c = 1; c < W - 1; c++) {
#define P(dr, dc) img[(size_t)(r + (dr)) * W + (c + (dc))]
      gr[(size_t)r * W + c] = (P(1, -1) + 2 * P(1, 0) + P(1, 1) - P(-1, -1) - 2 * P(-1, 0) - P(-1, 1)) / 8.f;
      gc[(size_t)r * W + c] = (P(-1, 1) + 2 * P(0, 1) + P(1, 1) - P(-1, -1) - 2 * P(0, -1) - P(1, -1)) / 8.f;
#undef P
    }
}

static void box_down(const float* in, int H, int W, float* out) {
  int H2 = H / 2, W2 = W / 2;
  for (int r = 0; r < H2; r++)
    for (int c = 0; c < W2; c++) {
      int s = (int)in[(size_t)(2 * r) * W + 2 * c] + (int)in[(size_t)(2 * r) * W + 2 * c + 1] +
              (int)in[(size_t)(2 * r + 1) * W + 2 * c] + (int)in[(size_t)(2 * r + 1) * W + 2 * c + 1];
      out[(size_t)r * W2 + c] = (float)(s / 4);
    }
}

/* Tracks `n` points (row, col; level-0 coordinates) from `prev` to `cur`
 * (H x W floats; integral values for pyr 0).  Writes the new positions,
 * status (1 accepted) and the match error. */
int oracle_lk_track(const float* prev, const float* cur, int H, int W, int L, int pyr, int ws, int npix,
                    int max_iter, float eps, float kerr, const float* pts, int n, float* out, int* status,
                    float* err) {
  if (L < 1 || ws < 3 || !(ws & 1)) return -1;
  lk_ctx k = {L, ws, npix, max_iter, pyr == 0, eps, kerr, NULL};
  k.lv = (lk_level*)calloc(L, sizeof(lk_level));
  int h = H, w = W;
  for (int l = 0; l < L; l++) {
    k.lv[l].H = h;
    k.lv[l].W = w;
    size_t np = (size_t)h * w;
    k.lv[l].prev = (float*)malloc(np * 4);
    k.lv[l].cur = (float*)malloc(np * 4);
    k.lv[l].gr = (float*)malloc(np * 4);
    k.lv[l].gc = (float*)malloc(np * 4);
    h /= 2;
    w /= 2;
  }
  memcpy(k.lv[0].prev, prev, (size_t)H * W * 4);
  memcpy(k.lv[0].cur, cur, (size_t)H * W * 4);
  if (pyr == 0) {
    for (int l = 1; l < L; l++) {
      box_down(k.lv[l - 1].prev, k.lv[l - 1].H, k.lv[l - 1].W, k.lv[l].prev);
      box_down(k.lv[l - 1].cur, k.lv[l - 1].H, k.lv[l - 1].W, k.lv[l].cur);
    }
  } else if (L > 1) {
    size_t np = (size_t)H * W, tot = 0;
    for (int l = 1; l < L; l++) tot += (size_t)k.lv[l].H * k.lv[l].W;
    float *tmp = (float*)malloc(np * 4), *blur = (float*)malloc(np * 4), *work = (float*)malloc(np * 4);
    float* o = (float*)malloc(tot * 4);
    for (int which = 0; which < 2; which++) {
      oracle_gauss_pyramid_f32(which ? cur : prev, H, W, L, tmp, blur, work, o);
      size_t off = 0;
      for (int l = 1; l < L; l++) {
        size_t m = (size_t)k.lv[l].H * k.lv[l].W;
        memcpy(which ? k.lv[l].cur : k.lv[l].prev, o + off, m * 4);
        off += m;
      }
    }
    free(tmp);
    free(blur);
    free(work);
    free(o);
  }
  for (int l = 0; l < L; l++) sobel8(k.lv[l].prev, k.lv[l].H, k.lv[l].W, k.lv[l].gr, k.lv[l].gc);

  for (int i = 0; i < n; i++) {
    float p[2] = {pts[2 * i], pts[2 * i + 1]};
    status[i] = 0;
    err[i] = 1000.f;
    out[2 * i] = p[0];
    out[2 * i + 1] = p[1];
    const lk_level* l0 = &k.lv[0];
    if (!box_has(l0->H, l0->W, 3, p[0], p[1])) continue;
    float pred_tr[2] = {0.f, 0.f};
    if (L > 1) {
      float q[2] = {p[0] / 2.f, p[1] / 2.f}, u[2];
      flow_at(&k, 1, q, u);
      pred_tr[0] = 2.f * u[0];
      pred_tr[1] = 2.f * u[1];
    }
    float pred[2] = {p[0] + pred_tr[0], p[1] + pred_tr[1]};
    if (!box_has(l0->H, l0->W, 3, pred[0], pred[1])) continue;
    float tr[2], e;
    lk_match(&k, l0, p, pred_tr, tr, &e);
    float m0 = (float)(int)(p[0] + tr[0]), m1 = (float)(int)(p[1] + tr[1]);
    float d0 = m0 - pred[0], d1 = m1 - pred[1];
    if (box_has(l0->H, l0->W, 3, p[0] + tr[0], p[1] + tr[1]) && e < kerr && sqrtf(d0 * d0 + d1 * d1) < 160.f) {
      status[i] = 1;
      out[2 * i] = p[0] + tr[0];
      out[2 * i + 1] = p[1] + tr[1];
    }
    err[i] = e;
  }
  for (int l = 0; l < L; l++) {
    free(k.lv[l].prev);
    free(k.lv[l].cur);
    free(k.lv[l].gr);
    free(k.lv[l].gc);
  }
  free(k.lv);
  return 0;
}

/* ===========================================================================
 * The reference's pyramidal LK tracker strategy over frames:
 * tracker<pyrlk_cpu<fast_detector<cpu>, iterative_lk_match_5x5>>
 * (cuimg/tracking2/pyrlk_tracker.h:16-82, pyrlk_tracker.hpp:772-1063), which
 * the reference never instantiates.  Per frame and scale, coarsest first
 * (tracker.hpp:83-91), pyrlk_cpu::update (:833-875):
 *   - prev_input_ = the previous frame's input_ (the first frame: the frame);
 *     input_ = a fresh copy of the tracker's level (see below);
 *   - frames > 0: match_particles (:902-971): the sparse index emptied, the
 *     Sobel/8 gradient of prev_input_, then pyrlk_match_particles_kernel
 *     (:677-769) over the slots in index order: the prediction through the
 *     upper scale's get_flow_at (:1027-1063; the top scale uses the motion
 *     prediction, predictions.h:61-74), the LK match, the acceptance and
 *     kernel_particle_container::move (particle_container.hpp:422-466);
 *   - detector frames: create_detector_mask (:878-887: every slot's position
 *     and its 8 neighbours, dead slots included), the FAST saliency
 *     (fast_detector.hpp:296-313), new_particles (:217-262) and compact
 *     (particle_container.hpp:215-252);
 *   - filtering frames: filter_bad_particles_kernel (tracking_strategies.hpp:
 *     482-523), which never removes a particle here because the strategy's
 *     multiscale_count_ image stays zero (it is only ever memset), then
 *     merge_trajectories (merge_trajectories.h:10-35) in index order.
 * input_ is `host_image2d(in.domain(), in.border())` filled by
 * copy(in, input_), which for equal borders copies nrows * pitch bytes from
 * the start of the allocation (cuimg/copy.h:30-40, host_image2d.hpp:76-110):
 * the top border rows and the domain rows 0 .. H - 1 - b come over (b = 3,
 * the FAST detector's border, pyrlk_tracker.hpp:822-827); rows H - b .. H - 1
 * and the bottom border stay zero.  The LK and the detector read that image.
 * Window samples outside the domain are clamped to the edge (undefined in the
 * reference), as in the LK restatement above.
 * ======================================================================== */
uint8_t oracle_fast_saliency_at(const uint8_t* p00, int pitch, int r, int c, int n_, int th);

#define PK_B 3 /* the tracker input's border: fast_detector::border_needed() */
#define PK_MB 4 /* the detector mask's border */
static const int PK_C8[8][2] = {{-1, 1}, {0, 1}, {1, 1}, {-1, 0}, {1, 0}, {-1, -1}, {0, -1}, {1, -1}};

typedef struct {
  int H, W, ipitch;      /* ipitch: input_'s row pitch ((W + 2b) rounded up to 4 bytes) */
  uint8_t* lvl;          /* the tracker's level (H x W) */
  uint8_t* inb;          /* input_: (H + 2b) rows of ipitch bytes */
  float *cur, *prev, *gr, *gc; /* H x W */
  uint8_t* mask;         /* (H + 2 PK_MB) x (W + 2 PK_MB) */
  uint8_t* sal;          /* H x W */
  uint8_t* newpts;       /* H x W */
  uint32_t* sparse;      /* H x W, 0xFFFFFFFF = none */
  int n, cap, nmatches, compact_has_run, frame_cpt;
  float *pos, *speed;    /* 2 per slot */
  uint16_t* age;
  int32_t* matches;
  int threshold, n_fast, det_freq, filt_freq, k, with_merge;
} pk_level;

typedef struct {
  int L;
  pk_level* lv;
  lk_level* lkl; /* the LK's view of every scale (prev, cur, gradient) */
  lk_ctx lk;
} pk_tracker;

static int pk_reserve(pk_level* l, int n) {
  if (n <= l->cap) return 0;
  int cap = l->cap ? l->cap : 1024;
  while (cap < n) cap *= 2;
  float* p = (float*)realloc(l->pos, sizeof(float) * 2 * cap);
  float* sp = (float*)realloc(l->speed, sizeof(float) * 2 * cap);
  uint16_t* a = (uint16_t*)realloc(l->age, sizeof(uint16_t) * cap);
  int32_t* m = (int32_t*)realloc(l->matches, sizeof(int32_t) * cap);
  if (!p || !sp || !a || !m) return -1;
  l->pos = p;
  l->speed = sp;
  l->age = a;
  l->matches = m;
  l->cap = cap;
  return 0;
}

void* oracle_pyrlk_create(int rows, int cols, int nscales, int threshold, int det_freq, int filt_freq) {
  if (nscales < 1 || nscales > 9 || det_freq < 1 || filt_freq < 1) return NULL;
  pk_tracker* t = (pk_tracker*)calloc(1, sizeof(pk_tracker));
  t->L = nscales;
  t->lv = (pk_level*)calloc(nscales, sizeof(pk_level));
  t->lkl = (lk_level*)calloc(nscales, sizeof(lk_level));
  int H = rows, W = cols;
  for (int s = 0; s < nscales; s++) {
    pk_level* l = &t->lv[s];
    if (H < 16 || W < 16) return NULL;
    l->H = H;
    l->W = W;
    l->ipitch = (W + 2 * PK_B + 3) / 4 * 4;
    size_t np = (size_t)H * W;
    l->lvl = (uint8_t*)calloc(np, 1);
    l->inb = (uint8_t*)calloc((size_t)(H + 2 * PK_B) * l->ipitch, 1);
    l->cur = (float*)calloc(np, 4);
    l->prev = (float*)calloc(np, 4);
    l->gr = (float*)calloc(np, 4);
    l->gc = (float*)calloc(np, 4);
    l->mask = (uint8_t*)calloc((size_t)(H + 2 * PK_MB) * (W + 2 * PK_MB), 1);
    l->sal = (uint8_t*)calloc(np, 1);
    l->newpts = (uint8_t*)calloc(np, 1);
    l->sparse = (uint32_t*)malloc(np * 4);
    memset(l->sparse, 0xFF, np * 4);
    l->threshold = threshold;
    l->n_fast = 9;
    l->det_freq = det_freq;
    l->filt_freq = filt_freq;
    l->k = 300;
    l->with_merge = 1;
    t->lkl[s].H = H;
    t->lkl[s].W = W;
    t->lkl[s].prev = l->prev;
    t->lkl[s].cur = l->cur;
    t->lkl[s].gr = l->gr;
    t->lkl[s].gc = l->gc;
    H /= 2;
    W /= 2;
  }
  lk_ctx k = {nscales, 11, 25, 30, 1, 0.1f, 300.f, t->lkl};
  t->lk = k;
  return t;
}

void oracle_pyrlk_destroy(void* h) {
  pk_tracker* t = (pk_tracker*)h;
  if (!t) return;
  for (int s = 0; s < t->L; s++) {
    pk_level* l = &t->lv[s];
    free(l->lvl);
    free(l->inb);
    free(l->cur);
    free(l->prev);
    free(l->gr);
    free(l->gc);
    free(l->mask);
    free(l->sal);
    free(l->newpts);
    free(l->sparse);
    free(l->pos);
    free(l->speed);
    free(l->age);
    free(l->matches);
  }
  free(t->lv);
  free(t->lkl);
  free(t);
}

/* Settings of scale s (every scale when s < 0), keys as oracle_set_param:
 * 0 threshold, 1 n, 2 detector frequency, 3 filtering frequency, 4 k,
 * 5 with_merge. */
int oracle_pyrlk_set_param(void* h, int s, int key, int value) {
  pk_tracker* t = (pk_tracker*)h;
  if (s >= t->L) return -1;
  for (int i = s < 0 ? 0 : s; i < (s < 0 ? t->L : s + 1); i++) {
    pk_level* l = &t->lv[i];
    switch (key) {
      case 0: l->threshold = value; break;
      case 1: l->n_fast = value; break;
      case 2: l->det_freq = value; break;
      case 3: l->filt_freq = value; break;
      case 4: l->k = value; break;
      case 5: l->with_merge = value; break;
      default: return -1;
    }
  }
  return 0;
}

#define PK_IN(l, r, c) ((l)->inb[(size_t)((r) + PK_B) * (l)->ipitch + ((c) + PK_B)])
#define PK_MASK(l, r, c) ((l)->mask[(size_t)((r) + PK_MB) * ((l)->W + 2 * PK_MB) + ((c) + PK_MB)])

/* input_ of a scale from the tracker's level (see the header above). */
static void pk_make_input(pk_level* l) {
  const int H = l->H, W = l->W, b = PK_B;
  memset(l->inb, 0, (size_t)(H + 2 * b) * l->ipitch);
  for (int r = -b; r < H - b; r++) /* the copied rows: bordered rows -b .. H - b - 1 */
    for (int c = -b; c < W + b; c++) {
      int rr = r < 0 ? 0 : r, cc = c < 0 ? 0 : (c > W - 1 ? W - 1 : c);
      PK_IN(l, r, c) = l->lvl[(size_t)rr * W + cc];
    }
}

static void pk_match(pk_tracker* t, int s) {
  pk_level* l = &t->lv[s];
  const int H = l->H, W = l->W;
  memset(l->sparse, 0xFF, (size_t)H * W * 4);
  l->compact_has_run = 0;
  sobel8(l->prev, H, W, l->gr, l->gc);
  lk_ctx k = t->lk;
  k.kerr = (float)l->k;
  for (int i = 0; i < l->n; i++) {
    float p[2] = {l->pos[2 * i], l->pos[2 * i + 1]};
    if (l->age[i] == 0 || !box_has(H, W, 3, p[0], p[1])) {
      l->age[i] = 0;
      continue;
    }
    float pred_tr[2] = {0.f, 0.f};
    if (s + 1 < t->L) {
      float q[2] = {p[0] / 2.f, p[1] / 2.f}, u[2];
      flow_at(&k, s + 1, q, u);
      pred_tr[0] = 2.f * u[0];
      pred_tr[1] = 2.f * u[1];
    } else if (l->age[i] != 1) {
      pred_tr[0] = l->speed[2 * i];
      pred_tr[1] = l->speed[2 * i + 1];
    }
    float pred[2] = {p[0] + pred_tr[0], p[1] + pred_tr[1]};
    if (!box_has(H, W, 3, pred[0], pred[1])) {
      l->age[i] = 0;
      continue;
    }
    float tr[2], e;
    lk_match(&k, &t->lkl[s], p, pred_tr, tr, &e);
    float m0 = (float)(int)(p[0] + tr[0]), m1 = (float)(int)(p[1] + tr[1]);
    float d0 = m0 - pred[0], d1 = m1 - pred[1];
    if (box_has(H, W, 3, p[0] + tr[0], p[1] + tr[1]) && e < (float)l->k && sqrtf(d0 * d0 + d1 * d1) < 160.f) {
      l->age[i]++;
      l->speed[2 * i] = tr[0];
      l->speed[2 * i + 1] = tr[1];
      l->pos[2 * i] = p[0] + tr[0];
      l->pos[2 * i + 1] = p[1] + tr[1];
      l->sparse[(size_t)(int)l->pos[2 * i] * W + (int)l->pos[2 * i + 1]] = (uint32_t)i;
    } else {
      l->age[i] = 0;
    }
  }
}

static int pk_detect_and_compact(pk_level* l) {
  const int H = l->H, W = l->W;
  memset(l->mask, 255, (size_t)(H + 2 * PK_MB) * (W + 2 * PK_MB));
  for (int i = 0; i < l->n; i++) { /* every slot, dead ones included */
    int pr = (int)l->pos[2 * i], pc = (int)l->pos[2 * i + 1];
    PK_MASK(l, pr, pc) = 0;
    for (int k = 0; k < 8; k++) PK_MASK(l, pr + PK_C8[k][0], pc + PK_C8[k][1]) = 0;
  }
  memset(l->sal, 0, (size_t)H * W);
  for (int r = 0; r < H; r++)
    for (int c = 0; c < W; c++)
      if (PK_MASK(l, r, c) != 0)
        l->sal[(size_t)r * W + c] = oracle_fast_saliency_at(&PK_IN(l, 0, 0), l->ipitch, r, c, l->n_fast, l->threshold);
  memset(l->newpts, 0, (size_t)H * W);
  for (int tr = 0; tr < H / 3; tr++)
    for (int tc = 0; tc < W / 3; tc++) {
      int pr = tr * 3 + 1, pc = tc * 3 + 1, skip = 0;
      for (int r = 0; r < 3 && !skip; r++)
        for (int c = 0; c < 3; c++)
          if (pr + r < H && pc + c < W && l->sparse[(size_t)(pr + r) * W + pc + c] != 0xFFFFFFFFu) {
            skip = 1;
            break;
          }
      if (skip) continue;
      float vmax = l->sal[(size_t)pr * W + pc];
      int mr = pr, mc = pc;
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
          if (pr + r < H && pc + c < W) {
            float v = l->sal[(size_t)(pr + r) * W + pc + c];
            if (vmax < v) {
              vmax = v;
              mr = pr + r;
              mc = pc + c;
            }
          }
      if (vmax < (float)l->threshold) continue;
      l->newpts[(size_t)mr * W + mc] = 1;
    }
  for (int r = 3; r <= H - 4; r++)
    for (int c = 3; c <= W - 4; c++)
      if (l->newpts[(size_t)r * W + c]) {
        if (pk_reserve(l, l->n + 1)) return -1;
        int i = l->n++;
        l->age[i] = 1;
        l->speed[2 * i] = l->speed[2 * i + 1] = 0.f;
        l->pos[2 * i] = (float)r;
        l->pos[2 * i + 1] = (float)c;
        l->sparse[(size_t)r * W + c] = (uint32_t)i;
      }
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
    l->sparse[(size_t)(int)l->pos[2 * o] * W + (int)l->pos[2 * o + 1]] = (uint32_t)o;
    l->matches[i] = o;
    o++;
  }
  l->n = o;
  return 0;
}

static void pk_merge(pk_level* l) {
  const int W = l->W;
  for (int i = 0; i < l->n; i++) {
    if (l->age[i] == 0) continue;
    int pr = (int)l->pos[2 * i], pc = (int)l->pos[2 * i + 1];
    for (int k = 0; k < 8; k++) {
      uint32_t j = l->sparse[(size_t)(pr + PK_C8[k][0]) * W + (pc + PK_C8[k][1])];
      if (j == 0xFFFFFFFFu) continue;
      float dx = l->speed[2 * i] - l->speed[2 * j], dy = l->speed[2 * i + 1] - l->speed[2 * j + 1];
      if ((int)l->age[j] > (int)l->age[i] + 2 && sqrtf(dx * dx + dy * dy) < 2.f) {
        l->age[j] = 0;
        break;
      }
    }
  }
}

int oracle_pyrlk_run(void* h, const uint8_t* frame) {
  pk_tracker* t = (pk_tracker*)h;
  memcpy(t->lv[0].lvl, frame, (size_t)t->lv[0].H * t->lv[0].W);
  for (int s = 1; s < t->L; s++) { /* tracker::subsample_input: 2x2 floor means of the level below */
    pk_level *a = &t->lv[s - 1], *o = &t->lv[s];
    for (int r = 0; r < o->H; r++)
      for (int c = 0; c < o->W; c++) {
        int v = a->lvl[(size_t)(2 * r) * a->W + 2 * c] + a->lvl[(size_t)(2 * r) * a->W + 2 * c + 1] +
                a->lvl[(size_t)(2 * r + 1) * a->W + 2 * c] + a->lvl[(size_t)(2 * r + 1) * a->W + 2 * c + 1];
        o->lvl[(size_t)r * o->W + c] = (uint8_t)(v / 4);
      }
  }
  for (int s = t->L - 1; s >= 0; s--) {
    pk_level* l = &t->lv[s];
    const size_t np = (size_t)l->H * l->W;
    if (l->frame_cpt > 0)
      memcpy(l->prev, l->cur, np * 4); /* copy(input_, prev_input_) before input_ is replaced */
    else
      for (size_t i = 0; i < np; i++) l->prev[i] = (float)l->lvl[i];
    pk_make_input(l);
    for (int r = 0; r < l->H; r++)
      for (int c = 0; c < l->W; c++) l->cur[(size_t)r * l->W + c] = (float)PK_IN(l, r, c);
    if (l->frame_cpt > 0) pk_match(t, s);
    if (!(l->frame_cpt % l->det_freq))
      if (pk_detect_and_compact(l)) return -1;
    if (!(l->frame_cpt % l->filt_freq) && l->with_merge) pk_merge(l);
    l->frame_cpt++;
  }
  return 0;
}

int oracle_pyrlk_nparticles(void* h, int s) { return ((pk_tracker*)h)->lv[s].n; }

/* Particle state of scale s: pos and speed (2 floats each), age; matches of
 * the last compaction (*nmatches of them) and whether this frame compacted. */
void oracle_pyrlk_get(void* h, int s, float* pos, float* speed, uint16_t* age, int32_t* matches, int* nmatches,
                      int* compact_has_run) {
  pk_level* l = &((pk_tracker*)h)->lv[s];
  if (pos) memcpy(pos, l->pos, (size_t)l->n * 8);
  if (speed) memcpy(speed, l->speed, (size_t)l->n * 8);
  if (age) memcpy(age, l->age, (size_t)l->n * 2);
  if (nmatches) *nmatches = l->nmatches;
  if (matches) memcpy(matches, l->matches, (size_t)l->nmatches * 4);
  if (compact_has_run) *compact_has_run = l->compact_has_run;
}

void oracle_pyrlk_get_sparse(void* h, int s, uint32_t* out) {
  pk_level* l = &((pk_tracker*)h)->lv[s];
  memcpy(out, l->sparse, (size_t)l->H * l->W * 4);
}
