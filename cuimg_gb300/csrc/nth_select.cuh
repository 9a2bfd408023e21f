// The reference's std::nth_element order among equal keys, for the LK
// strongest-gradient selection (cuimg/tracking2/pyrlk_tracker.hpp:207-228).
//
// The C++ standard leaves it to the library which of several equal keys end
// up before position nth; the reference's CPU build uses GNU libstdc++'s
// introselect (Musser 1997): while more than 3 elements remain, the median of
// the second, middle and last elements is moved to the front and the rest is
// partitioned around it by two inward scans that stop on elements not
// strictly on their side (so equal elements are exchanged); after
// 2 * floor(log2 n) partitions it falls back to a heap selection; the last
// <= 3 elements are insertion-sorted.  nth_select replays those steps on
// packed words (key << 32 | payload) ordered by key, largest first, the
// reference's comparator `norml2(gs[a]) > norml2(gs[b])`.
//
// Compiles as host code too (no CUDA qualifiers outside nvcc), so the CPU
// tests check this very code against std::nth_element.
#pragma once

#if defined(__CUDACC__)
#define GBT_HD __host__ __device__
#define GBT_NOINLINE __noinline__
#else
#define GBT_HD
#define GBT_NOINLINE
#endif

namespace gbt_sel {

GBT_HD inline bool ord_gt(unsigned long long a, unsigned long long b) { return (a >> 32) > (b >> 32); }

GBT_HD inline void heap_up(unsigned long long* h, int hole, int top, unsigned long long val) {
  int parent = (hole - 1) / 2;
  while (hole > top && ord_gt(h[parent], val)) {
    h[hole] = h[parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  h[hole] = val;
}

GBT_HD inline void heap_down(unsigned long long* h, int hole, int len, unsigned long long val) {
  const int top = hole;
  int child = hole;
  while (child < (len - 1) / 2) {
    child = 2 * (child + 1);
    if (ord_gt(h[child], h[child - 1])) child--;
    h[hole] = h[child];
    hole = child;
  }
  if ((len & 1) == 0 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    h[hole] = h[child - 1];
    hole = child - 1;
  }
  heap_up(h, hole, top, val);
}

GBT_HD GBT_NOINLINE inline void nth_select(unsigned long long* a, int n, int nth) {
  if (n == 0 || nth >= n) return;
  int first = 0, last = n, depth = 0;
  for (int m = n; m > 1; m >>= 1) depth++;
  depth *= 2;
  while (last - first > 3) {
    if (depth == 0) {
      unsigned long long* h = a + first;
      const int middle = nth + 1 - first, len = last - first;
      if (middle > 1)
        for (int parent = (middle - 2) / 2;; parent--) {
          heap_down(h, parent, middle, h[parent]);
          if (parent == 0) break;
        }
      for (int i = middle; i < len; i++)
        if (ord_gt(h[i], h[0])) {
          const unsigned long long v = h[i];
          h[i] = h[0];
          heap_down(h, 0, middle, v);
        }
      const unsigned long long t = a[first];
      a[first] = a[nth];
      a[nth] = t;
      return;
    }
    depth--;
    const int x = first + 1, y = first + (last - first) / 2, z = last - 1;
    const unsigned long long ax = a[x], ay = a[y], az = a[z];
    int m;
    if (ord_gt(ax, ay))
      m = ord_gt(ay, az) ? y : (ord_gt(ax, az) ? z : x);
    else
      m = ord_gt(ax, az) ? x : (ord_gt(ay, az) ? z : y);
    const unsigned long long piv = a[m];
    a[m] = a[first];
    a[first] = piv;
    int lo = first + 1, hi = last;
    for (;;) {
      while (ord_gt(a[lo], piv)) lo++;
      hi--;
      while (ord_gt(piv, a[hi])) hi--;
      if (!(lo < hi)) break;
      const unsigned long long t = a[lo];
      a[lo] = a[hi];
      a[hi] = t;
      lo++;
    }
    if (lo <= nth)
      first = lo;
    else
      last = lo;
  }
  for (int i = first + 1; i < last; i++) {
    const unsigned long long v = a[i];
    int j = i;
    if (ord_gt(v, a[first])) {
      for (; j > first; j--) a[j] = a[j - 1];
    } else {
      while (ord_gt(v, a[j - 1])) {
        a[j] = a[j - 1];
        j--;
      }
    }
    a[j] = v;
  }
}

}  // namespace gbt_sel
