/*
 * Plain C (C99) translation unit over include/cuimg_gb300.h: shows the header
 * is valid C and prints the struct layouts and the host-only calls' results,
 * which tests/test_cpp_boundary.py compares with the ctypes mirror
 * (cuimg_gb300/_native.py).  Needs no GPU.
 */
#include <stddef.h>
#include <stdio.h>

#include "cuimg_gb300.h"

#define FIELD(T, f) printf("%s.%s %zu\n", #T, #f, offsetof(T, f))

int main(void) {
  gbt_config c;
  gbt_lk_params p;
  float taps[2 * 12 + 1];
  int32_t radius = 0;
  printf("sizeof.gbt_config %zu\n", sizeof(gbt_config));
  FIELD(gbt_config, rows);
  FIELD(gbt_config, cols);
  FIELD(gbt_config, nscales);
  FIELD(gbt_config, detector_threshold);
  FIELD(gbt_config, detector_n);
  FIELD(gbt_config, detector_frequency);
  FIELD(gbt_config, filtering_frequency);
  FIELD(gbt_config, k);
  FIELD(gbt_config, with_merge);
  FIELD(gbt_config, detector);
  FIELD(gbt_config, detector_step);
  FIELD(gbt_config, detector_grad_th);
  FIELD(gbt_config, matcher);
  printf("sizeof.gbt_lk_params %zu\n", sizeof(gbt_lk_params));
  FIELD(gbt_lk_params, window);
  FIELD(gbt_lk_params, npix);
  FIELD(gbt_lk_params, max_iter);
  FIELD(gbt_lk_params, eps);
  FIELD(gbt_lk_params, max_err);
  FIELD(gbt_lk_params, warps_per_block);
  gbt_config_default(&c, 480, 640, 3);
  printf("default %d %d %d %d %d %d %d %d %d %d %d %d %d\n", c.rows, c.cols, c.nscales, c.detector_threshold,
         c.detector_n, c.detector_frequency, c.filtering_frequency, c.k, c.with_merge, c.detector, c.detector_step,
         c.detector_grad_th, c.matcher);
  gbt_lk_params_default(&p);
  printf("lk_default %d %d %d %.9g %.9g %d\n", p.window, p.npix, p.max_iter, p.eps, p.max_err, p.warps_per_block);
  printf("sizes_ok %d %d %d\n", gbt_sizes_ok(1080, 1920, 4), gbt_sizes_ok(97, 131, 3), gbt_sizes_ok(8, 8, 1));
  printf("lk_scratch %lld\n", (long long)gbt_lk_scratch_bytes(480, 640, 3, 2));
  if (gbt_gaussian_taps(4.0f, taps, &radius) != GBT_OK) return 1;
  printf("taps4 %d %.9g %.9g\n", radius, taps[0], taps[radius]);
  return 0;
}
