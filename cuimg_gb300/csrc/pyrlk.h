// Internal interface of the pyramidal LK tracker engine (pyrlk.cu), used by
// the C ABI entry points in tracker.cu for contexts created with
// gbt_config.matcher == GBT_MATCHER_LK.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "cuimg_gb300.h"

struct PkTracker;

int pk_create(const gbt_config* cfgs, int nstreams, int device, PkTracker** out, std::string& err);
void pk_destroy(PkTracker* t);
const std::string& pk_error(const PkTracker* t);
cudaStream_t pk_stream(const PkTracker* t);
int pk_run(PkTracker* t, const uint8_t* const* frames, const int64_t* pitches, int location);
int pk_sync(PkTracker* t);
int pk_set_param(PkTracker* t, int stream, int scale, int key, int value);
int pk_get_param(PkTracker* t, int stream, int scale, int key, int32_t* value);
int pk_nparticles(PkTracker* t, int stream, int scale, int32_t* n);
int pk_frame_count(PkTracker* t, int stream, int scale, int32_t* n);
int pk_get_particles(PkTracker* t, int stream, int scale, float* pos, float* speed, uint16_t* age, int32_t* matches,
                     int32_t* nmatches, int32_t* compact_has_run);
int pk_get_stage(PkTracker* t, int stream, int scale, int stage, int border, void* out);
int pk_read_counts(PkTracker* t, int32_t* counts, int n, bool async);
int pk_kernel_launches(PkTracker* t, int64_t* total);
int pk_kernels_per_frame(PkTracker* t, int32_t* n);
