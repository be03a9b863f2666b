// ntk_adi_f64.h -- FP64 ADI half steps over overlapping windows, one warp
// per window (ntk_adi_f64.cu), used by the ADI plan (ntk_adi.cu).
#pragma once
#include "ntk_internal.h"

namespace ntk {

struct AdiF64;

// N x N field, steps dx, dt.  NTK_ERR_UNSUPPORTED when N < 128 or the
// factors decay too slowly for the windows (the plan then uses the
// segmented sweeps).
int adi_f64_create(AdiF64** out, int N, double dx, double dt);
void adi_f64_destroy(AdiF64* af);
// rows each window writes back, halo (0 for one whole-system window) and
// windows per system
void adi_f64_windows(const AdiF64* af, int* L, int* H, int* P);
// one step (both half steps) in place
int adi_f64_step(AdiF64* af, double* u, double* d_x, const double* d_y, cudaStream_t st);

}  // namespace ntk
