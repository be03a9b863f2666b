// ntk_adi_refine.h -- the FP32 / FP32+refinement ADI half-steps
// (ntk_adi_refine.cu), used by the ADI plan (ntk_adi.cu).
#pragma once
#include "ntk_internal.h"

namespace ntk {

struct AdiRefine;

// N x N field, steps dx, dt; precision NTK_FP32 (no refinement) or
// NTK_FP32_REFINE (one sweep; two when the halo exceeds 32 rows).  NTK_ERR_UNSUPPORTED when N < 128 or the
// factors decay too slowly for the windows.
int adi_refine_create(AdiRefine** out, int N, double dx, double dt, int precision);
void adi_refine_destroy(AdiRefine* ar);
// the status words of the window kernels
void adi_refine_status_words(const AdiRefine* ar, std::vector<unsigned*>& out);
// rows each window writes back, halo (0 for one whole-system window) and
// windows per system
void adi_refine_windows(const AdiRefine* ar, int* L, int* H, int* P);
// one step (both half steps) in place
int adi_refine_step(AdiRefine* ar, double* u, double* d_x, const double* d_y, cudaStream_t st);

}  // namespace ntk
