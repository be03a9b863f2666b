// ntk_long_refine.h -- FP32 / FP32+refinement plans for n > 1024
// (ntk_long_refine.cu), used by the plan (ntk_refine.cu).
#pragma once
#include "ntk_internal.h"

namespace ntk {

struct Plan;
struct LongRefine;

// Windows for plan p (n > 1024); NTK_ERR_UNSUPPORTED when the LU multipliers
// decay too slowly for 512-row windows.
int long_refine_create(LongRefine** out, const Plan& p, int precision, int sweeps);
void long_refine_destroy(LongRefine* lr);
// the status words of the window plans' kernels
void long_refine_status_words(const LongRefine* lr, std::vector<unsigned*>& out);
// a plan's solve or compact derivative (RHS_IDENTITY / RHS_COMPACT), W warps
// per CTA (4 or 8); in place when in and out overlap (through a work array)
int long_refine_run(LongRefine* lr, const double* in, double* out, const Batch& b, const RhsParams& rp, double s,
                    int W, cudaStream_t st);

}  // namespace ntk
