// ntk_batch_refine.h -- uneven batches in FP32 / FP32+refinement
// (ntk_batch_refine.cu), used by ntk_batch.cu.
#pragma once
#include "ntk_internal.h"

namespace ntk {

struct BatchRefine;

// Windows for every system (arguments as ntk_batch_create's).
// NTK_ERR_UNSUPPORTED when some system's pivots decay too slowly.
int batch_refine_create(BatchRefine** out, long long nsys, const int* n, const long long* offset,
                        const double* interior, const double* head, const double* tail, int precision);
void batch_refine_destroy(BatchRefine* br);
// the status word of the window kernels
void batch_refine_status_words(const BatchRefine* br, std::vector<unsigned*>& out);
long long batch_refine_windows(const BatchRefine* br);
// of those, the windows on the paired-chunk solve
long long batch_refine_paired_windows(const BatchRefine* br);
// in place on d (elements [0, total)); work: a device array of total doubles
int batch_refine_solve(BatchRefine* br, double* d, double* work, cudaStream_t st);

}  // namespace ntk
