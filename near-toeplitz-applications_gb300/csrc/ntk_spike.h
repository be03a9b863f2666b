// ntk_spike.h -- FP32 + refinement solves of long systems whose LU
// multipliers decay too slowly for overlapping windows (ntk_spike.cu).
#pragma once
#include <vector>

#include "ntk_internal.h"
#include "ntk_plan.h"

namespace ntk {

struct SpikeSolver;

// Partitions of 512 rows, one warp each, coupled exactly through a reduced
// system of the partitions' end unknowns.  Needs n > 512 and at most
// SPIKE_MAX_PARTS partitions; NTK_ERR_UNSUPPORTED otherwise (or when a
// partition block or the reduced system is singular, or sweeps > 2).
// sweeps: 0 (FP32 only), 1 or 2 refinement sweeps.
constexpr int SPIKE_MAX_PARTS = 16;
int spike_create(SpikeSolver** out, const Matrix& m, int sweeps);
void spike_destroy(SpikeSolver* s);
// In place or out of place over the systems of b (plain solve: the RHS is
// in's values).
int spike_solve(SpikeSolver* s, const double* in, double* out, const Batch& b, cudaStream_t st);
int spike_partitions(const SpikeSolver* s);
int spike_sweeps(const SpikeSolver* s);
void spike_status_words(const SpikeSolver* s, std::vector<unsigned*>& out);

}  // namespace ntk
