// ntk_r2_adi.h -- ADI half steps on the paired-chunk FP32 + refinement
// solve (ntk_r2_adi.cu), for the ADI plan's windows (ntk_adi_refine.cu).
#pragma once
#include <string>
#include <vector>

#include "ntk_internal.h"

namespace ntk {
namespace r2 {

struct AdiR2;

// Window geometry of the ADI plan (ntk_adi_geom.h): N rows per system, L
// central rows and H halo rows per 512-row window, P windows per system
// (whole: N == 512).  The rows are scaled by dx^2: interior (1, beta, 1),
// RHS gamma u_mid - (u_lo + u_hi).  Returns null, with the reason in *why,
// where these kernels do not apply: beta not a power of two, factors that
// decay too slowly for 16-row carries, N or H not multiples of 16, more
// than one sweep.
AdiR2* adi_create(int N, int L, int H, int P, bool whole, double beta, double gamma, int sweeps, std::string* why);
void adi_destroy(AdiR2* r);
// One ADI step (experiments/run-adi.py:59-71): x half step from u into
// d_x (rows 1..N-2, boundary RHS d_x's own boundary columns), y half step
// from d_x into u's columns 1..N-2 (boundary RHS d_y's boundary columns).
int adi_step(AdiR2* r, double* u, double* d_x, const double* d_y, cudaStream_t st);
void adi_status_words(const AdiR2* r, std::vector<unsigned*>& out);

}  // namespace r2
}  // namespace ntk
