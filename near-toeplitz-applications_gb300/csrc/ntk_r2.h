// ntk_r2.h -- entry points of the paired-chunk solve (ntk_r2.cu) for the plan.
#pragma once
#include "ntk_internal.h"
#include "ntk_r2_host.h"

namespace ntk {
namespace r2 {

// Whether in, out and the batch layout fit the kernels' tensor maps
// (16-byte aligned buffers, even strides, whole planes).
bool layout_ok(const double* in, const double* out, const Batch& b);
// The solve (rhs: RHS_IDENTITY or RHS_COMPACT; sweeps 0 or 1), S systems
// per CTA for contiguous systems (4, 8 or 16); strided systems run
// persistent CTAs (one per SM, a tile loading while two are solved) or one
// group per CTA; prefetch (0 .. 4): how many half waves ahead a one-group
// CTA prefetches a tile into L2.
int launch(const double* in, double* out, const Batch& b, const Args& a, int rhs, int sweeps, int S, bool persistent,
           int prefetch, cudaStream_t st);

// dfdx, dfdy, dfdz of a 512^3 field f (compact RHS, a's scales set) in one
// launch: per z-plane the x and y groups next to each other (so the second
// read of a plane can come from L2), then the z groups.
int launch_grad(const double* f, double* ox, double* oy, double* oz, const Args& a, int sweeps, int prefetch,
                cudaStream_t st);

}  // namespace r2
}  // namespace ntk
