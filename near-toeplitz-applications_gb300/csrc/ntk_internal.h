// ntk_internal.h -- host-side declarations shared by the ntk translation units.
#pragma once
#include <cuda_runtime.h>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/ntk.h"

namespace ntk {

// How a batch of systems sits in memory: system s (0 <= s < nsys) starts at
// element (s / ni) * os + (s % ni) * is and its k-th unknown is at
// start + k * es.  Every direction of a C-ordered [nz][ny][nx] field is one
// of these without copies:
//   x: ni = nsys, is = nx, es = 1
//   y: ni = nx, is = 1, os = nx*ny, es = nx
//   z: ni = nx*ny, is = 1, es = nx*ny
struct Batch {
  long long nsys = 0;
  long long ni = 1;
  long long is = 0;
  long long os = 0;
  long long es = 1;
};

// Right-hand side applied inside the solve's load phase.
enum RhsKind : int {
  RHS_IDENTITY = 0,  // d is given (in place solve)
  RHS_COMPACT = 1,   // compact 4th-order first derivative of f along the system
  RHS_CROSS = 2,     // 3-point stencil across systems (ADI explicit half)
};

// Parameters of the fused right-hand sides, in the units the kernels use:
// the solve is carried out on eta = y / s (s the interior RHS scale) so the
// interior RHS needs no multiply.
struct RhsParams {
  int kind = RHS_IDENTITY;
  double sigma0 = 1.0;  // boundary-row scale, row 0   (compact: s_0 / s)
  double sigmaN = 1.0;  // boundary-row scale, row n-1
  // cross stencil: d_i = bottom * in[i - cs] + center * in[i] + top * in[i + cs]
  double bottom = 0, center = 0, top = 0;
  long long cs = 0;             // element offset of the stencil's neighbours across systems
  const double* bnd = nullptr;  // boundary-row values D_0, D_{n-1} (cross stencil)
  long long bnd_ss = 0;         // boundary values of system s start at bnd + s * bnd_ss
  long long bnd_es = 1;         // D_{n-1} is at (n-1) * bnd_es from D_0
};

// Decay-truncated segmentation of the Thomas sweeps: system s is cut into P
// segments of L rows; the forward sweep of segment g starts H rows early
// from zero and the backward sweep H rows late from zero.  Used only when
// the products of |l_i| (|w_i|) over every halo window are below 2^-64, so
// the truncation is below FP64 rounding.
struct SegParams {
  int L = 0;
  int H = 0;
  int P = 1;
};

// Segmentation of nsys systems of n rows for the segmented sweeps (the ADI
// half-steps: few, long systems).  l[n], w[n]: the FP64 LU factors.  Aims
// for ~16 warps per SM of (segment, system) threads and takes the largest
// power-of-two P up to that for which some halo H <= L/2 makes every
// truncated factor product (l over the H rows before a segment start, w over
// the H rows after a segment end) fall below 2^-64, i.e. the truncation is
// below FP64 rounding.  P = 1 (plain sweeps) when none qualifies.  Allocates
// nothing.
#ifndef NTK_SEG_THREADS
#define NTK_SEG_THREADS (152 * 512)
#endif
inline SegParams choose_segments(const double* l, const double* w, int n, long long nsys) {
  SegParams sp;
  sp.P = 1;
  sp.L = n;
  sp.H = 0;
  int Pmax = 1;
  while (nsys * Pmax < (long long)NTK_SEG_THREADS && Pmax < 64 && n / (2 * Pmax) >= 16) Pmax *= 2;
  const double lim = std::ldexp(1.0, -64);
  for (int P = Pmax; P >= 2; P /= 2) {
    const int L = (n + P - 1) / P;
    for (int H = 8; H <= L / 2; H += 2) {
      bool ok = true;
      for (int g = 1; g < P && ok; ++g) {
        double prod = 1.0;
        for (int i = (g * L - H > 1 ? g * L - H : 1); i < g * L; ++i) prod *= std::fabs(l[i]);
        ok = prod <= lim;
      }
      for (int g = 0; g < P - 1 && ok; ++g) {
        double prod = 1.0;
        const int e = ((g + 1) * L < n) ? (g + 1) * L : n;
        for (int i = e; i < ((e + H < n) ? e + H : n); ++i) prod *= std::fabs(w[i - 1]);
        ok = prod <= lim;
      }
      if (ok) {
        sp.P = P;
        sp.L = L;
        sp.H = H;
        return sp;
      }
    }
  }
  return sp;
}

// FP64 factor tables of the shared matrix (length n each), device memory.
struct TablesF64 {
  const double* l = nullptr;  // l_i = a_i / u_{i-1}
  const double* g = nullptr;  // g_i = s / u_i
  const double* w = nullptr;  // w_i = c_i / u_i
};

void set_error(const char* fmt, ...);
int cuda_status(cudaError_t e, const char* where);

// Status bits the FP32 / FP32+refinement kernels raise in their device
// status words (ntk.h NTK_STATUS_*).
constexpr unsigned STATUS_RANGE = 1u;  // an input outside the double-word range (|x| >= 2^128, inf, nan)

// Reads the device status words in `words` on stream st, clears them (both in
// stream order) and waits for the stream; *flags = the OR of the words.
// Returns NTK_ERR_RANGE when STATUS_RANGE is set, NTK_OK otherwise, or the
// CUDA error of a failed copy.
int read_clear_status(const std::vector<unsigned*>& words, cudaStream_t st, int* flags);

// kernels (ntk_solve_f64.cu)
// x_variant (contiguous systems): 0 = automatic (transposing tile ring),
// 1 = whole-system shared-memory tile, 2 = direct loads
int launch_thomas_f64(const double* in, double* out, int n, const Batch& b, const RhsParams& rp,
                      const TablesF64& t, int threads, cudaStream_t stream, int x_variant = 0);
int launch_thomas_f64_segmented(const double* in, double* eta, double* out, int n, const Batch& b,
                                const RhsParams& rp, const TablesF64& t, const SegParams& sp, cudaStream_t stream);

// standalone operators (ntk_ops.cu)
int launch_compact_rhs(const double* f, double* rhs, int nz, int ny, int nx, double dx, cudaStream_t s);
int launch_permute3d(const double* in, double* out, int o0, int o1, int o2, long long s0, long long s1,
                     long long s2, cudaStream_t s);
int launch_adi_rhs(const double* u, double* d, int N, double bottom, double center, double top, cudaStream_t s);
int launch_transpose2d(const double* a, double* b, int N, cudaStream_t s);

}  // namespace ntk
