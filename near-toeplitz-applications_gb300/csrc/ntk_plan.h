// ntk_plan.h -- the solver plan behind the opaque ntk_plan handle.
#pragma once
#include <map>
#include <mutex>
#include <vector>

#include "ntk_internal.h"

#define NTK_STR2(x) #x
#define NTK_STR(x) NTK_STR2(x)

namespace ntk {

// A near-Toeplitz tridiagonal matrix: up to two special rows at each end,
// constant (ai, bi, ci) in between.  The reference's model (neato.py:136-138)
// is one special row at each end.
struct Matrix {
  int n = 0;
  int nh = 1, nt = 1;                          // special rows at head / tail
  double ha[2] = {0, 0}, hb[2] = {1, 1}, hc[2] = {0, 0};
  double ta[2] = {0, 0}, tb[2] = {1, 1}, tc[2] = {0, 0};
  double ai = 0, bi = 1, ci = 0;

  void set_reference(const double co[7]) {
    nh = nt = 1;
    ha[0] = 0.0;
    hb[0] = co[0];
    hc[0] = co[1];
    ai = co[2];
    bi = co[3];
    ci = co[4];
    ta[0] = co[5];
    tb[0] = co[6];
    tc[0] = 0.0;
  }
  double a(int i) const {
    if (i == 0) return 0.0;
    if (i < nh) return ha[i];
    if (i >= n - nt) return ta[i - (n - nt)];
    return ai;
  }
  double b(int i) const {
    if (i < nh) return hb[i];
    if (i >= n - nt) return tb[i - (n - nt)];
    return bi;
  }
  double c(int i) const {
    if (i == n - 1) return 0.0;
    if (i < nh) return hc[i];
    if (i >= n - nt) return tc[i - (n - nt)];
    return ci;
  }
};

bool factor_host(const Matrix& m, std::vector<double>& l, std::vector<double>& u);

struct RefineState;  // ntk_refine.cu
struct LongRefine;   // ntk_long_refine.cu
struct SpikeSolver;  // ntk_spike.cu

struct Plan {
  int n = 0;
  long long nrhs = 0;
  double coeffs[7] = {0, 0, 0, 0, 0, 0, 0};
  Matrix mat;
  int precision = NTK_FP64;
  int sweeps = 1;
  int device = -1;
  std::vector<double> lu_l, lu_u;   // host LU factors (FP64)
  double* d_lw = nullptr;           // device: l[n], w[n]
  std::map<double, double*> g_by_scale;  // device g = s/u per RHS scale
  RefineState* refine = nullptr;
  LongRefine* long_refine = nullptr;  // FP32 / FP32+refine windows for n > 1024
  SpikeSolver* spike = nullptr;       // n > 1024 where the windows' halos do not decay: exact partitions
  LongRefine* long_alt = nullptr;     // 512 < n <= 1024: two-window solve (64 threads per system)
  std::mutex mu;
  // launch configuration (ntk_plan_set_tuning; chosen by the autotuner)
  int tune_f64_x_variant = 0;  // contiguous FP64 sweeps: 0 tile ring, 1 whole-system tile, 2 direct
  int tune_f64_threads = 128;  // threads per block of the one-thread-per-system FP64 kernel
  int tune_refine_w = 8;       // warps per CTA of the refinement kernel
  int tune_refine_spw = 1;     // systems per warp (2: strided layouts, 16 rows per lane)
  int tune_refine_kernel = 0;  // n = 512: paired-chunk TMA kernels where they apply (0: automatic, 2: one
                               // strided group per CTA, 3: persistent strided CTAs), 1: the chunked kernel
  int tune_refine_prefetch = 2;  // one-group strided CTAs: L2 prefetch 0 .. 4 half waves ahead
  int tune_refine_tps = 0;       // threads per system, 512 < n <= 1024: 32 (one warp, 32 rows per lane; 0 =
                                 // automatic) or 64 (two 512-row windows, 16 rows per lane)

  int init(int n, long long nrhs, const double co[7], int precision, int sweeps);
  ~Plan();
  int g_table(double s, const double** out);
  int check_device() const;
  int run(const double* in, double* out, const Batch& b, RhsParams rp, double s, cudaStream_t stream);

  // FP32 / FP32 + refinement (ntk_refine.cu)
  int init_refine();
  int run_refine(const double* in, double* out, const Batch& b, const RhsParams& rp, double s, cudaStream_t stream);
  void release_refine();
  // the three derivatives of an n^3 field in one launch (ntk_r2.cu);
  // NTK_ERR_UNSUPPORTED where that kernel does not apply
  int run_grad(const double* f, double* ox, double* oy, double* oz, double h, cudaStream_t stream);
  // device status words of this plan's FP32 kernels (none for NTK_FP64)
  void status_words(std::vector<unsigned*>& out) const;
};

}  // namespace ntk
