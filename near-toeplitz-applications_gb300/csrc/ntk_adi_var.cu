// ntk_adi_var.cu -- Peaceman-Rachford ADI steps with per-line coefficients.
//
// The reference's ADI (experiments/run-adi.py:50-71) has one matrix for
// every line: (1, 0, 1/dx^2, -2(1/dt + 1/dx^2), 1/dx^2, 0, 1), the model of
// neato.py:136-138.  Here the diffusivity of each direction may vary across
// the lines of that direction, u_t = kx(y) u_xx + ky(x) u_yy: the x operator
// has kx[j] on row j (constant along the row) and the y operator ky[i] on
// column i, so every line is still a near-Toeplitz system, each with its
// own coefficients:
//   x half step: d_x[j][i] = -b_i (u[j-1][i] + u[j+1][i]) + 2(-1/dt + b_i) u[j][i]
//                (b_i = ky[i] / dx^2, interior points; the reference's
//                stencil, adi/rhs.py:21-24, with per-column coefficients),
//                then row j (1..N-2) of d_x is solved with the matrix
//                (1, 0 | a_j, -2(1/dt + a_j), a_j | 0, 1), a_j = kx[j] / dx^2,
//                then u = d_x^T;
//   y half step: the same on u = d_x^T with the roles of kx and ky swapped,
//                into d_y, then u = d_y^T.
// With kx = ky = 1 this is the reference's step, operation for operation.
// The per-line solves are uneven batches (ntk_batch.cu: FP64 windows, or
// FP32 + double-word refinement windows) over the rows of d_x and d_y; the
// stencil and the transposes are one pass each, as in the reference.
#include <cmath>
#include <vector>

#include "ntk_internal.h"

namespace ntk {
namespace {

// Interior points of d: bt[i] u[j-1][i] + cen[i] u[j][i] + bt[i] u[j+1][i],
// in the reference's order, no contraction.
__global__ void var_stencil_kernel(const double* __restrict__ u, double* __restrict__ d, int N,
                                   const double* __restrict__ bt, const double* __restrict__ cen) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 1 || i > N - 2) return;
  const double b = bt[i], c = cen[i];
  for (int j = 1 + blockIdx.y * blockDim.y + threadIdx.y; j < N - 1; j += gridDim.y * blockDim.y) {
    const long long k = (long long)j * N + i;
    d[k] = __dadd_rn(__dadd_rn(__dmul_rn(b, u[k - N]), __dmul_rn(c, u[k])), __dmul_rn(b, u[k + N]));
  }
}

}  // namespace

struct AdiVar {
  int N = 0;
  int device = -1;
  ntk_batch* rows = nullptr;  // rows 1..N-2 of d_x, row j with kx[j]
  ntk_batch* cols = nullptr;  // rows 1..N-2 of d_y (columns of the field), row i with ky[i]
  double* d_coef = nullptr;   // [4][N]: stencil bt, cen of the x half step (from ky), of the y half step (from kx)
  ~AdiVar() {
    if (rows) ntk_batch_destroy(rows);
    if (cols) ntk_batch_destroy(cols);
    if (d_coef) cudaFree(d_coef);
  }
};

}  // namespace ntk

struct ntk_adi_var : public ntk::AdiVar {};

extern "C" {

int ntk_adi_var_create(ntk_adi_var** out, int N, double dx, double dt, const double* kx, const double* ky,
                       int precision) {
  if (!out || !kx || !ky) {
    ntk::set_error("ntk_adi_var_create: null argument");
    return NTK_ERR_INVALID;
  }
  *out = nullptr;
  if (N < 4 || !(dx > 0) || !(dt > 0) || !std::isfinite(dx) || !std::isfinite(dt)) {
    ntk::set_error("ntk_adi_var_create: need N >= 4 and positive finite dx, dt");
    return NTK_ERR_INVALID;
  }
  for (int i = 0; i < N; ++i)
    if (!std::isfinite(kx[i]) || !std::isfinite(ky[i])) {
      ntk::set_error("ntk_adi_var_create: coefficient %d is not finite", i);
      return NTK_ERR_INVALID;
    }
  ntk_adi_var* a = new (std::nothrow) ntk_adi_var();
  if (!a) {
    ntk::set_error("ntk_adi_var_create: out of host memory");
    return NTK_ERR_ALLOC;
  }
  a->N = N;
  int rc = ntk::cuda_status(cudaGetDevice(&a->device), "cudaGetDevice");
  const double rdx2 = 1. / (dx * dx);
  // per-line matrices: identity rows at both ends, (c, -2(1/dt + c), c) inside
  const long long ns = N - 2;
  std::vector<int> n(ns, N);
  std::vector<long long> off(ns);
  std::vector<double> inter(3 * ns), head(6 * ns), tail(6 * ns);
  auto build = [&](const double* k, ntk_batch** bt) {
    for (long long s = 0; s < ns; ++s) {
      const double c = k[s + 1] * rdx2;
      const double b = -2. * (1. / dt + c);
      off[s] = (s + 1) * (long long)N;
      inter[3 * s + 0] = c;
      inter[3 * s + 1] = b;
      inter[3 * s + 2] = c;
      const double h[6] = {0., 1., 0., c, b, c};
      const double t[6] = {c, b, c, 0., 1., 0.};
      for (int q = 0; q < 6; ++q) {
        head[6 * s + q] = h[q];
        tail[6 * s + q] = t[q];
      }
    }
    return ntk_batch_create(bt, ns, n.data(), off.data(), inter.data(), head.data(), tail.data(), precision);
  };
  if (!rc) rc = build(kx, &a->rows);
  if (!rc) rc = build(ky, &a->cols);
  if (!rc) {
    // stencil coefficients, adi/rhs.py:46-49 per line: bottom = top = -k/dx^2,
    // center = 2(-1/dt + k/dx^2)
    std::vector<double> coef(4 * (size_t)N);
    for (int i = 0; i < N; ++i) {
      const double by = ky[i] * rdx2, bx = kx[i] * rdx2;
      coef[i] = -by;
      coef[N + i] = 2 * (-1. / dt + by);
      coef[2 * N + i] = -bx;
      coef[3 * N + i] = 2 * (-1. / dt + bx);
    }
    rc = ntk::cuda_status(cudaMalloc(&a->d_coef, sizeof(double) * coef.size()), "cudaMalloc(ADI coefficients)");
    if (!rc)
      rc = ntk::cuda_status(
          cudaMemcpy(a->d_coef, coef.data(), sizeof(double) * coef.size(), cudaMemcpyHostToDevice),
          "cudaMemcpy(ADI coefficients)");
  }
  if (rc) {
    delete a;
    return rc;
  }
  *out = a;
  return NTK_OK;
}

int ntk_adi_var_destroy(ntk_adi_var* adi) {
  delete adi;
  return NTK_OK;
}

int ntk_adi_var_step(ntk_adi_var* a, double* u, double* d_x, double* d_y, void* stream) {
  if (!a || !u || !d_x || !d_y) {
    ntk::set_error("ntk_adi_var_step: null argument");
    return NTK_ERR_INVALID;
  }
  const int N = a->N;
  const long long total = (long long)N * N;
  if ((u < d_x + total && d_x < u + total) || (u < d_y + total && d_y < u + total) ||
      (d_x < d_y + total && d_y < d_x + total)) {
    ntk::set_error("ntk_adi_var_step: u, d_x and d_y must not overlap");
    return NTK_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const dim3 block(32, 8), grid((N + 31) / 32, (unsigned)((N + 7) / 8 < 1024 ? (N + 7) / 8 : 1024));
  // x half step
  ntk::var_stencil_kernel<<<grid, block, 0, st>>>(u, d_x, N, a->d_coef, a->d_coef + N);
  int rc = ntk::cuda_status(cudaGetLastError(), "var_stencil_kernel");
  if (!rc) rc = ntk_batch_solve(a->rows, d_x, stream);
  if (!rc) rc = ntk::launch_transpose2d(d_x, u, N, st);
  // y half step
  if (!rc) {
    ntk::var_stencil_kernel<<<grid, block, 0, st>>>(u, d_y, N, a->d_coef + 2 * N, a->d_coef + 3 * N);
    rc = ntk::cuda_status(cudaGetLastError(), "var_stencil_kernel");
  }
  if (!rc) rc = ntk_batch_solve(a->cols, d_y, stream);
  if (!rc) rc = ntk::launch_transpose2d(d_y, u, N, st);
  return rc;
}

int ntk_adi_var_status(ntk_adi_var* a, int* flags, void* stream) {
  if (!a) {
    ntk::set_error("ntk_adi_var_status: null plan");
    return NTK_ERR_INVALID;
  }
  int f1 = 0, f2 = 0;
  int rc = ntk_batch_status(a->rows, &f1, stream);
  const int rc2 = ntk_batch_status(a->cols, &f2, stream);
  if (flags) *flags = f1 | f2;
  if (rc == NTK_OK) rc = rc2;
  return rc;
}

}  // extern "C"
