/*
 * ntk_oracle.c -- CPU restatement of the reference's hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker: it may be
 * called from tests/, from __graft_entry__.smoke() and from the cpu_baseline
 * leg of bench.py, never from the product path (the CUDA library in
 * near-toeplitz-applications_gb300/csrc).
 *
 * Every function restates one piece of ashwinsrnth/near-toeplitz-applications
 * in plain sequential C, keeping the reference's order of floating-point
 * operations so that, compiled without FMA contraction (-ffp-contract=off),
 * the results are bit-identical to the reference's own kernels executed on
 * the CPU (oracle/ref_cpu.cpp) and to the golden vectors in tests/golden/.
 *
 *   ntko_precompute       neato.py:199-274  (_precompute_coefficients)
 *   ntko_cr_solve         neato.py:26-123   (sharedMemCyclicReduction, one
 *                                            block per system, n/2 threads)
 *   ntko_thomas           experiments/run-compact.py:14-28 restated as the
 *                         textbook Thomas algorithm (general tridiagonal)
 *   ntko_thomas_ld        the same in long double, many right-hand sides: the
 *                         accuracy reference for badly scaled matrices
 *   ntko_compact_rhs      compact/rhs.py:9-37 (computeRHS)
 *   ntko_permute          compact/permute.py:7-20,32-52 (permuteKernel)
 *   ntko_adi_rhs          adi/rhs.py:10-25,35-55 (applyVerticalStencil)
 *   ntko_transpose        adi/transpose.py:9-27,40-50 (transposeCoalesced)
 *   ntko_adi_step         experiments/run-adi.py:59-71 (one time step)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static int ilog2_exact(int n) {
  int l = 0;
  while ((1 << l) < n) ++l;
  return ((1 << l) == n) ? l : -1;
}

/* neato.py:199-274.  Arrays have length log2(n); the last-row a/b values are
 * stored in a[L-1], b[L-1] (neato.py:270-272).  Returns 0, or -1 when n is
 * not a power of two >= 4 (neato.py:145 asserts a power of two; n = 2 leaves
 * a_last undefined in the reference). */
int ntko_precompute(int n, const double coeffs[7], double* a, double* b, double* c, double* k1,
                    double* k2, double* b_first, double* k1_first, double* k1_last) {
  int L = ilog2_exact(n);
  if (L < 2) return -1;
  const double b1 = coeffs[0], c1 = coeffs[1], ai = coeffs[2], bi = coeffs[3], ci = coeffs[4],
               an = coeffs[5], bn = coeffs[6];
  for (int i = 0; i < L; ++i) a[i] = b[i] = c[i] = k1[i] = k2[i] = b_first[i] = k1_first[i] = k1_last[i] = 0.0;
  double a_last = 0.0, b_last = 0.0;
  for (int i = 0; i < L - 1; ++i) {
    if (i == 0) {
      k1[i] = ai / bi;
      k2[i] = ci / bi;
      a[i] = -ai * k1[i];
      b[i] = bi - ci * k1[i] - ai * k2[i];
      c[i] = -ci * k2[i];
      k1_first[i] = ai / b1;
      b_first[i] = bi - c1 * k1_first[i] - ai * k2[i];
      k1_last[i] = an / bi;
      a_last = -(ai)*k1_last[i];
      b_last = bn - (ci)*k1_last[i];
    } else {
      k1[i] = a[i - 1] / b[i - 1];
      k2[i] = c[i - 1] / b[i - 1];
      a[i] = -a[i - 1] * k1[i];
      b[i] = b[i - 1] - c[i - 1] * k1[i] - a[i - 1] * k2[i];
      c[i] = -c[i - 1] * k2[i];
      k1_first[i] = a[i - 1] / b_first[i - 1];
      b_first[i] = b[i - 1] - c[i - 1] * k1_first[i] - a[i - 1] * k2[i];
      k1_last[i] = a_last / b[i - 1];
      a_last = -a[i - 1] * k1_last[i];
      b_last = b_last - c[i - 1] * k1_last[i];
    }
  }
  a[L - 1] = a_last;
  b[L - 1] = b_last;
  return 0;
}

/* neato.py:26-123, executed for one system at a time with the thread loop
 * inside each level.  Within a level no thread reads a slot another thread
 * writes, so the sequential order gives the same values as the kernel.
 * Solves in place.  `work` must hold n/2 doubles. */
static void cr_one(int n, const double* a, const double* b, const double* c, const double* k1,
                   const double* k2, const double* b_first, const double* k1_first,
                   const double* k1_last, double b1, double c1, double ai, double bi, double ci,
                   double* d, double* d_l) {
  const int half = n / 2;
  int idx = 0;
  /* level 0 during the load (neato.py:36-50) */
  for (int tix = 0; tix < half; ++tix) {
    if (tix == 0) {
      d_l[tix] = d[2 * tix + 1] - d[2 * tix] * k1_first[idx] - d[2 * tix + 2] * k2[idx];
    } else if (tix == half - 1) {
      d_l[tix] = d[2 * tix + 1] - d[2 * tix] * k1_last[idx];
    } else {
      d_l[tix] = d[2 * tix + 1] - d[2 * tix] * k1[idx] - d[2 * tix + 2] * k2[idx];
    }
  }
  /* forward levels (neato.py:57-76) */
  for (int stride = 2; stride < half; stride = stride * 2) {
    idx = idx + 1;
    for (int tix = 0; tix < n / (2 * stride); ++tix) {
      int i = (stride - 1) + tix * stride;
      if (tix == 0) {
        d_l[i] = d_l[i] - d_l[i - stride / 2] * k1_first[idx] - d_l[i + stride / 2] * k2[idx];
      } else if (i == (n / 2 - 1)) {
        d_l[i] = d_l[i] - d_l[i - stride / 2] * k1_last[idx];
      } else {
        d_l[i] = d_l[i] - d_l[i - stride / 2] * k1[idx] - d_l[i + stride / 2] * k2[idx];
      }
    }
  }
  /* 2x2 solve (neato.py:78-92) */
  {
    int j = (int)rint(log2((float)half)) - 1;
    int k = (int)rint(log2((float)half));
    double d_j = (d_l[n / 4 - 1] * b[k] - c[j] * d_l[n / 2 - 1]) / (b_first[j] * b[k] - c[j] * a[k]);
    double d_k = (b_first[j] * d_l[n / 2 - 1] - d_l[n / 4 - 1] * a[k]) / (b_first[j] * b[k] - c[j] * a[k]);
    d_l[n / 4 - 1] = d_j;
    d_l[n / 2 - 1] = d_k;
  }
  /* back substitution (neato.py:95-110) */
  idx = (int)rint(log2((float)n)) - 2;
  for (int stride = n / 4; stride > 1; stride = stride / 2) {
    idx = idx - 1;
    for (int tix = 0; tix < n / (2 * stride); ++tix) {
      int i = (stride / 2 - 1) + tix * stride;
      if (tix == 0) {
        d_l[i] = (d_l[i] - c[idx] * d_l[i + stride / 2]) / b_first[idx];
      } else {
        d_l[i] = (d_l[i] - a[idx] * d_l[i - stride / 2] - c[idx] * d_l[i + stride / 2]) / b[idx];
      }
    }
  }
  /* even rows during the store (neato.py:114-122) */
  for (int tix = 0; tix < half; ++tix) {
    if (tix == 0) {
      d[2 * tix] = (d[2 * tix] - c1 * d_l[tix]) / b1;
      d[2 * tix + 1] = d_l[tix];
    } else {
      d[2 * tix] = (d[2 * tix] - ai * d_l[tix - 1] - ci * d_l[tix]) / bi;
      d[2 * tix + 1] = d_l[tix];
    }
  }
}

/* NearToeplitzSolver(n, nrhs, coeffs).solve(d) (neato.py:131-197): nrhs
 * contiguous systems of length n starting at d, solved in place. */
int ntko_cr_solve(int n, long nrhs, const double coeffs[7], double* d) {
  int L = ilog2_exact(n);
  if (L < 2 || nrhs < 0) return -1;
  double arr[8][32];
  if (ntko_precompute(n, coeffs, arr[0], arr[1], arr[2], arr[3], arr[4], arr[5], arr[6], arr[7])) return -1;
  double* d_l = (double*)malloc(sizeof(double) * (size_t)(n / 2));
  if (!d_l) return -2;
  for (long s = 0; s < nrhs; ++s)
    cr_one(n, arr[0], arr[1], arr[2], arr[3], arr[4], arr[5], arr[6], arr[7], coeffs[0], coeffs[1],
           coeffs[2], coeffs[3], coeffs[4], d + (size_t)s * (size_t)n, d_l);
  free(d_l);
  return 0;
}

/* General tridiagonal Thomas algorithm, the textbook restatement of the
 * banded LAPACK solve the reference uses on the CPU
 * (experiments/run-compact.py:14-28: a = sub-diagonal, first entry ignored;
 * c = super-diagonal, last entry ignored). x may alias d. */
int ntko_thomas(int n, const double* a, const double* b, const double* c, const double* d, double* x) {
  if (n < 1) return -1;
  double* cp = (double*)malloc(sizeof(double) * (size_t)n);
  double* dp = (double*)malloc(sizeof(double) * (size_t)n);
  if (!cp || !dp) { free(cp); free(dp); return -2; }
  cp[0] = (n > 1 ? c[0] : 0.0) / b[0];
  dp[0] = d[0] / b[0];
  for (int i = 1; i < n; ++i) {
    double den = b[i] - a[i] * cp[i - 1];
    cp[i] = (i < n - 1 ? c[i] : 0.0) / den;
    dp[i] = (d[i] - a[i] * dp[i - 1]) / den;
  }
  x[n - 1] = dp[n - 1];
  for (int i = n - 2; i >= 0; --i) x[i] = dp[i] - cp[i] * x[i + 1];
  free(cp);
  free(dp);
  return 0;
}

/* The same Thomas algorithm in long double (80-bit x87 on x86-64, IEEE quad
 * on AArch64) for nrhs right-hand sides stored one after another: the
 * accuracy reference for badly scaled matrices (the ADI tuples), where
 * LAPACK's pivoting banded solve and FP64 cyclic reduction both lose digits.
 * d and x hold nrhs * n values; x may alias d. */
int ntko_thomas_ld(int n, long nrhs, const double* a, const double* b, const double* c, const double* d, double* x) {
  if (n < 1 || nrhs < 0) return -1;
  long double* cp = (long double*)malloc(sizeof(long double) * (size_t)n);
  long double* den = (long double*)malloc(sizeof(long double) * (size_t)n);
  long double* dp = (long double*)malloc(sizeof(long double) * (size_t)n);
  if (!cp || !den || !dp) { free(cp); free(den); free(dp); return -2; }
  den[0] = (long double)b[0];
  cp[0] = (n > 1 ? (long double)c[0] : 0.0L) / den[0];
  for (int i = 1; i < n; ++i) {
    den[i] = (long double)b[i] - (long double)a[i] * cp[i - 1];
    cp[i] = (i < n - 1 ? (long double)c[i] : 0.0L) / den[i];
  }
  for (long s = 0; s < nrhs; ++s) {
    const double* ds = d + (size_t)s * n;
    double* xs = x + (size_t)s * n;
    dp[0] = (long double)ds[0] / den[0];
    for (int i = 1; i < n; ++i) dp[i] = ((long double)ds[i] - (long double)a[i] * dp[i - 1]) / den[i];
    long double xv = dp[n - 1];
    xs[n - 1] = (double)xv;
    for (int i = n - 2; i >= 0; --i) {
      xv = dp[i] - cp[i] * xv;
      xs[i] = (double)xv;
    }
  }
  free(cp);
  free(den);
  free(dp);
  return 0;
}

/* compact/rhs.py:9-37 over an [nz][ny][nx] field, derivative along x. */
void ntko_compact_rhs(const double* f, double* rhs, int nz, int ny, int nx, double dx) {
  for (int tiz = 0; tiz < nz; ++tiz)
    for (int tiy = 0; tiy < ny; ++tiy)
      for (int tix = 0; tix < nx; ++tix) {
        size_t i = (size_t)tiz * ((size_t)nx * ny) + (size_t)tiy * nx + tix;
        if (tix == 0) {
          rhs[i] = (1. / (2 * dx)) * (-5 * f[i] + 4 * f[i + 1] + f[i + 2]);
        } else if (tix == nx - 1) {
          rhs[i] = -(1. / (2 * dx)) * (-5 * f[i] + 4 * f[i - 1] + f[i - 2]);
        } else {
          rhs[i] = (3. / (4 * dx)) * (f[i + 1] - f[i - 1]);
        }
      }
}

/* compact/permute.py:7-20,32-52: out (shape o0 x o1 x o2, C order) gets
 * out[i0][i1][i2] = in[i0*s0 + i1*s1 + i2*s2], where s_k are the input's
 * element strides taken in the order of `permutation`.  This is
 * numpy.transpose(in, permutation).  (The reference kernel indexes the
 * output with the first output extent in place of the last, which agrees
 * with this for cubic arrays, the only shape its drivers use.) */
void ntko_permute(const double* in, double* out, int o0, int o1, int o2, long s0, long s1, long s2) {
  for (int i0 = 0; i0 < o0; ++i0)
    for (int i1 = 0; i1 < o1; ++i1)
      for (int i2 = 0; i2 < o2; ++i2)
        out[((size_t)i0 * o1 + i1) * o2 + i2] = in[(size_t)(i0 * s0 + i1 * s1 + i2 * s2)];
}

/* adi/rhs.py:10-25 with the coefficients of adi/rhs.py:46-49. Only interior
 * points of d are written. */
void ntko_adi_rhs(const double* u, double* d, int N, double dx, double dt) {
  const double bottom = -1. / (dx * dx);
  const double top = -1. / (dx * dx);
  const double center = 2 * (-1. / dt + 1. / (dx * dx));
  for (int tiy = 1; tiy < N - 1; ++tiy)
    for (int tix = 1; tix < N - 1; ++tix) {
      size_t i = (size_t)tiy * N + tix;
      d[i] = bottom * u[i - N] + center * u[i] + top * u[i + N];
    }
}

/* adi/transpose.py:40-50: b = transpose(a), N x N. */
void ntko_transpose(const double* a, double* b, int N) {
  for (int y = 0; y < N; ++y)
    for (int x = 0; x < N; ++x) b[(size_t)y * N + x] = a[(size_t)x * N + y];
}

/* experiments/run-adi.py:50-53,59-71: one Peaceman-Rachford step.  u, d_x,
 * d_y are N x N; d_x/d_y keep their boundary entries from the caller (the
 * reference initialises them as u and u^T).  Solver: the reference CR with
 * coefficients (1, 0, 1/dx^2, -2(1/dt + 1/dx^2), 1/dx^2, 0, 1) applied to the
 * N-2 rows starting at row 1. */
int ntko_adi_step(double* u, double* d_x, double* d_y, int N, double dx, double dt) {
  const double coeffs[7] = {1., 0., 1. / (dx * dx), -2. * (1. / dt + 1. / (dx * dx)), 1. / (dx * dx), 0., 1.};
  ntko_adi_rhs(u, d_x, N, dx, dt);
  if (ntko_cr_solve(N, N - 2, coeffs, d_x + N)) return -1;
  ntko_transpose(d_x, u, N);
  ntko_adi_rhs(u, d_y, N, dx, dt);
  if (ntko_cr_solve(N, N - 2, coeffs, d_y + N)) return -1;
  ntko_transpose(d_y, u, N);
  return 0;
}
