// Host emulation of the paired-chunk FP32 + refinement solve (the kernels of
// near-toeplitz-applications_gb300/csrc/ntk_r2.cu), built by the tests with
// g++: the same per-thread functions (ntk_r2.cuh) run chunk after chunk with
// the carries and edge values passed explicitly, so the kernels' outputs can
// be checked bit for bit and the algorithm's accuracy on the CPU.
#include <cstdio>
#include <cstring>
#include <string>

#include "ntk_r2_host.h"

using namespace ntk::r2;

namespace {

void emulate_system(const Args& a, bool compact, int sweeps, const double* f, double* out, unsigned* rmax_out,
                    int* edge_mismatch, bool gen = false) {
  const Consts& K = a.k;
  float2 v[CHUNKS][8], dh[CHUNKS][8], dl[CHUNKS][8];
  unsigned rmax = 0;
  for (int c = 0; c < CHUNKS; ++c)
    for (int k = 0; k < ROWS; ++k) {
      const int r = ROWS * c + k;
      float h, l;
      if (compact && r == 0) {
        boundary_rhs(f[0], f[1], f[2], a.sigma0, h, l, rmax);
      } else if (compact && r == NROWS - 1) {
        boundary_rhs(f[NROWS - 1], f[NROWS - 2], f[NROWS - 3], a.sigmaN, h, l, rmax);
      } else {
        split_f64(compact ? dsub_(f[r + 1], f[r - 1]) : f[r], h, l, rmax);
      }
      if (k < HALF) {
        dh[c][k].x = h;
        dl[c][k].x = l;
      } else {
        dh[c][k - HALF].y = h;
        dl[c][k - HALF].y = l;
      }
    }
  std::memcpy(v, dh, sizeof(v));
  // ---- FP32 solve ----
  float E[CHUNKS], S[CHUNKS], a0[CHUNKS], b0[CHUNKS], b7[CHUNKS];
  for (int c = 0; c < CHUNKS; ++c) E[c] = fwd_local(v[c], K);
  for (int c = 0; c < CHUNKS; ++c) {
    bwd_local(v[c], c > 0 ? E[c - 1] : 0.f, K);
    S[c] = start_comb(v[c], K);
    a0[c] = v[c][0].x;
    b0[c] = v[c][0].y;
    b7[c] = v[c][7].y;
  }
  for (int c = 0; c < CHUNKS; ++c) bwd_fix(v[c], c + 1 < CHUNKS ? S[c + 1] : 0.f, K);
  head_fix(v[0], K);
  tail_fix(v[CHUNKS - 1], K);
  if (sweeps == 0) {
    for (int c = 0; c < CHUNKS; ++c)
      for (int k = 0; k < HALF; ++k) out_pair0(v[c][k], a, out[ROWS * c + k], out[ROWS * c + k + HALF]);
    *rmax_out = rmax;
    return;
  }
  // ---- residual ----
  float2 r[CHUNKS][8];
  for (int c = 0; c < CHUNKS; ++c) {
    const float xl = c > 0 ? left_edge(b7[c - 1], S[c], K) : 0.f;
    const float xr =
        c + 1 < CHUNKS ? right_edge(a0[c + 1], b0[c + 1], c + 2 < CHUNKS ? S[c + 2] : 0.f, K) : 0.f;
    if (c > 0 && f2u(xl) != f2u(v[c - 1][7].y)) ++*edge_mismatch;
    if (c + 1 < CHUNKS && f2u(xr) != f2u(v[c + 1][0].x)) ++*edge_mismatch;
    const float2(&x)[8] = v[c];
    for (int k = 0; k < HALF; ++k) {
      const float2 xm = k == 0 ? pair(xl, x[HALF - 1].x) : x[k - 1];
      const float2 xp = k == HALF - 1 ? pair(x[0].y, xr) : x[k + 1];
      r[c][k] = gen ? res_pair_gen(dh[c][k], dl[c][k], xm, x[k], xp, a) : res_pair(dh[c][k], dl[c][k], xm, x[k], xp, a);
    }
  }
  {
    const float2(&x)[8] = v[0];
    for (int q = 0; q < 2 && q < a.nh; ++q) {
      const float xm = q == 0 ? 0.f : x[q - 1].x;
      r[0][q].x = res_row(dh[0][q].x, dl[0][q].x, xm, x[q].x, x[q + 1].x, a.hd[q][0], a.hd[q][1], a.hd[q][2]);
    }
  }
  {
    const float2(&x)[8] = v[CHUNKS - 1];
    for (int q = 0; q < 2 && q < a.nt; ++q) {
      const int k = HALF - 1 - q;  // row n-1-q is B[k] of the last chunk
      const float xp = q == 0 ? 0.f : x[k + 1].y;
      const int ti = a.nt - 1 - q;
      r[CHUNKS - 1][k].y =
          res_row(dh[CHUNKS - 1][k].y, dl[CHUNKS - 1][k].y, x[k - 1].y, x[k].y, xp, a.td[ti][0], a.td[ti][1],
                  a.td[ti][2]);
    }
  }
  // ---- FP32 correction solve ----
  for (int c = 0; c < CHUNKS; ++c) E[c] = fwd_local(r[c], K);
  for (int c = 0; c < CHUNKS; ++c) {
    bwd_local(r[c], c > 0 ? E[c - 1] : 0.f, K);
    S[c] = start_comb(r[c], K);
  }
  for (int c = 0; c < CHUNKS; ++c) bwd_fix(r[c], c + 1 < CHUNKS ? S[c + 1] : 0.f, K);
  head_fix(r[0], K);
  tail_fix(r[CHUNKS - 1], K);
  for (int c = 0; c < CHUNKS; ++c)
    for (int k = 0; k < HALF; ++k) out_pair(v[c][k], r[c][k], a, out[ROWS * c + k], out[ROWS * c + k + HALF]);
  *rmax_out = rmax;
}

}  // namespace

extern "C" {

// Solves nsys systems of 512 rows (f: nsys x 512, contiguous) of the matrix
// with head rows head[6] = rows 0, 1 (a, b, c), tail[6] = rows n-nt .. n-1,
// interior (ai, bi, ci).  compact != 0: the compact derivative of f with
// grid spacing h (the plan's scales); else the in-place solve of d = f.
// Returns 0, 1 when the solve does not apply (reason in why), 2 on a range
// error (|input| >= 2^128), 3 when an edge value did not match its owner's.
int r2emu_solve(int nh, int nt, const double* head, const double* tail, double ai, double bi, double ci, int compact,
                double h, int sweeps, long long nsys, const double* f, double* out, char* why, int whylen) {
  MatrixRows m;
  m.n = NROWS;
  m.nh = nh;
  m.nt = nt;
  for (int i = 0; i < 2; ++i)
    for (int q = 0; q < 3; ++q) {
      m.head[i][q] = head[3 * i + q];
      m.tail[i][q] = tail[3 * i + q];
    }
  m.ai = ai;
  m.bi = bi;
  m.ci = ci;
  Args a;
  std::string w;
  if (!prepare(m, &a, &w)) {
    if (why && whylen > 0) std::snprintf(why, whylen, "%s", w.c_str());
    return 1;
  }
  if (compact) {
    const double s = 3. / (4 * h);
    set_scales(&a, (1. / (2 * h)) / s, -(1. / (2 * h)) / s, s);
  }
  unsigned rmax = 0;
  int mism = 0;
  for (long long s = 0; s < nsys; ++s) {
    unsigned r = 0;
    emulate_system(a, compact != 0, sweeps, f + s * NROWS, out + s * NROWS, &r, &mism);
    rmax = umax(rmax, r);
  }
  if (mism) return 3;
  return rmax >= (1151u << 20) ? 2 : 0;
}

// The same solve (d = f in place) for interior coefficients of any value
// (prepare with PrepareLimits::general and the given truncation limits; the
// residual res_pair_gen), as the uneven-batch windows run it.
int r2emu_solve_general(int nh, int nt, const double* head, const double* tail, double ai, double bi, double ci,
                        double carry, double trunc, int sweeps, long long nsys, const double* f, double* out,
                        char* why, int whylen) {
  MatrixRows m;
  m.n = NROWS;
  m.nh = nh;
  m.nt = nt;
  for (int i = 0; i < 2; ++i)
    for (int q = 0; q < 3; ++q) {
      m.head[i][q] = head[3 * i + q];
      m.tail[i][q] = tail[3 * i + q];
    }
  m.ai = ai;
  m.bi = bi;
  m.ci = ci;
  PrepareLimits lim;
  lim.general = true;
  lim.carry = carry;
  lim.trunc = trunc;
  Args a;
  std::string w;
  if (!prepare(m, &a, &w, lim)) {
    if (why && whylen > 0) std::snprintf(why, whylen, "%s", w.c_str());
    return 1;
  }
  unsigned rmax = 0;
  int mism = 0;
  for (long long s = 0; s < nsys; ++s) {
    unsigned r = 0;
    emulate_system(a, false, sweeps, f + s * NROWS, out + s * NROWS, &r, &mism, true);
    rmax = umax(rmax, r);
  }
  if (mism) return 3;
  return rmax >= (1151u << 20) ? 2 : 0;
}

// split_f64 and dw_to_f64 element-wise
void r2emu_split(const double* x, long long n, float* hi, float* lo) {
  unsigned r = 0;
  for (long long i = 0; i < n; ++i) split_f64(x[i], hi[i], lo[i], r);
}
void r2emu_dw(const float* hi, const float* lo, long long n, double* out) {
  for (long long i = 0; i < n; ++i) out[i] = dw_to_f64(hi[i], lo[i]);
}

}  // extern "C"
