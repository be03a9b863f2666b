// ntk_r2_host.h -- host-side preparation of the paired-chunk solve
// (ntk_r2.cuh): the FP32 LU constants of the pure Toeplitz matrix T and the
// Woodbury end corrections, computed in FP64 once per plan.  Plain C++ (also
// compiled by the host emulation in tests/r2_emul.cpp).
#pragma once
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "ntk_r2.cuh"

namespace ntk {
namespace r2 {

// The near-Toeplitz matrix as the plans store it: up to two special rows at
// each end, (a, b, c) each; interior (ai, bi, ci).
struct MatrixRows {
  int n = 0;
  int nh = 1, nt = 1;
  double head[2][3] = {{0, 1, 0}, {0, 1, 0}};  // rows 0, 1: (a, b, c)
  double tail[2][3] = {{0, 1, 0}, {0, 1, 0}};  // rows n-nt .. n-1: (a, b, c)
  double ai = 0, bi = 1, ci = 0;
  double a(int i) const {
    if (i <= 0 || i >= n) return 0.0;
    if (i < nh) return head[i][0];
    if (i >= n - nt) return tail[i - (n - nt)][0];
    return ai;
  }
  double b(int i) const {
    if (i < nh) return head[i][1];
    if (i >= n - nt) return tail[i - (n - nt)][1];
    return bi;
  }
  double c(int i) const {
    if (i < 0 || i >= n - 1) return 0.0;
    if (i < nh) return head[i][2];
    if (i >= n - nt) return tail[i - (n - nt)][2];
    return ci;
  }
};

inline bool pow2_or_zero(double v) {
  if (v == 0.0) return true;
  int e;
  const double m = std::frexp(std::fabs(v), &e);
  return m == 0.5 && e > -100 && e < 100;
}

inline DWc to_dwc(double v) {
  DWc d;
  d.h = (float)v;
  d.l = (float)(v - (double)d.h);
  return d;
}

// What prepare() accepts.  general: interior coefficients of any value
// (the kernel then uses res_pair_gen); carry: the largest |l|^16, |w|^16
// (the weight of the carry the 16-row chunks drop); trunc: the largest part
// of an end correction beyond the 15 rows it is applied to.  Both limits
// bound the FP32 solve's own error, which the refinement removes.
struct PrepareLimits {
  bool general = false;
  double carry = std::ldexp(1.0, -26);
  double trunc = std::ldexp(1.0, -25);
};

// The matrix-dependent part of Args (Consts, interior and special rows).
// Returns false, with the reason in *why, when this solve does not apply:
// n != 512, interior coefficients that are not powers of two (unless
// lim.general), multipliers that decay too slowly for the 16-row carry
// truncation (|l|^16 or |w|^16 above lim.carry), end corrections that reach
// beyond the first / last 15 rows (lim.trunc), or an ill-conditioned
// capacitance matrix.
inline bool prepare(const MatrixRows& m, Args* out, std::string* why, const PrepareLimits& lim = PrepareLimits()) {
  Args a;
  std::memset(&a, 0, sizeof(a));
  auto fail = [&](const char* msg) {
    if (why) *why = msg;
    return false;
  };
  const int n = m.n;
  if (n != NROWS) return fail("paired-chunk solve serves n = 512 only");
  if (m.nh < 0 || m.nh > 2 || m.nt < 0 || m.nt > 2) return fail("more than two special rows");
  if (!lim.general && (!pow2_or_zero(m.ai) || !pow2_or_zero(m.bi) || !pow2_or_zero(m.ci)))
    return fail("interior coefficients are not powers of two");
  // pivot fixed point of the interior recurrence u = b - a c / u
  double u = m.bi;
  for (int it = 0; it < 100000; ++it) {
    const double un = m.bi - m.ai * m.ci / u;
    if (!std::isfinite(un) || un == 0.0) return fail("interior pivot recurrence breaks down");
    if (un == u) break;
    u = un;
  }
  if (std::fabs(m.bi - m.ai * m.ci / u - u) > 1e-15 * std::fabs(u)) return fail("interior pivots do not converge");
  const double l = m.ai / u, w = m.ci / u, g = 1.0 / u;
  if (std::pow(std::fabs(l), 16) > lim.carry || std::pow(std::fabs(w), 16) > lim.carry)
    return fail("multipliers decay too slowly for 16-row carries");
  Consts& k = a.k;
  k.nl = splat((float)-l);
  k.g = splat((float)g);
  k.nw = splat((float)-w);
  for (int i = 0; i < 8; ++i) {
    k.phi[i] = splat((float)std::pow(-l, i + 1));
    k.psi[i] = splat((float)std::pow(-w, 8 - i));
  }
  // T = A's interior everywhere, T[0][0] = u.  Its LU factors are the
  // constants above; solve T x = d in FP64.
  auto tsolve = [&](const std::vector<double>& d) {
    std::vector<double> y(n), x(n);
    y[0] = d[0];
    for (int i = 1; i < n; ++i) y[i] = d[i] - l * y[i - 1];
    x[n - 1] = g * y[n - 1];
    for (int i = n - 2; i >= 0; --i) x[i] = g * y[i] - w * x[i + 1];
    return x;
  };
  auto trow = [&](int i, int col) {  // T[i][col]
    if (col == i) return i == 0 ? u : m.bi;
    if (col == i - 1) return m.ai;
    if (col == i + 1) return m.ci;
    return 0.0;
  };
  auto arow = [&](int i, int col) {
    if (col == i) return m.b(i);
    if (col == i - 1) return m.a(i);
    if (col == i + 1) return m.c(i);
    return 0.0;
  };
  // head: rows 0 .. nh'-1 differ (row 0 always: T[0][0] = u)
  const int nh = m.nh < 1 ? 1 : m.nh;
  const int nt = m.nt;
  double hdel[2][3] = {{0}}, tdel[2][3] = {{0}};
  for (int j = 0; j < nh; ++j)
    for (int q = 0; q < 3; ++q) hdel[j][q] = arow(j, q) - trow(j, q);
  for (int j = 0; j < nt; ++j) {
    const int row = n - nt + j;
    for (int q = 0; q < 3; ++q) tdel[j][q] = arow(row, n - 3 + q) - trow(row, n - 3 + q);
  }
  std::vector<std::vector<double>> p(nh), qv(nt);
  for (int i = 0; i < nh; ++i) {
    std::vector<double> e(n, 0.0);
    e[i] = 1.0;
    p[i] = tsolve(e);
  }
  for (int j = 0; j < nt; ++j) {
    std::vector<double> e(n, 0.0);
    e[n - nt + j] = 1.0;
    qv[j] = tsolve(e);
  }
  // capacitance blocks C = I + delta^T T^-1 U; the head/tail cross terms
  // must vanish (they are ~ l^500 here)
  double Ch[2][2] = {{1, 0}, {0, 1}}, Ct[2][2] = {{1, 0}, {0, 1}};
  for (int jj = 0; jj < nh; ++jj)
    for (int i = 0; i < nh; ++i)
      for (int q = 0; q < 3; ++q) Ch[jj][i] += hdel[jj][q] * p[i][q];
  for (int jj = 0; jj < nt; ++jj)
    for (int i = 0; i < nt; ++i)
      for (int q = 0; q < 3; ++q) Ct[jj][i] += tdel[jj][q] * qv[i][n - 3 + q];
  double cross = 0.0;
  for (int jj = 0; jj < nh; ++jj)
    for (int i = 0; i < nt; ++i)
      for (int q = 0; q < 3; ++q) cross = std::fmax(cross, std::fabs(hdel[jj][q] * qv[i][q]));
  for (int jj = 0; jj < nt; ++jj)
    for (int i = 0; i < nh; ++i)
      for (int q = 0; q < 3; ++q) cross = std::fmax(cross, std::fabs(tdel[jj][q] * p[i][n - 3 + q]));
  if (cross > 1e-30) return fail("head and tail corrections interact");
  auto inv = [&](double C[2][2], int d, double R[2][2]) {
    if (d == 0) return true;
    if (d == 1) {
      if (!(std::fabs(C[0][0]) > 1e-6)) return false;
      R[0][0] = 1.0 / C[0][0];
      return true;
    }
    const double det = C[0][0] * C[1][1] - C[0][1] * C[1][0];
    const double sc = std::fabs(C[0][0]) + std::fabs(C[0][1]) + std::fabs(C[1][0]) + std::fabs(C[1][1]);
    if (!(std::fabs(det) > 1e-6 * sc * sc)) return false;
    R[0][0] = C[1][1] / det;
    R[0][1] = -C[0][1] / det;
    R[1][0] = -C[1][0] / det;
    R[1][1] = C[0][0] / det;
    return true;
  };
  double Rh[2][2] = {{0}}, Rt[2][2] = {{0}};
  if (!inv(Ch, nh, Rh) || !inv(Ct, nt, Rt)) return fail("end correction is ill-conditioned");
  // P_j = sum_i p_i (C_h^-1)_ij over rows 0..15; row 15 must be negligible
  const double trunc = lim.trunc;
  k.nh = nh;
  k.nt = nt;
  for (int jj = 0; jj < nh; ++jj) {
    std::vector<double> P(16, 0.0);
    double dn = 0.0;
    for (int q = 0; q < 3; ++q) dn += std::fabs(hdel[jj][q]);
    double rest = 0.0;
    for (int r = 0; r < n; ++r) {
      double s = 0.0;
      for (int i = 0; i < nh; ++i) s += p[i][r] * Rh[i][jj];
      if (r < 15) P[r] = s;
      else rest = std::fmax(rest, std::fabs(s));
    }
    if (rest * dn > trunc) return fail("head correction reaches beyond the first 15 rows");
    for (int q = 0; q < 3; ++q) k.hdel[jj][q] = (float)hdel[jj][q];
    for (int i = 0; i < 8; ++i) k.P[jj][i] = pair((float)P[i], (float)P[i + 8]);
  }
  for (int jj = 0; jj < nt; ++jj) {
    std::vector<double> Q(16, 0.0);
    double dn = 0.0;
    for (int q = 0; q < 3; ++q) dn += std::fabs(tdel[jj][q]);
    double rest = 0.0;
    for (int r = 0; r < n; ++r) {
      double s = 0.0;
      for (int i = 0; i < nt; ++i) s += qv[i][r] * Rt[i][jj];
      const int cr = r - (n - 16);  // row within the last chunk
      if (cr >= 1) Q[cr] = s;
      else rest = std::fmax(rest, std::fabs(s));
    }
    if (rest * dn > trunc) return fail("tail correction reaches beyond the last 15 rows");
    for (int q = 0; q < 3; ++q) k.tdel[jj][q] = (float)tdel[jj][q];
    for (int i = 0; i < 8; ++i) k.Q[jj][i] = pair((float)Q[i], (float)Q[i + 8]);
  }
  // A's own rows for the residual
  a.ca = splat((float)m.ai);
  a.cb = splat((float)m.bi);
  a.cc = splat((float)m.ci);
  a.cal = splat(to_dwc(m.ai).l);
  a.cbl = splat(to_dwc(m.bi).l);
  a.ccl = splat(to_dwc(m.ci).l);
  a.nca = splat(-(float)m.ai);
  a.ncb = splat(-(float)m.bi);
  a.ncc = splat(-(float)m.ci);
  a.nh = m.nh;
  a.nt = m.nt;
  for (int i = 0; i < 2; ++i) {
    const int hr = i, tr = n - m.nt + i;
    a.hd[i][0] = to_dwc(hr == 0 ? 0.0 : m.a(hr));
    a.hd[i][1] = to_dwc(m.b(hr));
    a.hd[i][2] = to_dwc(m.c(hr));
    a.td[i][0] = to_dwc(tr >= 0 && tr < n ? m.a(tr) : 0.0);
    a.td[i][1] = to_dwc(tr >= 0 && tr < n ? m.b(tr) : 1.0);
    a.td[i][2] = to_dwc(tr >= 0 && tr < n - 1 ? m.c(tr) : 0.0);
  }
  a.sigma0 = a.sigmaN = 1.0;
  a.unit_scale = 1;
  a.sh = splat(1.f);
  a.nsh = splat(-1.f);
  *out = a;
  return true;
}

// The call-dependent part: RHS scales of the compact boundary rows and the
// output scale s.
inline void set_scales(Args* a, double sigma0, double sigmaN, double s) {
  a->sigma0 = sigma0;
  a->sigmaN = sigmaN;
  const DWc d = to_dwc(s);
  a->sh = splat(d.h);
  a->sl = splat(d.l);
  a->nsh = splat(-d.h);
  a->nsl = splat(-d.l);
  a->unit_scale = (s == 1.0) ? 1 : 0;
}

}  // namespace r2
}  // namespace ntk
