// ntk_adi_geom.h -- window geometry of the ADI half steps that cut each
// system into overlapping windows (ntk_adi_refine.cu, ntk_adi_f64.cu).
#pragma once
#include "ntk_internal.h"

namespace ntk {

// Geometry of one half step: systems s = 0 .. ns-1, system s's row i at
// in[s * is + i * es]; windows g = 0 .. P-1 of Lw rows (see window_rows).
struct AdiGeom {
  long long ns = 0;             // systems (N - 2)
  long long is = 0, es = 0;     // line and row strides
  int N = 0, Lw = 0, L = 0, H = 0, P = 1;
  int whole = 0;                // N == Lw: one window, both identity rows
  double gamma = 0.0;           // FP32 windows (rows scaled by dx^2): d = gamma * mid - (lo + hi)
  double bottom = 0.0, center = 0.0, top = 0.0;  // FP64 windows: d = bottom lo + center mid + top hi
  const double* bnd = nullptr;  // identity-row right-hand sides: system s, row i at
  long long bnd_ss = 0;         //   bnd[s * bnd_ss + i * bnd_es]
  long long bnd_es = 0;
};

// Window g: first row, rows written back [lo, hi), and its kind (the
// matrix and tables it uses): 0 first, 1 middle, 2 last, 3 whole.
struct WinRows {
  int start, lo, hi, kind;
};
__host__ __device__ __forceinline__ WinRows window_rows(const AdiGeom& g, int w) {
  WinRows r;
  if (g.whole) {
    r.start = 0, r.lo = 0, r.hi = g.Lw, r.kind = 3;
  } else if (w == 0) {
    r.start = 0, r.lo = 0, r.hi = g.L, r.kind = 0;
  } else if (w < g.P - 1) {
    r.start = w * g.L - g.H, r.lo = g.H, r.hi = g.H + g.L, r.kind = 1;
  } else {
    r.start = g.N - g.Lw, r.lo = (g.P - 1) * g.L - (g.N - g.Lw), r.hi = g.Lw, r.kind = 2;
  }
  return r;
}

}  // namespace ntk
