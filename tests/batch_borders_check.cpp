// Host check of the uneven batches' border rows (ntk_batch_borders.h, the
// product's own header), built by the tests with g++: windows laid out as
// ntk_batch_refine.cu (paired-chunk / chunked windows: first, middles, a
// last window starting at n - 512) or ntk_batch.cu (FP64 windows) lay them
// out, per_cta windows to a CTA; every central row that a window of another
// CTA reads must be a border row, the central ranges must partition each
// system, the row list must hold each border row once, and the CTA counts
// must add up to the system's windows.
#include <cstdio>
#include <set>
#include <vector>

#include "ntk_batch_borders.h"

namespace {

struct Win {
  long long start = 0;  // absolute row of window row 0
  int lo = 0, hi = 0;   // central rows
  int blo = 0, bhi = 0, wfirst = 0, wcount = 1, ccount = 0, rfirst = 0, rcount = 0;
};

constexpr int LW = 512;

// ntk_batch_refine.cu: halo H, central L = LW - 2H per middle window
void refine_windows(long long off, int n, int H, std::vector<Win>& ws) {
  const int L = LW - 2 * H;
  const int first = (int)ws.size();
  if (n <= LW) {
    Win w;
    w.start = off, w.lo = 0, w.hi = n;
    ws.push_back(w);
  } else {
    const int P = (n - LW + H + L - 1) / L + 1;
    for (int g = 0; g < P; ++g) {
      Win w;
      if (g == 0) {
        w.start = off, w.lo = 0, w.hi = L;
      } else if (g < P - 1) {
        w.start = off + g * L - H, w.lo = H, w.hi = H + L;
      } else {
        const int st = n - LW;
        w.start = off + st, w.lo = (P - 1) * L - st, w.hi = LW;
      }
      ws.push_back(w);
    }
  }
  for (size_t k = first; k < ws.size(); ++k) ws[k].wfirst = first, ws[k].wcount = (int)ws.size() - first;
}

// ntk_batch.cu (FP64 windows): first window central [0, LW - H), middles
// of up to L central rows, the last window at n - LW
void f64_windows(long long off, int n, int H, std::vector<Win>& ws) {
  const int L = LW - 2 * H;
  const int first = (int)ws.size();
  if (n <= LW) {
    Win w;
    w.start = off, w.lo = 0, w.hi = n;
    ws.push_back(w);
  } else {
    auto add = [&](int w0, int lo, int hi) {
      Win w;
      w.start = off + w0, w.lo = lo, w.hi = hi;
      ws.push_back(w);
    };
    add(0, 0, LW - H);
    int pos = LW - H;
    const int last_w0 = n - LW, last_lo = last_w0 + H;
    while (pos < last_lo) {
      const int w0 = pos - H;
      const int hi = pos + L < last_lo ? pos + L : last_lo;
      add(w0, pos - w0, hi - w0);
      pos = hi;
    }
    add(last_w0, pos - last_w0, LW);
  }
  for (size_t k = first; k < ws.size(); ++k) ws[k].wfirst = first, ws[k].wcount = (int)ws.size() - first;
}

}  // namespace

extern "C" {

// Returns the number of violations (0: every check holds); *nborder = border
// rows in the list.
long long batch_borders_check(int layout, int nsys, const int* n, int H, int per_cta, long long* nborder) {
  std::vector<Win> ws;
  std::vector<long long> offs(nsys);
  long long off = 0;
  for (int s = 0; s < nsys; ++s) {
    offs[s] = off;
    if (layout == 0)
      refine_windows(off, n[s], H, ws);
    else
      f64_windows(off, n[s], H, ws);
    off += n[s] + 1;
  }
  std::vector<long long> rows;
  ntk::cta_borders(
      ws, per_cta, LW, [](const Win& w) { return w.start; }, [](const Win& w) { return w.lo; },
      [](const Win& w) { return w.hi; }, rows);
  long long bad = 0;
  std::set<long long> listed(rows.begin(), rows.end());
  if (listed.size() != rows.size()) ++bad;  // a row listed twice
  long long nb = 0;
  for (size_t i = 0; i < ws.size();) {
    const Win& f = ws[i];
    const size_t end = i + (size_t)f.wcount;
    // central ranges partition the system; counts add up
    long long next = f.start + f.lo;
    int counted = 0;
    for (size_t k = i; k < end; ++k) {
      const Win& w = ws[k];
      if (w.start + w.lo != next) ++bad;
      next = w.start + w.hi;
      counted += w.ccount;
      if (w.blo < w.lo || w.blo > w.hi || w.bhi < w.lo || w.bhi > w.hi) ++bad;
      for (int r = w.lo; r < w.hi; ++r) {
        const bool border = r < w.blo || r >= w.bhi;
        nb += border;
        if (border != (listed.count(w.start + r) == 1)) ++bad;
        for (size_t j = i; j < end; ++j) {  // every other CTA's window reading row r
          if (j / per_cta == k / per_cta) continue;
          const long long a = w.start + r;
          if (a >= ws[j].start && a < ws[j].start + LW && !border) ++bad;
        }
      }
    }
    if (counted != f.wcount) ++bad;
    i = end;
  }
  if (nb != (long long)rows.size()) ++bad;
  *nborder = (long long)rows.size();
  return bad;
}

}  // extern "C"
