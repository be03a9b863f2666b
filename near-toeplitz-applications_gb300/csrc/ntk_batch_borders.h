// ntk_batch_borders.h -- border rows of uneven-batch windows that run
// per_cta to a CTA (ntk_batch.cu, ntk_batch_refine.cu), host side.
//
// Windows are len rows long, listed system by system (a system's windows
// consecutive, their starts increasing), per_cta consecutive windows to a
// CTA.  Every window of a CTA reads its rows before any of them stores (a
// CTA barrier), so only the central rows that a window in another CTA reads
// are border rows (stored to the work array, copied into d once every window
// of the system has stored): the rows below the end of the system's last
// window in an earlier CTA and those from the start of its first window in a
// later CTA.  The row ranges grow with the window index, so these two bound
// every other CTA's reads; the last window of a system, which starts at
// n - len, can reach back past its neighbour into the window before it,
// which a rule against the immediate neighbours alone would miss.
#pragma once
#include <algorithm>
#include <vector>

namespace ntk {

// WIN has int blo, bhi, wfirst, wcount, ccount, rfirst, rcount; start(w) is
// the absolute row of window w's row 0, lo(w) / hi(w) its central rows.
// Sets blo / bhi, ccount (the system's windows in the CTA, on the first of
// them there; else 0) and each system's border rows (absolute, appended to
// rows; rfirst / rcount on every window of the system).
template <class WIN, class START, class LO, class HI>
void cta_borders(std::vector<WIN>& ws, int per_cta, int len, START start, LO lo, HI hi, std::vector<long long>& rows) {
  for (size_t i = 0; i < ws.size(); ++i) {
    WIN& w = ws[i];
    const size_t first = (size_t)w.wfirst, last = first + (size_t)w.wcount - 1;
    const size_t cta = i / per_cta;
    const size_t cta_lo = cta * per_cta, cta_hi = cta_lo + per_cta - 1;
    const long long s = start(w);
    w.blo = lo(w);
    w.bhi = hi(w);
    if (cta_lo > first) {  // the system's last window in an earlier CTA
      const long long end = start(ws[cta_lo - 1]) + len - s;
      w.blo = (int)std::min<long long>(hi(w), std::max<long long>(lo(w), end));
    }
    if (cta_hi < last) {  // the system's first window in a later CTA
      const long long from = start(ws[cta_hi + 1]) - s;
      w.bhi = (int)std::max<long long>(lo(w), std::min<long long>(hi(w), from));
    }
    w.ccount = 0;
    if (i == first || (i - 1) / per_cta != cta) {
      size_t e = i;
      while (e < last && (e + 1) / per_cta == cta) ++e;
      w.ccount = (int)(e - i + 1);
    }
  }
  for (size_t i = 0; i < ws.size();) {
    const size_t end = i + (size_t)ws[i].wcount;
    const int rf = (int)rows.size();
    for (size_t k = i; k < end; ++k) {
      const WIN& w = ws[k];
      const long long s = start(w);
      for (int r = lo(w); r < hi(w); ++r)  // the two ranges can overlap: each row once
        if (r < w.blo || r >= w.bhi) rows.push_back(s + r);
    }
    for (size_t k = i; k < end; ++k) {
      ws[k].rfirst = rf;
      ws[k].rcount = (int)rows.size() - rf;
    }
    i = end;
  }
}

}  // namespace ntk
