// ntk_batch_refine.cu -- uneven batches in FP32 + double-word refinement.
//
// Same windows as the ADI path (ntk_adi_refine.cu): a system longer than
// Lw = 512 rows is cut into windows overlapping by H-row halos (H: LU
// multiplier products below 2^-56 for the slowest-decaying system), each
// solved by one warp and writing back only its central rows; a shorter
// system is one window padded with identity rows.  Two solves share the
// launch:
//  * paired-chunk windows (the full windows of every system whose window
//    kinds qualify): the solve of ntk_r2_group.cuh with each window kind's
//    constants (the interior Toeplitz factors and the Woodbury end
//    corrections, prepared on the host once per batch by r2::prepare) and
//    interior coefficients of any value in the residual (res_pair_gen);
//  * chunked windows (short systems, and full windows of systems whose
//    factors decay too slowly for the paired-chunk limits): the refine
//    kernel's machinery (refine_system); every system has its own
//    coefficients, so each warp builds its window's FP32 factor tables
//    itself, lane-parallel: lane j runs the pivot recurrence over its 16
//    rows starting from the system's converged pivot carried through the
//    two rows before its chunk (lane 0 from the window's exact first row).
//    For these near-Toeplitz matrices the pivots reach the fixed point
//    within a few rows (the transient shrinks by ~(a c / u^2) per row), so
//    the tables are the window's FP32 LU; they only precondition the
//    refinement, whose residual uses the exact double-word rows.
//
// One launch, in place, no waiting.  A paired-chunk CTA stages its four
// windows before a CTA barrier, so only the central rows that a window of
// another CTA reads are border rows (ntk_batch_borders.h); they go to the
// work array, so d keeps every row another CTA reads unchanged while the
// system's windows run; after a second barrier the CTA counts its windows on
// the system's counter, and the CTA that completes the count copies the
// system's border rows from work into d and resets the counter.  Chunked
// windows count and copy per window against both neighbours (finish_system).
#include <algorithm>
#include <cmath>
#include <vector>

#include "ntk_batch_borders.h"
#include "ntk_batch_refine.h"
#include "ntk_r2_group.cuh"
#include "ntk_r2_host.h"
#include "ntk_refine.cuh"

namespace ntk {

// One window: rows [r0, r0 + nwin) of a system; written back: window rows
// [out_lo, out_hi).  Row coefficients as refine_system reads them.
struct BatchWin {
  long long off = 0;  // element offset of window row 0 in d
  int nwin = 0;
  int out_lo = 0, out_hi = 0;
  int nh = 1, nt = 1;  // special rows at the window's head / tail
  float uinf = 1.f;    // the system's converged pivot (FP32)
  DW ai, bi, ci;
  DW hd[2][3];
  DW td[2][3];
  DW s;                // output scale (1)
  int unit_scale = 1;
  // central rows r < blo or r >= bhi are border rows (a neighbouring window
  // reads them): written to work during the solve, copied into d at the end
  int blo = 0, bhi = 0;
  int sysi = 0;                // the system's counter
  int wfirst = 0, wcount = 1;  // the system's windows
  int args = -1;               // paired-chunk windows: index of the kind's constants
  int ccount = 0;              // paired-chunk windows: the system's windows in this window's CTA
                               // when it is the first of them there, else 0
  int rfirst = 0, rcount = 0;  // paired-chunk windows: the system's border rows in the row list
};

namespace refine_detail {

constexpr int BM = 16;                  // rows per lane
constexpr int BLW = 32 * BM;            // window rows
#ifndef NTK_BATCH_BW
#define NTK_BATCH_BW 4
#endif
constexpr int BW = NTK_BATCH_BW;        // warps (windows) per CTA (a build flag, for tuning experiments)
// Table slots of one warp: lanes whose chunks (and the three rows before
// them) see the same coefficients build identical tables, so they share a
// slot: 0 lane 0 (the window's head), 1 interior lanes, 2..4 the lanes
// around the system's tail rows, 5 lanes wholly in the padding.
constexpr int BSLOTS = 6;
constexpr int NROWS_R2 = 512;           // rows of a paired-chunk window
constexpr int BTAB = BSLOTS * class_pitch4<BM>();  // float4s of one warp's tables

__device__ __forceinline__ void row_coeffs(const BatchWin& w, int r, float& a, float& b, float& c) {
  if (r >= w.nwin) {
    a = 0.f;
    b = 1.f;
    c = 0.f;
  } else if (r < w.nh) {
    a = w.hd[r][0].h;
    b = w.hd[r][1].h;
    c = w.hd[r][2].h;
  } else if (r >= w.nwin - w.nt) {
    const int q = r - (w.nwin - w.nt);
    a = w.td[q][0].h;
    b = w.td[q][1].h;
    c = w.td[q][2].h;
  } else {
    a = w.ai.h;
    b = w.bi.h;
    c = w.ci.h;
  }
}

// Slot of lane j (its table depends on rows 16j - 3 .. 16j + 15): lane 0
// alone; lanes whose rows reach the tail rows or the padding start
// (16j + 15 >= nwin - nt and 16j - 3 < nwin) by position; lanes wholly in
// the padding (16j - 3 >= nwin) one slot; all other lanes one interior slot.
// The writer of a slot is the first lane that maps to it.
__device__ __forceinline__ void slot_of(const BatchWin& w, int j, int& slot, bool& writer) {
  const int r0 = j * BM;
  if (j == 0) {
    slot = 0;
    writer = true;
    return;
  }
  // first lane reaching the tail region
  const int jft = max(1, (w.nwin - w.nt - (BM - 1) + (BM - 1)) / BM);
  if (r0 - 3 >= w.nwin) {
    // wholly padding: the first such lane writes
    const int jpad = max(1, (w.nwin + 3 + BM - 1) / BM);
    slot = 5;
    writer = (j == jpad);
    return;
  }
  if (j >= jft) {
    slot = 2 + min(j - jft, 2);
    writer = (j - jft) <= 2;
    return;
  }
  slot = 1;
  writer = (j == 1);
}

// After window w of a multi-window system: count it done; the warp of the
// system's last window copies every border row of the system from work into
// d (by then no window of the system reads d any more) and resets the
// counter for the next launch.
template <class WIN>
__device__ __forceinline__ void finish_system(const double* work, double* d, const WIN* __restrict__ wins,
                                              const WIN& w, unsigned* done, unsigned lane) {
  __syncwarp();
  unsigned last = 0;
  if (lane == 0) {
    __threadfence();
    last = atomicAdd(done + w.sysi, 1u) == (unsigned)w.wcount - 1;
    if (last) __threadfence();
  }
  if (!__shfl_sync(0xffffffffu, last, 0)) return;
  border_copy(work, d, w.wfirst, w.wcount, lane, [&](int g, long long& base, int& lo, int& blo, int& bhi, int& hi) {
    const WIN* v = wins + g;
    base = __ldg(&v->off);
    lo = __ldg(&v->out_lo);
    hi = __ldg(&v->out_hi);
    blo = min(__ldg(&v->blo), hi);
    bhi = max(__ldg(&v->bhi), lo);
  });
  if (lane == 0) done[w.sysi] = 0u;
}

// Window `item` by one warp: all rows read from d, the central rows written
// to d except the border rows, which go to work.
template <int SWEEPS, bool PAD>
__device__ __forceinline__ void refine_window(double* work, double* dst, const BatchWin* __restrict__ wins,
                                           long long item, unsigned* status, unsigned* done, float4* tq,
                                           BatchWin* wa, double* trow, unsigned lane) {
  unsigned range = 0;

  // window descriptor into shared memory
  {
    const int* g = reinterpret_cast<const int*>(wins + item);
    int* sdst = reinterpret_cast<int*>(wa);
    constexpr int NW = (int)(sizeof(BatchWin) / sizeof(int));
    for (int i = lane; i < NW; i += 32) sdst[i] = __ldg(g + i);
  }
  __syncwarp();
  const BatchWin& w = *wa;
  // stage the window (rows lane + 32q; zero beyond nwin)
  {
#pragma unroll
    for (int q = 0; q < BM; ++q) {
      const int r = (int)lane + 32 * q;
      const bool ok = !PAD || r < w.nwin;
      cp_async8(trow + tile_off<BM>(r), ok ? dst + w.off + r : dst, ok ? 8u : 0u);
    }
  }
  // FP32 factor tables of this lane's 16 rows (layout of ChunkTabs)
  {
    const int r0 = (int)lane * BM;
    float l[BM], g[BM], wv[BM];
    float a, b, c, cprev;
    float u;
    if (lane == 0) {
      u = 0.f;
      cprev = 0.f;
    } else {
      // incoming pivot: the converged one, carried through the two rows
      // before the chunk (they may be the system's special tail rows)
      float ap, bp;
      row_coeffs(w, r0 - 3, ap, bp, cprev);
      u = w.uinf;
#pragma unroll
      for (int r = r0 - 2; r < r0; ++r) {
        row_coeffs(w, r, a, b, c);
        u = b - (a / u) * cprev;
        cprev = c;
      }
    }
#pragma unroll
    for (int k = 0; k < BM; ++k) {
      row_coeffs(w, r0 + k, a, b, c);
      const float lk = (r0 + k == 0) ? 0.f : a / u;
      u = b - lk * cprev;
      l[k] = lk;
      g[k] = 1.f / u;
      wv[k] = c * g[k];
      cprev = c;
    }
    float phi = 1.f, psi = 1.f;
    float ph[BM], ps[BM];
#pragma unroll
    for (int k = 0; k < BM; ++k) {
      phi *= -l[k];
      ph[k] = phi;
    }
#pragma unroll
    for (int k = BM - 1; k >= 0; --k) {
      psi *= -wv[k];
      ps[k] = psi;
    }
    // this lane's slot, and whether it writes it (one writer per slot)
    int slot;
    bool writer;
    slot_of(w, (int)lane, slot, writer);
    float4* t = tq + slot * class_pitch4<BM>();
    if (writer)
#pragma unroll
    for (int j = 0; j < BM / 4; ++j) {
      t[5 * j + 0] = make_float4(l[4 * j], l[4 * j + 1], l[4 * j + 2], l[4 * j + 3]);
      t[5 * j + 1] = make_float4(g[4 * j], g[4 * j + 1], g[4 * j + 2], g[4 * j + 3]);
      t[5 * j + 2] = make_float4(wv[4 * j], wv[4 * j + 1], wv[4 * j + 2], wv[4 * j + 3]);
      t[5 * j + 3] = make_float4(ph[4 * j], ph[4 * j + 1], ph[4 * j + 2], ph[4 * j + 3]);
      t[5 * j + 4] = make_float4(ps[4 * j], ps[4 * j + 1], ps[4 * j + 2], ps[4 * j + 3]);
    }
  }
  cp_async_wait_all();
  __syncwarp();
  ChunkTabs tabs;
  {
    int slot;
    bool writer;
    slot_of(w, (int)lane, slot, writer);
    tabs.q = tq + slot * class_pitch4<BM>();
  }
  refine_system<BM, RHS_IDENTITY, SWEEPS, false, PAD, false, BatchWin>(trow, nullptr, tabs, w.nwin, w, lane, range);
  __syncwarp();
  {
#pragma unroll 4
    for (int q = 0; q < BM; ++q) {
      const int r = (int)lane + 32 * q;
      if (r >= w.out_lo && r < w.out_hi) {
        const bool border = r < w.blo || r >= w.bhi;
        (border ? work : dst)[w.off + r] = trow[tile_off<BM>(r)];
      }
    }
  }
  if (range && status) atomicOr(status, 1u);
  if (w.wcount > 1) finish_system(work, dst, wins, w, done, lane);
}

// The chunked path's windows as separate (not inlined) functions: one kernel
// holding them inline beside the paired-chunk windows spills heavily.
template <int SWEEPS, bool PAD>
__device__ __noinline__ void refine_window_call(double* work, double* dst, const BatchWin* __restrict__ wins,
                                                long long item, unsigned* status, unsigned* done, float4* tq,
                                                BatchWin* wa, double* trow, unsigned lane) {
  refine_window<SWEEPS, PAD>(work, dst, wins, item, status, done, tq, wa, trow, lane);
}

// A full window whose system qualifies for the paired-chunk solve
// (ntk_r2_group.cuh): the FP32 solve of the pure Toeplitz matrix with the
// window kind's Woodbury end corrections (Args, computed on the host once per
// batch and copied into shared memory), interior coefficients of any value
// in the residual.  The warp stages its 512 rows with 8-byte copies into a
// 4 KB tile in the 128-byte-swizzled layout the solve reads (rows 2i, 2i + 1
// of chunk j at xpair(j, i)); after a CTA barrier (every window of the CTA
// has read its rows) it rewrites them as (hi, lo) pairs, solves, puts the
// results back into the tile and stores the window's central rows with
// coalesced stores.  Neighbouring windows in the same CTA have read their
// rows before the barrier, so only rows that a window in another CTA reads
// (border rows) go to the work array.
__device__ __forceinline__ void r2_stage(const double* d, const BatchWin* __restrict__ wp,
                                         const r2::Args* __restrict__ args, r2::Args* sa, double* tile,
                                         unsigned lane) {
  const long long off = __ldg(&wp->off);
  {
    const unsigned long long* g = reinterpret_cast<const unsigned long long*>(args + __ldg(&wp->args));
    unsigned long long* sd = reinterpret_cast<unsigned long long*>(sa);
    constexpr int NA = (int)(sizeof(r2::Args) / sizeof(unsigned long long));
    for (int i = (int)lane; i < NA; i += 32) sd[i] = __ldg(g + i);
  }
  const double* src = d + off;
#pragma unroll
  for (int q = 0; q < BM; ++q) {
    const int r = (int)lane + 32 * q;
    cp_async8(tile + r2::xpair(r >> 4, (r & 15) >> 1) + (r & 1), src + r, 8u);
  }
}

template <int SWEEPS>
__device__ __forceinline__ void r2_solve(double* work, double* dst, const BatchWin* __restrict__ wp,
                                         unsigned* status, const r2::Args* sa, double* tile, unsigned lane) {
  const int j = (int)lane;
  unsigned rmax = 0;
  float2 v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const double2 q = *reinterpret_cast<const double2*>(tile + r2::xpair(j, i));
    float h0, l0, h1, l1;
    r2::split_f64(q.x, h0, l0, rmax);
    r2::split_f64(q.y, h1, l1, rmax);
    if (SWEEPS > 0) *reinterpret_cast<float4*>(tile + r2::xpair(j, i)) = make_float4(h0, l0, h1, l1);
    if (i < 4) {
      v[2 * i].x = h0;
      v[2 * i + 1].x = h1;
    } else {
      v[2 * i - 8].y = h0;
      v[2 * i - 7].y = h1;
    }
  }
  r2::contiguous_solve<SWEEPS, true>(v, tile, j, *sa, [&](int i, double oa0, double oa1, double ob0, double ob1) {
    *reinterpret_cast<double2*>(tile + r2::xpair(j, i)) = make_double2(oa0, oa1);
    *reinterpret_cast<double2*>(tile + r2::xpair(j, i + 4)) = make_double2(ob0, ob1);
  });
  __syncwarp();
  {
    const long long off = __ldg(&wp->off);
    const int lo = __ldg(&wp->out_lo), hi = __ldg(&wp->out_hi);
    const int blo = __ldg(&wp->blo), bhi = __ldg(&wp->bhi);
#pragma unroll 4
    for (int q = 0; q < BM; ++q) {
      const int r = (int)lane + 32 * q;
      if (r >= lo && r < hi)
        ((r < blo || r >= bhi) ? work : dst)[off + r] = tile[r2::xpair(r >> 4, (r & 15) >> 1) + (r & 1)];
    }
  }
  if (__any_sync(0xffffffffu, rmax >= r2::RANGE_MAG) && lane == 0 && status) atomicOr(status, 1u);
}

// After a CTA barrier that follows every window's stores: the first window
// in this CTA of a system that other CTAs share adds the CTA's windows of
// that system to the system's counter.  Returns true (warp-uniform) in the
// warp that completes the count: every window of the system has stored.
__device__ __forceinline__ bool r2_count(const BatchWin* __restrict__ wp, unsigned* done, unsigned lane) {
  const int cc = __ldg(&wp->ccount);
  const int wcount = __ldg(&wp->wcount);
  if (cc == 0 || cc == wcount) return false;  // not the first here, or the whole system is in this CTA
  unsigned last = 0;
  if (lane == 0) {
    __threadfence();
    last = atomicAdd(done + __ldg(&wp->sysi), (unsigned)cc) == (unsigned)(wcount - cc);
    if (last) __threadfence();
  }
  return __shfl_sync(0xffffffffu, last, 0) != 0;
}

// L2 prefetch of window `item`'s rows (issued by one lane): the window the
// warp of the CTA one wave later solves, so its staging finds it in L2.
__device__ __forceinline__ void prefetch_window(const double* d, const BatchWin* __restrict__ wins, long long item) {
  const long long off = __ldg(&wins[item].off);
  const int nwin = __ldg(&wins[item].nwin);
  const uintptr_t a = reinterpret_cast<uintptr_t>(d + off) & ~(uintptr_t)15;
  const uintptr_t e = (reinterpret_cast<uintptr_t>(d + off + nwin) + 15) & ~(uintptr_t)15;
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"((unsigned)(e - a)) : "memory");
}

// The launch's windows: n_r2 paired-chunk windows, then n_old full windows
// of the chunked path (together the full array, one system's windows next
// to each other), then n_pad padded windows; BW per CTA, CTAs [0, c_r2) on
// the first kind, [c_r2, c_r2 + c_old) on the second, the rest on the third.
// (Running the slower chunked windows first measured slower: 0.081 against
// 0.075 ms for the 4096-system batch; at the end they run with fewer warps
// beside them.)
struct BatchGeo {
  int n_r2 = 0, n_old = 0, n_pad = 0;
  unsigned c_r2 = 0, c_old = 0;
  unsigned pf = 0;  // prefetch distance in CTAs (the CTAs resident at once)
};

// Index in wins of warp `warp`'s window in CTA b, kind 0 / 1 / 2 (paired
// chunk / chunked full / padded); -1: none.
__device__ __forceinline__ long long window_of(long long b, int warp, const BatchGeo& g, int& kind) {
  if (b < g.c_r2) {
    kind = 0;
    const long long it = b * BW + warp;
    return it < g.n_r2 ? it : -1;
  }
  b -= g.c_r2;
  if (b < g.c_old) {
    kind = 1;
    const long long it = b * BW + warp;
    return it < g.n_old ? g.n_r2 + it : -1;
  }
  b -= g.c_old;
  kind = 2;
  const long long it = b * BW + warp;
  return it < g.n_pad ? (long long)g.n_r2 + g.n_old + it : -1;
}

// shared memory of a paired-chunk CTA: BW tiles of 512 rows, then BW Args
constexpr size_t R2_ARGS_BYTES = (sizeof(r2::Args) + 15) / 16 * 16;
constexpr size_t r2_smem() { return (size_t)BW * NROWS_R2 * sizeof(double) + (size_t)BW * R2_ARGS_BYTES; }

// CTAs per SM the kernel is compiled for (registers per thread: 65536 /
// (32 BW x this)); a build flag, for tuning experiments.  Five (96
// registers) measured 0.068 ms for the 4096-system batch against 0.069-0.070
// with six (80 registers, more spilled) and 0.089 with one 16-warp CTA.
#ifndef NTK_BATCH_MINB
#define NTK_BATCH_MINB 5
#endif

// The whole batch in one launch.  Each warp first prefetches into L2 the
// window of the warp pf CTAs further on (pf = the CTAs resident at once).
template <int SWEEPS>
__global__ void __launch_bounds__(32 * BW, NTK_BATCH_MINB)
    batch_refine_kernel(double* work, double* d, const BatchWin* __restrict__ wins,
                        const r2::Args* __restrict__ args, const long long* __restrict__ border_rows,
                        unsigned* status, unsigned* done, const __grid_constant__ BatchGeo g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int P = sys_pitch<BM>();
  const int warp = threadIdx.x >> 5;
  const unsigned lane = threadIdx.x & 31;
  if (lane == 0 && g.pf > 0) {
    int k;
    const long long nb = window_of((long long)blockIdx.x + g.pf, warp, g, k);
    if (nb >= 0) prefetch_window(d, wins, nb);
  }
  int kind;
  const long long it = window_of(blockIdx.x, warp, g, kind);
  if (kind == 0) {  // the whole CTA: every thread reaches both barriers
    double* tile = reinterpret_cast<double*>(smem_raw) + (size_t)warp * NROWS_R2;
    r2::Args* sa = reinterpret_cast<r2::Args*>(smem_raw + (size_t)BW * NROWS_R2 * sizeof(double) +
                                               (size_t)warp * R2_ARGS_BYTES);
    __shared__ int last_win[BW];  // windows whose warp completed their system's count
    const BatchWin* wp = wins + (it >= 0 ? it : 0);
    if (it >= 0) r2_stage(d, wp, args, sa, tile, lane);
    cp_async_wait_all();
    __syncthreads();  // every window of the CTA has read its rows from d
    if (it >= 0) r2_solve<SWEEPS>(work, d, wp, status, sa, tile, lane);
    __syncthreads();  // every window of the CTA has stored its rows
    const bool last = it >= 0 && r2_count(wp, done, lane);
    if (lane == 0) last_win[warp] = last ? (int)it : -1;
    __syncthreads();
    // the systems this CTA completed: every window of theirs has stored, so
    // their border rows go from work into d (by then nothing reads them)
    for (int k = 0; k < BW; ++k) {
      const int wi = last_win[k];
      if (wi < 0) continue;
      const BatchWin* lw = wins + wi;
      row_copy(work, d, border_rows + __ldg(&lw->rfirst), __ldg(&lw->rcount), (int)threadIdx.x, 32 * BW);
      if (threadIdx.x == 0) done[__ldg(&lw->sysi)] = 0u;
    }
    return;
  }
  if (it < 0) return;
  float4* tq = reinterpret_cast<float4*>(smem_raw) + (size_t)warp * BTAB;
  BatchWin* wa = reinterpret_cast<BatchWin*>(reinterpret_cast<float4*>(smem_raw) + (size_t)BW * BTAB) + warp;
  double* trow = reinterpret_cast<double*>(reinterpret_cast<BatchWin*>(reinterpret_cast<float4*>(smem_raw) +
                                                                        (size_t)BW * BTAB) + BW) + (size_t)warp * P;
  if (kind == 1)
    refine_window_call<SWEEPS, false>(work, d, wins, it, status, done, tq, wa, trow, lane);
  else
    refine_window_call<SWEEPS, true>(work, d, wins, it, status, done, tq, wa, trow, lane);
}

constexpr size_t batch_smem() {
  return std::max((size_t)BW * BTAB * sizeof(float4) + (size_t)BW * sizeof(BatchWin) +
                      (size_t)BW * sys_pitch<BM>() * sizeof(double),
                  r2_smem());
}

}  // namespace refine_detail

struct BatchRefine {
  int sweeps = 1;
  refine_detail::BatchGeo geo;
  unsigned ctas = 0;
  BatchWin* d_wins = nullptr;
  r2::Args* d_args = nullptr;  // the paired-chunk window kinds' constants
  long long* d_rows = nullptr;  // the paired-chunk windows' border rows, grouped by system
  unsigned* d_status = nullptr;
  unsigned* d_done = nullptr;  // per system: its windows finished in the current launch
  ~BatchRefine() {
    if (d_wins) cudaFree(d_wins);
    if (d_args) cudaFree(d_args);
    if (d_rows) cudaFree(d_rows);
    if (d_status) cudaFree(d_status);
    if (d_done) cudaFree(d_done);
  }
};

namespace {

DW to_dw(double v) {
  DW d;
  d.h = (float)v;
  d.l = (float)(v - (double)d.h);
  return d;
}

}  // namespace

void batch_refine_status_words(const BatchRefine* br, std::vector<unsigned*>& out) {
  if (br && br->d_status) out.push_back(br->d_status);
}

int batch_refine_create(BatchRefine** out, long long nsys, const int* n, const long long* offset,
                        const double* interior, const double* head, const double* tail, int precision) {
  using namespace refine_detail;
  *out = nullptr;
  // halo for the slowest-decaying system: interior pivot fixed point and
  // the product of multipliers over H rows below 2^-56
  std::vector<double> uinf(nsys);
  double worst = 0.0;
  for (long long s = 0; s < nsys; ++s) {
    const double a = interior[3 * s], b = interior[3 * s + 1], c = interior[3 * s + 2];
    double u = b;
    for (int i = 0; i < 4096; ++i) {
      const double un = b - a * c / u;
      if (un == u || !std::isfinite(un)) break;
      u = un;
    }
    if (!(u != 0.0) || !std::isfinite(u)) {
      set_error("ntk_batch_create: system %lld has no finite pivot fixed point", s);
      return NTK_ERR_INVALID;
    }
    uinf[s] = u;
    worst = std::max(worst, std::max(std::fabs(a / u), std::fabs(c / u)));
  }
  if (!(worst < 0.75)) {
    set_error("ntk_batch_create: FP32/refine needs pivots that decay (|a/u|, |c/u| < 0.75; got %g); use NTK_FP64",
              worst);
    return NTK_ERR_UNSUPPORTED;
  }
  int H = 4;
  {
    double prod = 1.0;
    H = 0;
    while (prod > std::ldexp(1.0, -56)) {
      prod *= worst;
      ++H;
    }
    H = (H + 3) & ~1;
  }
  const int L = BLW - 2 * H;
  // Full windows of systems whose window kinds all qualify for the
  // paired-chunk solve go to r2w (their kinds' constants in r2args), the
  // other full windows to full, short systems to padded.  Limits: with
  // refinement the FP32 solve's truncations may reach 2^-22 (one sweep then
  // leaves ~2^-44); the FP32-only precision keeps the compact plans' limits.
  r2::PrepareLimits lim;
  lim.general = true;
  if (precision != NTK_FP32) {
    lim.carry = std::ldexp(1.0, -22);
    lim.trunc = std::ldexp(1.0, -22);
  }
  std::vector<BatchWin> r2w, full, padded;
  std::vector<r2::Args> r2args;
  for (long long s = 0; s < nsys; ++s) {
    const int ns = n[s];
    BatchWin base;
    base.uinf = (float)uinf[s];
    base.ai = to_dw(interior[3 * s]);
    base.bi = to_dw(interior[3 * s + 1]);
    base.ci = to_dw(interior[3 * s + 2]);
    base.s = to_dw(1.0);
    base.unit_scale = 1;
    base.sysi = (int)s;
    // the system's own head rows (0, 1) and tail rows (n-2, n-1); for n = 3
    // the middle row is head's second row (ntk_batch_create's rule)
    auto set_head = [&](BatchWin& w) {
      w.nh = 2;
      for (int r = 0; r < 2; ++r)
        for (int k = 0; k < 3; ++k) w.hd[r][k] = to_dw(head[6 * s + 3 * r + k]);
      w.hd[0][0] = to_dw(0.0);
    };
    auto set_tail = [&](BatchWin& w, int nrow) {
      w.nt = std::min(2, nrow - w.nh);
      for (int q = 0; q < w.nt; ++q) {
        const int r = 2 - w.nt + q;  // tail row index within (n-2, n-1)
        for (int k = 0; k < 3; ++k) w.td[q][k] = to_dw(tail[6 * s + 3 * r + k]);
      }
      w.td[w.nt - 1][2] = to_dw(0.0);
    };
    auto cut_head = [&](BatchWin& w) {
      w.nh = 1;
      w.hd[0][0] = to_dw(0.0);
      w.hd[0][1] = base.bi;
      w.hd[0][2] = base.ci;
    };
    auto cut_tail = [&](BatchWin& w) {
      w.nt = 1;
      w.td[0][0] = base.ai;
      w.td[0][1] = base.bi;
      w.td[0][2] = to_dw(0.0);
    };
    if (ns < BLW) {
      BatchWin w = base;
      w.off = offset[s];
      w.nwin = ns;
      w.out_lo = 0;
      w.out_hi = ns;
      set_head(w);
      if (ns >= 4) {
        set_tail(w, ns);
      } else {  // n = 3: rows 0, 1 from head, row 2 from tail's last row
        w.nt = 1;
        for (int k = 0; k < 3; ++k) w.td[0][k] = to_dw(tail[6 * s + 3 + k]);
        w.td[0][2] = to_dw(0.0);
      }
      w.blo = w.out_lo;  // a whole system: no border rows
      w.bhi = w.out_hi;
      padded.push_back(w);
      continue;
    }
    // windows of 512 rows: one whole window, or first, middle..., last
    // overlapping by the halos
    std::vector<BatchWin> sw;
    if (ns == BLW) {
      BatchWin w = base;
      w.off = offset[s];
      w.nwin = BLW;
      w.out_lo = 0;
      w.out_hi = BLW;
      set_head(w);
      set_tail(w, BLW);
      sw.push_back(w);
    } else {
      const int Pw = (ns - BLW + H + L - 1) / L + 1;
      for (int g = 0; g < Pw; ++g) {
        BatchWin w = base;
        w.nwin = BLW;
        int start;
        if (g == 0) {
          start = 0;
          w.out_lo = 0;
          w.out_hi = L;
          set_head(w);
          cut_tail(w);
        } else if (g < Pw - 1) {
          start = g * L - H;
          w.out_lo = H;
          w.out_hi = H + L;
          cut_head(w);
          cut_tail(w);
        } else {
          start = ns - BLW;
          w.out_lo = (Pw - 1) * L - start;
          w.out_hi = BLW;
          cut_head(w);
          set_tail(w, BLW);
        }
        w.off = offset[s] + start;
        sw.push_back(w);
      }
    }
    // border rows: central rows the neighbouring windows read
    const int Pw = (int)sw.size();
    for (int g = 0; g < Pw; ++g) {
      BatchWin& w = sw[g];
      w.wcount = Pw;
      const long long st = w.off - offset[s];
      w.blo = w.out_lo;
      w.bhi = w.out_hi;
      if (g > 0) w.blo = (int)std::min<long long>(w.out_hi, sw[g - 1].off - offset[s] + BLW - st);
      if (g + 1 < Pw) w.bhi = (int)std::max<long long>(w.out_lo, sw[g + 1].off - offset[s] - st);
    }
    // the paired-chunk constants of the system's window kinds (first,
    // middle, last, or whole): head rows cut (row 0 = (0, b, c)) or the
    // system's own, tail rows the system's own or none (the interior row
    // with c dropped, as the Toeplitz matrix has it)
    int kinds[3] = {-1, -1, -1};  // index in r2args of: the first (or whole), a middle, the last window
    bool ok = true;
    for (int g = 0; g < Pw && ok; ++g) {
      const int kind = (g == 0) ? 0 : (g == Pw - 1 ? 2 : 1);
      if (kinds[kind] >= 0) {
        sw[g].args = kinds[kind];
        continue;
      }
      r2::MatrixRows m;
      m.n = BLW;
      m.ai = interior[3 * s];
      m.bi = interior[3 * s + 1];
      m.ci = interior[3 * s + 2];
      if (g == 0) {
        m.nh = 2;
        for (int r = 0; r < 2; ++r)
          for (int k = 0; k < 3; ++k) m.head[r][k] = head[6 * s + 3 * r + k];
        m.head[0][0] = 0.0;
      } else {
        m.nh = 1;
        m.head[0][0] = 0.0;
        m.head[0][1] = m.bi;
        m.head[0][2] = m.ci;
      }
      if (g == Pw - 1) {
        m.nt = 2;
        for (int r = 0; r < 2; ++r)
          for (int k = 0; k < 3; ++k) m.tail[r][k] = tail[6 * s + 3 * r + k];
        m.tail[1][2] = 0.0;
      } else {
        m.nt = 0;
      }
      r2::Args a;
      if (!r2::prepare(m, &a, nullptr, lim)) {
        ok = false;
        break;
      }
      a.status = nullptr;
      kinds[kind] = (int)r2args.size();
      sw[g].args = kinds[kind];
      r2args.push_back(a);
    }
    if (!ok) {
      // unused constants of this system stay in r2args (harmless)
      for (BatchWin& w : sw) w.args = -1;
    }
    std::vector<BatchWin>& dst = ok ? r2w : full;
    const int first = (int)dst.size();
    for (BatchWin& w : sw) {
      w.wfirst = first;  // the chunked path's indices move past r2w below
      dst.push_back(w);
    }
  }
  for (BatchWin& w : full) w.wfirst += (int)r2w.size();
  // paired-chunk windows: border rows against other CTAs only (ntk_batch_borders.h)
  std::vector<long long> rows;
  cta_borders(
      r2w, BW, BLW, [](const BatchWin& w) { return w.off; }, [](const BatchWin& w) { return w.out_lo; },
      [](const BatchWin& w) { return w.out_hi; }, rows);
  BatchRefine* br = new (std::nothrow) BatchRefine();
  if (!br) {
    set_error("out of host memory");
    return NTK_ERR_ALLOC;
  }
  br->sweeps = (precision == NTK_FP32) ? 0 : 1;
  BatchGeo& geo = br->geo;
  geo.n_r2 = (int)r2w.size();
  geo.n_old = (int)full.size();
  geo.n_pad = (int)padded.size();
  geo.c_r2 = (unsigned)((geo.n_r2 + BW - 1) / BW);
  geo.c_old = (unsigned)((geo.n_old + BW - 1) / BW);
  br->ctas = geo.c_r2 + geo.c_old + (unsigned)((geo.n_pad + BW - 1) / BW);
  std::vector<BatchWin> all(r2w);
  all.insert(all.end(), full.begin(), full.end());
  all.insert(all.end(), padded.begin(), padded.end());
  int rc = NTK_OK;
  if (!all.empty()) {
    rc = cuda_status(cudaMalloc(&br->d_wins, sizeof(BatchWin) * all.size()), "cudaMalloc(batch windows)");
    if (!rc)
      rc = cuda_status(cudaMemcpy(br->d_wins, all.data(), sizeof(BatchWin) * all.size(), cudaMemcpyHostToDevice),
                       "cudaMemcpy(batch windows)");
  }
  if (!rc && !r2args.empty()) {
    rc = cuda_status(cudaMalloc(&br->d_args, sizeof(r2::Args) * r2args.size()), "cudaMalloc(window constants)");
    if (!rc)
      rc = cuda_status(
          cudaMemcpy(br->d_args, r2args.data(), sizeof(r2::Args) * r2args.size(), cudaMemcpyHostToDevice),
          "cudaMemcpy(window constants)");
  }
  if (!rc && !rows.empty()) {
    rc = cuda_status(cudaMalloc(&br->d_rows, sizeof(long long) * rows.size()), "cudaMalloc(border rows)");
    if (!rc)
      rc = cuda_status(cudaMemcpy(br->d_rows, rows.data(), sizeof(long long) * rows.size(), cudaMemcpyHostToDevice),
                       "cudaMemcpy(border rows)");
  }
  if (!rc) rc = cuda_status(cudaMalloc(&br->d_status, sizeof(unsigned)), "cudaMalloc(status)");
  if (!rc) rc = cuda_status(cudaMemset(br->d_status, 0, sizeof(unsigned)), "cudaMemset(status)");
  if (!rc) rc = cuda_status(cudaMalloc(&br->d_done, sizeof(unsigned) * (size_t)nsys), "cudaMalloc(system counters)");
  if (!rc) rc = cuda_status(cudaMemset(br->d_done, 0, sizeof(unsigned) * (size_t)nsys), "cudaMemset(system counters)");
  if (!rc) {
    auto kern = br->sweeps == 0 ? batch_refine_kernel<0> : batch_refine_kernel<1>;
    rc = cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)batch_smem()),
                     "cudaFuncSetAttribute(batch_refine_kernel)");
    int dev = 0, sms = 0, per_sm = 0;
    if (!rc) rc = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if (!rc) rc = cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
    if (!rc)
      rc = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * BW, batch_smem()),
                       "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    geo.pf = (unsigned)(per_sm * sms);
  }
  if (rc) {
    delete br;
    return rc;
  }
  *out = br;
  return NTK_OK;
}

void batch_refine_destroy(BatchRefine* br) { delete br; }

long long batch_refine_windows(const BatchRefine* br) {
  return (long long)br->geo.n_r2 + br->geo.n_old + br->geo.n_pad;
}

long long batch_refine_paired_windows(const BatchRefine* br) { return br->geo.n_r2; }

int batch_refine_solve(BatchRefine* br, double* d, double* work, cudaStream_t st) {
  using namespace refine_detail;
  if (br->ctas == 0) return NTK_OK;
  auto kern = br->sweeps == 0 ? batch_refine_kernel<0> : batch_refine_kernel<1>;
  kern<<<br->ctas, 32 * BW, batch_smem(), st>>>(work, d, br->d_wins, br->d_args, br->d_rows, br->d_status,
                                                br->d_done, br->geo);
  return cuda_status(cudaGetLastError(), "batch_refine_kernel");
}

}  // namespace ntk
