// ntk_r2.cu -- the paired-chunk FP32 + refinement solve for systems of 512
// rows (arithmetic in ntk_r2.cuh): the compact derivative and the plain
// solve of the plans' FP32 precisions on GB300, with the tiles moved by TMA.
//
// Two kernels, one per layout:
//
//  * r2x_kernel, contiguous systems (the x derivative, ntk_solve): a CTA
//    holds S systems, one warp per system, lane j owning rows [16j, 16j+16).
//    One TMA load brings the S x 4 KB box into shared memory with the
//    128-byte swizzle, so a lane reading two adjacent rows of its chunk
//    (16 bytes) and the other lanes of its quarter-warp hit eight different
//    16-byte bank groups; chunk carries and edge values move by shuffles.
//  * r2s_kernel, strided systems (the y and z derivatives): a CTA holds 16
//    adjacent systems (128 contiguous bytes per row), a dense [512][16] TMA
//    box; thread (warp w, lane l) owns system l % 16 and chunk 2w + l / 16,
//    so a half-warp reads one 128-byte row and the layout needs no permute
//    and no transpose.  Chunk carries and edge values go through shared
//    memory with CTA barriers.
//
// Each thread: compact RHS (one FP64 subtraction per row) split into a
// double-word, the FP32 solve of the pure Toeplitz factors with the Woodbury
// end corrections, the exact double-word residual, the FP32 correction
// solve, and the FP64 output assembled with integer operations: written in
// place into the tile and stored by TMA for contiguous systems, stored from
// registers (128-byte row segments per half-warp) for strided ones.  Out-of-range
// inputs raise a status bit; a bounded wait on the TMA barrier that runs out
// raises another and skips the group.
#include "ntk_internal.h"
#include "ntk_plan.h"
#include "ntk_r2.h"
#include "ntk_r2_group.cuh"
#include "ntk_r2_tma.cuh"

namespace ntk {
namespace r2 {

// ---------------------------------------------------------------------------
// contiguous systems
// ---------------------------------------------------------------------------
// S contiguous systems (one warp each) solved in place in their swizzled
// tile by the S * 32 threads gt = 0 .. of a group: TMA load of the box at
// coordinates (0, 0, c2, c3) of tin, solve, TMA store to tout.
template <int RHS, int SWEEPS, class SYNC>
__device__ __forceinline__ void contiguous_group(double* tile, float2* bnd, uint64_t* bar, const CUtensorMap* tin,
                                                 const CUtensorMap* tout, int S, int gt, int c2, int c3,
                                                 const Args& a, SYNC sync) {
  const int warp = gt >> 5, j = gt & 31;
  if (gt == 0) mbar_init(bar, 1);
  sync();
  if (gt == 0) {
    mbar_expect_tx(bar, (unsigned)S * NROWS * 8u);
    tma_load(tile, tin, 0, 0, c2, c3, bar);
  }
  // every thread waits (bounded); the group gives up together if any did
  if (!sync.all(mbar_wait(bar, 0))) {
    if (gt == 0 && a.status) atomicOr(a.status, STATUS_TIMEOUT);
    return;
  }
  const Consts& K = a.k;
  unsigned rmax = 0;
  if (RHS == RHS_COMPACT) {
    // one-sided boundary stencils of the S systems, one FP64 sequence for
    // the CTA: lane 2s -> row 0 of system s, lane 2s+1 -> row n-1
    if (warp == 0 && (j >> 1) < S) {
      const double* sy = tile + (j >> 1) * NROWS;
      const bool tl = j & 1;
      const double r0 = tl ? sy[xpair(31, 7) + 1] : sy[xpair(0, 0)];
      const double r1 = tl ? sy[xpair(31, 7)] : sy[xpair(0, 0) + 1];
      const double r2 = tl ? sy[xpair(31, 6) + 1] : sy[xpair(0, 1)];
      float h, l;
      boundary_rhs(r0, r1, r2, tl ? a.sigmaN : a.sigma0, h, l, rmax);
      bnd[j] = make_float2(h, l);
    }
    sync();
  }
  double* sy = tile + warp * NROWS;
  float2 v[8];
  // ---- right-hand side, written back in place as (hi, lo) per row ----
  if (RHS == RHS_COMPACT) {
    const double2 q0 = *reinterpret_cast<const double2*>(sy + xpair(j, 0));
    const double2 q7 = *reinterpret_cast<const double2*>(sy + xpair(j, 7));
    const double fl = __shfl_up_sync(FULL, q7.y, 1);    // row 16j - 1
    const double fr = __shfl_down_sync(FULL, q0.x, 1);  // row 16j + 16
    double prev = fl;
    double2 cur = q0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      double2 nxt;
      if (i < 6) nxt = *reinterpret_cast<const double2*>(sy + xpair(j, i + 1));
      else if (i == 6) nxt = q7;
      else nxt = make_double2(fr, 0.0);
      float h0, l0, h1, l1;
      split_f64(dsub_(cur.y, prev), h0, l0, rmax);
      split_f64(dsub_(nxt.x, cur.x), h1, l1, rmax);
      if (i == 0 && j == 0) {
        const float2 b = bnd[2 * warp];
        h0 = b.x;
        l0 = b.y;
      }
      if (i == 7 && j == 31) {
        const float2 b = bnd[2 * warp + 1];
        h1 = b.x;
        l1 = b.y;
      }
      *reinterpret_cast<float4*>(sy + xpair(j, i)) = make_float4(h0, l0, h1, l1);
      if (i < 4) {
        v[2 * i].x = h0;
        v[2 * i + 1].x = h1;
      } else {
        v[2 * i - 8].y = h0;
        v[2 * i - 7].y = h1;
      }
      prev = cur.y;
      cur = nxt;
    }
  } else {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const double2 q = *reinterpret_cast<const double2*>(sy + xpair(j, i));
      float h0, l0, h1, l1;
      split_f64(q.x, h0, l0, rmax);
      split_f64(q.y, h1, l1, rmax);
      *reinterpret_cast<float4*>(sy + xpair(j, i)) = make_float4(h0, l0, h1, l1);
      if (i < 4) {
        v[2 * i].x = h0;
        v[2 * i + 1].x = h1;
      } else {
        v[2 * i - 8].y = h0;
        v[2 * i - 7].y = h1;
      }
    }
  }
  contiguous_solve<SWEEPS>(v, sy, j, a, [&](int i, double oa0, double oa1, double ob0, double ob1) {
    *reinterpret_cast<double2*>(sy + xpair(j, i)) = make_double2(oa0, oa1);
    *reinterpret_cast<double2*>(sy + xpair(j, i + 4)) = make_double2(ob0, ob1);
  });
  if (__any_sync(FULL, rmax >= RANGE_MAG) && j == 0 && a.status) atomicOr(a.status, 1u);
  fence_proxy_async();
  sync();
  if (gt == 0) {
    tma_store(tout, 0, 0, c2, c3, tile);
    tma_store_commit_and_wait();
  }
}

// One group of S = blockDim.x / 32 contiguous systems per CTA.
template <int RHS, int SWEEPS>
__global__ void __launch_bounds__(512, 2)
    r2x_kernel(const __grid_constant__ CUtensorMap tin, const __grid_constant__ CUtensorMap tout,
               const __grid_constant__ Args a, int gpp) {
  extern __shared__ unsigned char smem_raw[];
  double* tile = reinterpret_cast<double*>(align1024(smem_raw));
  const int S = blockDim.x >> 5;
  float2* bnd = reinterpret_cast<float2*>(tile + S * NROWS);  // [S][2]: rows 0 and n-1
  uint64_t* bar = reinterpret_cast<uint64_t*>(bnd + 2 * S);
  const int plane = blockIdx.x / gpp;
  const int s0 = (blockIdx.x - plane * gpp) * S;
  contiguous_group<RHS, SWEEPS>(tile, bnd, bar, &tin, &tout, S, threadIdx.x, s0, plane, a, SyncAll());
}

// ---------------------------------------------------------------------------
// strided systems
// ---------------------------------------------------------------------------
constexpr size_t S_TILE_BYTES = (size_t)NROWS * SG * 8;
constexpr size_t S_XCH_FLOATS = (size_t)X_COUNT * CHUNKS * SG;
constexpr size_t S_SMEM = 1024 + S_TILE_BYTES + S_XCH_FLOATS * 4 + 16;
// the persistent kernel: two groups in compute, a third tile loading
constexpr int P_BUFS = 3;
constexpr size_t P_SMEM = 1024 + P_BUFS * S_TILE_BYTES + 2 * S_XCH_FLOATS * 4 + 8 * P_BUFS + 8;

// Where a strided group's results go: element (system x, row r, plane p) at
// p + plane * ps + x + r * es; systems at or beyond ni (a partial group) are
// not stored.
struct OutDesc {
  double* p;
  long long es, ps;
  int ni;
};
// Row r0 of system x0 + s of `plane`, or null beyond the last system.
__device__ __forceinline__ double* out_row(const OutDesc& o, int x0, int plane, int s, int r0) {
  return x0 + s < o.ni ? o.p + (long long)plane * o.ps + (x0 + s) + (long long)r0 * o.es : nullptr;
}

// One group of 16 systems in its [512][16] tile, solved by 512 threads:
// thread t owns system t % 16 and chunk t / 16.  DIRECT: the thread stores
// its 16 results from registers to out_of() (row r0 of its system, or null:
// nothing to store), rows es apart, a half-warp writing one 128-byte row
// segment; otherwise they are written in place into the tile.  With
// refinement the (hi, lo) split of each RHS row is kept in the tile for the
// residual; the first and last rows of a chunk are the halo rows its
// neighbours read for the compact RHS, so they are rewritten only after the
// first barrier.  Returns the thread's largest input magnitude (high word)
// for the range check.
template <int RHS, int SWEEPS, bool DIRECT, class SYNC, class OUTF>
__device__ __forceinline__ unsigned strided_group(double* tile, float* xch, int t, const Args& a, SYNC sync,
                                                  OUTF out_of, long long es) {
  const int s = t & 15;
  const int c = t >> 4;
  const int r0 = ROWS * c;
  auto X = [&](int which, int chunk) -> float& { return xch[(which * CHUNKS + chunk) * SG + s]; };
  const Consts& K = a.k;
  unsigned rmax = 0;
  double* col = tile + s;  // row r of this system: col[r * SG]
  float2 v[8];
  float2 edge0 = make_float2(0.f, 0.f), edge15 = edge0;  // (hi, lo) of rows r0 and r0 + 15
  if (RHS == RHS_COMPACT) {
    const double fl = c > 0 ? col[(r0 - 1) * SG] : 0.0;
    const double fr = c < CHUNKS - 1 ? col[(r0 + ROWS) * SG] : 0.0;
    float bh = 0.f, bl = 0.f;
    if (c == 0) boundary_rhs(col[0], col[SG], col[2 * SG], a.sigma0, bh, bl, rmax);
    if (c == CHUNKS - 1)
      boundary_rhs(col[(NROWS - 1) * SG], col[(NROWS - 2) * SG], col[(NROWS - 3) * SG], a.sigmaN, bh, bl, rmax);
    double prev = fl, cur = col[r0 * SG];
#pragma unroll
    for (int k = 0; k < ROWS; ++k) {
      const double nxt = (k < ROWS - 1) ? col[(r0 + k + 1) * SG] : fr;
      float h, l;
      split_f64(dsub_(nxt, prev), h, l, rmax);
      if (k == 0 && c == 0) {
        h = bh;
        l = bl;
      }
      if (k == ROWS - 1 && c == CHUNKS - 1) {
        h = bh;
        l = bl;
      }
      if (SWEEPS > 0) {
        if (k == 0) edge0 = make_float2(h, l);
        else if (k == ROWS - 1) edge15 = make_float2(h, l);
        else reinterpret_cast<float2*>(col + (r0 + k) * SG)[0] = make_float2(h, l);
      }
      if (k < HALF) v[k].x = h;
      else v[k - HALF].y = h;
      prev = cur;
      cur = nxt;
    }
  } else {
#pragma unroll
    for (int k = 0; k < ROWS; ++k) {
      float h, l;
      split_f64(col[(r0 + k) * SG], h, l, rmax);
      if (SWEEPS > 0) reinterpret_cast<float2*>(col + (r0 + k) * SG)[0] = make_float2(h, l);
      if (k < HALF) v[k].x = h;
      else v[k - HALF].y = h;
    }
  }
  strided_solve<SWEEPS, SG>(
      v, col, xch, s, c, a, sync,
      [&] {
        if (RHS == RHS_COMPACT && SWEEPS > 0) {
          reinterpret_cast<float2*>(col + r0 * SG)[0] = edge0;
          reinterpret_cast<float2*>(col + (r0 + ROWS - 1) * SG)[0] = edge15;
        }
      },
      [&](int k, double val) {
        double* out = DIRECT ? out_of() : col + r0 * SG;
        const long long step = DIRECT ? es : SG;
        if (out) out[k * step] = val;
      });
  return rmax;
}

// Group g of the strided layout: plane and first system.
__device__ __forceinline__ void group_coords(int g, int gpp, int& x0, int& plane) {
  plane = g / gpp;
  x0 = (g - plane * gpp) * SG;
}

// One 16-system strided group per CTA, boxes at (x0, 0 | 256, plane, 0):
// load, solve, store from registers.  prefetch() runs on thread 0 once its
// own load is issued.
template <int RHS, int SWEEPS, class PF>
__device__ __forceinline__ void strided_cta(double* tile, float* xch, uint64_t* bar, const CUtensorMap* tin,
                                            const OutDesc& o, int x0, int plane, const Args& a, PF prefetch) {
  const int tid = threadIdx.x;
  if (tid == 0) mbar_init(bar, 1);
  __syncthreads();
  if (tid == 0) {
    mbar_expect_tx(bar, (unsigned)S_TILE_BYTES);
    tma_load(tile, tin, x0, 0, plane, 0, bar);
    tma_load(tile + (NROWS / 2) * SG, tin, x0, NROWS / 2, plane, 0, bar);
    prefetch();
  }
  if (!__syncthreads_and(mbar_wait(bar, 0))) {
    if (tid == 0 && a.status) atomicOr(a.status, STATUS_TIMEOUT);
    return;
  }
  const unsigned rmax = strided_group<RHS, SWEEPS, true>(
      tile, xch, tid, a, SyncAll(), [&] { return out_row(o, x0, plane, tid & 15, ROWS * (tid >> 4)); }, o.es);
  if (__any_sync(FULL, rmax >= RANGE_MAG) && (tid & 31) == 0 && a.status) atomicOr(a.status, 1u);
}

// pf_dist > 0: on starting, a CTA prefetches into L2 the tile of the group
// pf_dist further on, which the CTA resident one wave later loads (pf_dist =
// the number of CTAs resident at once), so that load is served from L2.
template <int RHS, int SWEEPS>
__global__ void __launch_bounds__(512, 2)
    r2s_kernel(const __grid_constant__ CUtensorMap tin, const __grid_constant__ OutDesc o,
               const __grid_constant__ Args a, int gpp, int pf_dist) {
  extern __shared__ unsigned char smem_raw[];
  double* tile = reinterpret_cast<double*>(align1024(smem_raw));  // [512][16]
  float* xch = reinterpret_cast<float*>(tile + NROWS * SG);         // [X_COUNT][32][16]
  uint64_t* bar = reinterpret_cast<uint64_t*>(xch + S_XCH_FLOATS);
  int x0, plane;
  group_coords(blockIdx.x, gpp, x0, plane);
  strided_cta<RHS, SWEEPS>(tile, xch, bar, &tin, o, x0, plane, a, [&] {
    const long long gn = (long long)blockIdx.x + pf_dist;
    if (pf_dist > 0 && gn < (long long)gridDim.x) {
      int px, pp;
      group_coords((int)gn, gpp, px, pp);
      tma_prefetch_l2(&tin, px, 0, pp, 0);
      tma_prefetch_l2(&tin, px, NROWS / 2, pp, 0);
    }
  });
}

// ---------------------------------------------------------------------------
// the three directional derivatives of an n^3 field in one launch
// ---------------------------------------------------------------------------
// CTA b: for each z-plane p, the plane's x CTAs (cx of them, 16 x-lines each
// as four independent 4-system groups) and then its y CTAs (cy, 16 columns
// each) -- consecutive CTAs, so a plane read from HBM by one axis is in L2
// for the other -- and after all planes the z CTAs (gz, 16 columns each).
struct GradGeom {
  int nz, cx, cy, gz;
  int pf;        // prefetch distance in CTAs (0: none)
  OutDesc y, z;  // outputs of the y and z derivatives
};
constexpr int GX_SUB = 4;  // systems per x sub-group (one 128-thread group)
constexpr size_t G_SMEM = S_SMEM > 1024 + (size_t)4 * GX_SUB * NROWS * 8 + 4 * GX_SUB * 16 + 4 * 8 + 16
                              ? S_SMEM
                              : 1024 + (size_t)4 * GX_SUB * NROWS * 8 + 4 * GX_SUB * 16 + 4 * 8 + 16;

__device__ __forceinline__ void grad_prefetch(const CUtensorMap* mx, const CUtensorMap* my, const CUtensorMap* mz,
                                              const GradGeom& g, long long b) {
  const long long nxy = (long long)g.nz * (g.cx + g.cy);
  if (b < nxy) {
    const int p = (int)(b / (g.cx + g.cy)), r = (int)(b % (g.cx + g.cy));
    if (r < g.cx) {
      for (int q = 0; q < 4; ++q) tma_prefetch_l2(mx, 0, 0, r * 16 + q * GX_SUB, p);
    } else {
      tma_prefetch_l2(my, (r - g.cx) * SG, 0, p, 0);
      tma_prefetch_l2(my, (r - g.cx) * SG, NROWS / 2, p, 0);
    }
  } else if (b - nxy < g.gz) {
    const int c0 = (int)(b - nxy) * SG;
    tma_prefetch_l2(mz, c0, 0, 0, 0);
    tma_prefetch_l2(mz, c0, NROWS / 2, 0, 0);
  }
}

template <int SWEEPS>
__global__ void __launch_bounds__(512, 2)
    r2g_kernel(const __grid_constant__ CUtensorMap fx, const __grid_constant__ CUtensorMap ox,
               const __grid_constant__ CUtensorMap fy, const __grid_constant__ CUtensorMap fz,
               const __grid_constant__ Args ax, const __grid_constant__ GradGeom g) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base = align1024(smem_raw);
  const long long b = blockIdx.x;
  const long long nxy = (long long)g.nz * (g.cx + g.cy);
  auto prefetch = [&] {
    if (g.pf > 0) grad_prefetch(&fx, &fy, &fz, g, b + g.pf);
  };
  if (b < nxy) {
    const int p = (int)(b / (g.cx + g.cy)), r = (int)(b % (g.cx + g.cy));
    if (r < g.cx) {
      // x: four independent 4-warp groups, each with its own tile, barrier
      // and named CTA barrier
      const int q = threadIdx.x >> 7;
      double* tiles = reinterpret_cast<double*>(base);                     // [4][GX_SUB][512]
      float2* bnds = reinterpret_cast<float2*>(tiles + 4 * GX_SUB * NROWS);  // [4][2 GX_SUB]
      uint64_t* bars = reinterpret_cast<uint64_t*>(bnds + 4 * 2 * GX_SUB);   // [4]
      double* tile = tiles + (size_t)q * GX_SUB * NROWS;
      float2* bnd = bnds + q * 2 * GX_SUB;
      uint64_t* bar = bars + q;
      if (threadIdx.x == 0) prefetch();
      contiguous_group<RHS_COMPACT, SWEEPS>(tile, bnd, bar, &fx, &ox, GX_SUB, threadIdx.x & 127, r * 16 + q * GX_SUB,
                                            p, ax, SyncBar{1 + q, 128});
    } else {
      double* tile = reinterpret_cast<double*>(base);
      float* xch = reinterpret_cast<float*>(tile + NROWS * SG);
      uint64_t* bar = reinterpret_cast<uint64_t*>(xch + S_XCH_FLOATS);
      strided_cta<RHS_COMPACT, SWEEPS>(tile, xch, bar, &fy, g.y, (r - g.cx) * SG, p, ax, prefetch);
    }
  } else {
    double* tile = reinterpret_cast<double*>(base);
    float* xch = reinterpret_cast<float*>(tile + NROWS * SG);
    uint64_t* bar = reinterpret_cast<uint64_t*>(xch + S_XCH_FLOATS);
    strided_cta<RHS_COMPACT, SWEEPS>(tile, xch, bar, &fz, g.z, (int)(b - nxy) * SG, 0, ax, prefetch);
  }
}

// Persistent CTA (one per SM, 1024 threads): its groups are blockIdx.x +
// k * gridDim.x, k = 0, 1, ...; half h (512 threads) solves k = h, h + 2, ...
// in tile buffer k % 3, in place.  The half that finishes group k stores it
// by TMA, and once the store has read the tile it loads group k + 3 into the
// same buffer for the other half, so one tile is always loading while two
// are in compute.  Each buffer's mbarrier completes once per load: load n of
// buffer b is waited on with parity n & 1.
__device__ __forceinline__ void load_group(double* buf, uint64_t* bar, const CUtensorMap* map, int g, int gpp) {
  int x0, plane;
  group_coords(g, gpp, x0, plane);
  mbar_expect_tx(bar, (unsigned)S_TILE_BYTES);
  tma_load(buf, map, x0, 0, plane, 0, bar);
  tma_load(buf + (NROWS / 2) * SG, map, x0, NROWS / 2, plane, 0, bar);
}

// Layout of the persistent kernel's shared memory.
struct PSmem {
  double* bufs;    // [3][512][16] tiles
  float* xch;      // [2][X_COUNT][32][16] exchange arrays
  uint64_t* bars;  // [3] tile barriers
  int* knext;      // [2] next group index of each half
};
__device__ __forceinline__ PSmem psmem() {
  extern __shared__ unsigned char smem_raw[];
  PSmem p;
  p.bufs = reinterpret_cast<double*>(align1024(smem_raw));
  p.xch = reinterpret_cast<float*>(p.bufs + P_BUFS * NROWS * SG);
  p.bars = reinterpret_cast<uint64_t*>(p.xch + 2 * S_XCH_FLOATS);
  p.knext = reinterpret_cast<int*>(p.bars + P_BUFS);
  return p;
}

// Thread 0 of half h after the half's group: store it from its tile, and
// once the store has read the tile load the group three places further on
// into it for the other half.  Not inlined, so that nothing it needs stays
// in registers across the group's solve.
__device__ __noinline__ void finish_group(const CUtensorMap* tin, const CUtensorMap* tout, int gpp, int ngroups,
                                          int h) {
  const PSmem sm = psmem();
  const int G = gridDim.x;
  const int kcount = (ngroups - (int)blockIdx.x + G - 1) / G;
  const int k = sm.knext[h] - 2;
  const int b = k % P_BUFS;
  double* tile = sm.bufs + (size_t)b * NROWS * SG;
  int x0, plane;
  group_coords(blockIdx.x + k * G, gpp, x0, plane);
  tma_store(tout, x0, 0, plane, 0, tile);
  tma_store(tout, x0, NROWS / 2, plane, 0, tile + (NROWS / 2) * SG);
  tma_store_commit_and_wait();
  if (k + P_BUFS < kcount) load_group(tile, sm.bars + b, tin, blockIdx.x + (k + P_BUFS) * G, gpp);
}

template <int RHS, int SWEEPS>
__global__ void __launch_bounds__(1024, 1)
    r2sp_kernel(const __grid_constant__ CUtensorMap tin, const __grid_constant__ CUtensorMap tout,
                const __grid_constant__ Args a, int gpp, int ngroups) {
  const PSmem sm = psmem();
  const int tid = threadIdx.x;
  const int h = tid >> 9;
  const int t = tid & 511;
  const int G = gridDim.x;
  const int kcount = (ngroups - (int)blockIdx.x + G - 1) / G;  // groups of this CTA
  if (tid == 0) {
    for (int b = 0; b < P_BUFS; ++b) mbar_init(sm.bars + b, 1);
  }
  __syncthreads();
  if (tid == 0) {
    for (int k = 0; k < P_BUFS && k < kcount; ++k)
      load_group(sm.bufs + (size_t)k * NROWS * SG, sm.bars + k, &tin, blockIdx.x + k * G, gpp);
  }
  if (tid < 2) sm.knext[tid] = tid;
  __syncthreads();
  const SyncBar sync{1 + h, 512};
  for (;;) {
    const int k = sm.knext[h];
    if (k >= kcount) break;
    const int b = k % P_BUFS;
    double* tile = sm.bufs + (size_t)b * NROWS * SG;
    if (!sync.all(mbar_wait(sm.bars + b, (unsigned)(k / P_BUFS) & 1u))) {
      if (t == 0 && a.status) atomicOr(a.status, STATUS_TIMEOUT);
      return;
    }
    const unsigned rmax = strided_group<RHS, SWEEPS, false>(tile, sm.xch + h * S_XCH_FLOATS, t, a, sync,
                                                           [] { return (double*)nullptr; }, 0);
    if (__any_sync(FULL, rmax >= RANGE_MAG) && (t & 31) == 0 && a.status) atomicOr(a.status, 1u);
    fence_proxy_async();
    if (t == 0) sm.knext[h] = k + 2;
    sync();
    if (t == 0) finish_group(&tin, &tout, gpp, ngroups, h);
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

template <int RHS, int SWEEPS>
int launch_x(const double* in, double* out, const Batch& b, const Args& a, int S, cudaStream_t st) {
  // dims: row in chunk, chunk, system in plane, plane
  const long long nplanes = b.nsys > b.ni ? b.nsys / b.ni : 1;
  const long long ni = b.nsys > b.ni ? b.ni : b.nsys;
  const cuuint64_t dims[4] = {16, 32, (cuuint64_t)ni, (cuuint64_t)nplanes};
  const cuuint64_t strides[3] = {128, (cuuint64_t)b.is * 8, (cuuint64_t)(nplanes > 1 ? b.os : b.is * ni) * 8};
  const cuuint32_t box[4] = {16, 32, (cuuint32_t)S, 1};
  CUtensorMap mi, mo;
  int rc = encode(&mi, in, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_128B);
  if (!rc) rc = encode(&mo, out, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_128B);
  if (rc) return rc;
  const long long gpp = (ni + S - 1) / S;
  const long long grid = gpp * nplanes;
  if (grid > 0x7fffffffLL) {
    set_error("too many systems for one launch");
    return NTK_ERR_INVALID;
  }
  const size_t smem = 1024 + (size_t)S * NROWS * 8 + (size_t)2 * S * sizeof(float2) + 16;
  auto kern = r2x_kernel<RHS, SWEEPS>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute(r2x_kernel)");
  kern<<<(unsigned)grid, 32 * S, smem, st>>>(mi, mo, a, (int)gpp);
  return cuda_status(cudaGetLastError(), "r2x_kernel");
}

template <int RHS, int SWEEPS>
int launch_s(const double* in, double* out, const Batch& b, const Args& a, bool persistent, int prefetch,
             cudaStream_t st) {
  // dims: system in plane (contiguous), row, plane
  const long long nplanes = b.nsys > b.ni ? b.nsys / b.ni : 1;
  const long long ni = b.nsys > b.ni ? b.ni : b.nsys;
  const cuuint64_t dims[4] = {(cuuint64_t)ni, (cuuint64_t)NROWS, (cuuint64_t)nplanes, 1};
  const long long ps = nplanes > 1 ? b.os : b.es * NROWS;
  const cuuint64_t strides[3] = {(cuuint64_t)b.es * 8, (cuuint64_t)ps * 8, (cuuint64_t)ps * nplanes * 8};
  const cuuint32_t box[4] = {(cuuint32_t)SG, (cuuint32_t)(NROWS / 2), 1, 1};
  CUtensorMap mi;
  int rc = encode(&mi, in, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_NONE);
  if (rc) return rc;
  const long long gpp = (ni + SG - 1) / SG;
  const long long grid = gpp * nplanes;
  if (grid > 0x7fffffffLL) {
    set_error("too many systems for one launch");
    return NTK_ERR_INVALID;
  }
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_status(e, "cudaDeviceGetAttribute(SM count)");
  if (!persistent) {
    auto kern = r2s_kernel<RHS, SWEEPS>;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S_SMEM);
    if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute(r2s_kernel)");
    // two 512-thread CTAs per SM fill its registers: a wave is 2 * SMs
    // groups, prefetch counts half waves
    const int pf = prefetch * sms;
    const OutDesc mo{out, b.es, ps, (int)ni};
    kern<<<(unsigned)grid, 32 * CHUNKS / 2, S_SMEM, st>>>(mi, mo, a, (int)gpp, pf);
    return cuda_status(cudaGetLastError(), "r2s_kernel");
  }
  CUtensorMap mo;
  rc = encode(&mo, out, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_NONE);
  if (rc) return rc;
  auto kern = r2sp_kernel<RHS, SWEEPS>;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P_SMEM);
  if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute(r2sp_kernel)");
  const long long pgrid = grid < sms ? grid : sms;
  kern<<<(unsigned)pgrid, 32 * CHUNKS, P_SMEM, st>>>(mi, mo, a, (int)gpp, (int)grid);
  return cuda_status(cudaGetLastError(), "r2sp_kernel");
}

}  // namespace

// Whether (in, out, b) fit the tensor maps; the plan falls back to the
// chunked kernel of ntk_refine.cuh otherwise.
bool layout_ok(const double* in, const double* out, const Batch& b) {
  if (!aligned16(in) || !aligned16(out) || b.nsys < 1 || b.ni < 1) return false;
  if (b.nsys > b.ni && b.nsys % b.ni != 0) return false;
  const long long nplanes = b.nsys > b.ni ? b.nsys / b.ni : 1;
  const long long ni = b.nsys > b.ni ? b.ni : b.nsys;
  if (nplanes >= (1LL << 31) || ni >= (1LL << 31)) return false;
  if (b.es == 1) {  // contiguous systems: is >= n, is and os even
    if (b.is < NROWS || (b.is & 1)) return false;
    if (nplanes > 1 && ((b.os & 1) || b.os < b.is * ni)) return false;
    return true;
  }
  // strided systems: adjacent systems one element apart
  if (b.is != 1 || (b.es & 1) || b.es < ni) return false;
  if (nplanes > 1 && ((b.os & 1) || b.os < b.es * NROWS)) return false;
  return true;
}

int launch_grad(const double* f, double* ox, double* oy, double* oz, const Args& a, int sweeps, int prefetch,
                cudaStream_t st) {
  const cuuint64_t n = NROWS;
  if (!aligned16(f) || !aligned16(ox) || !aligned16(oy) || !aligned16(oz)) {
    set_error("one-launch gradient needs 16-byte aligned arrays");
    return NTK_ERR_UNSUPPORTED;
  }
  // x: row in chunk, chunk, line (y), plane (z); box = one 4-system group
  const cuuint64_t dx[4] = {16, 32, n, n};
  const cuuint64_t sx[3] = {128, n * 8, n * n * 8};
  const cuuint32_t bx[4] = {16, 32, (cuuint32_t)GX_SUB, 1};
  // y: x (contiguous), y rows, z planes; z: (x, y) flattened, z rows
  const cuuint64_t dy[4] = {n, n, n, 1};
  const cuuint64_t sy[3] = {n * 8, n * n * 8, n * n * n * 8};
  const cuuint64_t dz[4] = {n * n, n, 1, 1};
  const cuuint64_t sz[3] = {n * n * 8, n * n * n * 8, n * n * n * 8};
  const cuuint32_t bs[4] = {(cuuint32_t)SG, (cuuint32_t)(NROWS / 2), 1, 1};
  CUtensorMap m[4];
  int rc = encode(&m[0], f, dx, sx, bx, CU_TENSOR_MAP_SWIZZLE_128B);
  if (!rc) rc = encode(&m[1], ox, dx, sx, bx, CU_TENSOR_MAP_SWIZZLE_128B);
  if (!rc) rc = encode(&m[2], f, dy, sy, bs, CU_TENSOR_MAP_SWIZZLE_NONE);
  if (!rc) rc = encode(&m[3], f, dz, sz, bs, CU_TENSOR_MAP_SWIZZLE_NONE);
  if (rc) return rc;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_status(e, "cudaDeviceGetAttribute(SM count)");
  GradGeom g;
  g.nz = NROWS;
  g.cx = NROWS / 16;
  g.cy = NROWS / SG;
  g.gz = NROWS * NROWS / SG;
  g.pf = prefetch * sms;
  g.y = OutDesc{oy, (long long)n, (long long)(n * n), (int)n};
  g.z = OutDesc{oz, (long long)(n * n), 0, (int)(n * n)};
  const long long grid = (long long)g.nz * (g.cx + g.cy) + g.gz;
  auto kern = sweeps ? r2g_kernel<1> : r2g_kernel<0>;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G_SMEM);
  if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute(r2g_kernel)");
  kern<<<(unsigned)grid, 512, G_SMEM, st>>>(m[0], m[1], m[2], m[3], a, g);
  return cuda_status(cudaGetLastError(), "r2g_kernel");
}

int launch(const double* in, double* out, const Batch& b, const Args& a, int rhs, int sweeps, int S, bool persistent,
           int prefetch, cudaStream_t st) {
  if (S != 4 && S != 8 && S != 16) S = 8;
  if (b.es == 1) {
    if (rhs == RHS_COMPACT)
      return sweeps ? launch_x<RHS_COMPACT, 1>(in, out, b, a, S, st) : launch_x<RHS_COMPACT, 0>(in, out, b, a, S, st);
    return sweeps ? launch_x<RHS_IDENTITY, 1>(in, out, b, a, S, st) : launch_x<RHS_IDENTITY, 0>(in, out, b, a, S, st);
  }
  const bool p = persistent;
  const int f = prefetch;
  if (rhs == RHS_COMPACT)
    return sweeps ? launch_s<RHS_COMPACT, 1>(in, out, b, a, p, f, st) : launch_s<RHS_COMPACT, 0>(in, out, b, a, p, f, st);
  return sweeps ? launch_s<RHS_IDENTITY, 1>(in, out, b, a, p, f, st)
                : launch_s<RHS_IDENTITY, 0>(in, out, b, a, p, f, st);
}

}  // namespace r2
}  // namespace ntk
