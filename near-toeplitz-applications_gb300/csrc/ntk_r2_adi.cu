// ntk_r2_adi.cu -- the ADI half steps of experiments/run-adi.py:59-71 on the
// paired-chunk FP32 + refinement solve (ntk_r2.cuh, ntk_r2_group.cuh).
//
// The ADI plan cuts each system of N rows into overlapping 512-row windows
// (ntk_adi_geom.h: first, middle, last, or one whole window); every window
// kind is a near-Toeplitz matrix of 512 rows with the interior (1, beta, 1)
// (rows scaled by dx^2) and one special row at each end, so the paired-chunk
// solve applies to it as it does to the compact matrix: constant Toeplitz
// factors with Woodbury end corrections per kind.  The right-hand side is
// the vertical stencil of adi/rhs.py:21-24 in the scaled form
// d = gamma u_mid - (u_lo + u_hi) (one or two FP64 operations, as in
// ntk_adi_refine.cu), the identity rows take the boundary values.
//
//  * x half step (r2ax_kernel): the systems are rows 1..N-2 of the field;
//    a CTA solves S consecutive rows of one window.  One TMA box brings the
//    S + 2 rows of u its stencils read (512 columns each, 128-byte swizzle);
//    once every stencil has been formed (a CTA barrier, the pairs held in
//    registers across it) each system's (hi, lo) RHS pairs overwrite its
//    middle row, and each thread stores the window's central rows of its
//    chunk straight to d_x.
//  * y half step (r2ay_kernel): the systems are columns 1..N-2 of d_x; a CTA
//    solves 16 adjacent columns of one window from an [512][18] tile (the
//    16 columns and their two neighbours, two TMA boxes).  After a CTA
//    barrier every thread rewrites its own column in place with the (hi, lo)
//    pairs; the central rows go straight into u's columns, where the
//    reference's final transpose puts them.
#include <cmath>

#include "ntk_r2_adi.h"
#include "ntk_r2_group.cuh"
#include "ntk_r2_host.h"

namespace ntk {
namespace r2 {

namespace {

struct AdiKinds {
  Args k[4];  // first, middle, last, whole window
};

struct AdiWin {
  int N = 0, L = 0, H = 0, P = 1, whole = 0;
  int ns = 0;                   // systems, N - 2
  double gamma = 0.0;           // RHS: gamma u_mid - (u_lo + u_hi)
  const double* bnd = nullptr;  // identity-row RHS: system s, row i at bnd[s * N + i]
};

__device__ __forceinline__ void window(const AdiWin& g, int w, int& start, int& lo, int& hi, int& kind) {
  if (g.whole) {
    start = 0, lo = 0, hi = NROWS, kind = 3;
  } else if (w == 0) {
    start = 0, lo = 0, hi = g.L, kind = 0;
  } else if (w < g.P - 1) {
    start = w * g.L - g.H, lo = g.H, hi = g.H + g.L, kind = 1;
  } else {
    start = g.N - NROWS, lo = (g.P - 1) * g.L - (g.N - NROWS), hi = NROWS, kind = 2;
  }
}

template <bool GZ>
__device__ __forceinline__ double stencil(double lo, double mid, double hi, double gamma) {
  const double t = dsub_(-lo, hi);
  return GZ ? t : dfma_(gamma, mid, t);
}

// ---- x half step: S = 4 rows of the field per CTA, one window ----
// Seven 4-warp CTAs per SM (72 registers: the RHS pairs are held across the
// barrier that frees the stencil rows).
constexpr int AX_S = 4;
template <int SWEEPS, bool GZ>
__global__ void __launch_bounds__(32 * AX_S, 7)
    r2ax_kernel(const __grid_constant__ CUtensorMap tu, double* out, const __grid_constant__ AdiWin g,
                const __grid_constant__ AdiKinds ak) {
  extern __shared__ unsigned char smem_raw[];
  constexpr int S = AX_S;
  double* tile = reinterpret_cast<double*>(align1024(smem_raw));  // [S + 2][512] stencil rows
  uint64_t* bar = reinterpret_cast<uint64_t*>(tile + (size_t)(S + 2) * NROWS);
  const int nblk = (g.ns + S - 1) / S;
  const int w = blockIdx.x / nblk;
  const int s0 = (blockIdx.x - w * nblk) * S;
  int start, lo, hi, kind;
  window(g, w, start, lo, hi, kind);
  const Args& a = ak.k[kind];
  const int gt = threadIdx.x, warp = gt >> 5, j = gt & 31;
  if (gt == 0) mbar_init(bar, 1);
  __syncthreads();
  if (gt == 0) {
    mbar_expect_tx(bar, (unsigned)(S + 2) * NROWS * 8u);
    tma_load(tile, &tu, 0, start / 16, s0, 0, bar);  // rows s0 .. s0 + S + 1 of u
  }
  if (!__syncthreads_and(mbar_wait(bar, 0))) {
    if (gt == 0 && a.status) atomicOr(a.status, STATUS_TIMEOUT);
    return;
  }
  const int s = s0 + warp;  // system s: row s + 1 of the field
  const bool live = s < g.ns;
  const double* rlo = tile + (size_t)warp * NROWS;
  double* hl = tile + (size_t)(warp + 1) * NROWS;  // the middle row, rewritten with the pairs
  const double* rhi = hl + NROWS;
  unsigned rmax = 0;
  float2 v[8], lo8[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const double2 ql = *reinterpret_cast<const double2*>(rlo + xpair(j, i));
    const double2 qm = *reinterpret_cast<const double2*>(hl + xpair(j, i));
    const double2 qh = *reinterpret_cast<const double2*>(rhi + xpair(j, i));
    double d0 = stencil<GZ>(ql.x, qm.x, qh.x, g.gamma);
    double d1 = stencil<GZ>(ql.y, qm.y, qh.y, g.gamma);
    // identity rows take the boundary values (experiments/run-adi.py:50-53)
    if (live && i == 0 && j == 0 && (kind == 0 || kind == 3)) d0 = g.bnd[(long long)s * g.N];
    if (live && i == 7 && j == 31 && (kind == 2 || kind == 3)) d1 = g.bnd[(long long)s * g.N + g.N - 1];
    float h0, l0, h1, l1;
    split_f64(d0, h0, l0, rmax);
    split_f64(d1, h1, l1, rmax);
    if (i < 4) {
      v[2 * i].x = h0;
      v[2 * i + 1].x = h1;
      lo8[2 * i].x = l0;
      lo8[2 * i + 1].x = l1;
    } else {
      v[2 * i - 8].y = h0;
      v[2 * i - 7].y = h1;
      lo8[2 * i - 8].y = l0;
      lo8[2 * i - 7].y = l1;
    }
  }
  __syncthreads();  // every stencil row has been read
  if (!live) return;  // no CTA barrier follows
  if (SWEEPS > 0) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      *reinterpret_cast<float4*>(hl + xpair(j, i)) =
          make_float4(v[2 * i].x, lo8[2 * i].x, v[2 * i + 1].x, lo8[2 * i + 1].x);
      *reinterpret_cast<float4*>(hl + xpair(j, i + 4)) =
          make_float4(v[2 * i].y, lo8[2 * i].y, v[2 * i + 1].y, lo8[2 * i + 1].y);
    }
  }
  double* dst = out + (long long)s * g.N + start + ROWS * j;  // row 16 j of the window
  contiguous_solve<SWEEPS>(v, hl, j, a, [&](int i, double oa0, double oa1, double ob0, double ob1) {
    const int r = ROWS * j + 2 * i;  // rows r, r + 1 and r + 8, r + 9 (lo, hi, r even)
    if (r >= lo && r < hi) *reinterpret_cast<double2*>(dst + 2 * i) = make_double2(oa0, oa1);
    if (r + 8 >= lo && r + 8 < hi) *reinterpret_cast<double2*>(dst + 2 * i + 8) = make_double2(ob0, ob1);
  });
  if (__any_sync(FULL, rmax >= RANGE_MAG) && j == 0 && a.status) atomicOr(a.status, 1u);
}

// ---- y half step: 16 columns of d_x per CTA, one window ----
constexpr int YP = SG + 2;  // tile pitch: the 16 columns and their two neighbours
constexpr size_t Y_SMEM = 1024 + (size_t)NROWS * YP * 8 + (size_t)X_COUNT * CHUNKS * SG * 4 + 16;

template <int SWEEPS, bool GZ>
__global__ void __launch_bounds__(512, 2)
    r2ay_kernel(const __grid_constant__ CUtensorMap td, double* out, const __grid_constant__ AdiWin g,
                const __grid_constant__ AdiKinds ak) {
  extern __shared__ unsigned char smem_raw[];
  double* tile = reinterpret_cast<double*>(align1024(smem_raw));  // [512][18]
  float* xch = reinterpret_cast<float*>(tile + (size_t)NROWS * YP);
  uint64_t* bar = reinterpret_cast<uint64_t*>(xch + X_COUNT * CHUNKS * SG);
  const int ngr = (g.ns + SG - 1) / SG;
  const int w = blockIdx.x / ngr;
  const int grp = blockIdx.x - w * ngr;
  int start, lo, hi, kind;
  window(g, w, start, lo, hi, kind);
  const Args& a = ak.k[kind];
  const int t = threadIdx.x, s = t & 15, c = t >> 4;
  if (t == 0) mbar_init(bar, 1);
  __syncthreads();
  if (t == 0) {
    mbar_expect_tx(bar, (unsigned)(NROWS * YP * 8));
    // columns 16 grp .. 16 grp + 17 of d_x: the group's systems 16 grp + s
    // are columns 16 grp + s + 1, with their neighbours on either side
    tma_load(tile, &td, SG * grp, start, 0, 0, bar);
    tma_load(tile + (NROWS / 2) * YP, &td, SG * grp, start + NROWS / 2, 0, 0, bar);
  }
  if (!__syncthreads_and(mbar_wait(bar, 0))) {
    if (t == 0 && a.status) atomicOr(a.status, STATUS_TIMEOUT);
    return;
  }
  const int sys = SG * grp + s;
  const bool live = sys < g.ns;
  double* col = tile + 1 + s;  // own column, row r at col[r * YP]
  const int r0 = ROWS * c;
  unsigned rmax = 0;
  float2 v[8], lo8[8];
#pragma unroll
  for (int k = 0; k < ROWS; ++k) {
    const int r = r0 + k;
    const double d0 = col[r * YP - 1], m = col[r * YP], d2 = col[r * YP + 1];
    double d = stencil<GZ>(d0, m, d2, g.gamma);
    if (k == 0 && c == 0 && (kind == 0 || kind == 3)) d = live ? g.bnd[(long long)sys * g.N] : 0.0;
    if (k == ROWS - 1 && c == CHUNKS - 1 && (kind == 2 || kind == 3))
      d = live ? g.bnd[(long long)sys * g.N + g.N - 1] : 0.0;
    float h, l;
    split_f64(d, h, l, rmax);
    if (k < HALF) {
      v[k].x = h;
      lo8[k].x = l;
    } else {
      v[k - HALF].y = h;
      lo8[k - HALF].y = l;
    }
  }
  __syncthreads();  // every stencil column has been read
  if (SWEEPS > 0) {
#pragma unroll
    for (int k = 0; k < HALF; ++k) {
      reinterpret_cast<float2*>(col + (r0 + k) * YP)[0] = make_float2(v[k].x, lo8[k].x);
      reinterpret_cast<float2*>(col + (r0 + k + HALF) * YP)[0] = make_float2(v[k].y, lo8[k].y);
    }
  }
  double* dst = out + (long long)(start + r0) * g.N + sys;  // row r0 of column sys + 1 of u
  strided_solve<SWEEPS, YP>(v, col, xch, s, c, a, SyncAll(), [] {}, [&](int k, double val) {
    const int r = r0 + k;
    if (live && r >= lo && r < hi) dst[(long long)k * g.N] = val;
  });
  if (__any_sync(FULL, live && rmax >= RANGE_MAG) && (t & 31) == 0 && a.status) atomicOr(a.status, 1u);
}

}  // namespace

struct AdiR2 {
  AdiKinds kinds;
  AdiWin geo;
  int sweeps = 1;
  bool gz = false;
  unsigned* d_status = nullptr;
  ~AdiR2() {
    if (d_status) cudaFree(d_status);
  }
};

AdiR2* adi_create(int N, int L, int H, int P, bool whole, double beta, double gamma, int sweeps, std::string* why) {
  auto fail = [&](const char* m) -> AdiR2* {
    if (why) *why = m;
    return nullptr;
  };
  if (sweeps > 1) return fail("two refinement sweeps");
  if (N % 16 != 0 || (!whole && H % 16 != 0)) return fail("N and the halo must be multiples of 16");
  if (N < NROWS) return fail("N below 512");
  AdiR2* r = new (std::nothrow) AdiR2();
  if (!r) return fail("out of host memory");
  // window kinds: rows (a, b, c) at each end, interior (1, beta, 1)
  const double ident[3] = {0.0, 1.0, 0.0};
  const double cut_head[3] = {0.0, beta, 1.0};
  const double cut_tail[3] = {1.0, beta, 0.0};
  const double* heads[4] = {ident, cut_head, cut_head, ident};
  const double* tails[4] = {cut_tail, cut_tail, ident, ident};
  for (int k = 0; k < 4; ++k) {
    if ((k == 3) != whole) continue;
    MatrixRows m;
    m.n = NROWS;
    m.nh = 1;
    m.nt = 1;
    for (int q = 0; q < 3; ++q) {
      m.head[0][q] = heads[k][q];
      m.tail[0][q] = tails[k][q];
    }
    m.ai = 1.0;
    m.bi = beta;
    m.ci = 1.0;
    if (!prepare(m, &r->kinds.k[k], why)) {
      delete r;
      return nullptr;
    }
  }
  if (cudaMalloc(&r->d_status, sizeof(unsigned)) != cudaSuccess ||
      cudaMemset(r->d_status, 0, sizeof(unsigned)) != cudaSuccess) {
    delete r;
    return fail("cudaMalloc(status)");
  }
  for (int k = 0; k < 4; ++k) r->kinds.k[k].status = r->d_status;
  r->geo.N = N;
  r->geo.L = L;
  r->geo.H = H;
  r->geo.P = P;
  r->geo.whole = whole ? 1 : 0;
  r->geo.ns = N - 2;
  r->geo.gamma = gamma;
  r->gz = (gamma == 0.0);
  r->sweeps = sweeps;
  return r;
}

void adi_destroy(AdiR2* r) { delete r; }

void adi_status_words(const AdiR2* r, std::vector<unsigned*>& out) {
  if (r && r->d_status) out.push_back(r->d_status);
}

namespace {

template <class K>
int launch_kernel(K kern, unsigned grid, unsigned block, size_t smem, cudaStream_t st, const CUtensorMap& m,
                  double* out, const AdiWin& g, const AdiKinds& ak, const char* name) {
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e, name);
  kern<<<grid, block, smem, st>>>(m, out, g, ak);
  return cuda_status(cudaGetLastError(), name);
}

}  // namespace

int adi_step(AdiR2* r, double* u, double* d_x, const double* d_y, cudaStream_t st) {
  if (!aligned16(u) || !aligned16(d_x)) {
    set_error("ADI: u and d_x must be 16-byte aligned");
    return NTK_ERR_INVALID;
  }
  const int N = r->geo.N;
  constexpr int S = AX_S;
  const cuuint64_t n = (cuuint64_t)N;
  // x half step: u as (column in chunk, chunk, row), box of S + 2 rows
  CUtensorMap mu, md;
  {
    const cuuint64_t dims[4] = {16, n / 16, n, 1};
    const cuuint64_t strides[3] = {128, n * 8, n * n * 8};
    const cuuint32_t box[4] = {16, 32, (cuuint32_t)(S + 2), 1};
    int rc = encode(&mu, u, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_128B);
    if (rc) return rc;
  }
  {
    const cuuint64_t dims[4] = {n, n, 1, 1};
    const cuuint64_t strides[3] = {n * 8, n * n * 8, n * n * 8};
    const cuuint32_t box[4] = {(cuuint32_t)YP, (cuuint32_t)(NROWS / 2), 1, 1};
    int rc = encode(&md, d_x, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_NONE);
    if (rc) return rc;
  }
  AdiWin gx = r->geo, gy = r->geo;
  gx.bnd = d_x + N;  // system s, row i: d_x[(s + 1) N + i]
  gy.bnd = d_y + N;  // system s, row i: d_y[(s + 1) N + i]
  const int P = r->geo.whole ? 1 : r->geo.P;
  const size_t xsmem = 1024 + (size_t)(S + 2) * NROWS * 8 + 16;
  const unsigned xgrid = (unsigned)(P * ((r->geo.ns + S - 1) / S));
  const unsigned ygrid = (unsigned)(P * ((r->geo.ns + SG - 1) / SG));
  int rc;
  if (r->sweeps == 0) {
    rc = r->gz ? launch_kernel(r2ax_kernel<0, true>, xgrid, 32 * S, xsmem, st, mu, d_x + N, gx, r->kinds, "r2ax_kernel")
               : launch_kernel(r2ax_kernel<0, false>, xgrid, 32 * S, xsmem, st, mu, d_x + N, gx, r->kinds,
                               "r2ax_kernel");
    if (rc) return rc;
    return r->gz ? launch_kernel(r2ay_kernel<0, true>, ygrid, 512, Y_SMEM, st, md, u + 1, gy, r->kinds, "r2ay_kernel")
                 : launch_kernel(r2ay_kernel<0, false>, ygrid, 512, Y_SMEM, st, md, u + 1, gy, r->kinds,
                                 "r2ay_kernel");
  }
  rc = r->gz ? launch_kernel(r2ax_kernel<1, true>, xgrid, 32 * S, xsmem, st, mu, d_x + N, gx, r->kinds, "r2ax_kernel")
             : launch_kernel(r2ax_kernel<1, false>, xgrid, 32 * S, xsmem, st, mu, d_x + N, gx, r->kinds,
                             "r2ax_kernel");
  if (rc) return rc;
  return r->gz ? launch_kernel(r2ay_kernel<1, true>, ygrid, 512, Y_SMEM, st, md, u + 1, gy, r->kinds, "r2ay_kernel")
               : launch_kernel(r2ay_kernel<1, false>, ygrid, 512, Y_SMEM, st, md, u + 1, gy, r->kinds,
                               "r2ay_kernel");
}

}  // namespace r2
}  // namespace ntk
