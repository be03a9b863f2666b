// ntk_adi_refine.cu -- ADI half-steps (experiments/run-adi.py:59-71) with
// the FP32 solve + double-word refinement of ntk_refine.cuh.
//
// A half-step solves N-2 systems of N rows (2046 x 2048 at the benchmark
// size), too long for one warp's registers.  Each system is cut into
// windows of Lw = 32 M rows that overlap by halos of H rows: window g
// writes back only its central rows, and every row it writes is at least
// H rows from a cut end.  The refinement converges to the exact solution of
// the window's own (truncated) system, so the truncation itself must lie
// below the target accuracy: H is chosen so that the product of the LU
// multipliers over H rows is below 2^-56 (r = 0.5: |l| -> 0.268, H = 32).
// Four window kinds have their own matrices and FP32 tables:
//   first : row 0 is the system's identity row, row Lw-1 is cut (c = 0)
//   middle: both ends cut (row 0 has a = 0, row Lw-1 has c = 0)
//   last  : row 0 cut, row Lw-1 is the system's identity row
//   whole : N == Lw, both identity rows, no truncation.
//
// The rows are scaled by dx^2, so the interior matrix is (1, beta, 1) with
// beta = -2 (1 + dx^2/dt) (= -4 at r = 0.5: all powers of two, exact
// residual products) and the right-hand side of the vertical stencil
// (adi/rhs.py:21-24) becomes  d = gamma * u_mid - (u_lo + u_hi),
// gamma = 2 (1 - dx^2/dt): one or two FP64 instructions per row, the only
// FP64 work.  One launch per half step; a CTA takes W consecutive systems
// of one window, copies its window kind's arguments to shared memory and
// stages the W + 2 lines their stencils read with cp.async.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ntk_adi_geom.h"
#include "ntk_adi_refine.h"
#include "ntk_r2_adi.h"
#include "ntk_refine.cuh"

namespace ntk {

#ifndef NTK_ADI_WX
#define NTK_ADI_WX 4
#endif
#ifndef NTK_ADI_WY
#define NTK_ADI_WY 8
#endif
// launch bounds of adi_refine_kernel: CTAs of up to NTK_ADI_MAXT threads,
// NTK_ADI_MINB of them resident per SM (80 registers for 256 x 3 or 384 x 2)
#ifndef NTK_ADI_MAXT
#define NTK_ADI_MAXT 256
#endif
#ifndef NTK_ADI_MINB
#define NTK_ADI_MINB 3
#endif

namespace refine_detail {

template <int M>
__host__ __device__ constexpr size_t adi_smem(int W, int ncls) {
  // line buffer (W + 2 lines, padded chunk layout; system w's tile reuses
  // line w + 1 once the stencil is formed), the window kind's arguments and
  // tables
  return (size_t)(W + 2) * sys_pitch<M>() * sizeof(double) + 16 + ((sizeof(RefineArgs) + 15) & ~(size_t)15) +
         (size_t)ncls * class_pitch4<M>() * sizeof(float4);
}

// One launch per half step: CTA b solves window b / nblk of the W
// consecutive systems starting at (b % nblk) W; args[kind] are the window
// kinds' kernel arguments (device memory, copied to shared memory).
template <int M, int SWEEPS, bool POW2, bool DECAY>
__global__ void __launch_bounds__(NTK_ADI_MAXT, (M <= 16) ? NTK_ADI_MINB : 1)
    adi_refine_kernel(const double* in, double* out, AdiGeom geo, const RefineArgs* args) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int P = sys_pitch<M>();
  constexpr int LW = 32 * M;
  const int W = blockDim.x >> 5;
  double* lines = reinterpret_cast<double*>(smem_raw);  // [W + 2][P]
  unsigned char* after = smem_raw + (((size_t)(W + 2) * P * sizeof(double) + 15) & ~(size_t)15);
  RefineArgs* ra = reinterpret_cast<RefineArgs*>(after);
  float4* tq = reinterpret_cast<float4*>(after + ((sizeof(RefineArgs) + 15) & ~(size_t)15));
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const unsigned lane = tid & 31;
  const long long nblk = (geo.ns + W - 1) / W;  // CTAs per window
  const int wi = (int)(blockIdx.x / nblk);
  const long long s0 = (blockIdx.x % nblk) * W;  // first system of the CTA
  const int wc = (int)((geo.ns - s0) < W ? (geo.ns - s0) : W);
  const WinRows wr = window_rows(geo, wi);
  unsigned range = 0;

  // this window kind's arguments and FP32 tables
  {
    const int* src = reinterpret_cast<const int*>(args + wr.kind);
    int* dst = reinterpret_cast<int*>(ra);
    constexpr int NW = (int)(sizeof(RefineArgs) / sizeof(int));
    for (int i = tid; i < NW; i += blockDim.x) dst[i] = __ldg(src + i);
  }
  __syncthreads();
  const int TC = ra->ncls * class_pitch4<M>();
  const int cbase = __ldg(reinterpret_cast<const int*>(ra->tab) + lane) * class_pitch4<M>();
  {
    const float4* g4 = reinterpret_cast<const float4*>(ra->tab + 32);
    for (int i = tid; i < TC; i += blockDim.x) tq[i] = g4[i];
  }

  // ---- stage lines s0-1 .. s0+wc (the stencil's neighbours included) ----
  // Line j of the buffer is system line s0 - 1 + j; lanes walk rows for
  // unit element stride (256-byte rows of copies), lines otherwise.
  const double* wbase = in + (long long)wr.start * geo.es;
  const int nl = wc + 2;
  const int total = nl * LW;
  for (int idx = tid; idx < total; idx += blockDim.x) {
    int j, r;
    if (geo.es == 1) {
      j = idx / LW;
      r = idx - j * LW;
    } else {
      r = idx / nl;
      j = idx - r * nl;
    }
    const double* src = wbase + (s0 - 1 + j) * geo.is + (long long)r * geo.es;
    cp_async8(lines + (size_t)j * P + tile_off<M>(r), src, 8u);
  }
  cp_async_wait_all();
  __syncthreads();

  // ---- double-word right-hand side, first in registers: every warp reads
  // three lines, and system w's tile then reuses line w + 1 ----
  const int cb = (int)lane * (M + 1);
  const long long s = s0 + warp;
  float dh[M], dl[M];
  if (warp < wc) {
    const double* lo = lines + (size_t)warp * P;
    const double* mid = lo + P;
    const double* hi = mid + P;
    if (geo.gamma != 0.0) {
#pragma unroll
      for (int k = 0; k < M; ++k)
        split_f64(fma(geo.gamma, mid[cb + k], (-lo[cb + k]) - hi[cb + k]), dh[k], dl[k], range);
    } else {
#pragma unroll
      for (int k = 0; k < M; ++k) split_f64((-lo[cb + k]) - hi[cb + k], dh[k], dl[k], range);
    }
    // identity rows: x = the boundary value (adi/rhs.py leaves them to the
    // solve's first and last rows, experiments/run-adi.py:50-53)
    if ((wr.kind == 0 || wr.kind == 3) && lane == 0) split_f64(geo.bnd[s * geo.bnd_ss], dh[0], dl[0], range);
    if ((wr.kind == 2 || wr.kind == 3) && lane == 31)
      split_f64(geo.bnd[s * geo.bnd_ss + (long long)(geo.N - 1) * geo.bnd_es], dh[M - 1], dl[M - 1], range);
  }
  __syncthreads();  // all lines read
  if (warp < wc) {
    double* trow = lines + (size_t)(warp + 1) * P;
    float2* drow = reinterpret_cast<float2*>(trow);
#pragma unroll
    for (int k = 0; k < M; ++k) drow[cb + k] = make_float2(dh[k], dl[k]);
    __syncwarp();
    ChunkTabs tabs;
    tabs.q = tq + cbase;
    refine_system<M, RHS_PRESPLIT, SWEEPS, POW2, false, DECAY>(trow, nullptr, tabs, LW, *ra, lane, range);
    __syncwarp();
    // ---- write back the window's central rows (coalesced for unit stride) ----
    double* dst = out + (long long)wr.start * geo.es + s * geo.is;
#pragma unroll 4
    for (int q = 0; q < M; ++q) {
      const int r = (int)lane + 32 * q;
      if (r >= wr.lo && r < wr.hi) dst[(long long)r * geo.es] = trow[tile_off<M>(r)];
    }
  }
  if (range && ra->status) atomicOr(ra->status, 1u);
}

template <int M, int SWEEPS, bool POW2, bool DECAY>
int adi_launch(const double* in, double* out, const AdiGeom& geo, const RefineArgs* d_args, int max_ncls, int W,
               cudaStream_t st) {
  const size_t smem = adi_smem<M>(W, max_ncls);
  auto kern = adi_refine_kernel<M, SWEEPS, POW2, DECAY>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute(adi_refine_kernel)");
  const long long blocks = (long long)geo.P * ((geo.ns + W - 1) / W);
  if (blocks <= 0) return NTK_OK;
  if (blocks > 0x7fffffffLL) {
    set_error("too many ADI windows for one launch");
    return NTK_ERR_INVALID;
  }
  kern<<<(unsigned)blocks, W * 32, smem, st>>>(in, out, geo, d_args);
  return cuda_status(cudaGetLastError(), "adi_refine_kernel");
}

template <int M, bool DECAY>
int adi_dispatch(const double* in, double* out, const AdiGeom& geo, const RefineArgs* d_args, int max_ncls,
                 bool pow2, int sweeps, int W, cudaStream_t st) {
  if (sweeps == 0)
    return pow2 ? adi_launch<M, 0, true, DECAY>(in, out, geo, d_args, max_ncls, W, st)
                : adi_launch<M, 0, false, DECAY>(in, out, geo, d_args, max_ncls, W, st);
  if (sweeps == 1)
    return pow2 ? adi_launch<M, 1, true, DECAY>(in, out, geo, d_args, max_ncls, W, st)
                : adi_launch<M, 1, false, DECAY>(in, out, geo, d_args, max_ncls, W, st);
  return pow2 ? adi_launch<M, 2, true, DECAY>(in, out, geo, d_args, max_ncls, W, st)
              : adi_launch<M, 2, false, DECAY>(in, out, geo, d_args, max_ncls, W, st);
}

}  // namespace refine_detail

struct AdiRefine {
  int N = 0;
  int M = 0, Lw = 0, H = 0, L = 0, P = 0;  // rows per lane, window, halo, central rows, windows
  int sweeps = 1;
  double gamma = 0.0;
  bool whole = false;  // N == Lw: one window per system, no truncation
  Plan win[4];         // first, middle, last, whole window matrices (n = Lw)
  // systems per CTA: rows (x half step) are staged as 256-byte row segments
  // already; columns (y half step) gain from more adjacent columns per CTA
  int wx = NTK_ADI_WX, wy = NTK_ADI_WY;
  RefineArgs* d_args = nullptr;  // kernel arguments of the four kinds (device)
  int max_ncls = 1;
  bool pow2 = true, decay = true;
  r2::AdiR2* r2a = nullptr;  // the paired-chunk half steps (ntk_r2_adi.cu) where they apply
  ~AdiRefine() {
    if (d_args) cudaFree(d_args);
    if (r2a) r2::adi_destroy(r2a);
  }
};

void adi_refine_status_words(const AdiRefine* ar, std::vector<unsigned*>& out) {
  if (!ar) return;
  for (const Plan& w : ar->win) w.status_words(out);
  r2::adi_status_words(ar->r2a, out);
}

int adi_refine_create(AdiRefine** out, int N, double dx, double dt, int precision) {
  *out = nullptr;
  AdiRefine* ar = new (std::nothrow) AdiRefine();
  if (!ar) {
    set_error("out of host memory");
    return NTK_ERR_ALLOC;
  }
  ar->N = N;
  ar->sweeps = (precision == NTK_FP32) ? 0 : 1;
  const double q = dx * dx / dt;
  const double beta = -2.0 * (1.0 + q);
  ar->gamma = 2.0 * (1.0 - q);
  // window length: the largest 32 M <= N with M in {16, 8, 4}
  for (int m : {16, 8, 4})
    if (32 * m <= N) {
      ar->M = m;
      break;
    }
  if (ar->M == 0) {
    set_error("ADI in FP32/FP32+refine needs N >= 128 (got %d); use NTK_FP64", N);
    delete ar;
    return NTK_ERR_UNSUPPORTED;
  }
  ar->Lw = 32 * ar->M;
  // halo: rows until the product of the LU multipliers of a window cut
  // (|l_i| = |1/u_{i-1}|, starting from u = beta at the cut; |w_i| = |1/u_i|
  // is the same sequence one row on) falls below 2^-56, plus two
  double linf = 0.0;
  {
    const double lim = std::ldexp(1.0, -56);
    double u = beta, prod = 1.0;
    int H = 0;
    while (prod > lim && H < 4 * ar->Lw) {
      const double l = 1.0 / u;
      prod *= std::fabs(l);
      u = beta - l;
      linf = std::fabs(l);
      ++H;
    }
    ar->H = (H + 2 + 1) & ~1;
  }
  // a slowly decaying LU (|l| -> above 1/2) belongs to a badly conditioned
  // matrix (r = 40: |l| -> 0.85): one sweep then leaves ~1e-12, a second one
  // restores ~1e-14
  if (ar->sweeps > 0 && linf > 0.5) ar->sweeps = 2;
  ar->whole = (N == ar->Lw);
  ar->L = ar->whole ? ar->Lw : ar->Lw - 2 * ar->H;
  if (!ar->whole && ar->L < ar->Lw / 4) {
    set_error("ADI in FP32/FP32+refine: the factors decay too slowly for %d-row windows (halo %d); use NTK_FP64",
              ar->Lw, ar->H);
    delete ar;
    return NTK_ERR_UNSUPPORTED;
  }
  // windows: first [0, Lw) writes [0, L); middle g writes [gL, gL + L) from
  // [gL - H, gL + L + H); last [N - Lw, N) writes [(P-1) L, N)
  const int Pm1 = (N - ar->Lw + ar->H + ar->L - 1) / ar->L;  // ceil((N - Lw + H) / L)
  ar->P = ar->whole ? 1 : (Pm1 < 1 ? 1 : Pm1) + 1;
  // the paired-chunk kernels (ntk_r2_adi.cu: 512-row windows, power-of-two
  // interior, at most one sweep): their TMA boxes start on 16-row
  // boundaries, so the halo is rounded up to a multiple of 16
  if (ar->M == 16 && ar->sweeps <= 1) {
    const int H16 = ar->whole ? ar->H : (ar->H + 15) & ~15;
    const int L16 = ar->whole ? ar->Lw : ar->Lw - 2 * H16;
    if (ar->whole || L16 >= ar->Lw / 4) {
      const int Q = (N - ar->Lw + H16 + L16 - 1) / L16;
      const int P16 = ar->whole ? 1 : (Q < 1 ? 1 : Q) + 1;
      std::string why;
      ar->r2a = r2::adi_create(N, L16, H16, P16, ar->whole, beta, ar->gamma, ar->sweeps, &why);
      if (ar->r2a) {
        ar->H = H16;
        ar->L = L16;
        ar->P = P16;
      }
    }
  }
  // scaled rows: coeffs (b1, c1, ai, bi, ci, an, bn)
  const double first[7] = {1.0, 0.0, 1.0, beta, 1.0, 1.0, beta};
  const double middle[7] = {beta, 1.0, 1.0, beta, 1.0, 1.0, beta};
  const double last[7] = {beta, 1.0, 1.0, beta, 1.0, 0.0, 1.0};
  const double whole[7] = {1.0, 0.0, 1.0, beta, 1.0, 0.0, 1.0};
  const double* co[4] = {first, middle, last, whole};
  for (int k = 0; k < 4; ++k) {
    if ((k == 3) != ar->whole) continue;
    int rc = ar->win[k].init(ar->Lw, 1, co[k], NTK_FP32_REFINE, 1);
    if (rc == NTK_OK) rc = ar->win[k].init_refine();
    if (rc) {
      delete ar;
      return rc;
    }
  }
  // the kinds' kernel arguments, uploaded once; one kernel shape for all
  // (power-of-two rows and one-shuffle carries only if every kind has them)
  {
    RefineArgs host[4];
    for (int k = 0; k < 4; ++k) {
      if ((k == 3) != ar->whole) continue;
      int M = 0;
      bool p2 = false, dec = false;
      int rc = refine_args(ar->win[k], 1.0, 1.0, 1.0, &host[k], &M, &p2, &dec);
      if (rc) {
        delete ar;
        return rc;
      }
      ar->pow2 = ar->pow2 && p2;
      ar->decay = ar->decay && dec;
      ar->max_ncls = std::max(ar->max_ncls, host[k].ncls);
    }
    int rc = cuda_status(cudaMalloc(&ar->d_args, sizeof(host)), "cudaMalloc(ADI window arguments)");
    if (!rc) rc = cuda_status(cudaMemcpy(ar->d_args, host, sizeof(host), cudaMemcpyHostToDevice),
                              "cudaMemcpy(ADI window arguments)");
    if (rc) {
      delete ar;
      return rc;
    }
  }
  *out = ar;
  return NTK_OK;
}

void adi_refine_destroy(AdiRefine* ar) { delete ar; }

void adi_refine_windows(const AdiRefine* ar, int* L, int* H, int* P) {
  *L = ar->L;
  *H = ar->whole ? 0 : ar->H;
  *P = ar->P;
}

namespace {

// One half step: systems s = 0..N-3 are lines s+1 of the field; in/out point
// at system 0's row 0; `is` is the line stride, `es` the row stride.
int half_step(AdiRefine* ar, const double* in, double* out, long long is, long long es, const double* bnd,
              long long bnd_ss, long long bnd_es, int W, cudaStream_t st) {
  AdiGeom g;
  g.ns = ar->N - 2;
  g.is = is;
  g.es = es;
  g.N = ar->N;
  g.Lw = ar->Lw;
  g.L = ar->L;
  g.H = ar->H;
  g.P = ar->P;
  g.whole = ar->whole ? 1 : 0;
  g.gamma = ar->gamma;
  g.bnd = bnd;
  g.bnd_ss = bnd_ss;
  g.bnd_es = bnd_es;
  using namespace refine_detail;
  switch (ar->M) {
    case 4: return adi_dispatch<4, false>(in, out, g, ar->d_args, ar->max_ncls, ar->pow2, ar->sweeps, W, st);
    case 8: return adi_dispatch<8, false>(in, out, g, ar->d_args, ar->max_ncls, ar->pow2, ar->sweeps, W, st);
    default:
      return ar->decay ? adi_dispatch<16, true>(in, out, g, ar->d_args, ar->max_ncls, ar->pow2, ar->sweeps, W, st)
                       : adi_dispatch<16, false>(in, out, g, ar->d_args, ar->max_ncls, ar->pow2, ar->sweeps, W, st);
  }
}

}  // namespace

int adi_refine_step(AdiRefine* ar, double* u, double* d_x, const double* d_y, cudaStream_t st) {
  if (ar->r2a) return r2::adi_step(ar->r2a, u, d_x, d_y, st);
  const int N = ar->N;
  // x half: systems = rows 1..N-2, stencil of u's rows, boundary RHS from d_x
  int rc = half_step(ar, u + N, d_x + N, N, 1, d_x + N, N, 1, ar->wx, st);
  if (rc) return rc;
  // y half: systems = columns 1..N-2 of d_x, result into u, boundary RHS from d_y
  return half_step(ar, d_x + 1, u + 1, 1, N, d_y + N, N, 1, ar->wy, st);
}

}  // namespace ntk
