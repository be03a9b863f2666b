// ntk_adi_f64.cu -- FP64 ADI half steps (experiments/run-adi.py:59-71) over
// overlapping windows, one warp per window.
//
// The reference solves each half step's N-2 systems of N rows with one CUDA
// block per system (neato.py:8-124).  Here every system is cut into the
// windows of the FP32 + refinement path (ntk_adi_geom.h: Lw = 32 M rows,
// central rows written back, halos of H rows), with H chosen so that the
// product of the LU multipliers over H rows is below 2^-64: the truncation
// is below FP64 rounding.  Inside a window nothing is truncated: lane j of
// the warp holds rows [jM, (j+1)M) in registers and runs Thomas's forward
// and backward recurrences over its chunk from zero; the chunks' carries are
// an exact affine scan across the 32 lanes (5 shuffle steps), applied with
// tabulated carry responses:
//   forward   y_i = d_i - l_i y_{i-1}:      y_i = y'_i + phi_i y_{s-1},
//             phi_s = -l_s, phi_i = -l_i phi_{i-1}        (chunk start s)
//   backward  x_i = y_i / u_i - (c_i / u_i) x_{i+1}:  x_i = x'_i + psi_i x_{e+1},
//             psi_e = -c_e / u_e, psi_i = -(c_i / u_i) psi_{i+1}   (chunk end e)
// The matrices are the reference's unscaled rows (run-adi.py:50-53): identity
// rows at the system's ends, (1/dx^2, -2 (1/dt + 1/dx^2), 1/dx^2) inside; the
// right-hand side is the vertical stencil of adi/rhs.py:21-24 evaluated as
// the segmented kernel does, fma(top, hi, fma(center, mid, bottom * lo)).
// When the stencil's centre coefficient 2 (1/dx^2 - 1/dt) is exactly zero
// (dt = dx^2, r = 0.5), interior rows are divided by 1/dx^2 instead: the
// matrix becomes (1, -4, 1) and the right-hand side -(lo + hi), one FP64
// addition instead of three operations (the solution is the same system's).
// Window kinds (first, middle, last, whole) have their own tables, stored
// [table][row in chunk k][lane j] so a warp's load of row k of every chunk
// is 256 contiguous bytes.  (Folding 1/u into per-row stencil coefficients
// saves one FP64 multiply per row but needs two more tables: measured
// slower, and it moved the r = 40 error from below to above 1e-13.)
// FP64 work per row: 3 (stencil; 1 when scaled) + 3 (sweeps) + 2 (carries).
#include <algorithm>
#include <cmath>
#include <vector>

#include "ntk_adi_f64.h"
#include "ntk_adi_geom.h"
#include "ntk_plan.h"
#include "ntk_refine.cuh"

namespace ntk {

namespace adi_f64_detail {

using refine_detail::sys_pitch;
using refine_detail::tile_off;

constexpr int NTAB = 5;  // -l, phi, 1/u, -c/u, psi per row
constexpr unsigned FULL = 0xffffffffu;

template <int M>
__host__ __device__ constexpr size_t smem_bytes(int W) {
  return (size_t)(W + 2) * sys_pitch<M>() * sizeof(double);
}

// One launch per half step: CTA b solves window b / nblk of the W
// consecutive systems starting at (b % nblk) W.  tab: [kind][NTAB][M][32].
template <int M, bool SCALED>
__global__ void __launch_bounds__(256, 3)
    adi_f64_kernel(const double* __restrict__ in, double* __restrict__ out, AdiGeom geo,
                   const double* __restrict__ tab) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int P = sys_pitch<M>();
  constexpr int LW = 32 * M;
  const int W = blockDim.x >> 5;
  double* lines = reinterpret_cast<double*>(smem_raw);  // [W + 2][P]
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int lane = tid & 31;
  const long long nblk = (geo.ns + W - 1) / W;
  const int wi = (int)(blockIdx.x / nblk);
  const long long s0 = (blockIdx.x % nblk) * W;
  const int wc = (int)((geo.ns - s0) < W ? (geo.ns - s0) : W);
  const WinRows wr = window_rows(geo, wi);

  // ---- stage lines s0-1 .. s0+wc (the stencil's neighbours included);
  // lanes walk rows for unit element stride, lines otherwise ----
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
    cp_async8(lines + (size_t)j * P + tile_off<M>(r), wbase + (s0 - 1 + j) * geo.is + (long long)r * geo.es, 8u);
  }
  cp_async_wait_all();
  __syncthreads();

  const int cb = lane * (M + 1);
  const long long s = s0 + warp;
  // row k of this lane's chunk in table t: tk[t * LW + 32 k]
  const double* tk = tab + (size_t)wr.kind * NTAB * LW + lane;
  const double* t_ml = tk;
  const double* t_phi = tk + LW;
  const double* t_iu = tk + 2 * LW;
  const double* t_mcu = tk + 3 * LW;
  const double* t_psi = tk + 4 * LW;
  double v[M];
  if (warp < wc) {
    const double* lo = lines + (size_t)warp * P + cb;
    const double* mid = lo + P;
    const double* hi = mid + P;
    if (SCALED) {
#pragma unroll
      for (int k = 0; k < M; ++k) v[k] = (-lo[k]) - hi[k];
    } else {
#pragma unroll
      for (int k = 0; k < M; ++k) v[k] = fma(geo.top, hi[k], fma(geo.center, mid[k], geo.bottom * lo[k]));
    }
    // identity rows: x = the boundary value (experiments/run-adi.py:50-53)
    if ((wr.kind == 0 || wr.kind == 3) && lane == 0) v[0] = geo.bnd[s * geo.bnd_ss];
    if ((wr.kind == 2 || wr.kind == 3) && lane == 31)
      v[M - 1] = geo.bnd[s * geo.bnd_ss + (long long)(geo.N - 1) * geo.bnd_es];
  }
  __syncthreads();  // all lines read: line warp + 1 becomes this warp's output tile
  if (warp >= wc) return;

  // ---- forward: chunk-local sweep, carry scan, carry applied ----
#pragma unroll
  for (int k = 1; k < M; ++k) v[k] = fma(__ldg(t_ml + 32 * k), v[k - 1], v[k]);
  {
    double a = v[M - 1], b = __ldg(t_phi + 32 * (M - 1));
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double ap = __shfl_up_sync(FULL, a, o);
      const double bp = __shfl_up_sync(FULL, b, o);
      if (lane >= o) {
        a = fma(b, ap, a);
        b *= bp;
      }
    }
    double carry = __shfl_up_sync(FULL, a, 1);
    if (lane == 0) carry = 0.0;
#pragma unroll
    for (int k = 0; k < M; ++k) v[k] = fma(__ldg(t_phi + 32 * k), carry, v[k]);
  }
  // ---- backward ----
  v[M - 1] *= __ldg(t_iu + 32 * (M - 1));
#pragma unroll
  for (int k = M - 2; k >= 0; --k) v[k] = fma(__ldg(t_mcu + 32 * k), v[k + 1], v[k] * __ldg(t_iu + 32 * k));
  {
    double a = v[0], b = __ldg(t_psi);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double ap = __shfl_down_sync(FULL, a, o);
      const double bp = __shfl_down_sync(FULL, b, o);
      if (lane + o < 32) {
        a = fma(b, ap, a);
        b *= bp;
      }
    }
    double carry = __shfl_down_sync(FULL, a, 1);
    if (lane == 31) carry = 0.0;
#pragma unroll
    for (int k = 0; k < M; ++k) v[k] = fma(__ldg(t_psi + 32 * k), carry, v[k]);
  }

  // ---- write back the window's central rows through the tile (coalesced
  // for unit stride) ----
  double* trow = lines + (size_t)(warp + 1) * P;
#pragma unroll
  for (int k = 0; k < M; ++k) trow[cb + k] = v[k];
  __syncwarp();
  double* dst = out + (long long)wr.start * geo.es + s * geo.is;
#pragma unroll 4
  for (int q = 0; q < M; ++q) {
    const int r = lane + 32 * q;
    if (r >= wr.lo && r < wr.hi) dst[(long long)r * geo.es] = trow[tile_off<M>(r)];
  }
}

template <int M, bool SCALED>
int launch(const double* in, double* out, const AdiGeom& geo, const double* d_tab, int W, cudaStream_t st) {
  const size_t smem = smem_bytes<M>(W);
  auto kern = adi_f64_kernel<M, SCALED>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute(adi_f64_kernel)");
  const long long blocks = (long long)geo.P * ((geo.ns + W - 1) / W);
  if (blocks <= 0) return NTK_OK;
  if (blocks > 0x7fffffffLL) {
    set_error("too many ADI windows for one launch");
    return NTK_ERR_INVALID;
  }
  kern<<<(unsigned)blocks, W * 32, smem, st>>>(in, out, geo, d_tab);
  return cuda_status(cudaGetLastError(), "adi_f64_kernel");
}

}  // namespace adi_f64_detail

struct AdiF64 {
  int N = 0;
  int M = 0, Lw = 0, H = 0, L = 0, P = 0;  // rows per lane, window, halo, central rows, windows
  bool whole = false;
  bool scaled = false;         // centre coefficient 0: rows divided by 1/dx^2
  double bottom = 0.0, center = 0.0, top = 0.0;
  int wx = 4, wy = 8;          // systems per CTA: x half step (rows), y half step (columns)
  double* d_tab = nullptr;     // [4][NTAB][Lw]
  ~AdiF64() {
    if (d_tab) cudaFree(d_tab);
  }
};

namespace {

// Per-row tables of one window matrix (coefficient tuple as in neato.py:136-138),
// row i = jM + k of lane j's chunk stored at k * 32 + j.
bool window_tables(int Lw, int M, const double co[7], double* t) {
  Matrix m;
  m.n = Lw;
  m.set_reference(co);
  std::vector<double> l, u;
  if (!factor_host(m, l, u)) return false;
  std::vector<double> ml(Lw), phi(Lw), iu(Lw), mcu(Lw), psi(Lw);
  for (int i = 0; i < Lw; ++i) {
    ml[i] = -l[i];
    iu[i] = 1.0 / u[i];
    mcu[i] = -m.c(i) / u[i];
    phi[i] = (i % M == 0) ? ml[i] : ml[i] * phi[i - 1];
  }
  for (int i = Lw - 1; i >= 0; --i) psi[i] = (i % M == M - 1) ? mcu[i] : mcu[i] * psi[i + 1];
  const std::vector<double>* tabs[5] = {&ml, &phi, &iu, &mcu, &psi};
  for (int q = 0; q < 5; ++q)
    for (int i = 0; i < Lw; ++i) t[(size_t)q * Lw + (i % M) * 32 + i / M] = (*tabs[q])[i];
  return true;
}

int half_step(AdiF64* af, const double* in, double* out, long long is, long long es, const double* bnd,
              long long bnd_ss, long long bnd_es, int W, cudaStream_t st) {
  AdiGeom g;
  g.ns = af->N - 2;
  g.is = is;
  g.es = es;
  g.N = af->N;
  g.Lw = af->Lw;
  g.L = af->L;
  g.H = af->H;
  g.P = af->P;
  g.whole = af->whole ? 1 : 0;
  g.bottom = af->bottom;
  g.center = af->center;
  g.top = af->top;
  g.bnd = bnd;
  g.bnd_ss = bnd_ss;
  g.bnd_es = bnd_es;
  using namespace adi_f64_detail;
  if (af->scaled) {
    switch (af->M) {
      case 4: return launch<4, true>(in, out, g, af->d_tab, W, st);
      case 8: return launch<8, true>(in, out, g, af->d_tab, W, st);
      default: return launch<16, true>(in, out, g, af->d_tab, W, st);
    }
  }
  switch (af->M) {
    case 4: return launch<4, false>(in, out, g, af->d_tab, W, st);
    case 8: return launch<8, false>(in, out, g, af->d_tab, W, st);
    default: return launch<16, false>(in, out, g, af->d_tab, W, st);
  }
}

}  // namespace

int adi_f64_create(AdiF64** out, int N, double dx, double dt) {
  *out = nullptr;
  int M = 0;
  for (int m : {16, 8, 4})
    if (32 * m <= N) {
      M = m;
      break;
    }
  if (M == 0) {
    set_error("FP64 ADI windows need N >= 128 (got %d)", N);
    return NTK_ERR_UNSUPPORTED;
  }
  const int Lw = 32 * M;
  const double e = 1.0 / (dx * dx);
  const double b = -2.0 * (1.0 / dt + e);
  // halo: rows from a cut until the product of the multipliers |l_i| =
  // |e / u_{i-1}| falls below 2^-64 (the backward multipliers |c_i / u_i| are
  // the same sequence one row on), plus two
  int H = 0;
  {
    const double lim = std::ldexp(1.0, -64);
    double u = b, prod = 1.0;
    while (prod > lim && H < 4 * Lw) {
      const double l = e / u;
      prod *= std::fabs(l);
      u = b - l * e;
      ++H;
    }
    H = (H + 2 + 1) & ~1;
  }
  const bool whole = (N == Lw);
  const int L = whole ? Lw : Lw - 2 * H;
  if (!whole && L < Lw / 4) {
    set_error("FP64 ADI windows: the factors decay too slowly for %d-row windows (halo %d)", Lw, H);
    return NTK_ERR_UNSUPPORTED;
  }
  AdiF64* af = new (std::nothrow) AdiF64();
  if (!af) {
    set_error("out of host memory");
    return NTK_ERR_ALLOC;
  }
  af->N = N;
  af->M = M;
  af->Lw = Lw;
  af->H = H;
  af->whole = whole;
  af->L = L;
  const int Pm1 = (N - Lw + H + L - 1) / L;  // ceil((N - Lw + H) / L)
  af->P = whole ? 1 : (Pm1 < 1 ? 1 : Pm1) + 1;
  // adi/rhs.py:46-49
  af->bottom = -e;
  af->top = -e;
  af->center = 2 * (-1. / dt + e);
  // window matrices (b1, c1, ai, bi, ci, an, bn): identity rows at the
  // system's ends, cut rows (the outside neighbour dropped) elsewhere;
  // interior rows divided by e when the stencil's centre is zero
  af->scaled = (af->center == 0.0);
  const double ei = af->scaled ? 1.0 : e;
  const double bi = af->scaled ? b / e : b;
  const double first[7] = {1.0, 0.0, ei, bi, ei, ei, bi};
  const double middle[7] = {bi, ei, ei, bi, ei, ei, bi};
  const double last[7] = {bi, ei, ei, bi, ei, 0.0, 1.0};
  const double wholem[7] = {1.0, 0.0, ei, bi, ei, 0.0, 1.0};
  const double* co[4] = {first, middle, last, wholem};
  const size_t per = (size_t)adi_f64_detail::NTAB * Lw;
  std::vector<double> host(4 * per, 0.0);
  for (int k = 0; k < 4; ++k) {
    if ((k == 3) != whole) continue;
    if (!window_tables(Lw, M, co[k], host.data() + k * per)) {
      set_error("FP64 ADI window matrix has a zero or non-finite pivot");
      delete af;
      return NTK_ERR_INVALID;
    }
  }
  int rc = cuda_status(cudaMalloc(&af->d_tab, host.size() * sizeof(double)), "cudaMalloc(ADI window tables)");
  if (!rc)
    rc = cuda_status(cudaMemcpy(af->d_tab, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice),
                     "cudaMemcpy(ADI window tables)");
  if (rc) {
    delete af;
    return rc;
  }
  *out = af;
  return NTK_OK;
}

void adi_f64_destroy(AdiF64* af) { delete af; }

void adi_f64_windows(const AdiF64* af, int* L, int* H, int* P) {
  *L = af->L;
  *H = af->whole ? 0 : af->H;
  *P = af->P;
}

int adi_f64_step(AdiF64* af, double* u, double* d_x, const double* d_y, cudaStream_t st) {
  const int N = af->N;
  // x half: systems = rows 1..N-2, stencil of u's rows, boundary RHS from d_x
  int rc = half_step(af, u + N, d_x + N, N, 1, d_x + N, N, 1, af->wx, st);
  if (rc) return rc;
  // y half: systems = columns 1..N-2 of d_x, result into u, boundary RHS from d_y
  return half_step(af, d_x + 1, u + 1, 1, N, d_y + N, N, 1, af->wy, st);
}

}  // namespace ntk
