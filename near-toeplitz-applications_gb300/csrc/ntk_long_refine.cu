// ntk_long_refine.cu -- FP32 / FP32+refinement plans for systems longer than
// one warp's register tile (n > 1024): the window scheme of the ADI path
// (ntk_adi_refine.cu) applied to a plan's batches (neato.py:168-197 solves,
// compact/rhs.py + solve derivatives).
//
// Each system is cut into windows of Lw = 512 rows overlapping by H-row
// halos (H: product of the LU multipliers over H rows below 2^-56, so the
// truncation lies below the refinement's accuracy); window g writes back
// only its central rows.  The first window keeps the system's row 0 and the
// last its row n-1; the rows at cut ends are interior rows without their
// outer neighbour.  Each kind (first, middle, last) has its own FP32 tables
// and kernel arguments.  A CTA takes W consecutive systems of one window:
// it stages their window rows (plus one row on each side for the compact
// stencil) with cp.async -- lanes walk rows for contiguous systems, adjacent
// systems for strided ones -- forms the double-word right-hand side, solves
// with refine_system and stores the central rows with the staging map.
// Windows of a system overlap, so an in-place call first copies the input
// to the plan's work array.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ntk_long_refine.h"
#include "ntk_refine.cuh"

namespace ntk {

namespace refine_detail {

constexpr int LM = 16;        // rows per lane
constexpr int LLW = 32 * LM;  // window rows

struct LongGeom {
  Batch b;
  int n = 0, L = 0, H = 0, P = 0;
};

struct LongWin {
  int start, lo, hi, kind;  // first row, rows written back [lo, hi), 0 first / 1 middle / 2 last
};
__device__ __forceinline__ LongWin long_window(const LongGeom& g, int w) {
  LongWin r;
  if (w == 0) {
    r.start = 0, r.lo = 0, r.hi = g.L, r.kind = 0;
  } else if (w < g.P - 1) {
    r.start = w * g.L - g.H, r.lo = g.H, r.hi = g.H + g.L, r.kind = 1;
  } else {
    r.start = g.n - LLW, r.lo = (g.P - 1) * g.L - (g.n - LLW), r.hi = LLW, r.kind = 2;
  }
  return r;
}

__host__ __device__ constexpr size_t long_smem(int W, int ncls) {
  return (((size_t)W * sys_pitch<LM>() * sizeof(double) + 2 * W * sizeof(double) + 15) & ~(size_t)15) +
         ((sizeof(RefineArgs) + 15) & ~(size_t)15) + (size_t)ncls * class_pitch4<LM>() * sizeof(float4);
}

// staging (load) or store of the W systems' window rows; thread map: lanes
// walk rows (es == 1: warp w takes system w) or adjacent systems (strided:
// thread t takes system t % W and rows t / W + 32 k, W a power of two)
template <bool LOAD>
__device__ __forceinline__ void long_copy(const double* in, double* out, double* tiles, const LongGeom& g,
                                          long long s0, int wc, int W, int start, int lo, int hi) {
  constexpr int P = sys_pitch<LM>();
  const Batch& b = g.b;
  if (b.es == 1) {
    const int w = (int)(threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (w < wc) {
      const long long base = sys_offset(s0 + w, b) + start;
      double* t = tiles + (size_t)w * P;
#pragma unroll
      for (int q = 0; q < LM; ++q) {
        const int r = lane + 32 * q;
        if (LOAD)
          cp_async8(t + tile_off<LM>(r), in + base + r, 8u);
        else if (r >= lo && r < hi)
          out[base + r] = t[tile_off<LM>(r)];
      }
    }
  } else {
    const int w = (int)threadIdx.x & (W - 1);
    const int rb = (int)threadIdx.x / W;  // 0 .. 31
    if (w < wc) {
      const long long base = sys_offset(s0 + w, b) + (long long)start * b.es;
      double* t = tiles + (size_t)w * P;
#pragma unroll
      for (int q = 0; q < LM; ++q) {
        const int r = rb + 32 * q;
        if (LOAD)
          cp_async8(t + tile_off<LM>(r), in + base + (long long)r * b.es, 8u);
        else if (r >= lo && r < hi)
          out[base + (long long)r * b.es] = t[tile_off<LM>(r)];
      }
    }
  }
}

template <int SWEEPS, bool POW2, bool DECAY, int RHS>
__global__ void __launch_bounds__(256, RefineOcc<LM>::value)
    long_refine_kernel(const double* in, double* out, LongGeom g, const RefineArgs* args) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int P = sys_pitch<LM>();
  const int W = blockDim.x >> 5;
  double* tiles = reinterpret_cast<double*>(smem_raw);  // [W][P]
  double* halo = tiles + (size_t)W * P;                  // [W][2]: rows start-1, start+Lw
  unsigned char* after = smem_raw + (((size_t)W * P * sizeof(double) + 2 * W * sizeof(double) + 15) & ~(size_t)15);
  RefineArgs* ra = reinterpret_cast<RefineArgs*>(after);
  float4* tq = reinterpret_cast<float4*>(after + ((sizeof(RefineArgs) + 15) & ~(size_t)15));
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const unsigned lane = tid & 31;
  const long long nblk = (g.b.nsys + W - 1) / W;
  const int wi = (int)(blockIdx.x / nblk);
  const long long s0 = (blockIdx.x % nblk) * W;
  const int wc = (int)((g.b.nsys - s0) < W ? (g.b.nsys - s0) : W);
  const LongWin wr = long_window(g, wi);
  unsigned range = 0;

  {
    const int* src = reinterpret_cast<const int*>(args + wr.kind);
    int* dst = reinterpret_cast<int*>(ra);
    constexpr int NW = (int)(sizeof(RefineArgs) / sizeof(int));
    for (int i = tid; i < NW; i += blockDim.x) dst[i] = __ldg(src + i);
  }
  __syncthreads();
  const int TC = ra->ncls * class_pitch4<LM>();
  const int cbase = __ldg(reinterpret_cast<const int*>(ra->tab) + lane) * class_pitch4<LM>();
  for (int i = tid; i < TC; i += blockDim.x) tq[i] = __ldg(reinterpret_cast<const float4*>(ra->tab + 32) + i);

  long_copy<true>(in, nullptr, tiles, g, s0, wc, W, wr.start, 0, 0);
  if (RHS == RHS_COMPACT && tid < 2 * wc) {
    // the rows just outside the window (the cut rows' stencil neighbours)
    const int w = tid >> 1;
    const int r = (tid & 1) ? wr.start + LLW : wr.start - 1;
    const bool ok = r >= 0 && r < g.n;
    cp_async8(halo + tid, ok ? in + sys_offset(s0 + w, g.b) + (long long)r * g.b.es : in, ok ? 8u : 0u);
  }
  cp_async_wait_all();
  __syncthreads();

  const int cb = (int)lane * (LM + 1);
  if (warp < wc) {
    double* trow = tiles + (size_t)warp * P;
    float2* drow = reinterpret_cast<float2*>(trow);
    float dh[LM], dl[LM];
    if (RHS == RHS_COMPACT) {
      // D_r = f_{r+1} - f_{r-1} (one DADD, exact when it cancels); the
      // one-sided boundary stencils (compact/rhs.py:21-31) on the
      // system's own first and last rows, in FP64 by the owning lane
      const double* hl = halo + 2 * warp;
      double fprev = (lane > 0) ? trow[tile_off<LM>((int)lane * LM - 1)] : hl[0];
      const double fright = (lane < 31) ? trow[tile_off<LM>((int)lane * LM + LM)] : hl[1];
      double fcur = trow[cb];
#pragma unroll
      for (int k = 0; k < LM; ++k) {
        const double fnext = (k < LM - 1) ? trow[cb + k + 1] : fright;
        split_f64(fnext - fprev, dh[k], dl[k], range);
        fprev = fcur;
        fcur = fnext;
      }
      if (wr.kind == 0 && lane == 0) {
        const double v = ra->sigma0 * ((-5.0 * trow[0] + 4.0 * trow[1]) + trow[2]);
        split_f64(v, dh[0], dl[0], range);
        fast_two_sum(dh[0], dl[0], dh[0], dl[0]);
      }
      if (wr.kind == 2 && lane == 31) {
        const double v = ra->sigmaN * ((-5.0 * trow[tile_off<LM>(LLW - 1)] + 4.0 * trow[tile_off<LM>(LLW - 2)]) +
                                       trow[tile_off<LM>(LLW - 3)]);
        split_f64(v, dh[LM - 1], dl[LM - 1], range);
        fast_two_sum(dh[LM - 1], dl[LM - 1], dh[LM - 1], dl[LM - 1]);
      }
    } else {
#pragma unroll
      for (int k = 0; k < LM; ++k) split_f64(trow[cb + k], dh[k], dl[k], range);
    }
    __syncwarp();  // all stencil reads of the tile done
#pragma unroll
    for (int k = 0; k < LM; ++k) drow[cb + k] = make_float2(dh[k], dl[k]);
    __syncwarp();
    ChunkTabs tabs;
    tabs.q = tq + cbase;
    refine_system<LM, RHS_PRESPLIT, SWEEPS, POW2, false, DECAY>(trow, nullptr, tabs, LLW, *ra, lane, range);
  }
  __syncthreads();
  long_copy<false>(nullptr, out, tiles, g, s0, wc, W, wr.start, wr.lo, wr.hi);
  if (range && ra->status) atomicOr(ra->status, 1u);
}

template <int SWEEPS, bool POW2, bool DECAY, int RHS>
int long_launch(const double* in, double* out, const LongGeom& g, const RefineArgs* d_args, int max_ncls, int W,
                cudaStream_t st) {
  const size_t smem = long_smem(W, max_ncls);
  auto kern = long_refine_kernel<SWEEPS, POW2, DECAY, RHS>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute(long_refine_kernel)");
  const long long blocks = (long long)g.P * ((g.b.nsys + W - 1) / W);
  if (blocks <= 0) return NTK_OK;
  if (blocks > 0x7fffffffLL) {
    set_error("too many windows for one launch");
    return NTK_ERR_INVALID;
  }
  kern<<<(unsigned)blocks, W * 32, smem, st>>>(in, out, g, d_args);
  return cuda_status(cudaGetLastError(), "long_refine_kernel");
}

template <int SWEEPS, bool DECAY, int RHS>
int long_pow2(const double* in, double* out, const LongGeom& g, const RefineArgs* d_args, int max_ncls, bool pow2,
              int W, cudaStream_t st) {
  return pow2 ? long_launch<SWEEPS, true, DECAY, RHS>(in, out, g, d_args, max_ncls, W, st)
              : long_launch<SWEEPS, false, DECAY, RHS>(in, out, g, d_args, max_ncls, W, st);
}

template <bool DECAY, int RHS>
int long_sweeps(const double* in, double* out, const LongGeom& g, const RefineArgs* d_args, int max_ncls,
                bool pow2, int sweeps, int W, cudaStream_t st) {
  switch (sweeps) {
    case 0: return long_pow2<0, DECAY, RHS>(in, out, g, d_args, max_ncls, pow2, W, st);
    case 1: return long_pow2<1, DECAY, RHS>(in, out, g, d_args, max_ncls, pow2, W, st);
    default: return long_pow2<2, DECAY, RHS>(in, out, g, d_args, max_ncls, pow2, W, st);
  }
}

}  // namespace refine_detail

struct LongRefine {
  int n = 0, H = 0, L = 0, P = 0;
  int sweeps = 1;
  Plan win[3];  // first, middle, last window matrices (n = 512)
  // kernel arguments per (RHS scales, output scale): the compact derivative
  // and the plain solve need different ones
  std::vector<std::pair<std::vector<double>, RefineArgs*>> d_args;
  int max_ncls = 1;
  bool pow2 = true, decay = true;
  double* work = nullptr;  // input copy for in-place calls
  size_t work_elems = 0;
  ~LongRefine() {
    for (auto& kv : d_args) cudaFree(kv.second);
    if (work) cudaFree(work);
  }
};

void long_refine_status_words(const LongRefine* lr, std::vector<unsigned*>& out) {
  for (const Plan& w : lr->win) w.status_words(out);
}

int long_refine_create(LongRefine** out, const Plan& p, int precision, int sweeps) {
  using namespace refine_detail;
  *out = nullptr;
  const Matrix& m = p.mat;
  // interior pivot fixed point and the larger multiplier magnitude there
  double u = m.bi;
  for (int i = 0; i < 4096; ++i) {
    const double un = m.bi - m.ai * m.ci / u;
    if (un == u || !std::isfinite(un)) break;
    u = un;
  }
  const double mult = std::max(std::fabs(m.ai / u), std::fabs(m.ci / u));
  if (!std::isfinite(mult) || !(mult < 0.9)) {
    set_error("FP32/refine for n > 1024 needs decaying LU multipliers (|a/u|, |c/u| < 0.9; got %g); use NTK_FP64",
              mult);
    return NTK_ERR_UNSUPPORTED;
  }
  int H = 0;
  for (double prod = 1.0; prod > std::ldexp(1.0, -56); prod *= mult) ++H;
  H = (H + 3) & ~1;
  const int L = LLW - 2 * H;
  if (L < LLW / 4) {
    set_error("FP32/refine for n > 1024: the LU multipliers decay too slowly for 512-row windows (halo %d); "
              "use NTK_FP64", H);
    return NTK_ERR_UNSUPPORTED;
  }
  LongRefine* lr = new (std::nothrow) LongRefine();
  if (!lr) {
    set_error("out of host memory");
    return NTK_ERR_ALLOC;
  }
  lr->n = p.n;
  lr->H = H;
  lr->L = L;
  lr->P = (p.n - LLW + H + L - 1) / L + 1;
  lr->sweeps = (precision == NTK_FP32) ? 0 : sweeps;
  const double* co = p.coeffs;  // (b1, c1, ai, bi, ci, an, bn)
  const double first[7] = {co[0], co[1], co[2], co[3], co[4], co[2], co[3]};
  const double middle[7] = {co[3], co[4], co[2], co[3], co[4], co[2], co[3]};
  const double last[7] = {co[3], co[4], co[2], co[3], co[4], co[5], co[6]};
  const double* kc[3] = {first, middle, last};
  for (int k = 0; k < 3; ++k) {
    int rc = lr->win[k].init(LLW, 1, kc[k], NTK_FP32_REFINE, 1);
    if (rc == NTK_OK) rc = lr->win[k].init_refine();
    if (rc) {
      delete lr;
      return rc;
    }
  }
  *out = lr;
  return NTK_OK;
}

void long_refine_destroy(LongRefine* lr) { delete lr; }

namespace {

long long sys_offset_host(long long s, const Batch& b) {
  if (b.ni >= b.nsys) return s * b.is;
  return (s / b.ni) * b.os + (s % b.ni) * b.is;
}

int args_for(LongRefine* lr, double sigma0, double sigmaN, double s, const RefineArgs** out) {
  const std::vector<double> key = {sigma0, sigmaN, s};
  for (auto& kv : lr->d_args)
    if (kv.first == key) {
      *out = kv.second;
      return NTK_OK;
    }
  RefineArgs host[3];
  for (int k = 0; k < 3; ++k) {
    int M = 0;
    bool p2 = false, dec = false;
    int rc = refine_args(lr->win[k], sigma0, sigmaN, s, &host[k], &M, &p2, &dec);
    if (rc) return rc;
    lr->pow2 = lr->pow2 && p2;
    lr->decay = lr->decay && dec;
    lr->max_ncls = std::max(lr->max_ncls, host[k].ncls);
  }
  RefineArgs* d = nullptr;
  int rc = cuda_status(cudaMalloc(&d, sizeof(host)), "cudaMalloc(window arguments)");
  if (!rc) rc = cuda_status(cudaMemcpy(d, host, sizeof(host), cudaMemcpyHostToDevice), "cudaMemcpy(window arguments)");
  if (rc) {
    if (d) cudaFree(d);
    return rc;
  }
  lr->d_args.emplace_back(key, d);
  *out = d;
  return NTK_OK;
}

}  // namespace

int long_refine_run(LongRefine* lr, const double* in, double* out, const Batch& b, const RhsParams& rp, double s,
                    int W, cudaStream_t st) {
  using namespace refine_detail;
  if (b.nsys == 0) return NTK_OK;
  const RefineArgs* d_args = nullptr;
  int rc = args_for(lr, rp.kind == RHS_COMPACT ? rp.sigma0 : 1.0, rp.kind == RHS_COMPACT ? rp.sigmaN : 1.0, s,
                    &d_args);
  if (rc) return rc;
  if (W != 4 && W != 8) W = 8;
  // extent of the batch (elements from the first system's row 0)
  long long lo_off = sys_offset_host(0, b), hi_off = sys_offset_host(b.nsys - 1, b);
  const long long extent = std::max(lo_off, hi_off) + (long long)(lr->n - 1) * b.es + 1;
  const double* src = in;
  if (in + extent > out && out + extent > in) {
    // windows overlap: read from a copy
    if (lr->work_elems < (size_t)extent) {
      if (lr->work) cudaFree(lr->work);
      lr->work = nullptr;
      lr->work_elems = 0;
      rc = cuda_status(cudaMalloc(&lr->work, sizeof(double) * (size_t)extent), "cudaMalloc(window work array)");
      if (rc) return rc;
      lr->work_elems = (size_t)extent;
    }
    rc = cuda_status(cudaMemcpyAsync(lr->work, in, sizeof(double) * (size_t)extent, cudaMemcpyDeviceToDevice, st),
                     "cudaMemcpyAsync(window input copy)");
    if (rc) return rc;
    src = lr->work;
  }
  LongGeom g;
  g.b = b;
  g.n = lr->n;
  g.L = lr->L;
  g.H = lr->H;
  g.P = lr->P;
  if (rp.kind == RHS_COMPACT)
    return lr->decay ? long_sweeps<true, RHS_COMPACT>(src, out, g, d_args, lr->max_ncls, lr->pow2, lr->sweeps, W, st)
                     : long_sweeps<false, RHS_COMPACT>(src, out, g, d_args, lr->max_ncls, lr->pow2, lr->sweeps, W, st);
  return lr->decay ? long_sweeps<true, RHS_IDENTITY>(src, out, g, d_args, lr->max_ncls, lr->pow2, lr->sweeps, W, st)
                   : long_sweeps<false, RHS_IDENTITY>(src, out, g, d_args, lr->max_ncls, lr->pow2, lr->sweeps, W, st);
}

}  // namespace ntk
