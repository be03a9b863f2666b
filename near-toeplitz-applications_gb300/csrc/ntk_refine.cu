// ntk_refine.cu -- host side of the FP32 / FP32+refinement path: FP32
// factor tables in the padded chunk layout, dispatch to the kernel
// instances (ntk_refine_m*.cu, kernel in ntk_refine.cuh).
#include <cmath>
#include <cstring>
#include <vector>

#include "ntk_long_refine.h"
#include "ntk_spike.h"
#include "ntk_r2.h"
#include "ntk_refine.cuh"

namespace ntk {


struct RefineState {
  int M = 0;
  int n_pad = 0;
  int ncls = 32;
  unsigned char cls[32] = {0};
  float* d_tab = nullptr;
  unsigned* d_status = nullptr;
  bool pow2 = false;
  bool decay = false;  // chunk factor products below 2^-26: one-shuffle carries
  // n = 512: the paired-chunk solve (ntk_r2.cu) when the matrix qualifies
  bool r2_ok = false;
  r2::Args r2args;
};

namespace {

DW to_dw(double v) {
  DW d;
  d.h = (float)v;
  d.l = (float)(v - (double)d.h);
  return d;
}

bool is_pow2_or_zero(double v) {
  if (v == 0.0) return true;
  int e;
  double m = std::frexp(std::fabs(v), &e);
  return m == 0.5 && e > -100 && e < 100;
}

}  // namespace

int Plan::init_refine() {
  RefineState* st = new (std::nothrow) RefineState();
  if (!st) {
    set_error("out of host memory");
    return NTK_ERR_ALLOC;
  }
  refine = st;
  int M = 0;
  for (int m : {4, 8, 16, 32})
    if (n <= 32 * m) {
      M = m;
      break;
    }
  if (M == 0) {
    // longer than one warp's register tile: overlapping windows
    // (ntk_long_refine.cu); where the LU multipliers decay too slowly for
    // their halos, exact partitions coupled by a reduced system
    // (ntk_spike.cu); the plan keeps no per-row tables of its own
    const int rc = long_refine_create(&long_refine, *this, precision, sweeps);
    if (rc != NTK_ERR_UNSUPPORTED) return rc;
    return spike_create(&spike, mat, precision == NTK_FP32 ? 0 : sweeps);
  }
  st->M = M;
  st->n_pad = 32 * M;
  if (n > 512) {
    // the alternative for 512 < n <= 1024: two overlapping 512-row windows,
    // 64 threads per system (NTK_TUNE_REFINE_TPS); unavailable where the
    // factors decay too slowly for their halos
    if (long_refine_create(&long_alt, *this, precision, sweeps) != NTK_OK) long_alt = nullptr;
  }
  // FP32 tables in the padded chunk layout (ChunkTabs); rows >= n are
  // identity rows (l = w = 0, g = 1)
  std::vector<double> L(32 * M, 0.0), G(32 * M, 1.0), Wv(32 * M, 0.0);
  for (int r = 0; r < n; ++r) {
    L[r] = lu_l[r];
    G[r] = 1.0 / lu_u[r];
    Wv[r] = (r < n - 1 ? mat.c(r) : 0.0) / lu_u[r];
  }
  // per-lane chunk tables: g, w, phi, l, psi for each of the M rows
  std::vector<std::vector<float>> lane_tab(32, std::vector<float>(5 * (size_t)M, 0.f));
  for (int j = 0; j < 32; ++j) {
    std::vector<float>& t = lane_tab[j];
    double phi = 1.0;
    for (int k = 0; k < M; ++k) {
      const int r = j * M + k;
      phi *= -L[r];
      t[5 * k + 0] = (float)G[r];
      t[5 * k + 1] = (float)Wv[r];
      t[5 * k + 2] = (float)phi;
      t[5 * k + 3] = (float)L[r];
    }
    double psi = 1.0;
    for (int k = M - 1; k >= 0; --k) {
      const int r = j * M + k;
      psi *= -Wv[r];
      t[5 * k + 4] = (float)psi;
    }
  }
  // lanes with bitwise identical tables share one class
  std::vector<int> rep;
  for (int j = 0; j < 32; ++j) {
    int c = -1;
    for (size_t q = 0; q < rep.size() && c < 0; ++q)
      if (std::memcmp(lane_tab[rep[q]].data(), lane_tab[j].data(), sizeof(float) * 5 * M) == 0) c = (int)q;
    if (c < 0) {
      c = (int)rep.size();
      rep.push_back(j);
    }
    st->cls[j] = (unsigned char)c;
  }
  st->ncls = (int)rep.size();
  // lane map (32 ints) | per class: groups of four rows as float4s L, G, W,
  // PHI, PSI (refine_detail::ChunkTabs), pitch class_pitch4
  const int CP = 5 * (M / 4) + 1;  // refine_detail::class_pitch4<M>()
  std::vector<float> tab(32 + 4 * (size_t)st->ncls * CP, 0.f);
  for (int j = 0; j < 32; ++j) {
    const int c = st->cls[j];
    std::memcpy(&tab[j], &c, sizeof(int));
  }
  float* tf = tab.data() + 32;
  for (int c = 0; c < st->ncls; ++c) {
    const std::vector<float>& t = lane_tab[rep[c]];
    for (int k = 0; k < M; ++k) {
      float* grp = tf + 4 * ((size_t)c * CP + 5 * (k / 4));
      const int e = k % 4;
      grp[0 * 4 + e] = t[5 * k + 3];  // l
      grp[1 * 4 + e] = t[5 * k + 0];  // g
      grp[2 * 4 + e] = t[5 * k + 1];  // w
      grp[3 * 4 + e] = t[5 * k + 2];  // phi
      grp[4 * 4 + e] = t[5 * k + 4];  // psi
    }
  }
  int rc = cuda_status(cudaMalloc(&st->d_tab, tab.size() * sizeof(float)), "cudaMalloc(refine tables)");
  if (rc) return rc;
  rc = cuda_status(cudaMemcpy(st->d_tab, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice),
                   "cudaMemcpy(refine tables)");
  if (rc) return rc;
  rc = cuda_status(cudaMalloc(&st->d_status, sizeof(unsigned)), "cudaMalloc(status)");
  if (rc) return rc;
  rc = cuda_status(cudaMemset(st->d_status, 0, sizeof(unsigned)), "cudaMemset(status)");
  if (rc) return rc;
  bool p2 = true;
  for (int i = 0; i < n; ++i) {
    p2 = p2 && is_pow2_or_zero(mat.a(i)) && is_pow2_or_zero(mat.b(i)) && is_pow2_or_zero(mat.c(i));
  }
  st->pow2 = p2;
  // carry truncation is exact to FP32 rounding when every chunk's factor
  // products (over its M rows) are below 2^-26 (only offered for M >= 16)
  bool dec = (M >= 16);
  const double lim = std::ldexp(1.0, -26);
  for (int j = 0; j < 32 && dec; ++j) {
    double pl = 1.0, pw = 1.0;
    for (int k = 0; k < M; ++k) {
      const int r = j * M + k;
      const double l = r < n ? std::fabs(lu_l[r]) : 0.0;
      const double w = r < n ? std::fabs((r < n - 1 ? mat.c(r) : 0.0) / lu_u[r]) : 0.0;
      pl *= l;
      pw *= w;
    }
    dec = (pl <= lim) && (pw <= lim);
  }
  st->decay = dec;
  if (n == r2::NROWS) {
    r2::MatrixRows mr;
    mr.n = n;
    mr.nh = mat.nh;
    mr.nt = mat.nt;
    for (int i = 0; i < 2; ++i) {
      mr.head[i][0] = mat.ha[i];
      mr.head[i][1] = mat.hb[i];
      mr.head[i][2] = mat.hc[i];
      mr.tail[i][0] = mat.ta[i];
      mr.tail[i][1] = mat.tb[i];
      mr.tail[i][2] = mat.tc[i];
    }
    mr.ai = mat.ai;
    mr.bi = mat.bi;
    mr.ci = mat.ci;
    st->r2_ok = r2::prepare(mr, &st->r2args, nullptr);
  }
  return NTK_OK;
}

void Plan::status_words(std::vector<unsigned*>& out) const {
  if (refine && refine->d_status) out.push_back(refine->d_status);
  if (long_refine) long_refine_status_words(long_refine, out);
  if (spike) spike_status_words(spike, out);
  if (long_alt) long_refine_status_words(long_alt, out);
}

void Plan::release_refine() {
  if (long_refine) {
    long_refine_destroy(long_refine);
    long_refine = nullptr;
  }
  if (spike) {
    spike_destroy(spike);
    spike = nullptr;
  }
  if (long_alt) {
    long_refine_destroy(long_alt);
    long_alt = nullptr;
  }
  if (!refine) return;
  if (refine->d_tab) cudaFree(refine->d_tab);
  if (refine->d_status) cudaFree(refine->d_status);
  delete refine;
  refine = nullptr;
}

int Plan::run_refine(const double* in, double* out, const Batch& b, const RhsParams& rp, double s,
                     cudaStream_t stream) {
  if (spike) {
    if (rp.kind != RHS_IDENTITY || s != 1.0) {
      set_error("FP32/refine with slowly decaying LU factors (n > 1024) supports the plain solve only");
      return NTK_ERR_UNSUPPORTED;
    }
    return spike_solve(spike, in, out, b, stream);
  }
  if (long_refine) {
    if (rp.kind != RHS_IDENTITY && rp.kind != RHS_COMPACT) {
      set_error("FP32/refine supports the identity and compact right-hand sides");
      return NTK_ERR_UNSUPPORTED;
    }
    return long_refine_run(long_refine, in, out, b, rp, s, tune_refine_w, stream);
  }
  if (!refine || !refine->d_tab) {
    set_error("plan has no FP32 tables");
    return NTK_ERR_INVALID;
  }
  if (rp.kind != RHS_IDENTITY && rp.kind != RHS_COMPACT) {
    set_error("FP32/refine supports the identity and compact right-hand sides");
    return NTK_ERR_UNSUPPORTED;
  }
  if (long_alt && tune_refine_tps == 64) return long_refine_run(long_alt, in, out, b, rp, s, tune_refine_w, stream);
  if (rp.kind == RHS_COMPACT && n < 4) {
    set_error("compact derivative needs n >= 4");
    return NTK_ERR_INVALID;
  }
  const int sweeps_eff = (precision == NTK_FP32) ? 0 : sweeps;
  if (refine->r2_ok && tune_refine_kernel != 1 && sweeps_eff <= 1 && r2::layout_ok(in, out, b)) {
    r2::Args a2 = refine->r2args;
    r2::set_scales(&a2, rp.sigma0, rp.sigmaN, s);
    a2.status = refine->d_status;
    // strided layouts: persistent CTAs measured faster without refinement,
    // one group per CTA with it (GB300, 512^3 fields)
    const bool persistent = tune_refine_kernel == 3 || (tune_refine_kernel == 0 && sweeps_eff == 0);
    return r2::launch(in, out, b, a2, rp.kind, sweeps_eff, tune_refine_w, persistent, tune_refine_prefetch, stream);
  }
  RefineArgs ra;
  int M = 0;
  bool p2 = false, d = false;
  int rc = refine_args(*this, rp.sigma0, rp.sigmaN, s, &ra, &M, &p2, &d);
  if (rc) return rc;
  const int W = tune_refine_w;
  // two systems per warp: strided layouts with 16 rows per lane
  const bool spw2 = (tune_refine_spw == 2) && (M == 16) && (b.es != 1);
  switch (M) {
    case 4: return refine_dispatch<4, false, 1>(in, out, n, b, ra, p2, sweeps_eff, rp.kind, W, stream);
    case 8: return refine_dispatch<8, false, 1>(in, out, n, b, ra, p2, sweeps_eff, rp.kind, W, stream);
    case 16:
      if (spw2)
        return d ? refine_dispatch<16, true, 2>(in, out, n, b, ra, p2, sweeps_eff, rp.kind, W, stream)
                 : refine_dispatch<16, false, 2>(in, out, n, b, ra, p2, sweeps_eff, rp.kind, W, stream);
      return d ? refine_dispatch<16, true, 1>(in, out, n, b, ra, p2, sweeps_eff, rp.kind, W, stream)
               : refine_dispatch<16, false, 1>(in, out, n, b, ra, p2, sweeps_eff, rp.kind, W, stream);
    default:
      return d ? refine_dispatch<32, true, 1>(in, out, n, b, ra, p2, sweeps_eff, rp.kind, W, stream)
               : refine_dispatch<32, false, 1>(in, out, n, b, ra, p2, sweeps_eff, rp.kind, W, stream);
  }
}

int Plan::run_grad(const double* f, double* ox, double* oy, double* oz, double h, cudaStream_t stream) {
  const int sweeps_eff = (precision == NTK_FP32) ? 0 : sweeps;
  if (!refine || !refine->r2_ok || n != r2::NROWS || sweeps_eff > 1 || tune_refine_kernel == 1) {
    set_error("the one-launch gradient serves n = 512 FP32 / FP32+refine plans of the paired-chunk solve");
    return NTK_ERR_UNSUPPORTED;
  }
  r2::Args a2 = refine->r2args;
  // compact/rhs.py:21-36: interior scale 3/(4h), boundary rows +-1/(2h)
  const double s = 3. / (4 * h);
  r2::set_scales(&a2, (1. / (2 * h)) / s, -(1. / (2 * h)) / s, s);
  a2.status = refine->d_status;
  return r2::launch_grad(f, ox, oy, oz, a2, sweeps_eff, tune_refine_prefetch, stream);
}

int refine_args(const Plan& p, double sigma0, double sigmaN, double s, RefineArgs* out, int* Mout, bool* pow2,
                bool* decay) {
  const RefineState* st = p.refine;
  if (!st || !st->d_tab) {
    set_error("plan has no FP32 tables");
    return NTK_ERR_INVALID;
  }
  const Matrix& mat = p.mat;
  const int n = p.n;
  RefineArgs ra;
  ra.tab = st->d_tab;
  ra.ncls = st->ncls;
  ra.ai = to_dw(mat.ai);
  ra.bi = to_dw(mat.bi);
  ra.ci = to_dw(mat.ci);
  ra.nh = mat.nh;
  ra.nt = mat.nt;
  // special rows as double-word coefficients; row 0 has no a, row n-1 no c
  for (int i = 0; i < 2; ++i) {
    const int hr = i, tr = n - mat.nt + i;
    ra.hd[i][0] = to_dw(hr == 0 ? 0.0 : mat.a(hr));
    ra.hd[i][1] = to_dw(mat.b(hr));
    ra.hd[i][2] = to_dw(mat.c(hr));
    ra.td[i][0] = to_dw(tr >= 0 && tr < n ? mat.a(tr) : 0.0);
    ra.td[i][1] = to_dw(tr >= 0 && tr < n ? mat.b(tr) : 1.0);
    ra.td[i][2] = to_dw(tr >= 0 && tr < n - 1 ? mat.c(tr) : 0.0);
  }
  ra.sigma0 = sigma0;
  ra.sigmaN = sigmaN;
  ra.s = to_dw(s);
  ra.unit_scale = (s == 1.0) ? 1 : 0;
  ra.status = st->d_status;
  *out = ra;
  *Mout = st->M;
  *pow2 = st->pow2;
  *decay = st->decay;
  return NTK_OK;
}

}  // namespace ntk
