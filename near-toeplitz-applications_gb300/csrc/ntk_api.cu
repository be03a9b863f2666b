// ntk_api.cu -- the C ABI (include/ntk.h): plans, validation, dispatch.
//
// A plan is the GB300 counterpart of the reference's NearToeplitzSolver
// (neato.py:129-197).  The reference precomputes per-level cyclic-reduction
// coefficients on the host (neato.py:199-274) and renders/compiles one
// kernel per system size; here the shared matrix is factored once on the
// host in FP64 (l_i, u_i), the factor tables are uploaded, and precompiled
// kernels take n as an argument.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "ntk_internal.h"
#include "ntk_plan.h"

namespace ntk {

namespace {
thread_local std::string g_last_error;
}

void set_error(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

int cuda_status(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return NTK_OK;
  set_error("%s: %s", where, cudaGetErrorString(e));
  return NTK_ERR_CUDA;
}

int read_clear_status(const std::vector<unsigned*>& words, cudaStream_t st, int* flags) {
  unsigned acc = 0;
  for (unsigned* w : words) {
    if (!w) continue;
    unsigned h = 0;
    int rc = cuda_status(cudaMemcpyAsync(&h, w, sizeof(unsigned), cudaMemcpyDeviceToHost, st),
                         "cudaMemcpyAsync(status word)");
    if (!rc) rc = cuda_status(cudaMemsetAsync(w, 0, sizeof(unsigned), st), "cudaMemsetAsync(status word)");
    if (!rc) rc = cuda_status(cudaStreamSynchronize(st), "cudaStreamSynchronize(status)");
    if (rc) return rc;
    acc |= h;
  }
  if (flags) *flags = (int)acc;
  if (acc & STATUS_RANGE) {
    set_error("input outside the FP32 + refinement range (|x| >= 2^128, inf or nan) in a solve since the last "
              "status read");
    return NTK_ERR_RANGE;
  }
  return NTK_OK;
}

// LU factors of the near-Toeplitz matrix; false on a zero pivot.
bool factor_host(const Matrix& m, std::vector<double>& l, std::vector<double>& u) {
  const int n = m.n;
  l.assign(n, 0.0);
  u.assign(n, 0.0);
  u[0] = m.b(0);
  if (!(u[0] != 0.0) || !std::isfinite(u[0])) return false;
  for (int i = 1; i < n; ++i) {
    l[i] = m.a(i) / u[i - 1];
    u[i] = m.b(i) - l[i] * m.c(i - 1);
    if (!(u[i] != 0.0) || !std::isfinite(u[i])) return false;
  }
  return true;
}

int Plan::init(int n_, long long nrhs_, const double co[7], int prec, int sweeps_) {
  n = n_;
  nrhs = nrhs_;
  for (int i = 0; i < 7; ++i) coeffs[i] = co[i];
  mat.n = n;
  mat.set_reference(co);
  precision = prec;
  sweeps = sweeps_;
  if (cudaGetDevice(&device) != cudaSuccess) {
    set_error("no CUDA device");
    return NTK_ERR_CUDA;
  }
  if (!factor_host(mat, lu_l, lu_u)) {
    set_error("matrix has a zero or non-finite pivot (LU breakdown)");
    return NTK_ERR_INVALID;
  }
  // l and w are independent of the RHS scale
  std::vector<double> host(2 * (size_t)n);
  for (int i = 0; i < n; ++i) {
    host[i] = lu_l[i];
    host[n + i] = (i < n - 1 ? mat.c(i) : 0.0) / lu_u[i];
  }
  int rc = cuda_status(cudaMalloc(&d_lw, sizeof(double) * 2 * (size_t)n), "cudaMalloc(factor tables)");
  if (rc) return rc;
  rc = cuda_status(cudaMemcpy(d_lw, host.data(), sizeof(double) * 2 * (size_t)n, cudaMemcpyHostToDevice),
                   "cudaMemcpy(factor tables)");
  if (rc) return rc;
  return NTK_OK;
}

Plan::~Plan() {
  if (d_lw) cudaFree(d_lw);
  for (auto& kv : g_by_scale) cudaFree(kv.second);
  release_refine();
}

// g_i = s / u_i for the requested scale, uploaded once per distinct s.
int Plan::g_table(double s, const double** out) {
  std::lock_guard<std::mutex> lk(mu);
  auto it = g_by_scale.find(s);
  if (it != g_by_scale.end()) {
    *out = it->second;
    return NTK_OK;
  }
  if (g_by_scale.size() >= 16) {
    set_error("more than 16 distinct RHS scales used with one plan");
    return NTK_ERR_UNSUPPORTED;
  }
  std::vector<double> g(n);
  for (int i = 0; i < n; ++i) g[i] = s / lu_u[i];
  double* d = nullptr;
  int rc = cuda_status(cudaMalloc(&d, sizeof(double) * (size_t)n), "cudaMalloc(g table)");
  if (rc) return rc;
  rc = cuda_status(cudaMemcpy(d, g.data(), sizeof(double) * (size_t)n, cudaMemcpyHostToDevice), "cudaMemcpy(g)");
  if (rc) {
    cudaFree(d);
    return rc;
  }
  g_by_scale[s] = d;
  *out = d;
  return NTK_OK;
}

int Plan::check_device() const {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev != device) {
    set_error("plan was created on device %d but the current device is %d", device, dev);
    return NTK_ERR_INVALID;
  }
  return NTK_OK;
}

// Dispatch of one batched solve with a fused RHS.
int Plan::run(const double* in, double* out, const Batch& b, RhsParams rp, double s, cudaStream_t stream) {
  int rc = check_device();
  if (rc) return rc;
  if (b.nsys == 0) return NTK_OK;
  if (precision == NTK_FP64) {
    TablesF64 t;
    t.l = d_lw;
    t.w = d_lw + n;
    rc = g_table(s, &t.g);
    if (rc) return rc;
    return launch_thomas_f64(in, out, n, b, rp, t, tune_f64_threads, stream, tune_f64_x_variant);
  }
  return run_refine(in, out, b, rp, s, stream);
}

static bool bad_ptr(const void* p) { return p == nullptr || (reinterpret_cast<uintptr_t>(p) & 7) != 0; }

}  // namespace ntk

using ntk::Batch;
using ntk::Plan;
using ntk::RhsParams;

struct ntk_plan : public Plan {};

extern "C" {

const char* ntk_version(void) { return "ntk 0.1.0 (sm_103a, CUDA " NTK_STR(__CUDACC_VER_MAJOR__) ")"; }

int ntk_last_error(char* buf, int len) {
  const std::string& e = ntk::g_last_error;
  if (buf && len > 0) {
    size_t k = e.size() < (size_t)(len - 1) ? e.size() : (size_t)(len - 1);
    memcpy(buf, e.data(), k);
    buf[k] = '\0';
  }
  return (int)e.size();
}

int ntk_plan_create(ntk_plan** out, int n, long long nrhs, const double coeffs[7], int precision,
                    int refine_sweeps) {
  if (!out || !coeffs) {
    ntk::set_error("ntk_plan_create: null argument");
    return NTK_ERR_INVALID;
  }
  *out = nullptr;
  if (n < 3) {
    ntk::set_error("ntk_plan_create: n must be >= 3 (got %d)", n);
    return NTK_ERR_INVALID;
  }
  if (nrhs < 0) {
    ntk::set_error("ntk_plan_create: nrhs must be >= 0");
    return NTK_ERR_INVALID;
  }
  if (precision != NTK_FP64 && precision != NTK_FP32 && precision != NTK_FP32_REFINE) {
    ntk::set_error("ntk_plan_create: unknown precision %d", precision);
    return NTK_ERR_INVALID;
  }
  if (precision == NTK_FP32_REFINE && (refine_sweeps < 1 || refine_sweeps > 4)) {
    ntk::set_error("ntk_plan_create: refine_sweeps must be in 1..4 (got %d)", refine_sweeps);
    return NTK_ERR_INVALID;
  }
  for (int i = 0; i < 7; ++i)
    if (!std::isfinite(coeffs[i])) {
      ntk::set_error("ntk_plan_create: coefficient %d is not finite", i);
      return NTK_ERR_INVALID;
    }
  ntk_plan* p = new (std::nothrow) ntk_plan();
  if (!p) {
    ntk::set_error("ntk_plan_create: out of host memory");
    return NTK_ERR_ALLOC;
  }
  int rc = p->init(n, nrhs, coeffs, precision, precision == NTK_FP32 ? 0 : refine_sweeps);
  if (rc == NTK_OK && precision != NTK_FP64) rc = p->init_refine();
  if (rc) {
    delete p;
    return rc;
  }
  *out = p;
  return NTK_OK;
}

int ntk_plan_set_tuning(ntk_plan* plan, int key, int value) {
  if (!plan) {
    ntk::set_error("ntk_plan_set_tuning: null plan");
    return NTK_ERR_INVALID;
  }
  switch (key) {
    case NTK_TUNE_F64_X_VARIANT:
      if (value < 0 || value > 2) break;
      plan->tune_f64_x_variant = value;
      return NTK_OK;
    case NTK_TUNE_F64_THREADS:
      if (value != 32 && value != 64 && value != 128) break;
      plan->tune_f64_threads = value;
      return NTK_OK;
    case NTK_TUNE_REFINE_W:
      if (value != 4 && value != 8 && value != 16) break;
      plan->tune_refine_w = value;
      return NTK_OK;
    case NTK_TUNE_REFINE_SPW:
      if (value != 1 && value != 2) break;
      plan->tune_refine_spw = value;
      return NTK_OK;
    case NTK_TUNE_REFINE_KERNEL:
      if (value < 0 || value > 3) break;
      plan->tune_refine_kernel = value;
      return NTK_OK;
    case NTK_TUNE_REFINE_PREFETCH:
      if (value < 0 || value > 4) break;
      plan->tune_refine_prefetch = value;
      return NTK_OK;
    case NTK_TUNE_REFINE_TPS:
      if (value != 0 && value != 32 && value != 64) break;
      plan->tune_refine_tps = value;
      return NTK_OK;
    default:
      ntk::set_error("ntk_plan_set_tuning: unknown key %d", key);
      return NTK_ERR_INVALID;
  }
  ntk::set_error("ntk_plan_set_tuning: value %d out of range for key %d", value, key);
  return NTK_ERR_INVALID;
}

int ntk_plan_get_tuning(const ntk_plan* plan, int key, int* value) {
  if (!plan || !value) {
    ntk::set_error("ntk_plan_get_tuning: null argument");
    return NTK_ERR_INVALID;
  }
  switch (key) {
    case NTK_TUNE_F64_X_VARIANT: *value = plan->tune_f64_x_variant; return NTK_OK;
    case NTK_TUNE_F64_THREADS: *value = plan->tune_f64_threads; return NTK_OK;
    case NTK_TUNE_REFINE_W: *value = plan->tune_refine_w; return NTK_OK;
    case NTK_TUNE_REFINE_SPW: *value = plan->tune_refine_spw; return NTK_OK;
    case NTK_TUNE_REFINE_KERNEL: *value = plan->tune_refine_kernel; return NTK_OK;
    case NTK_TUNE_REFINE_PREFETCH: *value = plan->tune_refine_prefetch; return NTK_OK;
    case NTK_TUNE_REFINE_TPS: *value = plan->tune_refine_tps; return NTK_OK;
    default:
      ntk::set_error("ntk_plan_get_tuning: unknown key %d", key);
      return NTK_ERR_INVALID;
  }
}

int ntk_plan_status(ntk_plan* plan, int* flags, void* stream) {
  if (!plan) {
    ntk::set_error("ntk_plan_status: null plan");
    return NTK_ERR_INVALID;
  }
  std::vector<unsigned*> words;
  plan->status_words(words);
  return ntk::read_clear_status(words, (cudaStream_t)stream, flags);
}

int ntk_plan_destroy(ntk_plan* plan) {
  delete plan;
  return NTK_OK;
}

int ntk_solve(ntk_plan* plan, double* d, void* stream) {
  if (!plan || ntk::bad_ptr(d)) {
    ntk::set_error("ntk_solve: null plan or null/misaligned d");
    return NTK_ERR_INVALID;
  }
  Batch b;
  b.nsys = plan->nrhs;
  b.ni = plan->nrhs > 0 ? plan->nrhs : 1;
  b.is = plan->n;
  b.os = 0;
  b.es = 1;
  RhsParams rp;
  rp.kind = ntk::RHS_IDENTITY;
  return plan->run(d, d, b, rp, 1.0, (cudaStream_t)stream);
}

int ntk_solve_strided(ntk_plan* plan, const double* d_in, double* d_out, long long nsys, long long ni,
                      long long is, long long os, long long es, void* stream) {
  if (!plan || ntk::bad_ptr(d_in) || ntk::bad_ptr(d_out)) {
    ntk::set_error("ntk_solve_strided: null plan or null/misaligned pointer");
    return NTK_ERR_INVALID;
  }
  if (nsys < 0 || ni < 1 || es < 1 || is < 0 || os < 0) {
    ntk::set_error("ntk_solve_strided: bad layout (nsys=%lld ni=%lld is=%lld os=%lld es=%lld)", nsys, ni, is, os,
                   es);
    return NTK_ERR_INVALID;
  }
  Batch b;
  b.nsys = nsys;
  b.ni = ni;
  b.is = is;
  b.os = os;
  b.es = es;
  RhsParams rp;
  rp.kind = ntk::RHS_IDENTITY;
  return plan->run(d_in, d_out, b, rp, 1.0, (cudaStream_t)stream);
}

int ntk_compact_deriv(ntk_plan* plan, const double* f, double* out, int nz, int ny, int nx, int axis, double h,
                      void* stream) {
  if (!plan || ntk::bad_ptr(f) || ntk::bad_ptr(out)) {
    ntk::set_error("ntk_compact_deriv: null plan or null/misaligned pointer");
    return NTK_ERR_INVALID;
  }
  if (nz < 1 || ny < 1 || nx < 1 || axis < 0 || axis > 2 || !(h > 0) || !std::isfinite(h)) {
    ntk::set_error("ntk_compact_deriv: bad shape/axis/h");
    return NTK_ERR_INVALID;
  }
  const long long ext[3] = {nz, ny, nx};
  if (ext[axis] != plan->n) {
    ntk::set_error("ntk_compact_deriv: extent %lld of axis %d does not match the plan's n = %d", ext[axis], axis,
                   plan->n);
    return NTK_ERR_INVALID;
  }
  const long long total = (long long)nz * ny * nx;
  if (f != out && ((f < out + total) && (out < f + total))) {
    ntk::set_error("ntk_compact_deriv: out partially overlaps f");
    return NTK_ERR_INVALID;
  }
  Batch b;
  if (axis == 2) {
    b.nsys = (long long)nz * ny;
    b.ni = b.nsys;
    b.is = nx;
    b.os = 0;
    b.es = 1;
  } else if (axis == 1) {
    b.nsys = (long long)nz * nx;
    b.ni = nx;
    b.is = 1;
    b.os = (long long)nx * ny;
    b.es = nx;
  } else {
    b.nsys = (long long)ny * nx;
    b.ni = b.nsys;
    b.is = 1;
    b.os = 0;
    b.es = (long long)nx * ny;
  }
  // compact/rhs.py:21-36: interior scale 3/(4h), boundary rows 1/(2h) and -1/(2h)
  const double s = 3. / (4 * h);
  RhsParams rp;
  rp.kind = ntk::RHS_COMPACT;
  rp.sigma0 = (1. / (2 * h)) / s;
  rp.sigmaN = -(1. / (2 * h)) / s;
  return plan->run(f, out, b, rp, s, (cudaStream_t)stream);
}

int ntk_compact_grad(ntk_plan* plan, const double* f, double* dfdx, double* dfdy, double* dfdz, int nz, int ny,
                     int nx, double h, void* stream) {
  if (!plan || ntk::bad_ptr(f) || ntk::bad_ptr(dfdx) || ntk::bad_ptr(dfdy) || ntk::bad_ptr(dfdz)) {
    ntk::set_error("ntk_compact_grad: null plan or null/misaligned pointer");
    return NTK_ERR_INVALID;
  }
  if (nz != plan->n || ny != plan->n || nx != plan->n || !(h > 0) || !std::isfinite(h)) {
    ntk::set_error("ntk_compact_grad: the field must be n x n x n with the plan's n = %d, h > 0", plan->n);
    return NTK_ERR_INVALID;
  }
  const long long total = (long long)nz * ny * nx;
  const double* arr[4] = {f, dfdx, dfdy, dfdz};
  for (int i = 0; i < 4; ++i)
    for (int k = i + 1; k < 4; ++k)
      if (arr[i] < arr[k] + total && arr[k] < arr[i] + total) {
        ntk::set_error("ntk_compact_grad: f and the three outputs must not overlap");
        return NTK_ERR_INVALID;
      }
  const cudaStream_t st = (cudaStream_t)stream;
  if (plan->precision != NTK_FP64) {
    const int rc = plan->run_grad(f, dfdx, dfdy, dfdz, h, st);
    if (rc != NTK_ERR_UNSUPPORTED) return rc;
  }
  int rc = ntk_compact_deriv(plan, f, dfdx, nz, ny, nx, 2, h, stream);
  if (!rc) rc = ntk_compact_deriv(plan, f, dfdy, nz, ny, nx, 1, h, stream);
  if (!rc) rc = ntk_compact_deriv(plan, f, dfdz, nz, ny, nx, 0, h, stream);
  return rc;
}

int ntk_compact_rhs(const double* f, double* rhs, int nz, int ny, int nx, double dx, void* stream) {
  if (ntk::bad_ptr(f) || ntk::bad_ptr(rhs)) {
    ntk::set_error("ntk_compact_rhs: null/misaligned pointer");
    return NTK_ERR_INVALID;
  }
  return ntk::launch_compact_rhs(f, rhs, nz, ny, nx, dx, (cudaStream_t)stream);
}

int ntk_permute3d(const double* in, double* out, int o0, int o1, int o2, long long s0, long long s1, long long s2,
                  void* stream) {
  if (ntk::bad_ptr(in) || ntk::bad_ptr(out)) {
    ntk::set_error("ntk_permute3d: null/misaligned pointer");
    return NTK_ERR_INVALID;
  }
  return ntk::launch_permute3d(in, out, o0, o1, o2, s0, s1, s2, (cudaStream_t)stream);
}

int ntk_adi_rhs(const double* u, double* d, int N, double dx, double dt, void* stream) {
  if (ntk::bad_ptr(u) || ntk::bad_ptr(d)) {
    ntk::set_error("ntk_adi_rhs: null/misaligned pointer");
    return NTK_ERR_INVALID;
  }
  // adi/rhs.py:46-49
  const double bottom = -1. / (dx * dx);
  const double top = -1. / (dx * dx);
  const double center = 2 * (-1. / dt + 1. / (dx * dx));
  return ntk::launch_adi_rhs(u, d, N, bottom, center, top, (cudaStream_t)stream);
}

int ntk_transpose2d(const double* a, double* b, int N, void* stream) {
  if (ntk::bad_ptr(a) || ntk::bad_ptr(b)) {
    ntk::set_error("ntk_transpose2d: null/misaligned pointer");
    return NTK_ERR_INVALID;
  }
  return ntk::launch_transpose2d(a, b, N, (cudaStream_t)stream);
}

}  // extern "C"
