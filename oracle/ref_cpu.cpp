// ref_cpu.cpp -- the reference's own CUDA kernels executed on the CPU.
//
// TEST INFRASTRUCTURE ONLY (parity checker).  Includes the kernels rendered
// by oracle/render_ref.py from the reference's source strings and runs them
// under a small emulation of the CUDA execution model: one OS thread per
// CUDA thread of a block, blocks run one after another, __shared__ arrays
// are function statics shared by the block's threads, __syncthreads() is a
// barrier.  Built with -ffp-contract=off so that no multiply-add is fused:
// the results are what the reference's arithmetic gives in strict IEEE
// double precision, and the golden vectors in tests/golden/ come from here.
//
// The launch shapes follow the reference's launch sites:
//   ntkref_cpu_cr            neato.py:181-197   grid nrhs, block n/2
//   ntkref_cpu_compact_rhs   compact/rhs.py:47-53  grid (nx/8, ny/8, nz/8), block 8^3
//   ntkref_cpu_permute       compact/permute.py:32-52
//   ntkref_cpu_adi_rhs       adi/rhs.py:35-55   grid (N/32, N/32), block 32x32
//   ntkref_cpu_transpose     adi/transpose.py:40-50 grid (N/32, N/32), block 32x32
#include <cmath>
#include <pthread.h>
#include <vector>

struct ntk_dim3 {
  unsigned x, y, z;
};
static thread_local ntk_dim3 threadIdx;
static ntk_dim3 blockIdx, blockDim, gridDim;
static pthread_barrier_t g_bar;
static inline void ntk_cpu_syncthreads() { pthread_barrier_wait(&g_bar); }

#define __global__ static
#define __shared__ static
#define __syncthreads() ntk_cpu_syncthreads()

#include "_ref/ref_kernels.cuh"

#undef __global__
#undef __shared__
#undef __syncthreads

namespace {

template <class Body>
struct Team {
  Body body;
  unsigned nthreads;
};

template <class Body>
struct ThreadArg {
  Team<Body>* team;
  unsigned tid;
};

// Runs `body()` for every block of the grid with one OS thread per CUDA
// thread.  Thread 0 advances blockIdx between two barriers.
template <class Body>
void* team_main(void* p) {
  ThreadArg<Body>* a = static_cast<ThreadArg<Body>*>(p);
  unsigned t = a->tid;
  threadIdx.x = t % blockDim.x;
  threadIdx.y = (t / blockDim.x) % blockDim.y;
  threadIdx.z = t / (blockDim.x * blockDim.y);
  for (unsigned bz = 0; bz < gridDim.z; ++bz)
    for (unsigned by = 0; by < gridDim.y; ++by)
      for (unsigned bx = 0; bx < gridDim.x; ++bx) {
        if (t == 0) blockIdx = ntk_dim3{bx, by, bz};
        pthread_barrier_wait(&g_bar);
        a->team->body();
        pthread_barrier_wait(&g_bar);
      }
  return nullptr;
}

template <class Body>
int launch(ntk_dim3 grid, ntk_dim3 block, Body body) {
  gridDim = grid;
  blockDim = block;
  unsigned nt = block.x * block.y * block.z;
  if (nt == 0 || grid.x == 0 || grid.y == 0 || grid.z == 0) return 0;
  Team<Body> team{body, nt};
  std::vector<pthread_t> th(nt);
  std::vector<ThreadArg<Body>> args(nt);
  if (pthread_barrier_init(&g_bar, nullptr, nt)) return -3;
  pthread_attr_t attr;
  pthread_attr_init(&attr);
  pthread_attr_setstacksize(&attr, 1 << 18);
  unsigned started = 0;
  int rc = 0;
  for (unsigned t = 0; t < nt; ++t) {
    args[t] = ThreadArg<Body>{&team, t};
    if (pthread_create(&th[t], &attr, &team_main<Body>, &args[t])) { rc = -4; break; }
    ++started;
  }
  pthread_attr_destroy(&attr);
  if (rc) {
    // a partial team would wait forever at the barrier; this only happens
    // when the OS refuses threads, before any block ran
    for (unsigned t = 0; t < started; ++t) pthread_cancel(th[t]);
  }
  for (unsigned t = 0; t < started; ++t) pthread_join(th[t], nullptr);
  pthread_barrier_destroy(&g_bar);
  return rc;
}

}  // namespace

extern "C" {

int ntkref_cpu_cr(int n, long nrhs, const double* a, const double* b, const double* c, const double* k1,
                  const double* k2, const double* b_first, const double* k1_first, const double* k1_last,
                  double b1, double c1, double ai, double bi, double ci, double* d) {
  double* A = const_cast<double*>(a);
  double* B = const_cast<double*>(b);
  double* C = const_cast<double*>(c);
  double* K1 = const_cast<double*>(k1);
  double* K2 = const_cast<double*>(k2);
  double* BF = const_cast<double*>(b_first);
  double* K1F = const_cast<double*>(k1_first);
  double* K1L = const_cast<double*>(k1_last);
  ntk_dim3 grid{(unsigned)nrhs, 1, 1}, block{(unsigned)(n / 2), 1, 1};
#define NTKREF_CASE(N)                                                                                   \
  if (n == N)                                                                                            \
    return launch(grid, block, [=] {                                                                     \
      ntkref_cr_n##N::sharedMemCyclicReduction(A, B, C, d, K1, K2, BF, K1F, K1L, b1, c1, ai, bi, ci);    \
    });
  NTKREF_CR_SIZES(NTKREF_CASE)
#undef NTKREF_CASE
  return -1;
}

int ntkref_cpu_compact_rhs(const double* f, double* rhs, int nz, int ny, int nx, double dx) {
  if (nx % 8 || ny % 8 || nz % 8) return -1;
  return launch(ntk_dim3{(unsigned)nx / 8, (unsigned)ny / 8, (unsigned)nz / 8}, ntk_dim3{8, 8, 8},
                [=] { ntkref_rhs::computeRHS(f, rhs, dx); });
}

// b has shape (b0, b1, b2); s0, s1, s2 are the input strides in elements
// taken in the order of the permutation (compact/permute.py:45-46).
int ntkref_cpu_permute(const double* in, double* out, int b0, int b1, int b2, int s0, int s1, int s2) {
  if (b0 % 8 || b1 % 8 || b2 % 8) return -1;
  double* I = const_cast<double*>(in);
  return launch(ntk_dim3{(unsigned)b2 / 8, (unsigned)b1 / 8, (unsigned)b0 / 8}, ntk_dim3{8, 8, 8},
                [=] { ntkref_permute::permuteKernel(I, out, b2, b1, b0, s2, s1, s0); });
}

int ntkref_cpu_adi_rhs(const double* u, double* d, int N, double dx, double dt) {
  if (N % 32) return -1;
  // adi/rhs.py:46-49
  double bottom = -1. / (dx * dx);
  double top = -1. / (dx * dx);
  double center = 2 * (-1. / dt + 1. / (dx * dx));
  return launch(ntk_dim3{(unsigned)N / 32, (unsigned)N / 32, 1}, ntk_dim3{32, 32, 1},
                [=] { ntkref_adi_rhs::applyVerticalStencil(u, d, bottom, center, top, N); });
}

int ntkref_cpu_transpose(const double* a, double* b, int N) {
  if (N % 32) return -1;
  return launch(ntk_dim3{(unsigned)N / 32, (unsigned)N / 32, 1}, ntk_dim3{32, 32, 1},
                [=] { ntkref_transpose::transposeCoalesced(b, a); });
}

}  // extern "C"
