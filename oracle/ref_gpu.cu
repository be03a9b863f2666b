// ref_gpu.cu -- the reference's own CUDA kernels, compiled for this GPU.
//
// TEST INFRASTRUCTURE ONLY (parity checker and the reference timing arm).
// Includes the kernels rendered by oracle/render_ref.py from the reference's
// source strings and launches them with the reference's grid and block
// shapes, on the stream passed in (the reference uses the default stream):
//   ntkref_gpu_cr            neato.py:181-197      grid nrhs, block n/2
//   ntkref_gpu_compact_rhs   compact/rhs.py:47-53  grid (nx/8, ny/8, nz/8), block 8^3
//   ntkref_gpu_permute       compact/permute.py:32-52
//   ntkref_gpu_adi_rhs       adi/rhs.py:35-55      grid (N/32, N/32), block 32x32
//   ntkref_gpu_transpose     adi/transpose.py:40-50
// The reference compiles with PyCUDA's SourceModule(options=['-O2']); this
// file is compiled by nvcc -O2 for sm_103a.
#include <cuda_runtime.h>

#include "_ref/ref_kernels.cuh"

extern "C" {

int ntkref_gpu_cr(int n, long nrhs, const double* a, const double* b, const double* c, const double* k1,
                  const double* k2, const double* b_first, const double* k1_first, const double* k1_last,
                  double b1, double c1, double ai, double bi, double ci, double* d, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (nrhs <= 0) return 0;
  dim3 grid((unsigned)nrhs), block((unsigned)(n / 2));
#define NTKREF_CASE(N)                                                                                       \
  if (n == N) {                                                                                              \
    ntkref_cr_n##N::sharedMemCyclicReduction<<<grid, block, 0, s>>>(                                         \
        (double*)a, (double*)b, (double*)c, d, (double*)k1, (double*)k2, (double*)b_first, (double*)k1_first, \
        (double*)k1_last, b1, c1, ai, bi, ci);                                                               \
    return (int)cudaGetLastError();                                                                          \
  }
  NTKREF_CR_SIZES(NTKREF_CASE)
#undef NTKREF_CASE
  return -1;
}

int ntkref_gpu_compact_rhs(const double* f, double* rhs, int nz, int ny, int nx, double dx, void* stream) {
  if (nx % 8 || ny % 8 || nz % 8) return -1;
  ntkref_rhs::computeRHS<<<dim3(nx / 8, ny / 8, nz / 8), dim3(8, 8, 8), 0, (cudaStream_t)stream>>>(f, rhs, dx);
  return (int)cudaGetLastError();
}

int ntkref_gpu_permute(const double* in, double* out, int b0, int b1, int b2, int s0, int s1, int s2,
                       void* stream) {
  if (b0 % 8 || b1 % 8 || b2 % 8) return -1;
  ntkref_permute::permuteKernel<<<dim3(b2 / 8, b1 / 8, b0 / 8), dim3(8, 8, 8), 0, (cudaStream_t)stream>>>(
      (double*)in, out, b2, b1, b0, s2, s1, s0);
  return (int)cudaGetLastError();
}

int ntkref_gpu_adi_rhs(const double* u, double* d, int N, double dx, double dt, void* stream) {
  if (N % 32) return -1;
  double bottom = -1. / (dx * dx);  // adi/rhs.py:46-49
  double top = -1. / (dx * dx);
  double center = 2 * (-1. / dt + 1. / (dx * dx));
  ntkref_adi_rhs::applyVerticalStencil<<<dim3(N / 32, N / 32, 1), dim3(32, 32, 1), 0, (cudaStream_t)stream>>>(
      u, d, bottom, center, top, N);
  return (int)cudaGetLastError();
}

int ntkref_gpu_transpose(const double* a, double* b, int N, void* stream) {
  if (N % 32) return -1;
  ntkref_transpose::transposeCoalesced<<<dim3(N / 32, N / 32, 1), dim3(32, 32, 1), 0, (cudaStream_t)stream>>>(
      b, a);
  return (int)cudaGetLastError();
}

}  // extern "C"
