// ntk_ops.cu -- the reference's stand-alone data-parallel operators.
//
//   compact_rhs  <- compact/rhs.py:9-37,47-53   (computeRHS)
//   permute3d    <- compact/permute.py:7-20,32-52 (permuteKernel)
//   adi_rhs      <- adi/rhs.py:10-25,35-55       (applyVerticalStencil)
//   transpose2d  <- adi/transpose.py:9-27,40-50  (transposeCoalesced)
//
// The fused solves (ntk_solve_f64.cu, ntk_refine.cu) make these passes
// unnecessary on the hot path; they are kept for drop-in use of the
// reference's free functions.  Arithmetic uses the _rn intrinsics so no
// multiply-add is contracted: results are bit-identical to the reference's
// arithmetic in strict IEEE double precision (the CPU oracle).  All are
// HBM-bound; they read 8 B and write 8 B per element with coalesced access,
// permute and transpose through 32x33 shared-memory tiles.
#include "ntk_device.cuh"
#include "ntk_internal.h"

namespace ntk {
namespace {

// rhs along the last (contiguous) axis of an [nz][ny][nx] field; one thread
// per element, grid-stride loop.
__global__ void compact_rhs_kernel(const double* __restrict__ f, double* __restrict__ rhs, long long total,
                                   int nx, double c34, double c12) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
    const int tix = (int)(i % nx);
    double r;
    if (tix == 0) {
      r = __dmul_rn(c12, __dadd_rn(__dadd_rn(__dmul_rn(-5.0, f[i]), __dmul_rn(4.0, f[i + 1])), f[i + 2]));
    } else if (tix == nx - 1) {
      r = -__dmul_rn(c12, __dadd_rn(__dadd_rn(__dmul_rn(-5.0, f[i]), __dmul_rn(4.0, f[i - 1])), f[i - 2]));
    } else {
      r = __dmul_rn(c34, __dsub_rn(f[i + 1], f[i - 1]));
    }
    rhs[i] = r;
  }
}

// out[i0][i1][i2] = in[i0*s0 + i1*s1 + i2*s2]; tiles over (i2, ia) where ia
// is the output axis whose input stride is 1, so both the gather and the
// store are coalesced.
template <int TRANSPOSED>
__global__ void permute_kernel(const double* __restrict__ in, double* __restrict__ out, int o0, int o1, int o2,
                               long long s0, long long s1, long long s2) {
  __shared__ double tile[32][33];
  if constexpr (TRANSPOSED == 0) {
    // s2 == 1 (or no unit stride): straight row gather
    const long long total = (long long)o0 * o1 * o2;
    const long long stride = (long long)gridDim.x * blockDim.x * blockDim.y;
    for (long long e = ((long long)blockIdx.x * blockDim.y + threadIdx.y) * blockDim.x + threadIdx.x; e < total;
         e += stride) {
      const int i2 = (int)(e % o2);
      const long long r = e / o2;
      const int i1 = (int)(r % o1);
      const int i0 = (int)(r / o1);
      out[e] = in[i0 * s0 + i1 * s1 + (long long)i2 * s2];
    }
  } else {
    // TRANSPOSED == 1: axis 1 has unit input stride; TRANSPOSED == 2: axis 0
    // blockIdx.x tiles i2, blockIdx.y tiles ia, blockIdx.z the remaining axis
    const int na = (TRANSPOSED == 1) ? o1 : o0;
    const long long sa = (TRANSPOSED == 1) ? s1 : s0;  // == 1
    const long long sb = (TRANSPOSED == 1) ? s0 : s1;
    const int i2b = blockIdx.x * 32;
    const int iab = blockIdx.y * 32;
    const int ib = blockIdx.z;
    // load: threads along ia (unit input stride)
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
      const int i2 = i2b + j;
      const int ia = iab + threadIdx.x;
      if (i2 < o2 && ia < na) tile[j][threadIdx.x] = in[(long long)ib * sb + (long long)ia * sa + (long long)i2 * s2];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
      const int ia = iab + j;
      const int i2 = i2b + threadIdx.x;
      if (i2 < o2 && ia < na) {
        long long o;
        if (TRANSPOSED == 1)
          o = ((long long)ib * o1 + ia) * o2 + i2;
        else
          o = ((long long)ia * o1 + ib) * o2 + i2;
        out[o] = tile[threadIdx.x][j];
      }
    }
  }
}

__global__ void adi_rhs_kernel(const double* __restrict__ u, double* __restrict__ d, int N, double bottom,
                               double center, double top) {
  const int tix = blockIdx.x * blockDim.x + threadIdx.x;
  const int tiy = blockIdx.y * blockDim.y + threadIdx.y;
  if (tix > 0 && tix < N - 1 && tiy > 0 && tiy < N - 1) {
    const long long i = (long long)tiy * N + tix;
    d[i] = __dadd_rn(__dadd_rn(__dmul_rn(bottom, u[i - N]), __dmul_rn(center, u[i])), __dmul_rn(top, u[i + N]));
  }
}

__global__ void transpose_kernel(const double* __restrict__ a, double* __restrict__ b, int N) {
  __shared__ double tile[32][33];
  const int x = blockIdx.x * 32 + threadIdx.x;
  const int y0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y)
    if (x < N && y0 + j < N) tile[j][threadIdx.x] = a[(long long)(y0 + j) * N + x];
  __syncthreads();
  const int xo = blockIdx.y * 32 + threadIdx.x;
  const int yo0 = blockIdx.x * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y)
    if (xo < N && yo0 + j < N) b[(long long)(yo0 + j) * N + xo] = tile[threadIdx.x][j];
}

int grid_for(long long total, int threads) {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long want = (total + threads - 1) / threads;
  long long cap = (long long)sms * 16;
  return (int)(want < cap ? (want > 0 ? want : 1) : cap);
}

}  // namespace

int launch_compact_rhs(const double* f, double* rhs, int nz, int ny, int nx, double dx, cudaStream_t s) {
  if (nx < 3 || ny < 1 || nz < 1) {
    set_error("compact_rhs: need nx >= 3 (got nz=%d ny=%d nx=%d)", nz, ny, nx);
    return NTK_ERR_INVALID;
  }
  const long long total = (long long)nz * ny * nx;
  const double c34 = 3. / (4 * dx);
  const double c12 = 1. / (2 * dx);
  compact_rhs_kernel<<<grid_for(total, 256), 256, 0, s>>>(f, rhs, total, nx, c34, c12);
  return cuda_status(cudaGetLastError(), "compact_rhs_kernel");
}

int launch_permute3d(const double* in, double* out, int o0, int o1, int o2, long long s0, long long s1,
                     long long s2, cudaStream_t s) {
  if (o0 < 1 || o1 < 1 || o2 < 1) {
    set_error("permute3d: bad shape");
    return NTK_ERR_INVALID;
  }
  if (s2 != 1 && (s1 == 1 || s0 == 1)) {
    dim3 block(32, 8);
    if (s1 == 1) {
      dim3 grid((o2 + 31) / 32, (o1 + 31) / 32, o0);
      permute_kernel<1><<<grid, block, 0, s>>>(in, out, o0, o1, o2, s0, s1, s2);
    } else {
      dim3 grid((o2 + 31) / 32, (o0 + 31) / 32, o1);
      permute_kernel<2><<<grid, block, 0, s>>>(in, out, o0, o1, o2, s0, s1, s2);
    }
  } else {
    const long long total = (long long)o0 * o1 * o2;
    permute_kernel<0><<<grid_for(total, 256), dim3(32, 8), 0, s>>>(in, out, o0, o1, o2, s0, s1, s2);
  }
  return cuda_status(cudaGetLastError(), "permute_kernel");
}

int launch_adi_rhs(const double* u, double* d, int N, double bottom, double center, double top, cudaStream_t s) {
  if (N < 3) {
    set_error("adi_rhs: need N >= 3");
    return NTK_ERR_INVALID;
  }
  dim3 block(32, 8), grid((N + 31) / 32, (N + 7) / 8);
  adi_rhs_kernel<<<grid, block, 0, s>>>(u, d, N, bottom, center, top);
  return cuda_status(cudaGetLastError(), "adi_rhs_kernel");
}

int launch_transpose2d(const double* a, double* b, int N, cudaStream_t s) {
  if (N < 1) {
    set_error("transpose2d: need N >= 1");
    return NTK_ERR_INVALID;
  }
  dim3 block(32, 8), grid((N + 31) / 32, (N + 31) / 32);
  transpose_kernel<<<grid, block, 0, s>>>(a, b, N);
  return cuda_status(cudaGetLastError(), "transpose_kernel");
}

}  // namespace ntk
