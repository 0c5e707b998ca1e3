// Batched vector building blocks of MatFlat's Blas class (strided batches of equal shapes):
// MulMatVec (Blas.MulMatVec.cs:138-236), Dot (Blas.VectorOperations.cs:143-174), L2Norm (:50-60)
// and Outer (:292-334), each in MatFlat's arithmetic: every dot is Internals.Dot's pairwise tree
// (Internals.cs:265-292), L2Norm the square root of that tree over x*x, Outer one product per entry
// (y_j * x_i).  They are the pieces the refinement residuals and the gradients are built from.
#include <cuda_runtime.h>

#include "mf_device.cuh"
#include "mf_kernels.h"

namespace mfg {

// One warp per matrix (grid-stride over the batch), one lane per output entry:
// NoTrans y_i = Dot(n, A(i,:), x); Trans y_j = Dot(m, A(:,j), x).
__global__ void gemv_strided_kernel(int trans, int m, int n, const double* a, int lda,
                                    long long sa, const double* x, int incx, long long sx,
                                    double* y, int incy, long long sy, int count) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  const int outs = trans == 111 ? m : n;
  for (long long b = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); b < count;
       b += warps) {
    const double* ab = a + b * sa;
    const double* xb = x + b * sx;
    double* yb = y + b * sy;
    for (int o = lane; o < outs; o += 32) {
      const double v = trans == 111 ? exact_dot<1>(n, ab + o, lda, xb, incx)
                                    : exact_dot<1>(m, ab + (long long)o * lda, 1, xb, incx);
      yb[(long long)o * incy] = v;
    }
  }
}

// One thread per vector pair: out[b] = Dot(n, x_b, y_b), or sqrt(Dot(n, x_b, x_b)) for norms.
__global__ void dot_strided_kernel(int n, const double* x, int incx, long long sx, const double* y,
                                   int incy, long long sy, double* out, int count, int norm) {
  for (long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x; b < count;
       b += (long long)gridDim.x * blockDim.x) {
    const double* xb = x + b * sx;
    const double s = norm ? exact_dot<1>(n, xb, incx, xb, incx)
                          : exact_dot<1>(n, xb, incx, y + b * sy, incy);
    out[b] = norm ? __dsqrt_rn(s) : s;
  }
}

// One thread per entry: a_b(i,j) = y_b[j] * x_b[i].
__global__ void ger_strided_kernel(int m, int n, const double* x, int incx, long long sx,
                                   const double* y, int incy, long long sy, double* a, int lda,
                                   long long sa, int count) {
  const long long per = (long long)m * n;
  const long long total = per * count;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / per;
    const long long r = e - b * per;
    const int j = (int)(r / m);
    const int i = (int)(r - (long long)j * m);
    a[b * sa + (long long)j * lda + i] =
        __dmul_rn(y[b * sy + (long long)j * incy], x[b * sx + (long long)i * incx]);
  }
}

static unsigned grid_for(long long items, int per_block) {
  long long g = (items + per_block - 1) / per_block;
  if (g < 1) g = 1;
  if (g > 65535) g = 65535;
  return (unsigned)g;
}

cudaError_t launch_gemv_strided(int trans, int m, int n, const double* a, int lda, long long sa,
                                const double* x, int incx, long long sx, double* y, int incy,
                                long long sy, int count, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  gemv_strided_kernel<<<grid_for(count, 8), 256, 0, s>>>(trans, m, n, a, lda, sa, x, incx, sx, y,
                                                          incy, sy, count);
  return cudaGetLastError();
}

cudaError_t launch_dot_strided(int n, const double* x, int incx, long long sx, const double* y,
                               int incy, long long sy, double* out, int count, int norm,
                               cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  dot_strided_kernel<<<grid_for(count, 128), 128, 0, s>>>(n, x, incx, sx, y, incy, sy, out, count,
                                                          norm);
  return cudaGetLastError();
}

cudaError_t launch_ger_strided(int m, int n, const double* x, int incx, long long sx,
                               const double* y, int incy, long long sy, double* a, int lda,
                               long long sa, int count, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  ger_strided_kernel<<<grid_for((long long)m * n * count, 256), 256, 0, s>>>(
      m, n, x, incx, sx, y, incy, sy, a, lda, sa, count);
  return cudaGetLastError();
}

}  // namespace mfg
