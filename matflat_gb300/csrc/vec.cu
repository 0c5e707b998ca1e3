// Batched vector building blocks of MatFlat's Blas class (strided batches of equal shapes):
// MulMatVec (Blas.MulMatVec.cs:138-236), Dot (Blas.VectorOperations.cs:143-174), L2Norm (:50-60)
// and Outer (:292-334), each in MatFlat's arithmetic: every dot is Internals.Dot's pairwise tree
// (Internals.cs:265-292), L2Norm the square root of that tree over x*x, Outer one product per entry
// (y_j * x_i).  They are the pieces the refinement residuals and the gradients are built from.
#include <cuda_runtime.h>

#include "mf_device.cuh"
#include "mf_kernels.h"
#include "mf_scalar.cuh"

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

// ---- The float and Complex overloads --------------------------------------------------------
// Float: dots and norms summed in double by Internals.Dot's tree over widened operands, the result
// cast to float (Blas.MulMatVec.cs:38-136, Blas.VectorOperations.cs:23-48, :110-141); Outer one
// float product per entry (:248-290).  Complex: Internals.Dot / DotConj (Internals.cs:294-379)
// for MulMatVec (:238-336, the Conj modes use DotConj) and Dot / DotConj (:176-246); L2Norm the
// square root of sum |x_i|^2 in Internals.Norm's order (Internals.cs:489-541), a double; Outer
// y_j * x_i and OuterConj conj(y_j) * x_i (:336-420).

// Internals.Norm over Complex, strided: an odd length seeds with |x_0|^2 = re^2 + im^2, then
// every pair adds ((re0^2 + im0^2) + re1^2) + im1^2.
__device__ __forceinline__ double znorm2(int len, const zdouble* x, long long inc) {
  double s = 0.0;
  if (len & 1) {
    s = __dadd_rn(__dmul_rn(x[0].re, x[0].re), __dmul_rn(x[0].im, x[0].im));
    x += inc;
  }
  for (int p = 0; p < (len >> 1); ++p) {
    const zdouble a = x[0], b = x[inc];
    double t = __dadd_rn(__dmul_rn(a.re, a.re), __dmul_rn(a.im, a.im));
    t = __dadd_rn(t, __dmul_rn(b.re, b.re));
    t = __dadd_rn(t, __dmul_rn(b.im, b.im));
    s = __dadd_rn(s, t);
    x += 2 * inc;
  }
  return __dsqrt_rn(s);
}

__global__ void sgemv_strided_kernel(int trans, int m, int n, const float* a, int lda,
                                     long long sa, const float* x, int incx, long long sx,
                                     float* y, int incy, long long sy, int count) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  const int outs = trans == 111 ? m : n;
  for (long long b = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); b < count;
       b += warps) {
    const float* ab = a + b * sa;
    const float* xb = x + b * sx;
    for (int o = lane; o < outs; o += 32) {
      const double v = trans == 111 ? exact_dot_f(n, ab + o, lda, xb, incx)
                                    : exact_dot_f(m, ab + (long long)o * lda, 1, xb, incx);
      y[b * sy + (long long)o * incy] = __double2float_rn(v);
    }
  }
}

__global__ void zgemv_strided_kernel(int trans, int m, int n, const zdouble* a, int lda,
                                     long long sa, const zdouble* x, int incx, long long sx,
                                     zdouble* y, int incy, long long sy, int count) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  const bool rows = trans == 111 || trans == 114;   // NoTrans, ConjNoTrans: dots over rows
  const bool conj = trans == 113 || trans == 114;
  const int outs = rows ? m : n;
  for (long long b = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); b < count;
       b += warps) {
    const zdouble* ab = a + b * sa;
    const zdouble* xb = x + b * sx;
    for (int o = lane; o < outs; o += 32) {
      const zdouble* ao = rows ? ab + o : ab + (long long)o * lda;
      const int len = rows ? n : m;
      const long long inc = rows ? lda : 1;
      y[b * sy + (long long)o * incy] =
          conj ? zdot<true>(len, ao, inc, xb, incx) : zdot<false>(len, ao, inc, xb, incx);
    }
  }
}

// One thread per vector (pair).  mode: 0 dot, 1 norm, 2 DotConj (Complex).
__global__ void sdot_strided_kernel(int n, const float* x, int incx, long long sx, const float* y,
                                    int incy, long long sy, float* out, int count, int norm) {
  for (long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x; b < count;
       b += (long long)gridDim.x * blockDim.x) {
    const float* xb = x + b * sx;
    const double s = norm ? exact_dot_f(n, xb, incx, xb, incx)
                          : exact_dot_f(n, xb, incx, y + b * sy, incy);
    out[b] = __double2float_rn(norm ? __dsqrt_rn(s) : s);
  }
}

__global__ void zdot_strided_kernel(int n, const zdouble* x, int incx, long long sx,
                                    const zdouble* y, int incy, long long sy, void* out,
                                    int count, int mode) {
  for (long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x; b < count;
       b += (long long)gridDim.x * blockDim.x) {
    const zdouble* xb = x + b * sx;
    if (mode == 1) {
      ((double*)out)[b] = znorm2(n, xb, incx);
    } else {
      const zdouble* yb = y + b * sy;
      ((zdouble*)out)[b] = mode == 2 ? zdot<true>(n, xb, incx, yb, incy)
                                     : zdot<false>(n, xb, incx, yb, incy);
    }
  }
}

__global__ void sger_strided_kernel(int m, int n, const float* x, int incx, long long sx,
                                    const float* y, int incy, long long sy, float* a, int lda,
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
        __fmul_rn(y[b * sy + (long long)j * incy], x[b * sx + (long long)i * incx]);
  }
}

__global__ void zger_strided_kernel(int m, int n, const zdouble* x, int incx, long long sx,
                                    const zdouble* y, int incy, long long sy, zdouble* a, int lda,
                                    long long sa, int count, int conj) {
  const long long per = (long long)m * n;
  const long long total = per * count;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / per;
    const long long r = e - b * per;
    const int j = (int)(r / m);
    const int i = (int)(r - (long long)j * m);
    const zdouble yj = y[b * sy + (long long)j * incy];
    a[b * sa + (long long)j * lda + i] = zmul(conj ? zconj(yj) : yj, x[b * sx + (long long)i * incx]);
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

cudaError_t launch_gemv_strided_t(int elem, int trans, int m, int n, const void* a, int lda,
                                  long long sa, const void* x, int incx, long long sx, void* y,
                                  int incy, long long sy, int count, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  if (elem == 1)
    sgemv_strided_kernel<<<grid_for(count, 8), 256, 0, s>>>(trans, m, n, (const float*)a, lda, sa,
                                                             (const float*)x, incx, sx, (float*)y,
                                                             incy, sy, count);
  else
    zgemv_strided_kernel<<<grid_for(count, 8), 256, 0, s>>>(
        trans, m, n, (const zdouble*)a, lda, sa, (const zdouble*)x, incx, sx, (zdouble*)y, incy,
        sy, count);
  return cudaGetLastError();
}

cudaError_t launch_dot_strided_t(int elem, int n, const void* x, int incx, long long sx,
                                 const void* y, int incy, long long sy, void* out, int count,
                                 int mode, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  if (elem == 1)
    sdot_strided_kernel<<<grid_for(count, 128), 128, 0, s>>>(n, (const float*)x, incx, sx,
                                                             (const float*)y, incy, sy,
                                                             (float*)out, count, mode == 1);
  else
    zdot_strided_kernel<<<grid_for(count, 128), 128, 0, s>>>(n, (const zdouble*)x, incx, sx,
                                                             (const zdouble*)y, incy, sy, out,
                                                             count, mode);
  return cudaGetLastError();
}

cudaError_t launch_ger_strided_t(int elem, int m, int n, const void* x, int incx, long long sx,
                                 const void* y, int incy, long long sy, void* a, int lda,
                                 long long sa, int count, int conj, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  const unsigned g = grid_for((long long)m * n * count, 256);
  if (elem == 1)
    sger_strided_kernel<<<g, 256, 0, s>>>(m, n, (const float*)x, incx, sx, (const float*)y, incy,
                                          sy, (float*)a, lda, sa, count);
  else
    zger_strided_kernel<<<g, 256, 0, s>>>(m, n, (const zdouble*)x, incx, sx, (const zdouble*)y,
                                          incy, sy, (zdouble*)a, lda, sa, count, conj);
  return cudaGetLastError();
}

}  // namespace mfg
