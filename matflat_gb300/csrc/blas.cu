// Single-matrix BLAS drop-ins in MatFlat's arithmetic:
//   Blas.SolveTriangular (MatFlat/Blas.SolveTriangular.cs:162-242),
//   Blas.MulMatMat       (MatFlat/Blas.MulMatMat.cs:226-368),
//   Factorization.LuInverse (MatFlat/Factorization.LuInverse.cs:123-199).
#include <cuda_runtime.h>

#include "mf_device.cuh"
#include "mf_kernels.h"
#include "mf_solve.cuh"

namespace mfg {

// One warp solves one triangular system.  x (stride incx) is staged into scratch, solved with
// the loop shape MatFlat uses for (uplo, trans), and written back.
__global__ void __launch_bounds__(32) trsv_single_kernel(int uplo, int trans, int n,
                                                         const double* a, int lda, double* x,
                                                         int incx, double* scratch) {
  const int lane = threadIdx.x & 31;
  const int ldx = n | 1;
  double* xs = scratch;
  double* acc = scratch + ldx;
  for (int i = lane; i < n; i += 32) xs[i] = x[(long long)i * incx];
  __syncwarp();
  const long long l = lda;
  if (uplo == 121) {         // Upper
    if (trans == 111) {      // NoTrans: column sweep over columns of U
      warp_solve_sweep(a, n, l, 1, xs, ldx, 1);
    } else {                 // Trans: dot form over columns of U
      warp_solve_dot(a, n, l, 1, false, xs, ldx, acc, 1);
    }
  } else {                   // Lower
    if (trans == 111) {      // NoTrans: dot form over rows of L
      warp_solve_dot(a, n, 1, l, false, xs, ldx, acc, 1);
    } else {                 // Trans: column sweep over rows of L
      warp_solve_sweep(a, n, 1, l, xs, ldx, 1);
    }
  }
  for (int i = lane; i < n; i += 32) x[(long long)i * incx] = xs[i];
}

// C = op(A) op(B): every element is one Internals.Dot of length k (Blas.MulMatMat.cs:306-367).
__global__ void gemm_single_kernel(int transa, int transb, int m, int n, int k, const double* a,
                                   int lda, const double* b, int ldb, double* c, int ldc) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)m * n) return;
  const int j = (int)(e / m);
  const int i = (int)(e - (long long)j * m);
  const double* x;
  long long incx;
  if (transa == 111) {
    x = a + i;
    incx = lda;
  } else {
    x = a + (long long)lda * i;
    incx = 1;
  }
  const double* y;
  long long incy;
  if (transb == 111) {
    y = b + (long long)ldb * j;
    incy = 1;
  } else {
    y = b + j;
    incy = ldb;
  }
  c[(long long)ldc * j + i] = exact_dot(k, x, incx, y, incy);
}

// LuInverse: work <- LU (leading dimension n); a <- the columns of P^T (a[piv[j], ...] pattern
// of LuInverse.cs:160-172); then every column is solved with the unit lower factor (the LuInverse
// idiom sets L's diagonal to 1.0, :174-182; dividing by 1.0 is exact, so the unit solve skips it)
// and then the upper factor (:184-192).  One CTA; warp w solves columns w, w+W, ... in chunks.
__global__ void getri_single_kernel(double* a, int n, int lda, const int* piv, double* work,
                                    double* scratch, long long scratch_stride) {
  const int tid = threadIdx.x;
  const int nthreads = blockDim.x;
  for (long long e = tid; e < (long long)n * n; e += nthreads) {
    const int j = (int)(e / n);
    const int i = (int)(e - (long long)j * n);
    work[e] = a[(long long)j * lda + i];
  }
  __syncthreads();
  for (long long e = tid; e < (long long)n * n; e += nthreads) {
    const int j = (int)(e / n);
    const int i = (int)(e - (long long)j * n);
    a[(long long)j * lda + i] = 0.0;
  }
  __syncthreads();
  for (int j = tid; j < n; j += nthreads) a[(long long)lda * piv[j] + j] = 1.0;
  __syncthreads();
  const int warp = tid >> 5;
  const int lane = tid & 31;
  const int nwarps = nthreads >> 5;
  const int ldx = n | 1;
  double* xs = scratch + warp * scratch_stride;
  double* acc = xs + RHS_CHUNK * ldx;
  for (int c0 = warp * RHS_CHUNK; c0 < n; c0 += nwarps * RHS_CHUNK) {
    const int nr = n - c0 < RHS_CHUNK ? n - c0 : RHS_CHUNK;
    for (int e = lane; e < nr * n; e += 32) {
      const int r = e / n;
      const int i = e - r * n;
      xs[r * ldx + i] = a[(long long)(c0 + r) * lda + i];
    }
    __syncwarp();
    warp_solve_dot(work, n, 1, n, true, xs, ldx, acc, nr);
    warp_solve_sweep(work, n, n, 1, xs, ldx, nr);
    for (int e = lane; e < nr * n; e += 32) {
      const int r = e / n;
      const int i = e - r * n;
      a[(long long)(c0 + r) * lda + i] = xs[r * ldx + i];
    }
    __syncwarp();
  }
}

__global__ void selftest_mul_kernel(const double* a, const double* b, double* out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = imul_rn(a[i], b[i]);
}

cudaError_t launch_selftest_mul(const double* a, const double* b, double* out, long long n,
                                cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  long long blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  selftest_mul_kernel<<<(unsigned)blocks, 256, 0, s>>>(a, b, out, n);
  return cudaGetLastError();
}

cudaError_t launch_trsv_single(int uplo, int trans, int n, const double* a, int lda, double* x,
                               int incx, double* scratch, cudaStream_t s) {
  trsv_single_kernel<<<1, 32, 0, s>>>(uplo, trans, n, a, lda, x, incx, scratch);
  return cudaGetLastError();
}

cudaError_t launch_gemm_single(int transa, int transb, int m, int n, int k, const double* a,
                               int lda, const double* b, int ldb, double* c, int ldc,
                               cudaStream_t s) {
  const long long total = (long long)m * n;
  const int threads = 128;
  const long long blocks = (total + threads - 1) / threads;
  gemm_single_kernel<<<(unsigned)blocks, threads, 0, s>>>(transa, transb, m, n, k, a, lda, b, ldb,
                                                          c, ldc);
  return cudaGetLastError();
}

cudaError_t launch_getri_single(double* a, int n, int lda, const int* piv, double* work,
                                double* scratch, int warps, cudaStream_t s) {
  const long long stride = 2LL * RHS_CHUNK * (n | 1);
  getri_single_kernel<<<1, warps * 32, 0, s>>>(a, n, lda, piv, work, scratch, stride);
  return cudaGetLastError();
}

}  // namespace mfg
