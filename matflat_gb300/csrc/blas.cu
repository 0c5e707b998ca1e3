// Single-matrix BLAS drop-ins in MatFlat's arithmetic:
//   Blas.SolveTriangular (MatFlat/Blas.SolveTriangular.cs:162-242),
//   Blas.MulMatMat       (MatFlat/Blas.MulMatMat.cs:226-368),
//   Factorization.LuInverse (MatFlat/Factorization.LuInverse.cs:123-199).
#include <cuda_runtime.h>

#include "mf_device.cuh"
#include "mf_kernels.h"
#include "mf_scalar.cuh"
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
// idiom sets L's diagonal to 1.0, :174-182; dividing by 1.0 is exact for double and float, so the
// unit solve skips it, and done as a division for Complex) and then the upper factor (:184-192).
// One CTA; warp w solves columns w, w+W, ... in chunks.  S: the element type's solve arithmetic
// (DSolve, SSolve or ZSolve<false>: the double, float and Complex overloads).
template <class S>
__device__ __forceinline__ typename S::T elem_of(double v);
template <>
__device__ __forceinline__ double elem_of<DSolve>(double v) { return v; }
template <>
__device__ __forceinline__ float elem_of<SSolve>(double v) { return (float)v; }
template <>
__device__ __forceinline__ zdouble elem_of<ZSolve<false>>(double v) { return zmake(v, 0.0); }

template <class S>
__global__ void getri_single_kernel(typename S::T* a, int n, int lda, const int* piv,
                                    typename S::T* work, void* scratch,
                                    long long scratch_bytes) {
  using T = typename S::T;
  using Acc = typename S::Acc;
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
    a[(long long)j * lda + i] = elem_of<S>(0.0);
  }
  __syncthreads();
  for (int j = tid; j < n; j += nthreads) a[(long long)lda * piv[j] + j] = elem_of<S>(1.0);
  __syncthreads();
  const int warp = tid >> 5;
  const int lane = tid & 31;
  const int nwarps = nthreads >> 5;
  const int ldx = n | 1;
  Acc* acc = (Acc*)((char*)scratch + warp * scratch_bytes);
  T* xs = (T*)(acc + RHS_CHUNK * ldx);
  for (int c0 = warp * RHS_CHUNK; c0 < n; c0 += nwarps * RHS_CHUNK) {
    const int nr = n - c0 < RHS_CHUNK ? n - c0 : RHS_CHUNK;
    for (int e = lane; e < nr * n; e += 32) {
      const int r = e / n;
      const int i = e - r * n;
      xs[r * ldx + i] = a[(long long)(c0 + r) * lda + i];
    }
    __syncwarp();
    warp_solve_dot<32, S>(work, n, 1, n, true, xs, ldx, acc, nr);
    warp_solve_sweep<32, S>(work, n, n, 1, xs, ldx, nr);
    for (int e = lane; e < nr * n; e += 32) {
      const int r = e / n;
      const int i = e - r * n;
      a[(long long)(c0 + r) * lda + i] = xs[r * ldx + i];
    }
    __syncwarp();
  }
}

// Both variants of the integer-pipe product must agree bit for bit; a disagreement is reported
// as a NaN in the output, which the IEEE comparison then flags.
__global__ void selftest_mul_kernel(const double* a, const double* b, double* out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double r0 = imul_rn<false>(a[i], b[i]);
    const double r1 = imul_rn<true>(a[i], b[i]);
    out[i] = dbits(r0) == dbits(r1) ? r0 : __longlong_as_double(0x7FF8DEAD0000DEADll);
  }
}

cudaError_t launch_selftest_mul(const double* a, const double* b, double* out, long long n,
                                cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  long long blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  selftest_mul_kernel<<<(unsigned)blocks, 256, 0, s>>>(a, b, out, n);
  return cudaGetLastError();
}

// The integer-pipe quotient with its per-divisor reciprocal, as the factorizations use it.
__global__ void selftest_div_kernel(const double* a, const double* b, double* out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double d = b[i];
    out[i] = idiv_rn(a[i], d, __drcp_rn(d));
  }
}

cudaError_t launch_selftest_div(const double* a, const double* b, double* out, long long n,
                                cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  long long blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  selftest_div_kernel<<<(unsigned)blocks, 256, 0, s>>>(a, b, out, n);
  return cudaGetLastError();
}

// Float and Complex overloads of SolveTriangular (Blas.SolveTriangular.cs:44-124, :280-395).
// TrP: plain element arithmetic, TrC: the Conj modes (Complex only; float uses TrP for both).
template <class TrP, class TrC>
__global__ void __launch_bounds__(32) trsv_t_kernel(int uplo, int trans, int n,
                                                    const typename TrP::T* a, int lda,
                                                    typename TrP::T* x, int incx, void* scratch) {
  using T = typename TrP::T;
  using Acc = typename TrP::Acc;
  const int lane = threadIdx.x & 31;
  const int ldx = n | 1;
  Acc* acc = (Acc*)scratch;
  T* xs = (T*)(acc + ldx);
  for (int i = lane; i < n; i += 32) xs[i] = x[(long long)i * incx];
  __syncwarp();
  const long long l = lda;
  const bool conj = trans == 113 || trans == 114;
  const bool tr = trans == 112 || trans == 113;   // Trans, ConjTrans
  if (uplo == 121) {   // Upper
    if (!tr) {         // NoTrans / ConjNoTrans: column sweep over the columns of U
      if (conj) warp_solve_sweep<32, TrC>(a, n, l, 1, xs, ldx, 1);
      else warp_solve_sweep<32, TrP>(a, n, l, 1, xs, ldx, 1);
    } else {           // Trans / ConjTrans: dot form over the columns of U
      if (conj) warp_solve_dot<32, TrC>(a, n, l, 1, false, xs, ldx, acc, 1);
      else warp_solve_dot<32, TrP>(a, n, l, 1, false, xs, ldx, acc, 1);
    }
  } else {             // Lower
    if (!tr) {         // NoTrans / ConjNoTrans: dot form over the rows of L
      if (conj) warp_solve_dot<32, TrC>(a, n, 1, l, false, xs, ldx, acc, 1);
      else warp_solve_dot<32, TrP>(a, n, 1, l, false, xs, ldx, acc, 1);
    } else {           // Trans / ConjTrans: column sweep over the rows of L
      if (conj) warp_solve_sweep<32, TrC>(a, n, 1, l, xs, ldx, 1);
      else warp_solve_sweep<32, TrP>(a, n, 1, l, xs, ldx, 1);
    }
  }
  for (int i = lane; i < n; i += 32) x[(long long)i * incx] = xs[i];
}

// Float MulMatMat (Blas.MulMatMat.cs:45-187): c = (float)Dot with the double tree.
__global__ void sgemm_single_kernel(int transa, int transb, int m, int n, int k, const float* a,
                                    int lda, const float* b, int ldb, float* c, int ldc) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)m * n) return;
  const int j = (int)(e / m);
  const int i = (int)(e - (long long)j * m);
  const float* x = transa == 111 ? a + i : a + (long long)lda * i;
  const long long incx = transa == 111 ? lda : 1;
  const float* y = transb == 111 ? b + (long long)ldb * j : b + j;
  const long long incy = transb == 111 ? 1 : ldb;
  c[(long long)ldc * j + i] = __double2float_rn(exact_dot_f(k, x, incx, y, incy));
}

// Complex MulMatMat (Blas.MulMatMat.cs:407-575): unpaired sequential sums Dot_NN/CN/NC/CC
// (:598-648) starting from Complex.Zero.
__global__ void zgemm_single_kernel(int transa, int transb, int m, int n, int k, const zdouble* a,
                                    int lda, const zdouble* b, int ldb, zdouble* c, int ldc) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)m * n) return;
  const int j = (int)(e / m);
  const int i = (int)(e - (long long)j * m);
  const bool ca = transa == 113 || transa == 114, cb = transb == 113 || transb == 114;
  const bool ta = transa == 112 || transa == 113, tb = transb == 112 || transb == 113;
  const zdouble* x = ta ? a + (long long)lda * i : a + i;
  const long long incx = ta ? 1 : lda;
  const zdouble* y = tb ? b + j : b + (long long)ldb * j;
  const long long incy = tb ? ldb : 1;
  zdouble sum = zmake(0.0, 0.0);
  for (int t = 0; t < k; ++t) {
    const zdouble xv = x[t * incx], yv = y[t * incy];
    zdouble p;
    if (ca && cb) p = zmulconjconj(xv, yv);
    else if (ca) p = zmulconj(xv, yv);
    else if (cb) p = zmulconj(yv, xv);
    else p = zmul(xv, yv);
    sum = zadd(sum, p);
  }
  c[(long long)ldc * j + i] = sum;
}

cudaError_t launch_strsv_single(int uplo, int trans, int n, const float* a, int lda, float* x,
                                int incx, double* scratch, cudaStream_t s) {
  trsv_t_kernel<SSolve, SSolve><<<1, 32, 0, s>>>(uplo, trans, n, a, lda, x, incx, scratch);
  return cudaGetLastError();
}

cudaError_t launch_ztrsv_single(int uplo, int trans, int n, const double* a, int lda, double* x,
                                int incx, double* scratch, cudaStream_t s) {
  trsv_t_kernel<ZSolve<false>, ZSolve<true>><<<1, 32, 0, s>>>(
      uplo, trans, n, (const zdouble*)a, lda, (zdouble*)x, incx, scratch);
  return cudaGetLastError();
}

cudaError_t launch_sgemm_single(int transa, int transb, int m, int n, int k, const float* a,
                                int lda, const float* b, int ldb, float* c, int ldc,
                                cudaStream_t s) {
  const long long total = (long long)m * n;
  sgemm_single_kernel<<<(unsigned)((total + 127) / 128), 128, 0, s>>>(transa, transb, m, n, k, a,
                                                                      lda, b, ldb, c, ldc);
  return cudaGetLastError();
}

cudaError_t launch_zgemm_single(int transa, int transb, int m, int n, int k, const double* a,
                                int lda, const double* b, int ldb, double* c, int ldc,
                                cudaStream_t s) {
  const long long total = (long long)m * n;
  zgemm_single_kernel<<<(unsigned)((total + 127) / 128), 128, 0, s>>>(
      transa, transb, m, n, k, (const zdouble*)a, lda, (const zdouble*)b, ldb, (zdouble*)c, ldc);
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

// Scratch per warp: RHS_CHUNK * (n|1) accumulators and as many staged entries, 8-byte aligned.
template <class S>
static long long getri_single_scratch_bytes(int n) {
  const long long ld = n | 1;
  const long long b = RHS_CHUNK * ld * (long long)(sizeof(typename S::Acc) + sizeof(typename S::T));
  return (b + 15) / 16 * 16;
}

long long getri_single_scratch_bytes_per_warp(int n, int elem) {
  return elem == 1 ? getri_single_scratch_bytes<SSolve>(n)
         : elem == 2 ? getri_single_scratch_bytes<ZSolve<false>>(n)
                     : getri_single_scratch_bytes<DSolve>(n);
}

cudaError_t launch_getri_single(double* a, int n, int lda, const int* piv, double* work,
                                double* scratch, int warps, cudaStream_t s) {
  getri_single_kernel<DSolve><<<1, warps * 32, 0, s>>>(a, n, lda, piv, work, scratch,
                                                       getri_single_scratch_bytes<DSolve>(n));
  return cudaGetLastError();
}
cudaError_t launch_sgetri_single(float* a, int n, int lda, const int* piv, float* work,
                                 void* scratch, int warps, cudaStream_t s) {
  getri_single_kernel<SSolve><<<1, warps * 32, 0, s>>>(a, n, lda, piv, work, scratch,
                                                       getri_single_scratch_bytes<SSolve>(n));
  return cudaGetLastError();
}
cudaError_t launch_zgetri_single(double* a, int n, int lda, const int* piv, double* work,
                                 void* scratch, int warps, cudaStream_t s) {
  getri_single_kernel<ZSolve<false>><<<1, warps * 32, 0, s>>>(
      (zdouble*)a, n, lda, piv, (zdouble*)work, scratch,
      getri_single_scratch_bytes<ZSolve<false>>(n));
  return cudaGetLastError();
}

}  // namespace mfg
