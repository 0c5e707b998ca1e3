/*
 * matflat_gpu.h — C ABI of the GB300 (sm_103a) implementation of MatFlat's factorization path.
 *
 * The reference is the pure-C# library MatFlat 0.8.2 (sinshu/matflat).  Its hot path is a set of
 * `public static unsafe` methods on `MatFlat.Factorization` and `MatFlat.Blas` that take raw
 * column-major pointers, a leading dimension and CBLAS-valued enums.  Each single-matrix entry
 * point below replaces one of those methods one for one (cited per function) and keeps its
 * argument meaning; a C# facade binds them with [LibraryImport] (the binding is shown in the
 * integration notes of this repository).  The batched entry points are new overloads beside
 * them: one call factors tens of thousands of matrices of uneven size.
 *
 * Conventions shared by every entry point:
 *  - Column-major storage with an explicit leading dimension, as in MatFlat.
 *  - Return value: MFG_OK (0); a negative value -i when argument i (1-based, counting the
 *    context as argument 1) is invalid, checked in the same order MatFlat checks its arguments;
 *    or one of the MFG_ERR_* codes below.  No exception crosses the ABI.  Numerical failure that
 *    MatFlat reports by throwing MatrixFactorizationException is reported through an `info`
 *    output (0 = success, k+1 = first failing column k), never by a failing status.
 *  - Single-matrix entry points take the arrays MatFlat's callers pass in HOST memory, or the
 *    same arrays in DEVICE memory (told apart through unified addressing); the library stages
 *    them through its workspace and returns after the result is in place.  Scalar outputs
 *    (sign, info) are host pointers.
 *  - Batched entry points take DEVICE pointers and are asynchronous on the context's stream.
 *  - The plain FP64 path reproduces MatFlat's arithmetic operation by operation (same summation
 *    trees, no fused multiply-add, IEEE division and square root), so factors, pivots and
 *    solutions are bit-identical to MatFlat's.
 *  - A context is not thread-safe; use one context per host thread.  Distinct contexts are
 *    independent.
 */
#ifndef MATFLAT_GPU_H
#define MATFLAT_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define MFG_API __declspec(dllexport)
#else
#define MFG_API __attribute__((visibility("default")))
#endif

/* MatFlat.Uplo (MatFlat/Uplo.cs:13,18) and MatFlat.Transpose (MatFlat/Transpose.cs:13-28);
 * CBLAS-compatible values. */
enum mfg_uplo { MFG_UPPER = 121, MFG_LOWER = 122 };
enum mfg_transpose {
  MFG_NOTRANS = 111,
  MFG_TRANS = 112,
  MFG_CONJTRANS = 113,
  MFG_CONJNOTRANS = 114
};

enum mfg_status {
  MFG_OK = 0,
  MFG_ERR_CUDA = -1000,        /* a CUDA runtime call failed; see mfg_last_error */
  MFG_ERR_NO_DEVICE = -1001,   /* no CUDA device, or the kernels are not built for it */
  MFG_ERR_ALLOC = -1002,       /* device or pinned allocation failed */
  MFG_ERR_INPLACE = -1003,     /* MulMatMat: a == c or b == c ("In-place operation is not
                                  supported.", Blas.MulMatMat.cs:301-304) */
  MFG_ERR_TIMEOUT = -1004,     /* a bounded device-side wait of the mixed solver's tensor-core
                                  update gave up; reported by mfg_plan_status */
  MFG_ERR_UNSUPPORTED = -1005  /* size or option outside what the library supports */
};

typedef struct mfg_ctx mfg_ctx;
typedef struct mfg_plan mfg_plan;

/* ---------------------------------------------------------------------------------------------
 * Context: owns a CUDA stream, a device workspace, the CUDA-graph cache and the tuning table.
 * ------------------------------------------------------------------------------------------- */
MFG_API int mfg_create(mfg_ctx** ctx);
MFG_API int mfg_destroy(mfg_ctx* ctx);
/* Use `stream` (a cudaStream_t) for all later work; NULL selects the context's own stream. */
MFG_API int mfg_set_stream(mfg_ctx* ctx, void* stream);
MFG_API int mfg_synchronize(mfg_ctx* ctx);
/* The CUDA device the context was created on (the device current at mfg_create).  Every later
 * call on the context makes that device current while it runs and restores the caller's device
 * before returning, so a thread may switch devices between calls. */
MFG_API int mfg_get_device(mfg_ctx* ctx, int* device);
/* Text of the last failure on this context (empty when none).  Valid until the next call. */
MFG_API const char* mfg_last_error(mfg_ctx* ctx);
/* Library version, e.g. "0.1.0"; the MatFlat version whose arithmetic it reproduces is 0.8.2. */
MFG_API const char* mfg_version(void);

/* ---------------------------------------------------------------------------------------------
 * Single-matrix drop-ins (host or device arrays).  Same argument meaning as the MatFlat method
 * cited.
 * ------------------------------------------------------------------------------------------- */

/* Factorization.Lu(int m, int n, double* a, int lda, int* piv) -> pivot sign
 * (MatFlat/Factorization.Lu.cs:122-161; LuCore :296-350).  piv has m entries and is a
 * permutation vector: row i of P*A is row piv[i] of A.  *sign receives Lu's return value.
 * Like MatFlat, a zero pivot is not an error (the column is left undivided). */
MFG_API int mfg_dgetrf(mfg_ctx* ctx, int m, int n, double* a, int lda, int* piv, int* sign);

/* Factorization.Cholesky(int n, double* a, int lda) (MatFlat/Factorization.Cholesky.cs:114-168).
 * Reads the upper triangle, writes L to the lower triangle and zeroes the strict upper triangle.
 * *info = 0 on success, or k+1 when the matrix is not positive definite at column k (where
 * MatFlat throws MatrixFactorizationException; the content of a is then unspecified). */
MFG_API int mfg_dpotrf(mfg_ctx* ctx, int n, double* a, int lda, int* info);

/* Factorization.Qr(int m, int n, double* a, int lda, double* rdiag)
 * (MatFlat/Factorization.Qr.cs:115-172): Householder QR in the Mapack format, m >= n. */
MFG_API int mfg_dgeqrf(mfg_ctx* ctx, int m, int n, double* a, int lda, double* rdiag);
/* Factorization.QrOrthogonalFactor (MatFlat/Factorization.Qr.cs:357-413): thin m-by-n Q. */
MFG_API int mfg_dorgqr(mfg_ctx* ctx, int m, int n, const double* a, int lda, double* q, int ldq);
/* Factorization.QrUpperTriangularFactor (MatFlat/Factorization.Qr.cs:597-650): n-by-n R. */
MFG_API int mfg_dqr_r(mfg_ctx* ctx, int m, int n, const double* a, int lda, double* r, int ldr,
                      const double* rdiag);

/* Float overloads of the three QR routines (MatFlat/Factorization.Qr.cs:32-89, :278-334,
 * :518-571): float storage, dots and norms summed in double as MatFlat does. */
MFG_API int mfg_sgeqrf(mfg_ctx* ctx, int m, int n, float* a, int lda, float* rdiag);
MFG_API int mfg_sorgqr(mfg_ctx* ctx, int m, int n, const float* a, int lda, float* q, int ldq);
MFG_API int mfg_sqr_r(mfg_ctx* ctx, int m, int n, const float* a, int lda, float* r, int ldr,
                      const float* rdiag);

/* Float and Complex overloads of Lu, Cholesky, Qr, SolveTriangular and MulMatMat, with the
 * reference arithmetic of each overload: float storage with dots accumulated in double
 * (Internals.cs:149-176, 236-263); Complex = System.Numerics.Complex as interleaved (re, im)
 * doubles, every product and sum separately rounded, division by Smith's algorithm, LU pivots by
 * FastMagnitude |re| + |im| (Internals.cs:16-19).  Complex transposes also accept ConjTrans and
 * ConjNoTrans.
 *   Factorization.Lu (Factorization.Lu.cs:45-84 float, :199-238 Complex)
 *   Factorization.Cholesky (Factorization.Cholesky.cs:33-87 float, :195-249 Complex: A = L L^H)
 *   Factorization.Qr / QrOrthogonalFactor / QrUpperTriangularFactor Complex
 *     (Factorization.Qr.cs:198-255, :436-492, :677-730; rdiag is real)
 *   Blas.SolveTriangular (Blas.SolveTriangular.cs:44-124 float, :280-395 Complex)
 *   Blas.MulMatMat (Blas.MulMatMat.cs:45-187 float, :407-648 Complex) */
MFG_API int mfg_sgetrf(mfg_ctx* ctx, int m, int n, float* a, int lda, int* piv, int* sign);
MFG_API int mfg_zgetrf(mfg_ctx* ctx, int m, int n, double* a, int lda, int* piv, int* sign);
MFG_API int mfg_spotrf(mfg_ctx* ctx, int n, float* a, int lda, int* info);
MFG_API int mfg_zpotrf(mfg_ctx* ctx, int n, double* a, int lda, int* info);
MFG_API int mfg_zgeqrf(mfg_ctx* ctx, int m, int n, double* a, int lda, double* rdiag);
MFG_API int mfg_zorgqr(mfg_ctx* ctx, int m, int n, const double* a, int lda, double* q, int ldq);
MFG_API int mfg_zqr_r(mfg_ctx* ctx, int m, int n, const double* a, int lda, double* r, int ldr,
                      const double* rdiag);
MFG_API int mfg_strsv(mfg_ctx* ctx, int uplo, int trans, int n, const float* a, int lda, float* x,
                      int incx);
MFG_API int mfg_ztrsv(mfg_ctx* ctx, int uplo, int trans, int n, const double* a, int lda,
                      double* x, int incx);
MFG_API int mfg_sgemm(mfg_ctx* ctx, int transa, int transb, int m, int n, int k, const float* a,
                      int lda, const float* b, int ldb, float* c, int ldc);
MFG_API int mfg_zgemm(mfg_ctx* ctx, int transa, int transb, int m, int n, int k, const double* a,
                      int lda, const double* b, int ldb, double* c, int ldc);

/* Blas.SolveTriangular(Uplo, Transpose, int n, double* a, int lda, double* x, int incx)
 * (MatFlat/Blas.SolveTriangular.cs:162-242): non-unit diagonal, NoTrans or Trans. */
MFG_API int mfg_dtrsv(mfg_ctx* ctx, int uplo, int trans, int n, const double* a, int lda,
                      double* x, int incx);

/* Blas.MulMatMat(Transpose, Transpose, int m, int n, int k, double* a, int lda, double* b,
 * int ldb, double* c, int ldc) (MatFlat/Blas.MulMatMat.cs:226-368): C = op(A) op(B), C is
 * overwritten, aliasing of C with A or B is rejected with MFG_ERR_INPLACE. */
MFG_API int mfg_dgemm(mfg_ctx* ctx, int transa, int transb, int m, int n, int k, const double* a,
                      int lda, const double* b, int ldb, double* c, int ldc);

/* Factorization.LuInverse(int n, double* a, int lda, int* piv)
 * (MatFlat/Factorization.LuInverse.cs:123-199): overwrites the LU factors with A^-1.
 * *info = 1 when a diagonal entry of U is zero (MatFlat throws "The matrix is not invertible."),
 * in which case a is left unchanged. */
MFG_API int mfg_dgetri(mfg_ctx* ctx, int n, double* a, int lda, const int* piv, int* info);
/* The float and Complex overloads (MatFlat/Factorization.LuInverse.cs:27-103, :219-295; Complex
 * as interleaved (re, im) doubles, singular when a diagonal entry is exactly 0 + 0i). */
MFG_API int mfg_sgetri(mfg_ctx* ctx, int n, float* a, int lda, const int* piv, int* info);
MFG_API int mfg_zgetri(mfg_ctx* ctx, int n, double* a, int lda, const int* piv, int* info);

/* ---------------------------------------------------------------------------------------------
 * Batched overloads (new).  A plan fixes the shapes of a batch once: the host runtime sorts the
 * matrices by work (longest first), uploads the descriptors, picks the launch shape from the
 * tuning table and captures the launch sequence as a CUDA graph on first execution.  Executing a
 * plan is then a single graph replay on the context's stream, with device pointers only.
 *
 * Layout of a batch: matrix i is square of order n[i], stored column-major at
 * a + a_off[i] with leading dimension lda[i] (lda may be NULL: lda[i] = n[i]); its pivot vector
 * at piv + piv_off[i] (n[i] ints); its right-hand sides at b + b_off[i], nrhs columns with
 * leading dimension n[i].  Offsets are in elements.  All descriptor arrays are HOST arrays,
 * read during plan creation only.
 * ------------------------------------------------------------------------------------------- */

/* LU with partial pivoting of every matrix (Factorization.Lu), then, when nrhs > 0, the solve
 * A x = b for nrhs right-hand sides: b' = P b, the unit-lower solve in MatFlat's LuInverse
 * idiom (MatFlat/Factorization.LuInverse.cs:174-182) and the upper solve
 * (Blas.SolveTriangular Upper/NoTrans, MatFlat/Blas.SolveTriangular.cs:191-199). */
MFG_API int mfg_plan_getrf_batched(mfg_ctx* ctx, mfg_plan** plan, int count, const int* n,
                                   const int* lda, const int64_t* a_off, const int64_t* piv_off,
                                   int nrhs, const int64_t* b_off);
/* Executes a getrf plan.  a: in/out factors; piv: out; b: in/out solutions (NULL if nrhs = 0);
 * sign: out, one per matrix (Lu's return value); info: out, one per matrix (0, or k+1 for the
 * first exactly-zero pivot U(k,k), LAPACK's convention; the factorization still completes). */
MFG_API int mfg_dgetrf_batched(mfg_plan* plan, double* a, int* piv, double* b, int* sign,
                               int* info);
/* The same factor + solve on HOST buffers (the arrays a C# caller pins), laid out exactly as the
 * plan describes: the batch is cut into contiguous chunks of about equal work, and each chunk's
 * upload, factorization and download overlap with its neighbours' on separate streams, so the
 * copies hide behind the compute.  Synchronous: returns when a, piv, b, sign and info hold the
 * results (bit-identical to mfg_dgetrf_batched).  Page-locked host memory gives full copy speed.
 * The first call allocates device mirrors of the arrays and per-chunk plans (kept by the plan). */
MFG_API int mfg_dgetrf_batched_host(mfg_plan* plan, double* a, int* piv, double* b, int* sign,
                                    int* info);
/* The same pipelined host-buffer form of the other batched operations (arguments as in their
 * device-buffer forms; every array is a HOST array, synchronous, bit-identical results). */
MFG_API int mfg_dpotrf_batched_host(mfg_plan* plan, double* a, double* b, int* info);
MFG_API int mfg_dgetri_batched_host(mfg_plan* plan, double* a, const int* piv, int* info);
MFG_API int mfg_dgeqrf_batched_host(mfg_plan* plan, double* a, double* rdiag, double* b);
MFG_API int mfg_sgeqrf_batched_host(mfg_plan* plan, float* a, float* rdiag, float* b);
MFG_API int mfg_dgevd_front_batched_host(mfg_plan* plan, const double* a, double* b, double* c,
                                         int* info);
MFG_API int mfg_sgevd_front_batched_host(mfg_plan* plan, const float* a, float* b, float* c,
                                         int* info);
MFG_API int mfg_zgevd_front_batched_host(mfg_plan* plan, const double* a, double* b, double* c,
                                         int* info);
MFG_API int mfg_dpotrf_logdet_solve_grad_batched_host(mfg_plan* plan, double* k, double* y,
                                                     double* loss, double* grad, int* info,
                                                     int keep_factor);
/* The float and Complex overloads' host-buffer forms (Complex: interleaved (re, im) doubles;
 * the Complex QR's rdiag is real). */
MFG_API int mfg_sgetrf_batched_host(mfg_plan* plan, float* a, int* piv, float* b, int* sign,
                                    int* info);
MFG_API int mfg_zgetrf_batched_host(mfg_plan* plan, double* a, int* piv, double* b, int* sign,
                                    int* info);
MFG_API int mfg_spotrf_batched_host(mfg_plan* plan, float* a, float* b, int* info);
MFG_API int mfg_zpotrf_batched_host(mfg_plan* plan, double* a, double* b, int* info);
MFG_API int mfg_zgeqrf_batched_host(mfg_plan* plan, double* a, double* rdiag, double* b);
/* Solve only, with factors and pivots already in a and piv (from mfg_dgetrf_batched or
 * Factorization.Lu): b' = P b, the unit-lower solve (LuInverse idiom, Factorization.LuInverse.cs:
 * 174-182) and the upper solve (Blas.SolveTriangular.cs:191-199), for the plan's nrhs (>= 1)
 * right-hand sides; bit-identical to the fused path.  a and piv are read only. */
MFG_API int mfg_dgetrs_batched(mfg_plan* plan, const double* a, const int* piv, double* b);
/* The float and Complex overloads of the batched factor + solve and of the solve alone, on the
 * same plan (offsets count elements of the type; Complex arrays are interleaved (re, im) doubles,
 * element e at doubles 2e and 2e+1).  Bit-identical to Factorization.Lu's float / Complex
 * overloads (MatFlat/Factorization.Lu.cs:240-294 float, :352-406 Complex: float storage with
 * double dot sums; Complex pivots by FastMagnitude) followed by the unit-lower and upper
 * SolveTriangular of the same type (MatFlat/Blas.SolveTriangular.cs:44-124 float, :280-395
 * Complex).  sign, info and piv as in mfg_dgetrf_batched. */
MFG_API int mfg_sgetrf_batched(mfg_plan* plan, float* a, int* piv, float* b, int* sign,
                               int* info);
MFG_API int mfg_zgetrf_batched(mfg_plan* plan, double* a, int* piv, double* b, int* sign,
                               int* info);
MFG_API int mfg_sgetrs_batched(mfg_plan* plan, const float* a, const int* piv, float* b);
MFG_API int mfg_zgetrs_batched(mfg_plan* plan, const double* a, const int* piv, double* b);

/* Cholesky of every matrix (Factorization.Cholesky), then, when nrhs > 0, L y = b
 * (SolveTriangular Lower/NoTrans) and L^T x = y (SolveTriangular Lower/Trans) per right-hand
 * side.  info: 0, or k+1 for a matrix that is not positive definite at column k (its b is left
 * unchanged and its a unspecified). */
MFG_API int mfg_plan_potrf_batched(mfg_ctx* ctx, mfg_plan** plan, int count, const int* n,
                                   const int* lda, const int64_t* a_off, int nrhs,
                                   const int64_t* b_off);
MFG_API int mfg_dpotrf_batched(mfg_plan* plan, double* a, double* b, int* info);
/* Solve only with Cholesky factors already in a (lower triangle): L y = b, L^T x = y
 * (Blas.SolveTriangular Lower/NoTrans then Lower/Trans, Blas.SolveTriangular.cs:215-238) for the
 * plan's nrhs (>= 1) right-hand sides. */
MFG_API int mfg_dpotrs_batched(mfg_plan* plan, const double* a, double* b);
/* The float and Complex overloads on the same plan (offsets count elements; Complex arrays are
 * interleaved (re, im) doubles).  Bit-identical to Factorization.Cholesky's float / Complex
 * overloads (MatFlat/Factorization.Cholesky.cs:33-87, :195-249; Complex A = L L^H with a real
 * diagonal) followed by SolveTriangular of the same type: Lower/NoTrans, then Lower/Trans (float)
 * or Lower/ConjTrans (Complex) (MatFlat/Blas.SolveTriangular.cs:44-124, :280-395).  One warp per
 * matrix whatever the plan's lanes per matrix; info as in mfg_dpotrf_batched. */
MFG_API int mfg_spotrf_batched(mfg_plan* plan, float* a, float* b, int* info);
MFG_API int mfg_zpotrf_batched(mfg_plan* plan, double* a, double* b, int* info);
MFG_API int mfg_spotrs_batched(mfg_plan* plan, const float* a, float* b);
MFG_API int mfg_zpotrs_batched(mfg_plan* plan, const double* a, double* b);

/* Strided batches of MatFlat's vector building blocks (device pointers, asynchronous on the
 * context's stream; item b of every operand at base + b*stride), in MatFlat's arithmetic:
 *   Blas.MulMatVec (Blas.MulMatVec.cs:138-236): y = A x (NoTrans: y_i = Dot(n, A(i,:), x)) or
 *     A^T x (Trans: y_j = Dot(m, A(:,j), x)); same checks and messages (a or x aliasing y is
 *     MFG_ERR_INPLACE);
 *   Blas.Dot (Blas.VectorOperations.cs:143-174) and Blas.L2Norm (:50-60: Math.Sqrt of the same
 *     tree over x*x): one result per item;
 *   Blas.Outer (:292-334): a(i,j) = y_j * x_i. */
MFG_API int mfg_dgemv_strided_batched(mfg_ctx* ctx, int trans, int m, int n, const double* a,
                                      int lda, int64_t stride_a, const double* x, int incx,
                                      int64_t stride_x, double* y, int incy, int64_t stride_y,
                                      int count);
MFG_API int mfg_ddot_strided_batched(mfg_ctx* ctx, int n, const double* x, int incx,
                                     int64_t stride_x, const double* y, int incy,
                                     int64_t stride_y, double* result, int count);
MFG_API int mfg_dnrm2_strided_batched(mfg_ctx* ctx, int n, const double* x, int incx,
                                      int64_t stride_x, double* result, int count);
MFG_API int mfg_dger_strided_batched(mfg_ctx* ctx, int m, int n, const double* x, int incx,
                                     int64_t stride_x, const double* y, int incy,
                                     int64_t stride_y, double* a, int lda, int64_t stride_a,
                                     int count);
/* The float and Complex overloads of the same strided batches (Complex as interleaved (re, im)
 * doubles, strides and increments in elements):
 *   MulMatVec float (Blas.MulMatVec.cs:38-136: the double tree over widened operands, cast to
 *     float) and Complex (:238-336: Internals.Dot, and DotConj for ConjNoTrans / ConjTrans);
 *   Dot float (Blas.VectorOperations.cs:110-141), Dot / DotConj Complex (:176-246);
 *   L2Norm float (:23-48, cast to float) and Complex (:77-108, a double: Internals.Norm's order,
 *     ((re0^2 + im0^2) + re1^2) + im1^2 per pair);
 *   Outer float (:248-290), Outer / OuterConj Complex (:336-420: y_j * x_i, conj(y_j) * x_i). */
MFG_API int mfg_sgemv_strided_batched(mfg_ctx* ctx, int trans, int m, int n, const float* a,
                                      int lda, int64_t stride_a, const float* x, int incx,
                                      int64_t stride_x, float* y, int incy, int64_t stride_y,
                                      int count);
MFG_API int mfg_zgemv_strided_batched(mfg_ctx* ctx, int trans, int m, int n, const double* a,
                                      int lda, int64_t stride_a, const double* x, int incx,
                                      int64_t stride_x, double* y, int incy, int64_t stride_y,
                                      int count);
MFG_API int mfg_sdot_strided_batched(mfg_ctx* ctx, int n, const float* x, int incx,
                                     int64_t stride_x, const float* y, int incy,
                                     int64_t stride_y, float* result, int count);
MFG_API int mfg_zdot_strided_batched(mfg_ctx* ctx, int n, const double* x, int incx,
                                     int64_t stride_x, const double* y, int incy,
                                     int64_t stride_y, double* result, int count);
MFG_API int mfg_zdotc_strided_batched(mfg_ctx* ctx, int n, const double* x, int incx,
                                      int64_t stride_x, const double* y, int incy,
                                      int64_t stride_y, double* result, int count);
MFG_API int mfg_snrm2_strided_batched(mfg_ctx* ctx, int n, const float* x, int incx,
                                      int64_t stride_x, float* result, int count);
MFG_API int mfg_dznrm2_strided_batched(mfg_ctx* ctx, int n, const double* x, int incx,
                                       int64_t stride_x, double* result, int count);
MFG_API int mfg_sger_strided_batched(mfg_ctx* ctx, int m, int n, const float* x, int incx,
                                     int64_t stride_x, const float* y, int incy,
                                     int64_t stride_y, float* a, int lda, int64_t stride_a,
                                     int count);
MFG_API int mfg_zger_strided_batched(mfg_ctx* ctx, int m, int n, const double* x, int incx,
                                     int64_t stride_x, const double* y, int incy,
                                     int64_t stride_y, double* a, int lda, int64_t stride_a,
                                     int count);
MFG_API int mfg_zgerc_strided_batched(mfg_ctx* ctx, int m, int n, const double* x, int incx,
                                      int64_t stride_x, const double* y, int incy,
                                      int64_t stride_y, double* a, int lda, int64_t stride_a,
                                      int count);

/* Front half of Factorization.Gevd for a batch of pairs (Factorization.GevdCore,
 * Factorization.Gevd.cs:330-365; the reference has no batched form): B = L L^T in place
 * (Factorization.Cholesky), then C = L^-1 A L^-T from A's upper triangle by MatFlat's two passes of
 * SolveTriangular(Lower, NoTrans) over the rows and then the columns of C, bit-identical.  C is
 * what the eigen-solver of the back half takes (MatFlat runs its Svd on it; out of scope here).
 * Pair i: A of order n[i] (<= 128) at a + a_off[i] (leading dimension lda[i], NULL: n), B at
 * b + b_off[i] (ldb[i]), C at c + c_off[i] (leading dimension n[i]).  info: 0, or k+1 when B is not
 * positive definite at column k (MatFlat throws "The right-hand side matrix is not positive
 * definite."; B and C are then unspecified). */
MFG_API int mfg_plan_gevd_front_batched(mfg_ctx* ctx, mfg_plan** plan, int count, const int* n,
                                        const int* lda, const int64_t* a_off, const int* ldb,
                                        const int64_t* b_off, const int64_t* c_off);
MFG_API int mfg_dgevd_front_batched(mfg_plan* plan, const double* a, double* b, double* c,
                                    int* info);
/* The float and Complex overloads on the same plan (GevdCore float, Factorization.Gevd.cs:282-318;
 * Complex, :378-422, Complex as interleaved (re, im) doubles).  The float overload computes in
 * float storage with double dots, as MatFlat's float Cholesky and SolveTriangular do.  The
 * Complex one factors B = L L^H, fills C Hermitian from A's upper triangle (the diagonal taken as
 * stored) and solves each row of C conjugated, conjugating the solution back, as MatFlat does:
 * C = L^-1 A L^-H. */
MFG_API int mfg_sgevd_front_batched(mfg_plan* plan, const float* a, float* b, float* c,
                                    int* info);
MFG_API int mfg_zgevd_front_batched(mfg_plan* plan, const double* a, double* b, double* c,
                                    int* info);

/* Batched Factorization.LuInverse (Factorization.LuInverse.cs:123-199): replaces every matrix's
 * LU factors (as left by mfg_dgetrf_batched / Factorization.Lu) with A^-1, bit-identical to
 * MatFlat.  piv at piv + piv_off[i] is the matrix's pivot vector (read only).  info: 0, or j+1
 * when U(j,j) == 0 for the first such j (MatFlat throws "The matrix is not invertible."), or -1
 * when piv is not a permutation of 0..n-1; in both cases that matrix is left unchanged. */
MFG_API int mfg_plan_getri_batched(mfg_ctx* ctx, mfg_plan** plan, int count, const int* n,
                                   const int* lda, const int64_t* a_off, const int64_t* piv_off);
MFG_API int mfg_dgetri_batched(mfg_plan* plan, double* a, const int* piv, int* info);
/* The float and Complex overloads on the same plan (Factorization.LuInverse.cs:27-103, :219-295;
 * Complex as interleaved (re, im) doubles, offsets in elements): bit-identical to MatFlat, info
 * as above (a diagonal entry counts as zero when it is exactly 0, or 0 + 0i). */
MFG_API int mfg_sgetri_batched(mfg_plan* plan, float* a, const int* piv, int* info);
MFG_API int mfg_zgetri_batched(mfg_plan* plan, double* a, const int* piv, int* info);

/* Householder QR of every tall matrix (Factorization.Qr; m[i] >= n[i], lda[i] >= m[i]), then,
 * when nrhs > 0, the least-squares solve min ||A x - b|| of nrhs right-hand sides per matrix
 * (b: nrhs columns of m[i] entries, leading dimension m[i]).  MatFlat has no QR solve; the
 * solver applies the same reflector updates to b (Qr.cs:160-165) and then solves R x = (Q^T b)
 * with SolveTriangular Upper/NoTrans (Blas.SolveTriangular.cs:191-199).  On exit b[0:n] holds
 * x and b[n:m] the residual components; a and rdiag hold the factorization in MatFlat's format.
 * The same plan runs in double (mfg_dgeqrf_batched) or float (mfg_sgeqrf_batched, MatFlat's
 * float overload: float storage, double-accumulated dots). */
MFG_API int mfg_plan_geqrf_batched(mfg_ctx* ctx, mfg_plan** plan, int count, const int* m,
                                   const int* n, const int* lda, const int64_t* a_off,
                                   const int64_t* rdiag_off, int nrhs, const int64_t* b_off);
MFG_API int mfg_dgeqrf_batched(mfg_plan* plan, double* a, double* rdiag, double* b);
MFG_API int mfg_sgeqrf_batched(mfg_plan* plan, float* a, float* rdiag, float* b);
/* Least-squares solve only, with the factorization already in a and rdiag (Factorization.Qr's
 * format): the stored reflectors applied to b in the factorization's order (Qr.cs:160-165), then
 * R x = Q^T b (Blas.SolveTriangular.cs:191-199); bit-identical to the fused path.  nrhs >= 1. */
MFG_API int mfg_dgeqrs_batched(mfg_plan* plan, const double* a, const double* rdiag, double* b);
MFG_API int mfg_sgeqrs_batched(mfg_plan* plan, const float* a, const float* rdiag, float* b);
/* The Complex overload of the batched QR (+ least squares) and of the solve alone, on the same
 * plan: a and b are interleaved (re, im) doubles (offsets count complex elements), rdiag is real
 * as in Factorization.Qr(Complex) (MatFlat/Factorization.Qr.cs:198-255: DotConj coefficients,
 * division by Complex(norm, 0)); factors and rdiag bit-identical to it.  The right-hand sides get
 * Q^H b from the same reflector updates, then R x = y with Complex SolveTriangular Upper/NoTrans
 * arithmetic (Blas.SolveTriangular.cs:280-395; R's diagonal is Complex(rdiag, 0)). */
MFG_API int mfg_zgeqrf_batched(mfg_plan* plan, double* a, double* rdiag, double* b);
MFG_API int mfg_zgeqrs_batched(mfg_plan* plan, const double* a, const double* rdiag, double* b);

/* Differentiable Cholesky / log-determinant / solve over a potrf plan with nrhs = 1 (n <= 128).
 * For every SPD matrix K (upper triangle read, as Factorization.Cholesky) and vector y:
 *   loss[i] = y^T K^-1 y + log det K,
 *   grad    = d loss / d K = K^-1 - alpha alpha^T (full symmetric n-by-n, same layout as k),
 *   y       <- alpha = K^-1 y.
 * Built from MatFlat's own routines in MatFlat's arithmetic: L = Cholesky(K)
 * (Factorization.Cholesky.cs:114-168), z = SolveTriangular(Lower, NoTrans), alpha =
 * SolveTriangular(Lower, Trans) (Blas.SolveTriangular.cs:216-231), K^-1 by the same two solves on
 * the columns of the identity (the LuInverse idiom, Factorization.LuInverse.cs:174-192), taken
 * from its upper triangle and mirrored; log det K = 2 * sum log L_ii.
 * keep_factor = 1: k is overwritten with L.  keep_factor = 0: k is left untouched and L is
 * recomputed inside grad's storage (no extra memory for the factor).
 * info[i] = 0, or j+1 when K is not positive definite at column j (loss NaN, grad unspecified). */
MFG_API int mfg_dpotrf_logdet_solve_grad_batched(mfg_plan* plan, double* k, double* y,
                                                double* loss, double* grad, int* info,
                                                int keep_factor);

/* Reverse mode (vector-Jacobian product) of Factorization.Cholesky
 * (MatFlat/Factorization.Cholesky.cs:114-168), its log-determinant and the solve A x = b done with
 * the two Blas.SolveTriangular calls (MatFlat/Blas.SolveTriangular.cs:162-242), over a potrf plan
 * (n <= 128).  Forward, per matrix: L = Cholesky(A), logdet = 2 sum log L_ii, x = A^-1 b.
 * Given the cotangents lbar (dloss/dL, lower triangle, same layout as a; NULL = 0), logdet_bar
 * (one per matrix; NULL = 0) and xbar (dloss/dx, laid out like b; NULL = 0, then x may be NULL),
 * writes the symmetric gradient dloss/dA to abar (same layout as a; d loss = <abar, dA> for
 * symmetric dA, so the derivative by an upper-triangle entry A_ij, i < j, that Cholesky reads is
 * 2 abar_ij):
 *   abar = sym(L^-T Phi(L^T lbar) L^-1) + logdet_bar A^-1 - sym(bbar x^T),  bbar = A^-1 xbar,
 * Phi = lower triangle with the diagonal halved, sym(M) = (M + M^T)/2, and bbar (dloss/db) to
 * bbar when not NULL (b layout; zero when xbar is NULL).  xbar needs a plan with nrhs >= 1.
 * recompute = 1: a holds A and the factor is recomputed in place (a <- L, bit-identical to
 * mfg_dpotrf_batched), so nothing is stored between the forward and the backward pass;
 * recompute = 0: a holds L from mfg_dpotrf_batched.  info[i] = j+1 when the recomputed
 * factorization fails at column j (abar then unspecified).  The backward pass uses fused
 * multiply-adds (MatFlat defines no derivative order).  Device pointers; asynchronous. */
MFG_API int mfg_dpotrf_backward_batched(mfg_plan* plan, double* a, const double* lbar,
                                        const double* logdet_bar, const double* x,
                                        const double* xbar, double* abar, double* bbar,
                                        int* info, int recompute);

/* Mixed-precision LU solve with FP64 iterative refinement (new; no MatFlat counterpart).
 * A plan for `count` systems of one order n (a multiple of 32, at most 1024); matrices packed
 * column-major with lda = n at stride n*n, right-hand sides and solutions at stride n.
 * The solver factors FP32 copies of A with partial pivoting (trailing updates on the tensor cores
 * in TF32 or BF16 with FP32 accumulation, hand-written tcgen05 + TMA, or on the FP32 cores),
 * then refines in FP64:
 * r = b - A x, d = (LU)^-1 r in FP32, x += d, until the normwise backward error
 * berr = |b - A x|_inf / (|A|_inf |x|_inf + |b|_inf) <= tol, stalls, or max_iter sweeps pass.
 * Systems that do not converge are solved again with the exact FP64 LU (Factorization.Lu's
 * arithmetic).  Outputs per system: x, berr, iters (refinement sweeps), info (0 refined to tol,
 * 1 solved by the FP64 fallback, 2 singular).  a, b, x, berr, iters and info are device
 * pointers.  The call is asynchronous on the context's stream and allocates nothing: the plan owns
 * the FP32 factors, the operand copies and the fallback's buffers (about 4 n^2 count bytes of
 * factors, 4 copies of n x 32 values per system, and the FP64 fallback copy of A, 8 n^2 count
 * bytes).  Check mfg_plan_status after it. */
/* lowp: FP32 (trailing updates on the FP32 cores), TF32 or BF16 (tensor cores, FP32
 * accumulation), TF32X3 (tensor cores, each operand split into a TF32 high and low part and the
 * three leading products accumulated: about FP32's accuracy, so refinement converges where the
 * FP32 mode does). */
enum mfg_lowp { MFG_LOWP_FP32 = 0, MFG_LOWP_TF32 = 1, MFG_LOWP_BF16 = 2, MFG_LOWP_TF32X3 = 3 };
MFG_API int mfg_plan_gesv_mixed_batched(mfg_ctx* ctx, mfg_plan** plan, int count, int n);
MFG_API int mfg_dgesv_mixed_batched(mfg_plan* plan, const double* a, const double* b, double* x,
                                    int lowp, int max_iter, double tol, double* berr, int* iters,
                                    int* info);

/* Launch-shape autotuner (no counterpart in the reference) for getrf, potrf and geqrf plans.
 * Times candidate shapes on a synthetic batch with the plan's size mix (sampled evenly: up to
 * 100,000 matrices, 50,000 for QR), installs the fastest in the plan and records it in the
 * context's tuning table under the plan's size bucket, so later plans of that bucket on this
 * context start from it.  getrf: the lanes-per-matrix table of its size buckets (8, 16 or 32
 * lanes per matrix by order; -1 one matrix per warp), warps per SM, dot-product block; potrf:
 * lanes per matrix, warps per SM, multiply pipe; geqrf: lanes per matrix and warps per SM, keyed
 * by the (largest m, largest n) bucket.  Synchronous; allocates and frees its own buffers; every
 * shape gives the same bits.  config (may be NULL) receives 5 ints: {warps per CTA, warps per
 * SM, lanes per matrix (getrf: the lanes table), multiply mode, dot-product pairs per pipelined
 * block}.  Environment overrides of the shape (MFG_WARPS_PER_*, MFG_HW_MUL, MFG_CHOL_GROUP,
 * MFG_LU_GROUPS, MFG_QR_GROUP) take precedence over the table for new plans. */
MFG_API int mfg_plan_autotune(mfg_plan* plan, int* config);

/* Arithmetic form of a batched Cholesky, QR or LU plan (no counterpart in the reference; MatFlat
 * has one form).  MFG_FORM_EXACT (default): MatFlat's arithmetic, bit-identical factors, info and
 * solutions.  MFG_FORM_FMA, Cholesky (double overload): the same column order and failure test,
 * with fused multiply-adds in any order and the column scaled by the reciprocal of its
 * diagonal: the factor satisfies the Cholesky backward-error bound
 * |A - L L^T| <= gamma_(n+2) |L| |L^T| instead of MatFlat's bits, the solves are fused
 * multiply-add column sweeps with that reciprocal diagonal (solve-only calls give the same
 * bits), and info reports a column whose computed pivot is not positive, which differs from
 * MatFlat only for matrices within rounding of the positive-definite boundary.  MFG_FORM_FMA, QR
 * (double overload): MatFlat's Householder algorithm and storage (no sign choice,
 * rdiag = -norm, the same degenerate-reflector rules) with fused multiply-add dots, norms and
 * updates and the column scaled by the reciprocal of its norm: backward-stable factors and
 * least-squares solutions instead of MatFlat's bits.  MFG_FORM_FMA, LU (double overload):
 * MatFlat's pivot rule with fused multiply-add arithmetic and reciprocal column scaling (the
 * Crout schedule up to order 152, a blocked right-looking LU with one CTA per matrix above it,
 * whatever the batch size), and a screen at every column that keeps MatFlat's
 * pivots: a matrix whose pivot could depend on rounding (the runner-up within about 1.5e-8 of the
 * pivot, ties, a zero pivot, NaN or infinite candidates) is redone in MatFlat's arithmetic
 * (mfg_plan_form_fallbacks counts them); factors satisfy |PA - LU| <= gamma_n |L| |U|, solutions
 * come from fused multiply-add column sweeps.
 * The screen is not a proof that every pivot is MatFlat's.  MFG_ERR_UNSUPPORTED for other
 * plans.
 * Drops the plan's cached graph. */
enum mfg_form { MFG_FORM_EXACT = 0, MFG_FORM_FMA = 1 };
MFG_API int mfg_plan_set_form(mfg_plan* plan, int form);

/* Matrices of a getrf plan's last execution (device or host-buffer call) that the FMA form
 * redid in MatFlat's arithmetic because their pivot choice did not pass its screen (no
 * counterpart in the reference).  Synchronizes with the plan's work; 0 for the exact form and
 * for other plans. */
MFG_API int mfg_plan_form_fallbacks(mfg_plan* plan, long long* count);

MFG_API int mfg_plan_destroy(mfg_plan* plan);

/* Waits for the context's stream and reports an asynchronous failure of the work queued so far
 * (including the last execution of `plan`): MFG_OK, MFG_ERR_CUDA (text in mfg_last_error), or,
 * for a mixed-precision plan, MFG_ERR_TIMEOUT when one of the tensor-core update's bounded waits
 * (TMA tile arrival, tensor-core completion; 0.2 s each) gave up, in which case that execution's
 * solutions are not valid (the status is cleared by reading it).  Numerical failures are not
 * statuses: they are in the `info` arrays. */
MFG_API int mfg_plan_status(mfg_plan* plan);

/* Allocation-free batched LU + solve (no counterpart in the reference: MatFlat has no batched
 * or GPU API).  For callers that cannot allocate device memory — code running inside a stream
 * capture they do not own, real-time paths whose memory is fixed at start-up, hosts that hand the
 * library a fixed arena — this entry point calls no cudaMalloc, cudaFree or allocating library
 * routine.  It factors `count` matrices of one order n (Factorization.Lu) and, when nrhs > 0,
 * solves A x = b exactly as mfg_dgetrf_batched does, bit for bit.  Matrix i is at
 * a + i*stride_a (leading dimension lda), its pivots at piv + i*stride_piv, its nrhs right-hand
 * sides at b + i*stride_b (leading dimension n); sign[i] and info[i] as in mfg_dgetrf_batched.
 * All pointers are device pointers; the call is asynchronous on the context's stream.
 * Limit: n <= 256 (larger n returns MFG_ERR_UNSUPPORTED before anything is launched).
 * The kernel's scratch lives in one static device array of 11.4 MB (10.8 MiB) that every GPU
 * loading the library keeps until exit.  Every call looks up that array's address on the
 * context's device (a look-up allocates nothing); the first call on a device may load the
 * library's kernels onto it and should come before any stream capture.  For n > 128 at most
 * 608 warps work on the batch, so those orders can run below the plan path's rate on a GPU
 * with more than 152 SMs.  Calls share the array: calls that overlap on the GPU (different
 * streams or contexts on one device) race and must be serialised by the caller. */
MFG_API int mfg_dgetrf_strided_batched_noalloc(mfg_ctx* ctx, int n, int count, double* a,
                                              int lda, int64_t stride_a, int* piv,
                                              int64_t stride_piv, int nrhs, double* b,
                                              int64_t stride_b, int* sign, int* info);

/* Diagnostics (no MatFlat counterpart): out[i] = a[i] * b[i] computed by the integer-pipe
 * product the dot products use, for n elements (device pointers, asynchronous on the context's
 * stream).  It must equal the IEEE round-to-nearest product bit for bit; the tests check it on
 * random and edge-case operands. */
MFG_API int mfg_selftest_dmul(mfg_ctx* ctx, const double* a, const double* b, double* out,
                              int64_t n);

/* Diagnostics (no MatFlat counterpart): out[i] = a[i] / b[i] computed by the integer-pipe
 * quotient the LU and Cholesky column scalings use (with the reciprocal of b[i] as its per-divisor
 * input), for n elements (device pointers, asynchronous on the context's stream).  It must equal
 * the IEEE round-to-nearest quotient bit for bit. */
MFG_API int mfg_selftest_ddiv(mfg_ctx* ctx, const double* a, const double* b, double* out,
                              int64_t n);

#ifdef __cplusplus
}
#endif

#endif /* MATFLAT_GPU_H */
