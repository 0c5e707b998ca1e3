// Host-side declarations of the kernel launchers (implemented in the .cu files beside this one).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace mfg {

// Per-warp shared-memory budget of the batched warp kernels: matrices up to SMEM_N keep their
// per-warp vectors in shared memory; larger ones use a slice of a global scratch buffer.
constexpr int SMEM_N = 128;
// Right-hand sides solved together per pass of the warp solvers.
constexpr int RHS_CHUNK = 4;
// Doubles of per-warp scratch needed for a matrix of order n (column sums (two arrays: the LU
// task kernel keeps even and odd columns apart), staged right-hand sides and their accumulators).
inline long long warp_scratch_doubles(int n) {
  const long long ld = (long long)(n | 1);
  return 2LL * n + 2LL * RHS_CHUNK * ld + 2;
}

struct BatchArgs {
  const int* order;          // execution order (longest first)
  const int* n;              // order of each matrix
  const int* lda;            // leading dimension of each matrix
  const long long* a_off;    // element offset of each matrix
  const long long* piv_off;  // element offset of each pivot vector (getrf)
  const long long* b_off;    // element offset of each right-hand-side block
  double* a;
  int* piv;
  double* b;
  int* sign;
  int* info;
  int count;
  int nrhs;
  int* queue;                // work counter, zeroed before every launch
  double* gscratch;          // per-warp scratch for n > SMEM_N
  long long gscratch_stride; // doubles per warp in gscratch
  int hw_mul;                // getrf/potrf: 0 products on the integer pipes, 1 on the FP64 pipe
                             // (DMUL), 2 (getrf) alternating; all give identical bits
  int group;                 // potrf: lanes per matrix (4, 8, 16 or 32)
  int dot_block;             // getrf: pairs per software-pipelined block of the dot loop (2, 4)
  int solve_only;            // getrf/potrf: a holds the factors already; only solve the b blocks
  int split;                 // potrf: split every dot in two halves a step apart
                             // (potrf_group_split; 4n doubles of per-group scratch)
  const int* task_first;     // getrf (double): size-bucketed tasks; task t covers order[first ..
  const int* task_gc;        // first + cnt) worked on by groups of G lanes (gc = G | cnt << 8);
  int ntasks;                // null task_first: one matrix per warp through `order`
  const int* dcount;         // getrf: when set, the number of matrices to take from `order` is
                             // read from device memory (a list built on the device); count
                             // stays the upper bound the grid was sized for
  int minb;                  // getrf (double, size-bucketed tasks): CTAs per SM of the launch
                             // shape (7 or 8 select variants compiled for that occupancy)
  int fma;                   // potrf, getrf (double): the FMA form (fused multiply-adds in any
                             // order, reciprocal scaling): backward-stable factors, not MatFlat's
                             // bits (getrf keeps MatFlat's pivots, see lu_fma.cu)
  double* fbackup;           // getrf FMA form: per-warp copies of the matrices being factored,
  long long fbackup_stride;  // fbackup_stride doubles per warp (32/G groups share it evenly)
  int* fcount;               // getrf FMA form: matrices redone in MatFlat's arithmetic
  double* gsolve;            // getrf/potrf: per-warp global staging of the solves (GSOLVE_STRIDE
                             // / GSOLVE_STRIDE_C doubles per warp) for the orders whose column
                             // sums fit in shared memory, which then holds only those sums and
                             // leaves the rest of the SM's L1 to the matrices; null: the solves
                             // are staged in shared memory too
};
// Doubles per matrix group of BatchArgs::gsolve for getrf (a warp holds up to GETRF_GROUPS groups,
// one matrix each), and per warp for potrf (32/G groups of G lanes, each with
// gsolve_group_doubles(G)).
constexpr long long GSOLVE_STRIDE = (2LL * RHS_CHUNK * (SMEM_N + 1) + 31) / 32 * 32;
constexpr int GETRF_GROUPS = 4;   // 8 lanes per matrix at the smallest
constexpr long long gsolve_group_doubles(int g) {
  return (2LL * RHS_CHUNK * (4 * g + 1) + 31) / 32 * 32;
}
constexpr long long GSOLVE_STRIDE_C = 1280;
static_assert(8 * gsolve_group_doubles(4) <= GSOLVE_STRIDE_C &&
                  4 * gsolve_group_doubles(8) <= GSOLVE_STRIDE_C &&
                  2 * gsolve_group_doubles(16) <= GSOLVE_STRIDE_C &&
                  gsolve_group_doubles(32) <= GSOLVE_STRIDE_C,
              "potrf solve staging");

// Batched Householder QR (+ least-squares solve of nrhs right-hand sides, ldb = m).
template <typename T>
struct QrBatchArgs {
  const int* order;
  const int* m;
  const int* n;
  const int* lda;
  const long long* a_off;
  const long long* rdiag_off;
  const long long* b_off;
  T* a;
  T* rdiag;
  T* b;
  int count;
  int nrhs;
  int* queue;
  T* gscratch;               // per-group coefficient scratch when n + nrhs > qr_smem_coefs
  long long gscratch_stride;
  int group;                 // lanes per matrix: 32 (one warp) or 16, 8, 4
  int solve_only;            // a and rdiag hold the factorization; only solve the b blocks
  int fused;                 // one pass per trailing column and step (qr_warp_fused); the
                             // coefficient scratch then holds 2 (n + nrhs) values
  int fma;                   // double: the FMA form (fused multiply-adds, reciprocal column
                             // scaling): backward-stable factors, not MatFlat's bits
};
// Shared-memory coefficients per matrix of the batched QR for a group size.
int qr_smem_coefs(int group);

template <typename T>
cudaError_t launch_qr_batched(const QrBatchArgs<T>& args, int ctas, int warps, cudaStream_t s);
// Complex batched QR (+ least squares): args holds interleaved (re, im) arrays as doubles with
// complex-element offsets and a real rdiag; one warp per matrix; coefficients of matrices with
// n + nrhs > zqr_smem_coefs() in global scratch (gscratch_stride doubles per warp, 2 per
// coefficient).
int zqr_smem_coefs();
cudaError_t launch_zqr_batched(const QrBatchArgs<double>& args, int ctas, int warps,
                               cudaStream_t s);
// Single-matrix QR kernels; scratch: n + 1 elements.
template <typename T>
cudaError_t launch_qr_single(T* a, int m, int n, int lda, T* rdiag, T* scratch, cudaStream_t s);
template <typename T>
cudaError_t launch_qr_q_single(const T* a, int m, int n, int lda, T* q, int ldq, T* scratch,
                               cudaStream_t s);
template <typename T>
cudaError_t launch_qr_r_single(const T* a, int n, int lda, T* r, int ldr, const T* rdiag,
                               cudaStream_t s);

// Diagnostics: out[i] = the integer-pipe product of a[i] and b[i] (device pointers).
cudaError_t launch_selftest_mul(const double* a, const double* b, double* out, long long n,
                                cudaStream_t s);
cudaError_t launch_selftest_div(const double* a, const double* b, double* out, long long n,
                                cudaStream_t s);

// Batched loss = y^T K^-1 y + log det K and its gradient K^-1 - alpha alpha^T (n <= 128; see
// chol.cu).  Uses args.a (K), args.b (y -> alpha), args.info.
cudaError_t launch_chol_grad_batched(const BatchArgs& args, double* loss, double* grad,
                                     int keep_factor, int ctas, cudaStream_t s);
cudaError_t init_grad_attributes();

// Reverse mode of Cholesky / log-determinant / solve (chol_bwd.cu), one CTA per matrix, n <= 128.
struct CholBwdArgs {
  const int* order;
  const int* n;
  const int* lda;
  const long long* a_off;
  const long long* b_off;
  const double* l;           // the factor L (lower triangle), a_off / lda layout
  const double* lbar;        // cotangent of L (lower triangle), same layout; null: zero
  const double* logdet_bar;  // one per matrix; null: zero
  const double* x;           // forward solution (b_off layout); needed with xbar
  const double* xbar;        // cotangent of x; null: zero
  double* abar;              // output: symmetric gradient, a_off / lda layout
  double* bbar;              // output (optional): A^-1 xbar
  const int* info;           // matrices with info != 0 are skipped; null: none
  int count;
  int* queue;
};
int chol_backward_max_n();
cudaError_t launch_chol_backward(const CholBwdArgs& args, int ctas, cudaStream_t s);

// Batched GEVD front half (chol.cu): B -> L (Cholesky), C = L^-1 A L^-T (leading dimension n).
struct GevdArgs {
  const int* order;
  const int* n;
  const int* lda;
  const int* ldb;
  const long long* a_off;
  const long long* b_off;
  const long long* c_off;
  const double* a;
  double* b;
  double* c;
  int* info;
  int count;
  int* queue;
};
cudaError_t launch_gevd_front_batched(const GevdArgs& args, int ctas, cudaStream_t s);
// Float (elem 1) and Complex (elem 2) overloads: a, b and c point at float / interleaved Complex.
cudaError_t launch_gevd_front_batched_t(const GevdArgs& args, int elem, int ctas, cudaStream_t s);
int gevd_t_ctas_per_sm(int elem);
int gevd_t_warps_per_cta();
int gevd_max_n();
int grad_ctas_per_sm();
int grad_warps_per_cta();

// Strided batches of MulMatVec / Dot / L2Norm / Outer (vec.cu).
cudaError_t launch_gemv_strided(int trans, int m, int n, const double* a, int lda, long long sa,
                                const double* x, int incx, long long sx, double* y, int incy,
                                long long sy, int count, cudaStream_t s);
cudaError_t launch_dot_strided(int n, const double* x, int incx, long long sx, const double* y,
                               int incy, long long sy, double* out, int count, int norm,
                               cudaStream_t s);
cudaError_t launch_ger_strided(int m, int n, const double* x, int incx, long long sx,
                               const double* y, int incy, long long sy, double* a, int lda,
                               long long sa, int count, cudaStream_t s);

// The float (elem 1) and Complex (elem 2, interleaved doubles) overloads of the same strided
// batches.  Dot mode: 0 Dot, 1 L2Norm (float result for float, double for Complex), 2 DotConj.
cudaError_t launch_gemv_strided_t(int elem, int trans, int m, int n, const void* a, int lda,
                                  long long sa, const void* x, int incx, long long sx, void* y,
                                  int incy, long long sy, int count, cudaStream_t s);
cudaError_t launch_dot_strided_t(int elem, int n, const void* x, int incx, long long sx,
                                 const void* y, int incy, long long sy, void* out, int count,
                                 int mode, cudaStream_t s);
cudaError_t launch_ger_strided_t(int elem, int m, int n, const void* x, int incx, long long sx,
                                 const void* y, int incy, long long sy, void* a, int lda,
                                 long long sa, int count, int conj, cudaStream_t s);

// Fills a QR plan's matrices and right-hand sides with the autotuner's synthetic batch (tune.cu).
cudaError_t launch_tune_fill_qr(const QrBatchArgs<double>& args, cudaStream_t s);
// Fills args.a (and args.b when nrhs > 0) with the autotuner's synthetic batch (tune.cu).
cudaError_t launch_tune_fill(const BatchArgs& args, int spd, cudaStream_t s);

// Allocation-free strided batched LU + solve (scratch in a static device array; see lu.cu).
int noalloc_max_n();
cudaError_t launch_getrf_strided_noalloc(double* a, int n, int lda, long long stride_a, int* piv,
                                         long long stride_piv, int nrhs, double* b,
                                         long long stride_b, int* sign, int* info, int count,
                                         int device, int sm_count, cudaStream_t s);

// Mixed-precision LU solve with FP64 refinement (mixed.cu).
int mx_panel_width();
cudaError_t mx_panel_attr(int nmax);
cudaError_t mx_round(const double* a, float* a32, long long total, cudaStream_t s);
// opfmt: 0 no operand copies (FP32 mode), 1 TF32 (FP32 storage), 2 BF16, 3 split TF32 (low
// parts in op_a2 / op_b2); R = mx_op_rows(n).
cudaError_t mx_panel(float* a32, int n, int k, int* ipiv, const int* active, int count,
                     void* op_a, void* op_b, void* op_a2, void* op_b2, int opfmt, int R,
                     cudaStream_t s);
cudaError_t mx_update_fp32(float* a32, int n, int k, const int* active, int count,
                           cudaStream_t s);
int mx_op_rows(int n);
}  // namespace mfg
struct CUtensorMap_st;
namespace mfg {
// Tensor-core trailing update (tcgen05 + TMA); the maps describe the operand copies.  *status is
// set when a bounded device-side wait gives up.
cudaError_t mx_make_tensor_maps(void* op_a, void* op_b, int n, int count, bool tf32,
                                CUtensorMap_st* tm_a, CUtensorMap_st* tm_b);
// mode 0 TF32, 1 BF16, 2 split TF32; tm: the maps of op_a, op_b (and op_a2, op_b2 for mode 2).
cudaError_t mx_update_tc(const CUtensorMap_st* tm, float* a32, int n, int k, int mode, int count,
                         int* status, cudaStream_t s);
cudaError_t mx_tc_attr();
// The exact FP64 fallback of the systems that did not converge, on the device.
cudaError_t mx_fb_gather(const double* a, const double* b, double* x, double* fa, const int* state,
                         int n, int count, int* order, int* fb_count, cudaStream_t s);
cudaError_t mx_fb_finish(int* state, int* info, const int* fb_info, int count, cudaStream_t s);
cudaError_t mx_refine(const double* a, const double* b, double* x, const float* lu,
                      const int* ipiv, int n, int count, int iter, double tol, double* berr,
                      int* iters, int* state, double* anorm, int* active, cudaStream_t s);

// One-time per-device set-up of kernel attributes (dynamic shared-memory limits).
cudaError_t init_getrf_attributes();
cudaError_t init_potrf_attributes();
// Batched LuInverse (getri.cu): per-warp global scratch of getri_scratch_doubles(max n),
// getri_warps_per_cta() warps per CTA, getri_ctas_per_sm() resident CTAs per SM.
long long getri_scratch_doubles(int n);
int getri_warps_per_cta();
int getri_ctas_per_sm();
int getri_max_n();
cudaError_t init_getri_attributes();
cudaError_t launch_getri_batched(const BatchArgs& args, int ctas, cudaStream_t s);
// Float (elem 1) and Complex (elem 2) batched LuInverse: same plan and launch shape, per-warp
// global scratch of getri_t_scratch_bytes(max n, elem) bytes (args.gscratch_stride in doubles).
long long getri_t_scratch_bytes(int n, int elem);
cudaError_t launch_getri_batched_t(const BatchArgs& args, int elem, int ctas, cudaStream_t s);

// Batched LU (+ solve); launched persistent: grid = ctas, WARPS warps per CTA.
// Size-bucketed batched LU (+ solve): one launch per lanes-per-matrix bucket g (8, 16 or 32) over
// the bucket's tasks (args.task_first / task_gc / ntasks / queue).
cudaError_t launch_getrf_tasks(const BatchArgs& args, int ctas, int warps, int g, cudaStream_t s);
// One CTA per matrix (getrf_cta_warps() warps) over `order` (or, with args.task_first, over the
// listed order positions); nmax = the largest order.  Its column sums and, up to order ~2,800,
// the solve's staging live in shared memory; above that the solve is staged in args.gscratch, one
// slice of warp_scratch_doubles(nmax) per CTA (cudaErrorInvalidValue if it is missing).
cudaError_t launch_getrf_cta(const BatchArgs& args, int ctas, int nmax, cudaStream_t s);
int getrf_cta_warps();
// FMA form of the size-bucketed LU (+ solve) (lu_fma.cu): the same tasks and queue as
// launch_getrf_tasks; needs args.fbackup (args.fbackup_stride doubles per launched warp, at least
// (32/g) n^2 for the bucket's largest n) and args.fcount.
cudaError_t launch_getrf_tasks_fma(const BatchArgs& args, int ctas, int warps, int g,
                                   cudaStream_t s);
cudaError_t init_getrf_fma_attributes();
// FMA form for orders above SMEM_N (lu_big.cu): one matrix per CTA, blocked right-looking, over
// the task list (one matrix per task).  Needs args.fbackup (getrf_big_backup_doubles(nmax) per
// launched CTA), args.fcount and args.gscratch (a slice of warp_scratch_doubles(nmax) per CTA).
// cps: CTAs per SM the launch is sized for (2 or 3: selects the register bound); mma: trailing
// updates on the FP64 tensor pipe (mma.sync m8n8k4) instead of fused multiply-adds.
cudaError_t launch_getrf_big_fma(const BatchArgs& args, int ctas, int nmax, int cps, bool mma,
                                 cudaStream_t s);
long long getrf_big_backup_doubles(int nmax);
// Resident form: one matrix per CTA of w warps (2, 4 or 8) over the task list (one matrix per
// task), the matrix held in smem_bytes of dynamic shared memory when it fits.
cudaError_t launch_getrf_blk(const BatchArgs& args, int ctas, int w, int smem_bytes,
                             cudaStream_t s);
// Shared memory (doubles) the resident form needs for one matrix of order n (resident: with the
// copy of the matrix), and the largest dynamic shared memory it may be given (bytes).
long long getrf_blk_smem_doubles(int n, int nrhs, int w, bool resident);
int getrf_blk_smem_max();
cudaError_t launch_getrf_batched(const BatchArgs& args, int ctas, int warps, cudaStream_t s);
// Float and Complex overloads of the batched LU (+ solve): args.a / args.b point at float or
// interleaved (re, im) double arrays, offsets count elements; per-warp global scratch (orders
// above SMEM_N) of W * warp_scratch_doubles(max n) doubles, W = 1 (float) or 2 (Complex).
cudaError_t launch_sgetrf_batched(const BatchArgs& args, int ctas, int warps, cudaStream_t s);
cudaError_t launch_zgetrf_batched(const BatchArgs& args, int ctas, int warps, cudaStream_t s);
// Float and Complex overloads of the batched Cholesky (+ L y = b, then L^T x = y or L^H x = y):
// one warp per matrix; per-warp global scratch (orders above SMEM_N) of W * warp_scratch_doubles
// doubles, W = 1 (float) or 2 (Complex).
cudaError_t launch_spotrf_batched(const BatchArgs& args, int ctas, int warps, cudaStream_t s);
cudaError_t launch_zpotrf_batched(const BatchArgs& args, int ctas, int warps, cudaStream_t s);
cudaError_t init_potrf_t_attributes();
// Batched Cholesky (+ two triangular solves).
cudaError_t launch_potrf_batched(const BatchArgs& args, int ctas, int warps, cudaStream_t s);

// Single-matrix kernels (device pointers).  scratch: at least warp_scratch_doubles(max(m,n))
// doubles of device memory.  out2[0] = sign (getrf) / info (potrf); out2[1] = info (getrf).
cudaError_t launch_getrf_single(double* a, int m, int n, int lda, int* piv, int* out2,
                                double* scratch, cudaStream_t s);
cudaError_t launch_potrf_single(double* a, int n, int lda, int* out1, double* scratch,
                                cudaStream_t s);
// Float and Complex overloads (Complex as interleaved re/im doubles).  LU scratch: m doubles
// (float) or 2m doubles (Complex).
cudaError_t launch_sgetrf_single(float* a, int m, int n, int lda, int* piv, int* out2,
                                 double* scratch, cudaStream_t s);
cudaError_t launch_zgetrf_single(double* a, int m, int n, int lda, int* piv, int* out2,
                                 double* scratch, cudaStream_t s);
// Complex QR (interleaved re/im doubles; rdiag real).  Scratch: 2(n+1) doubles.
cudaError_t launch_zqr_single(double* a, int m, int n, int lda, double* rdiag, double* scratch,
                              cudaStream_t s);
cudaError_t launch_zqr_q_single(const double* a, int m, int n, int lda, double* q, int ldq,
                                double* scratch, cudaStream_t s);
cudaError_t launch_zqr_r_single(const double* a, int n, int lda, double* r, int ldr,
                                const double* rdiag, cudaStream_t s);
// Triangular solve scratch: 4 * (n|1) doubles.
cudaError_t launch_strsv_single(int uplo, int trans, int n, const float* a, int lda, float* x,
                                int incx, double* scratch, cudaStream_t s);
cudaError_t launch_ztrsv_single(int uplo, int trans, int n, const double* a, int lda, double* x,
                                int incx, double* scratch, cudaStream_t s);
cudaError_t launch_sgemm_single(int transa, int transb, int m, int n, int k, const float* a,
                                int lda, const float* b, int ldb, float* c, int ldc,
                                cudaStream_t s);
cudaError_t launch_zgemm_single(int transa, int transb, int m, int n, int k, const double* a,
                                int lda, const double* b, int ldb, double* c, int ldc,
                                cudaStream_t s);
// Cholesky scratch: n doubles.
cudaError_t launch_spotrf_single(float* a, int n, int lda, int* out1, double* scratch,
                                 cudaStream_t s);
cudaError_t launch_zpotrf_single(double* a, int n, int lda, int* out1, double* scratch,
                                 cudaStream_t s);
cudaError_t launch_trsv_single(int uplo, int trans, int n, const double* a, int lda, double* x,
                               int incx, double* scratch, cudaStream_t s);
cudaError_t launch_gemm_single(int transa, int transb, int m, int n, int k, const double* a,
                               int lda, const double* b, int ldb, double* c, int ldc,
                               cudaStream_t s);
// LuInverse after the zero-diagonal check: a holds the LU factors on entry and A^-1 on exit;
// work: n*n doubles.  scratch: warps * 2 * RHS_CHUNK * (n|1) doubles.
cudaError_t launch_getri_single(double* a, int n, int lda, const int* piv, double* work,
                                double* scratch, int warps, cudaStream_t s);
// Float and Complex overloads (Complex as interleaved doubles; work: n*n elements).  Scratch:
// warps * getri_single_scratch_bytes_per_warp(n, elem) bytes (elem 0 double, 1 float, 2 Complex).
long long getri_single_scratch_bytes_per_warp(int n, int elem);
cudaError_t launch_sgetri_single(float* a, int n, int lda, const int* piv, float* work,
                                 void* scratch, int warps, cudaStream_t s);
cudaError_t launch_zgetri_single(double* a, int n, int lda, const int* piv, double* work,
                                 void* scratch, int warps, cudaStream_t s);

}  // namespace mfg
