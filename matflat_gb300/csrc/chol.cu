// Cholesky factorization A = L*L^T in MatFlat's arithmetic (Factorization.Cholesky,
// MatFlat/Factorization.Cholesky.cs:114-168), plus the fused triangular solves of the batched
// solver.
//
// MatFlat computes L row by row: for row j and k < j
//     t = (A(k,j) - Dot(k, L(j,0:), L(k,0:))) / L(k,k);  L(j,k) = t;  s = s + t*t   (:139-146)
// then L(j,j) = sqrt(A(j,j) - s) if that is > 0, else it throws (:148-157); finally the strict
// upper triangle is cleared (:162-167).  A is read from the upper triangle only.  Each L(j,k) is
// one dot with Internals.Dot's pairwise tree and the diagonal sum s is plain sequential, so the
// kernel may compute L column by column (all L(j,k), j > k, of step k in parallel across lanes)
// and accumulate every row's s as its entries appear, in the same order (k ascending): the values
// are bit-identical.
#include <cuda_runtime.h>

#include "mf_device.cuh"
#include "mf_kernels.h"
#include "mf_solve.cuh"

namespace mfg {

// Factors the n-by-n matrix a (leading dimension lda) in place.  dsum: n doubles of per-warp
// scratch.  Returns 0, or k+1 when A is not positive definite at column k.
template <bool IM>
__device__ int potrf_warp(double* a, int n, long long lda, double* dsum) {
  const int lane = threadIdx.x & 31;
  for (int j = lane; j < n; j += 32) dsum[j] = 0.0;
  __syncwarp();
  for (int k = 0; k < n; ++k) {
    double* colk = a + (long long)k * lda;
    const double s = __dsub_rn(colk[k], dsum[k]);
    if (!positive(s)) return k + 1;  // uniform across the warp
    const double lkk = __dsqrt_rn(s);
    __syncwarp();
    if (lane == 0) colk[k] = lkk;
    for (int j = k + 1 + lane; j < n; j += 32) {
      // Dot(k, a + j, lda, a + k, lda): row j of L against row k of L.
      const double d = exact_dot<IM>(k, a + j, lda, a + k, lda);
      const double t = __ddiv_rn(__dsub_rn(a[(long long)j * lda + k], d), lkk);
      colk[j] = t;
      dsum[j] = __dadd_rn(dsum[j], __dmul_rn(t, t));
    }
    __syncwarp();
  }
  // Clear the strict upper triangle.
  for (int c = 1; c < n; ++c) {
    double* col = a + (long long)c * lda;
    for (int r = lane; r < c; r += 32) col[r] = 0.0;
  }
  __syncwarp();
  return 0;
}

// L y = b (SolveTriangular Lower/NoTrans) then L^T x = y (Lower/Trans) for nrhs right-hand
// sides stored column-major with leading dimension ldb.
__device__ void potrs_warp(const double* l, int n, long long lda, double* b, long long ldb,
                           int nrhs, double* xs, double* acc) {
  const int lane = threadIdx.x & 31;
  const int ldx = n | 1;
  for (int r0 = 0; r0 < nrhs; r0 += RHS_CHUNK) {
    const int nr = nrhs - r0 < RHS_CHUNK ? nrhs - r0 : RHS_CHUNK;
    for (int e = lane; e < nr * n; e += 32) {
      const int r = e / n;
      const int i = e - r * n;
      xs[r * ldx + i] = b[(long long)(r0 + r) * ldb + i];
    }
    __syncwarp();
    warp_solve_dot(l, n, 1, lda, false, xs, ldx, acc, nr);
    warp_solve_sweep(l, n, 1, lda, xs, ldx, nr);
    for (int e = lane; e < nr * n; e += 32) {
      const int r = e / n;
      const int i = e - r * n;
      b[(long long)(r0 + r) * ldb + i] = xs[r * ldx + i];
    }
    __syncwarp();
  }
}

constexpr int SMEM_WARP_DOUBLES_C = SMEM_N + 2 * RHS_CHUNK * (SMEM_N + 1) + 2;

template <int WARPS, bool IM>
__global__ void __launch_bounds__(WARPS * 32) potrf_batched_kernel(BatchArgs p) {
  extern __shared__ double sm_dyn[];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const long long gw = (long long)blockIdx.x * WARPS + warp;
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(p.queue, 1);
    idx = __shfl_sync(FULL_MASK, idx, 0);
    if (idx >= p.count) break;
    const int mat = p.order[idx];
    const int n = p.n[mat];
    const long long lda = p.lda[mat];
    double* a = p.a + p.a_off[mat];
    double* scr = (n <= SMEM_N) ? sm_dyn + warp * SMEM_WARP_DOUBLES_C
                                 : p.gscratch + gw * p.gscratch_stride;
    const int ldx = n | 1;
    const int info = potrf_warp<IM>(a, n, lda, scr);
    if (info == 0 && p.nrhs > 0)
      potrs_warp(a, n, lda, p.b + p.b_off[mat], n, p.nrhs, scr + n, scr + n + RHS_CHUNK * ldx);
    if (lane == 0) p.info[mat] = info;
    __syncwarp();
  }
}

__global__ void __launch_bounds__(32) potrf_single_kernel(double* a, int n, int lda, int* out1,
                                                          double* scratch) {
  const int info = potrf_warp<true>(a, n, lda, scratch);
  if (threadIdx.x == 0) out1[0] = info;
}

template <int WARPS>
static cudaError_t launch_potrf_w(const BatchArgs& args, int ctas, cudaStream_t s) {
  const size_t smem = sizeof(double) * SMEM_WARP_DOUBLES_C * WARPS;
  if (args.hw_mul)
    potrf_batched_kernel<WARPS, false><<<ctas, WARPS * 32, smem, s>>>(args);
  else
    potrf_batched_kernel<WARPS, true><<<ctas, WARPS * 32, smem, s>>>(args);
  return cudaGetLastError();
}

template <int WARPS>
static cudaError_t set_potrf_attr() {
  const size_t smem = sizeof(double) * SMEM_WARP_DOUBLES_C * WARPS;
  cudaError_t e = cudaFuncSetAttribute(potrf_batched_kernel<WARPS, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(potrf_batched_kernel<WARPS, false>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

// Raises the dynamic shared-memory limit of every variant; called once per device, outside any
// stream capture.
cudaError_t init_potrf_attributes() {
  cudaError_t e;
  if ((e = set_potrf_attr<1>()) != cudaSuccess) return e;
  if ((e = set_potrf_attr<2>()) != cudaSuccess) return e;
  if ((e = set_potrf_attr<4>()) != cudaSuccess) return e;
  if ((e = set_potrf_attr<8>()) != cudaSuccess) return e;
  return set_potrf_attr<16>();
}

cudaError_t launch_potrf_batched(const BatchArgs& args, int ctas, int warps, cudaStream_t s) {
  switch (warps) {
    case 1: return launch_potrf_w<1>(args, ctas, s);
    case 2: return launch_potrf_w<2>(args, ctas, s);
    case 4: return launch_potrf_w<4>(args, ctas, s);
    case 8: return launch_potrf_w<8>(args, ctas, s);
    case 16: return launch_potrf_w<16>(args, ctas, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_potrf_single(double* a, int n, int lda, int* out1, double* scratch,
                                cudaStream_t s) {
  potrf_single_kernel<<<1, 32, 0, s>>>(a, n, lda, out1, scratch);
  return cudaGetLastError();
}

}  // namespace mfg
