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

// Factors the n-by-n matrix a (leading dimension lda) in place with a group of G lanes (G = 32:
// one warp per matrix; G < 32: 32/G matrices per warp, which amortises the per-column square root
// and the serial solve steps over several matrices).  dsum: n doubles of per-group scratch.
// Returns 0, or k+1 when A is not positive definite at column k.
template <int G, bool IM>
__device__ int potrf_group(double* a, int n, long long lda, double* dsum) {
  const int lane = group_lane<G>();
  const unsigned gm = group_mask<G>();
  for (int j = lane; j < n; j += G) dsum[j] = 0.0;
  __syncwarp(gm);
  for (int k = 0; k < n; ++k) {
    double* colk = a + (long long)k * lda;
    const double s = __dsub_rn(colk[k], dsum[k]);
    if (!positive(s)) return k + 1;  // uniform across the group
    const double lkk = __dsqrt_rn(s);
    __syncwarp(gm);
    if (lane == 0) colk[k] = lkk;
    for (int j = k + 1 + lane; j < n; j += G) {
      // Dot(k, a + j, lda, a + k, lda): row j of L against row k of L.
      const double d = exact_dot<IM>(k, a + j, lda, a + k, lda);
      const double t = __ddiv_rn(__dsub_rn(a[(long long)j * lda + k], d), lkk);
      colk[j] = t;
      dsum[j] = __dadd_rn(dsum[j], __dmul_rn(t, t));
    }
    __syncwarp(gm);
  }
  // Clear the strict upper triangle.
  for (int c = 1; c < n; ++c) {
    double* col = a + (long long)c * lda;
    for (int r = lane; r < c; r += G) col[r] = 0.0;
  }
  __syncwarp(gm);
  return 0;
}

// L y = b (SolveTriangular Lower/NoTrans) then L^T x = y (Lower/Trans) for nrhs right-hand
// sides stored column-major with leading dimension ldb.
template <int G>
__device__ void potrs_group(const double* l, int n, long long lda, double* b, long long ldb,
                            int nrhs, double* xs, double* acc) {
  const int lane = group_lane<G>();
  const unsigned gm = group_mask<G>();
  const int ldx = n | 1;
  for (int r0 = 0; r0 < nrhs; r0 += RHS_CHUNK) {
    const int nr = nrhs - r0 < RHS_CHUNK ? nrhs - r0 : RHS_CHUNK;
    for (int e = lane; e < nr * n; e += G) {
      const int r = e / n;
      const int i = e - r * n;
      xs[r * ldx + i] = b[(long long)(r0 + r) * ldb + i];
    }
    __syncwarp(gm);
    warp_solve_dot<G>(l, n, 1, lda, false, xs, ldx, acc, nr);
    warp_solve_sweep<G>(l, n, 1, lda, xs, ldx, nr);
    for (int e = lane; e < nr * n; e += G) {
      const int r = e / n;
      const int i = e - r * n;
      b[(long long)(r0 + r) * ldb + i] = xs[r * ldx + i];
    }
    __syncwarp(gm);
  }
}

// Per-warp shared memory: every group keeps its column sums and staged right-hand sides there
// for n <= 4G (G = 32: n <= 128); larger matrices use the group's slice of global scratch.
template <int G>
constexpr int chol_group_doubles() {
  return 4 * G + 2 * RHS_CHUNK * (4 * G + 1) + 2;
}
constexpr int SMEM_WARP_DOUBLES_C = 1240;
static_assert(chol_group_doubles<32>() <= SMEM_WARP_DOUBLES_C, "smem layout");
static_assert(4 * chol_group_doubles<8>() <= SMEM_WARP_DOUBLES_C, "smem layout");
static_assert(8 * chol_group_doubles<4>() <= SMEM_WARP_DOUBLES_C, "smem layout");

template <int WARPS, bool IM, int G>
__global__ void __launch_bounds__(WARPS * 32) potrf_batched_kernel(BatchArgs p) {
  extern __shared__ double sm_dyn[];
  constexpr int GPW = 32 / G;  // groups (matrices in flight) per warp
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int group = lane / G;
  const long long gg = ((long long)blockIdx.x * WARPS + warp) * GPW + group;
  double* smem_group = sm_dyn + warp * SMEM_WARP_DOUBLES_C + group * chol_group_doubles<G>();
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(p.queue, GPW);
    base = __shfl_sync(FULL_MASK, base, 0);
    if (base >= p.count) break;
    const int idx = base + group;
    if (idx < p.count) {
      const int mat = p.order[idx];
      const int n = p.n[mat];
      const long long lda = p.lda[mat];
      double* a = p.a + p.a_off[mat];
      double* scr = (n <= 4 * G) ? smem_group : p.gscratch + gg * p.gscratch_stride;
      const int ldx = n | 1;
      const int info = potrf_group<G, IM>(a, n, lda, scr);
      if (info == 0 && p.nrhs > 0)
        potrs_group<G>(a, n, lda, p.b + p.b_off[mat], n, p.nrhs, scr + n,
                       scr + n + RHS_CHUNK * ldx);
      if ((lane & (G - 1)) == 0) p.info[mat] = info;
    }
    __syncwarp();
  }
}

__global__ void __launch_bounds__(32) potrf_single_kernel(double* a, int n, int lda, int* out1,
                                                          double* scratch) {
  const int info = potrf_group<32, true>(a, n, lda, scratch);
  if (threadIdx.x == 0) out1[0] = info;
}

template <int WARPS, int G>
static cudaError_t launch_potrf_wg(const BatchArgs& args, int ctas, cudaStream_t s) {
  const size_t smem = sizeof(double) * SMEM_WARP_DOUBLES_C * WARPS;
  if (args.hw_mul)
    potrf_batched_kernel<WARPS, false, G><<<ctas, WARPS * 32, smem, s>>>(args);
  else
    potrf_batched_kernel<WARPS, true, G><<<ctas, WARPS * 32, smem, s>>>(args);
  return cudaGetLastError();
}

template <int WARPS>
static cudaError_t launch_potrf_w(const BatchArgs& args, int ctas, cudaStream_t s) {
  switch (args.group) {
    case 4: return launch_potrf_wg<WARPS, 4>(args, ctas, s);
    case 8: return launch_potrf_wg<WARPS, 8>(args, ctas, s);
    case 16: return launch_potrf_wg<WARPS, 16>(args, ctas, s);
    case 32: return launch_potrf_wg<WARPS, 32>(args, ctas, s);
    default: return cudaErrorInvalidValue;
  }
}

template <int WARPS, int G>
static cudaError_t set_potrf_attr_g() {
  const size_t smem = sizeof(double) * SMEM_WARP_DOUBLES_C * WARPS;
  cudaError_t e = cudaFuncSetAttribute(potrf_batched_kernel<WARPS, true, G>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(potrf_batched_kernel<WARPS, false, G>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <int WARPS>
static cudaError_t set_potrf_attr() {
  cudaError_t e;
  if ((e = set_potrf_attr_g<WARPS, 4>()) != cudaSuccess) return e;
  if ((e = set_potrf_attr_g<WARPS, 8>()) != cudaSuccess) return e;
  if ((e = set_potrf_attr_g<WARPS, 16>()) != cudaSuccess) return e;
  return set_potrf_attr_g<WARPS, 32>();
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
