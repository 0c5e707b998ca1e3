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

#include <cstdlib>
#include <type_traits>

#include "mf_device.cuh"
#include "mf_kernels.h"
#include "mf_scalar.cuh"
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

// The same factorization with every column's dots split in two halves computed one step apart,
// so that a step's lanes hold twice as many (half as long) dot items.  Column c's dot for row j,
// Dot(c, L(j,:), L(c,:)), is split at the pair boundary h(c) (about c/2, with c's parity: an odd
// length keeps its lone first product in the first half); the first half runs at step c-2 (it
// reads columns below h(c) <= c-2 only), the second half, continued from the first half's sum,
// at step c-1 right after column c-1 is finished, and column c finishes at step c.  The sums are
// MatFlat's tree in MatFlat's order, so L is bit-identical to potrf_group's.
// scratch: 4n doubles (the diagonal sums, the complete dots of the next column, and the
// first-half sums of the two columns after it, by parity).
__device__ __forceinline__ int split_point(int c) {
  return (c & 1) ? ((c >> 1) | 1) : ((c >> 1) & ~1);
}

template <int G, bool IM>
__device__ int potrf_group_split(double* a, int n, long long lda, double* dsum) {
  const int lane = group_lane<G>();
  const unsigned gm = group_mask<G>();
  double* full = dsum + n;   // Dot(k, ...) of the column finished next
  double* half = dsum + 2 * n;  // first halves, column parity p at half + p * n
  for (int j = lane; j < n; j += G) {
    dsum[j] = 0.0;
    full[j] = 0.0;
  }
  __syncwarp(gm);
  for (int k = 0; k < n; ++k) {
    double* colk = a + (long long)k * lda;
    const double s = __dsub_rn(colk[k], dsum[k]);
    if (!positive(s)) return k + 1;  // uniform across the group
    const double lkk = __dsqrt_rn(s);
    __syncwarp(gm);
    if (lane == 0) colk[k] = lkk;
    for (int j = k + 1 + lane; j < n; j += G) {
      const double t = __ddiv_rn(__dsub_rn(a[(long long)j * lda + k], full[j]), lkk);
      colk[j] = t;
      dsum[j] = __dadd_rn(dsum[j], __dmul_rn(t, t));
    }
    __syncwarp(gm);
    // Second halves of column c1 = k+1 (rows j > c1) and first halves of c2 = k+2 (rows j > c2).
    const int c1 = k + 1, c2 = k + 2;
    const int r1 = c1 < n ? n - c1 - 1 : 0;
    const int r2 = c2 < n ? n - c2 - 1 : 0;
    const int h1 = split_point(c1), h2 = split_point(c2);
    const double* row1 = a + c1;  // L(c1, t) = row1[t * lda]
    const double* row2 = a + c2;
    for (int d = lane; d < r1 + r2; d += G) {
      const bool second = d < r1;
      const int j = second ? c1 + 1 + d : c2 + 1 + (d - r1);
      const double* rj = a + j;
      const double* rc = second ? row1 : row2;
      double s0;
      int t0, pairs;
      double* dst;
      if (second) {
        // Dot(1) is its lone product; otherwise continue from the first half's sum.
        s0 = c1 == 1 ? xmul<IM>(rj[0], rc[0]) : half[(c1 & 1) * n + j];
        t0 = c1 == 1 ? 1 : h1;
        pairs = (c1 - t0) >> 1;
        dst = full + j;
      } else {
        s0 = (c2 & 1) ? xmul<IM>(rj[0], rc[0]) : 0.0;
        t0 = c2 & 1;
        pairs = (h2 - t0) >> 1;
        dst = half + (c2 & 1) * n + j;
      }
      *dst = exact_dot_pairs<IM>(s0, pairs, rj + (long long)t0 * lda, lda,
                                 rc + (long long)t0 * lda, lda);
    }
    __syncwarp(gm);
  }
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

// The FMA form of the factorization (selected per plan; not MatFlat's bits): the same column
// order and the same failure test (A(k,k) - sum of squares <= 0 -> k+1) as potrf_group, but every
// dot runs as fused multiply-adds in four chains, the column is scaled by the reciprocal of its
// diagonal and the sums of squares accumulate with fused multiply-adds.  The result satisfies the
// usual Cholesky backward-error bound |A - L L^T| <= gamma_(n+2) |L| |L^T|.
// C4: four-chain dots (fma_dot), else two chains (fma_dot2: fewer registers).
template <int G, bool C4 = true>
__device__ int potrf_group_fma(double* a, int n, long long lda, double* dsum, double* rcp) {
  const int lane = group_lane<G>();
  const unsigned gm = group_mask<G>();
  for (int j = lane; j < n; j += G) dsum[j] = 0.0;
  __syncwarp(gm);
  for (int k = 0; k < n; ++k) {
    double* colk = a + (long long)k * lda;
    const double s = __dsub_rn(colk[k], dsum[k]);
    if (!positive(s)) return k + 1;  // uniform across the group
    const double lkk = __dsqrt_rn(s);
    const double rk = __drcp_rn(lkk);
    __syncwarp(gm);
    if (lane == 0) {
      colk[k] = lkk;
      rcp[k] = rk;
    }
    // S lanes per row: 1 while the step has at least half as many rows as the group has lanes,
    // else 2 or 4 lanes share each row's dot (a contiguous part of it each), combined with
    // shuffles within the S lanes.  Every lane runs the same number of rounds (convergent
    // shuffles); lanes past the last row contribute zero.
    const int rows = n - k - 1;
    const int S = (rows * 2 > G || k < 8) ? 1 : (rows * 4 <= G ? 4 : 2);
    const int len = (k + S - 1) / S;
    const int part = lane & (S - 1);
    const int t0 = part * len;
    const int cnt = max(0, min(len, k - t0));
    for (int j0 = k + 1; j0 < n; j0 += G / S) {
      const int j = j0 + lane / S;
      const bool live = j < n;
      double d = 0.0;
      if (live && cnt > 0)
        d = C4 ? fma_dot(cnt, a + j + (long long)t0 * lda, lda, a + k + (long long)t0 * lda, lda)
               : fma_dot2(cnt, a + j + (long long)t0 * lda, lda, a + k + (long long)t0 * lda,
                          lda);
      if (S > 1) {
        d = __dadd_rn(d, __shfl_xor_sync(gm, d, 1, G));
        if (S > 2) d = __dadd_rn(d, __shfl_xor_sync(gm, d, 2, G));
      }
      if (live && part == 0) {
        const double t = __dmul_rn(__dsub_rn(a[(long long)j * lda + k], d), rk);
        colk[j] = t;
        dsum[j] = __fma_rn(t, t, dsum[j]);
      }
    }
    __syncwarp(gm);
  }
  for (int c = 1; c < n; ++c) {
    double* col = a + (long long)c * lda;
    for (int r = lane; r < c; r += G) col[r] = 0.0;
  }
  __syncwarp(gm);
  return 0;
}

// The FMA form's solves, L y = b then L^T x = y, on the factor potrf_group_fma left (rcp[k] =
// 1 / L(k,k) rounded, from the factorization): column sweeps with fused multiply-adds and
// multiplications by the reciprocal diagonal, backward stable like the factorization (not
// MatFlat's bits).  Right-hand sides are staged in xs (leading dimension n | 1).
template <int G>
__device__ void potrs_group_fma(const double* l, int n, long long lda, const double* rcp,
                                double* b, long long ldb, int nrhs, double* xs) {
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
    // Forward: x_t = x_t / L(t,t), then x_i -= L(i,t) x_t below it (column t of L, contiguous).
    for (int t = 0; t < n; ++t) {
      const double rt = rcp[t];
      const double* colt = l + (long long)t * lda;
      double xt[RHS_CHUNK];
#pragma unroll
      for (int r = 0; r < RHS_CHUNK; ++r) xt[r] = r < nr ? __dmul_rn(xs[r * ldx + t], rt) : 0.0;
      __syncwarp(gm);
      if (lane == 0)
        for (int r = 0; r < nr; ++r) xs[r * ldx + t] = xt[r];
      for (int i = t + 1 + lane; i < n; i += G) {
        const double lit = colt[i];
#pragma unroll
        for (int r = 0; r < RHS_CHUNK; ++r)
          if (r < nr) xs[r * ldx + i] = __fma_rn(-lit, xt[r], xs[r * ldx + i]);
      }
      __syncwarp(gm);
    }
    // Backward: x_t = x_t / L(t,t), then x_i -= L(t,i) x_t above it (row t of L).
    for (int t = n - 1; t >= 0; --t) {
      const double rt = rcp[t];
      double xt[RHS_CHUNK];
#pragma unroll
      for (int r = 0; r < RHS_CHUNK; ++r) xt[r] = r < nr ? __dmul_rn(xs[r * ldx + t], rt) : 0.0;
      __syncwarp(gm);
      if (lane == 0)
        for (int r = 0; r < nr; ++r) xs[r * ldx + t] = xt[r];
      for (int i = lane; i < t; i += G) {
        const double lti = l[(long long)i * lda + t];
#pragma unroll
        for (int r = 0; r < RHS_CHUNK; ++r)
          if (r < nr) xs[r * ldx + i] = __fma_rn(-lti, xt[r], xs[r * ldx + i]);
      }
      __syncwarp(gm);
    }
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

// Per-warp shared memory when the solves are staged in global memory (BatchArgs::gsolve): the
// column sums and dot buffers of the warp's groups (4 x 4G doubles each).
constexpr int SMEM_WARP_DOUBLES_CG = 4 * 4 * 32 + 2;

static size_t potrf_smem_bytes(const BatchArgs& args, int warps) {
  return sizeof(double) * (args.gsolve ? SMEM_WARP_DOUBLES_CG : SMEM_WARP_DOUBLES_C) * warps;
}

// Resident warps per SM the FMA and the exact variants are compiled for (caps their registers at
// 65536 / (32 x this)).  Without a bound the exact variants took 130-159 registers, 12 warps/SM.
#ifndef MFG_CHOL_FMA_WARPS
#define MFG_CHOL_FMA_WARPS 24
#endif
#ifndef MFG_CHOL_WARPS
#define MFG_CHOL_WARPS 20
#endif

// FMA = true: the FMA form of the factorization (potrf_group_fma) and of the solves
// (potrs_group_fma); IM then selects four-chain (true) or two-chain (false) dots.
template <int WARPS, bool IM, int G, bool SPLIT = false, bool FMA = false>
__global__ void __launch_bounds__(WARPS * 32, (FMA ? MFG_CHOL_FMA_WARPS : MFG_CHOL_WARPS) / WARPS > 0 ? (FMA ? MFG_CHOL_FMA_WARPS : MFG_CHOL_WARPS) / WARPS : 1)
    potrf_batched_kernel(BatchArgs p) {
  extern __shared__ double sm_dyn[];
  constexpr int GPW = 32 / G;  // groups (matrices in flight) per warp
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int group = lane / G;
  const long long gg = ((long long)blockIdx.x * WARPS + warp) * GPW + group;
  const bool gs = p.gsolve != nullptr;
  double* smem_group = gs ? sm_dyn + warp * SMEM_WARP_DOUBLES_CG + group * 4 * 4 * G
                          : sm_dyn + warp * SMEM_WARP_DOUBLES_C + group * chol_group_doubles<G>();
  double* gsol = gs ? p.gsolve + ((long long)blockIdx.x * WARPS + warp) * GSOLVE_STRIDE_C +
                          group * gsolve_group_doubles(G)
                    : nullptr;
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
      double* sol = (n <= 4 * G && gs) ? gsol : scr + n;
      // FMA form: the reciprocal diagonal for its solves (after the column sums in the group's
      // shared area, or in the solve accumulator the FMA solves do not use).
      double* rcp = (n <= 4 * G && gs) ? scr + n : sol + RHS_CHUNK * ldx;
      int info = 0;
      if (!p.solve_only) {
        if constexpr (FMA)
          info = potrf_group_fma<G, IM>(a, n, lda, scr, rcp);
        else if constexpr (SPLIT)
          info = potrf_group_split<G, IM>(a, n, lda, scr);
        else
          info = potrf_group<G, IM>(a, n, lda, scr);
      }
      if constexpr (FMA) {
        if (info == 0 && p.nrhs > 0) {
          // Solve-only calls form the reciprocals from the stored diagonal: the same values
          // as the factorization's.
          if (p.solve_only) {
            for (int t = lane & (G - 1); t < n; t += G) rcp[t] = __drcp_rn(a[(long long)t * lda + t]);
            __syncwarp(group_mask<G>());
          }
          potrs_group_fma<G>(a, n, lda, rcp, p.b + p.b_off[mat], n, p.nrhs, sol);
        }
      } else if (info == 0 && p.nrhs > 0) {
        potrs_group<G>(a, n, lda, p.b + p.b_off[mat], n, p.nrhs, sol, sol + RHS_CHUNK * ldx);
      }
      if ((lane & (G - 1)) == 0 && !p.solve_only) p.info[mat] = info;
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
  const size_t smem = potrf_smem_bytes(args, WARPS);
  if (args.fma) {
    // dot_block 1: two-chain dots.
    if (args.dot_block == 1)
      potrf_batched_kernel<WARPS, false, G, false, true><<<ctas, WARPS * 32, smem, s>>>(args);
    else
      potrf_batched_kernel<WARPS, true, G, false, true><<<ctas, WARPS * 32, smem, s>>>(args);
    return cudaGetLastError();
  }
  if constexpr (G == 32) {
    if (args.split && !args.hw_mul) {
      potrf_batched_kernel<WARPS, true, G, true><<<ctas, WARPS * 32, smem, s>>>(args);
      return cudaGetLastError();
    }
  }
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
  e = cudaFuncSetAttribute(potrf_batched_kernel<WARPS, true, G, false, true>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(potrf_batched_kernel<WARPS, false, G, false, true>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if constexpr (G == 32) {
    e = cudaFuncSetAttribute(potrf_batched_kernel<WARPS, true, G, true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
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

namespace mfg {

// ---------------------------------------------------------------------------------------------
// Differentiable Cholesky / log-determinant / solve.
//
// For each SPD matrix K and vector y the kernel evaluates
//     loss = y^T K^-1 y + log det K
// and its gradient with respect to K,
//     dloss/dK = K^-1 - alpha alpha^T,   alpha = K^-1 y,
// which is what reverse mode through K = L L^T, z = L^-1 y, loss = z^T z + 2 sum log L_ii gives
// (L-bar = diag(2/L_ii) - 2 tril(alpha z^T), K-bar = L^-T Phi(L^T L-bar) L^-1, symmetrised).
// Every quantity is built from MatFlat's own routines, in MatFlat's arithmetic: L by Cholesky,
// z by SolveTriangular(Lower, NoTrans), alpha by SolveTriangular(Lower, Trans), z^T z by the
// Internals.Dot tree, and K^-1 column by column by the same two solves applied to the columns of
// the identity (MatFlat's LuInverse idiom).  K^-1 is taken from its upper triangle (entries i <= j
// of column j) and mirrored, so the gradient is exactly symmetric; log det K = 2 * sum log L_ii,
// summed in index order.
//
// keep_factor = 1: K is overwritten with L (as Cholesky does) and G receives the gradient.
// keep_factor = 0: K is left untouched and the factor is recomputed inside G's lower triangle
// (no buffer for L), K^-1's strict upper triangle goes to G's strict upper triangle and its
// diagonal to shared memory, and G is completed at the end.
// Per-warp shared memory of the gradient kernel: the 32 staged columns of the identity solves
// (row stride 33), two staged rows of L, the Cholesky diagonal sums and K^-1's diagonal.
constexpr int GRAD_LDX = 33;
constexpr int GRAD_MAX_N = 128;
constexpr int GRAD_SMEM_DOUBLES = GRAD_LDX * GRAD_MAX_N + 4 * GRAD_MAX_N;
constexpr int GRAD_WARPS = 6;   // 6 x 37.9 KB per CTA, one CTA per SM

// SolveTriangular(Lower, NoTrans) in MatFlat's dot form (Blas.SolveTriangular.cs:215-222) on
// every lane's own right-hand side x (x = xs + lane, row stride GRAD_LDX):
// x_i = (x_i - Dot(i, L(i,:), x)) / L(i,i) for i = k0 .. n-1, the dots starting at k0 (k0 = 0: the
// full dots; k0 > 0 only where x_0..x_{k0-1} are known to be +0 and L finite, see chol_w_lanes).
// Rows of L are staged in shared memory (vb, 2n doubles) one ahead of use; products on the FP64
// pipe, blocks of four pairs.
__device__ void lanes_lower_solve(const double* L, int n, long long ld, int k0, double* x,
                                  double* vb) {
  stage_async(vb + (k0 & 1) * n, L + k0, k0, k0 + 1, ld);
  stage_wait();
  for (int i = k0; i < n; i++) {
    const double* li = vb + (i & 1) * n;
    if (i + 1 < n) stage_async(vb + ((i + 1) & 1) * n, L + i + 1, k0, i + 2, ld);
    double s = 0.0;
    int k = k0;
    if ((i - k0) & 1) {
      s = __dmul_rn(li[k0], x[k0 * GRAD_LDX]);
      k = k0 + 1;
    }
    for (; k + 8 <= i; k += 8) {
      double l8[8], v8[8], pr[8];
#pragma unroll
      for (int r = 0; r < 8; r++) {
        l8[r] = li[k + r];
        v8[r] = x[(k + r) * GRAD_LDX];
      }
      mul_block<0, 8, false>(l8, v8, pr);
#pragma unroll
      for (int r = 0; r < 4; r++) s = __dadd_rn(s, __dadd_rn(pr[2 * r], pr[2 * r + 1]));
    }
    for (; k < i; k += 2)
      s = __dadd_rn(s, __dadd_rn(__dmul_rn(li[k], x[k * GRAD_LDX]),
                                 __dmul_rn(li[k + 1], x[(k + 1) * GRAD_LDX])));
    x[i * GRAD_LDX] = __ddiv_rn(__dsub_rn(x[i * GRAD_LDX], s), li[i]);
    stage_wait();
  }
}

// W = L^-1, column by column: MatFlat's SolveTriangular(Lower, NoTrans) (Blas.SolveTriangular.cs:
// 215-222) applied to the columns of the identity, one lane per column (lane l of chunk j0 solves
// column c = j0 + l): x_i = (x_i - Dot(i, L(i,:), x)) / L(i,i).  For i < c, x_i = +0 exactly (0
// minus a signed-zero dot, divided by L(i,i) > 0), so with a finite L the dots of a chunk start at
// k0 = j0 (as in the batched LuInverse: the skipped terms are signed zeros); otherwise at 0.  Rows
// of L are staged in shared memory one ahead of use; products on the FP64 pipe.
// Output layout (G is free above its diagonal): W(i,c), i > c, goes to G(c,i) = G[i*ld + c] (a
// coalesced row of lanes), W(c,c) to wdiag[c].
__device__ void chol_w_lanes(const double* L, int n, long long ld, double* G, double* wdiag,
                             double* xs, double* vb) {
  const int lane = threadIdx.x & 31;
  int nonfinite = 0;
  for (int c = 0; c < n; ++c)
    for (int r = c + 1 + lane; r < n; r += 32)
      nonfinite |= ((dbits(L[(long long)c * ld + r]) >> 52) & 0x7FF) == 0x7FF;
  nonfinite = __any_sync(FULL_MASK, nonfinite);
  for (int j0 = 0; j0 < n; j0 += 32) {
    const bool active = j0 + lane < n;
    const int t = active ? j0 + lane : j0;  // lanes past n repeat lane 0's column
    const int k0 = nonfinite ? 0 : j0;
    double* x = xs + lane;
    for (int i = 0; i < n; i++) x[i * GRAD_LDX] = (i == t) ? 1.0 : 0.0;
    lanes_lower_solve(L, n, ld, k0, x, vb);
    if (active) wdiag[t] = x[t * GRAD_LDX];
    for (int i = j0 + 1; i < n; i++)          // one coalesced row segment per i
      if (active && i > t) G[(long long)i * ld + t] = x[i * GRAD_LDX];
    __syncwarp();
  }
}

// Entry (k, c) of W in the layout chol_w_lanes leaves (W is lower triangular; its structural
// zeros are +0, as the solve produces them).
__device__ __forceinline__ double w_at(const double* G, long long ld, const double* wdiag, int k,
                                       int c) {
  return k == c ? wdiag[c] : (k > c ? G[(long long)k * ld + c] : 0.0);
}

// C(i,j) = Internals.Dot(n, W(:,i), W(:,j)), i <= j, in MatFlat's pairwise order (MulMatMat's
// dot).  W(k,j) = +0 for k < j, so the sum starts at k = j: an even offset from the first pair
// starts with pair (j, j+1), an odd one seeds with the product at j (its pair partner is a zero).
// The skipped terms are signed zeros, which can only change the sign of a zero result; a zero
// result is therefore recomputed over all n terms.
__device__ double wtw_dot(const double* G, long long ld, const double* wdiag, int n, int i, int j) {
  const int p0 = n & 1;
  double s = 0.0;
  int k;
  if (j == 0 && p0) {
    s = __dmul_rn(w_at(G, ld, wdiag, 0, i), w_at(G, ld, wdiag, 0, j));
    k = 1;
  } else if (((j - p0) & 1) == 0) {
    k = j;
  } else {
    s = __dmul_rn(w_at(G, ld, wdiag, j, i), wdiag[j]);
    k = j + 1;
  }
  // Pairs (k, k+1) ... (n-2, n-1); here k > j >= i, so both factors are stored entries (k > i).
  if (k == j && k + 1 < n) {
    // First pair holds the diagonal of column j (and of column i when i == j).
    const double a0 = w_at(G, ld, wdiag, j, i), b0 = wdiag[j];
    const double a1 = G[(long long)(j + 1) * ld + i], b1 = G[(long long)(j + 1) * ld + j];
    s = __dadd_rn(s, __dadd_rn(__dmul_rn(a0, b0), __dmul_rn(a1, b1)));
    k += 2;
  }
  for (; k + 8 <= n; k += 8) {
    double a8[8], b8[8], pr[8];
#pragma unroll
    for (int r = 0; r < 8; r++) {
      a8[r] = G[(long long)(k + r) * ld + i];
      b8[r] = G[(long long)(k + r) * ld + j];
    }
    mul_block<0, 8, false>(a8, b8, pr);
#pragma unroll
    for (int r = 0; r < 4; r++) s = __dadd_rn(s, __dadd_rn(pr[2 * r], pr[2 * r + 1]));
  }
  for (; k + 1 < n; k += 2)
    s = __dadd_rn(s, __dadd_rn(__dmul_rn(G[(long long)k * ld + i], G[(long long)k * ld + j]),
                               __dmul_rn(G[(long long)(k + 1) * ld + i],
                                         G[(long long)(k + 1) * ld + j])));
  if (!nonzero(s)) {
    // The sign of a zero sum depends on the skipped terms: MatFlat's full dot.
    s = 0.0;
    k = 0;
    if (p0) {
      s = __dmul_rn(w_at(G, ld, wdiag, 0, i), w_at(G, ld, wdiag, 0, j));
      k = 1;
    }
    for (; k < n; k += 2)
      s = __dadd_rn(s, __dadd_rn(__dmul_rn(w_at(G, ld, wdiag, k, i), w_at(G, ld, wdiag, k, j)),
                                 __dmul_rn(w_at(G, ld, wdiag, k + 1, i),
                                           w_at(G, ld, wdiag, k + 1, j))));
  }
  return s;
}

// K^-1 = W^T W (MatFlat's MulMatMat(Trans, NoTrans)) for the upper triangle i <= j, one entry per
// lane over the triangle flattened column by column.  C(i,j), i < j, goes to G(j,i) = G[i*ld + j]
// (below G's diagonal: L, if it lived there, is no longer needed), C(j,j) to kdiag[j].
__device__ void chol_wtw_lanes(double* G, int n, long long ld, const double* wdiag, double* kdiag) {
  const int lane = threadIdx.x & 31;
  const long long total = (long long)n * (n + 1) / 2;
  // entry e of column j is (i, j) with e = j(j+1)/2 + i
  int j = 0;
  while ((long long)(j + 1) * (j + 2) / 2 <= lane) j++;
  int i = lane - j * (j + 1) / 2;
  for (long long e = lane; e < total; e += 32) {
    const double c = wtw_dot(G, ld, wdiag, n, i, j);
    if (i == j)
      kdiag[j] = c;
    else
      G[(long long)i * ld + j] = c;
    i += 32;
    while (i > j) {
      i -= j + 1;
      j++;
    }
  }
  __syncwarp();
}

__device__ void chol_grad_warp(double* K, double* G, int n, long long ld, double* y, double* loss,
                               int* info_out, int keep_factor, double* smem) {
  const int lane = threadIdx.x & 31;
  double* xs = smem;                                 // GRAD_LDX * n
  double* vb = smem + GRAD_LDX * GRAD_MAX_N;         // 2n
  double* dsum = vb + 2 * GRAD_MAX_N;                // n
  double* kdiag = dsum + GRAD_MAX_N;                 // n
  double* L;
  if (keep_factor) {
    L = K;
  } else {
    // Copy K's upper triangle into G and factor there.
    for (int c = 0; c < n; ++c)
      for (int r = lane; r <= c; r += 32) G[(long long)c * ld + r] = K[(long long)c * ld + r];
    __syncwarp();
    L = G;
  }
  // Cholesky in place; for keep_factor = 0 the strict upper triangle of G is cleared by potrf,
  // which is fine: it is overwritten below.
  const int info = potrf_group<32, true>(L, n, ld, dsum);
  if (info != 0) {
    if (lane == 0) {
      *info_out = info;
      *loss = __longlong_as_double(0x7FF8000000000000LL);
    }
    __syncwarp();
    return;
  }
  // z = L^-1 y (Lower/NoTrans), quad = z^T z, alpha = L^-T z (Lower/Trans).
  const int ldx = n | 1;
  double* acc = xs + ldx;
  for (int i = lane; i < n; i += 32) xs[i] = y[i];
  __syncwarp();
  warp_solve_dot<32>(L, n, 1, ld, false, xs, ldx, acc, 1);
  const double quad = exact_dot<true>(n, xs, 1, xs, 1);
  double logsum = 0.0;
  for (int i = 0; i < n; ++i) logsum = __dadd_rn(logsum, log(L[(long long)i * ld + i]));
  warp_solve_sweep<32>(L, n, 1, ld, xs, ldx, 1);
  for (int i = lane; i < n; i += 32) y[i] = xs[i];  // alpha
  __syncwarp();
  if (lane == 0) {
    *loss = __dadd_rn(quad, __dmul_rn(2.0, logsum));
    *info_out = 0;
  }
  // W = L^-1 above G's diagonal (and in wdiag, reusing the Cholesky sums' space), then
  // K^-1 = W^T W below it (and in kdiag).
  double* wdiag = dsum;
  chol_w_lanes(L, n, ld, G, wdiag, xs, vb);
  chol_wtw_lanes(G, n, ld, wdiag, kdiag);
  // G = K^-1 - alpha alpha^T (alpha is in y), written to both triangles.
  for (int c = 0; c < n; ++c) {
    for (int r = lane; r <= c; r += 32) {
      const double kinv = (r == c) ? kdiag[c] : G[(long long)r * ld + c];
      const double g = __dsub_rn(kinv, __dmul_rn(y[r], y[c]));
      G[(long long)c * ld + r] = g;
      G[(long long)r * ld + c] = g;
    }
  }
  __syncwarp();
}

__global__ void __launch_bounds__(GRAD_WARPS * 32) chol_grad_batched_kernel(BatchArgs p,
                                                                             double* loss,
                                                                             double* grad,
                                                                             int keep_factor) {
  extern __shared__ double sm_grad[];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(p.queue, 1);
    idx = __shfl_sync(FULL_MASK, idx, 0);
    if (idx >= p.count) break;
    const int mat = p.order[idx];
    const int n = p.n[mat];
    const long long lda = p.lda[mat];
    chol_grad_warp(p.a + p.a_off[mat], grad + p.a_off[mat], n, lda, p.b + p.b_off[mat],
                   loss + mat, p.info + mat, keep_factor, sm_grad + warp * GRAD_SMEM_DOUBLES);
    __syncwarp();
  }
}

static size_t grad_smem_bytes() { return sizeof(double) * GRAD_WARPS * GRAD_SMEM_DOUBLES; }

__global__ void gevd_front_batched_kernel(GevdArgs p);

cudaError_t init_grad_attributes() {
  const cudaError_t e = cudaFuncSetAttribute(chol_grad_batched_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)grad_smem_bytes());
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(gevd_front_batched_kernel,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)grad_smem_bytes());
}

int grad_ctas_per_sm() {
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, chol_grad_batched_kernel,
                                                    GRAD_WARPS * 32, grad_smem_bytes()) !=
      cudaSuccess)
    return 1;
  return blocks < 1 ? 1 : blocks;
}

int grad_warps_per_cta() { return GRAD_WARPS; }

// Front half of the generalized symmetric eigenproblem (Factorization.GevdCore,
// MatFlat/Factorization.Gevd.cs:330-365) for one pair: B = L L^T in place (Cholesky), C filled
// symmetrically from A's upper triangle, every row of C solved with L (SolveTriangular Lower/
// NoTrans at stride n), then every column: C = L^-1 A L^-T (leading dimension n).  One lane per
// row (first pass) and per column (second pass), each running MatFlat's sequential solve.
__device__ void gevd_front_warp(const double* A, long long lda, double* B, long long ldb,
                                double* C, int n, int* info_out, double* smem) {
  const int lane = threadIdx.x & 31;
  double* xs = smem;
  double* vb = smem + GRAD_LDX * GRAD_MAX_N;
  double* dsum = vb + 2 * GRAD_MAX_N;
  const int info = potrf_group<32, true>(B, n, ldb, dsum);
  if (info != 0) {
    if (lane == 0) *info_out = info;
    __syncwarp();
    return;
  }
  for (long long e = lane; e < (long long)n * n; e += 32) {
    const int j = (int)(e / n);
    const int i = (int)(e - (long long)j * n);
    C[(long long)j * n + i] = i <= j ? A[(long long)j * lda + i] : A[(long long)i * lda + j];
  }
  __syncwarp();
  // Rows of C: lane l of a pass solves row r0 + l (lanes past n repeat row r0, not written back).
  for (int r0 = 0; r0 < n; r0 += 32) {
    const bool active = r0 + lane < n;
    const int r = active ? r0 + lane : r0;
    double* x = xs + lane;
    for (int k = 0; k < n; k++) x[k * GRAD_LDX] = C[(long long)k * n + r];
    lanes_lower_solve(B, n, ldb, 0, x, vb);
    if (active)
      for (int k = 0; k < n; k++) C[(long long)k * n + r] = x[k * GRAD_LDX];
    __syncwarp();
  }
  // Columns of C: staged transposed (coalesced reads of each column).
  for (int c0 = 0; c0 < n; c0 += 32) {
    const int nc = min(32, n - c0);
    for (int l = 0; l < 32; l++) {
      const double* col = C + (long long)(c0 + (l < nc ? l : 0)) * n;
      for (int k = lane; k < n; k += 32) xs[k * GRAD_LDX + l] = col[k];
    }
    __syncwarp();
    lanes_lower_solve(B, n, ldb, 0, xs + lane, vb);
    __syncwarp();
    for (int l = 0; l < nc; l++) {
      double* col = C + (long long)(c0 + l) * n;
      for (int k = lane; k < n; k += 32) col[k] = xs[k * GRAD_LDX + l];
    }
    __syncwarp();
  }
  if (lane == 0) *info_out = 0;
  __syncwarp();
}

__global__ void __launch_bounds__(GRAD_WARPS * 32) gevd_front_batched_kernel(GevdArgs p) {
  extern __shared__ double sm_gevd[];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(p.queue, 1);
    idx = __shfl_sync(FULL_MASK, idx, 0);
    if (idx >= p.count) break;
    const int mat = p.order[idx];
    gevd_front_warp(p.a + p.a_off[mat], p.lda[mat], p.b + p.b_off[mat], p.ldb[mat],
                    p.c + p.c_off[mat], p.n[mat], p.info + mat, sm_gevd + warp * GRAD_SMEM_DOUBLES);
  }
}

cudaError_t launch_gevd_front_batched(const GevdArgs& args, int ctas, cudaStream_t s) {
  gevd_front_batched_kernel<<<ctas, GRAD_WARPS * 32, grad_smem_bytes(), s>>>(args);
  return cudaGetLastError();
}

int gevd_max_n() { return GRAD_MAX_N; }

cudaError_t launch_chol_grad_batched(const BatchArgs& args, double* loss, double* grad,
                                     int keep_factor, int ctas, cudaStream_t s) {
  chol_grad_batched_kernel<<<ctas, GRAD_WARPS * 32, grad_smem_bytes(), s>>>(args, loss, grad,
                                                                             keep_factor);
  return cudaGetLastError();
}

}  // namespace mfg

namespace mfg {

// Float overload of Factorization.Cholesky (MatFlat/Factorization.Cholesky.cs:33-87): float
// storage; t = ((double)A(k,j) - Dot) / (double)L(k,k) in double, stored as (float)t; the
// diagonal sum s += t*t stays in double with the unrounded t; L(j,j) = (float)sqrt(s).
// One warp per matrix; dsum: n doubles.  Returns 0, or k+1 (not positive definite at column k).
__device__ int spotrf_warp(float* a, int n, long long lda, double* dsum) {
  const int lane = threadIdx.x & 31;
  for (int j = lane; j < n; j += 32) dsum[j] = 0.0;
  __syncwarp();
  for (int k = 0; k < n; ++k) {
    float* colk = a + (long long)k * lda;
    const double s = __dsub_rn((double)colk[k], dsum[k]);
    if (!positive(s)) return k + 1;  // uniform across the warp
    const float lkk = __double2float_rn(__dsqrt_rn(s));
    __syncwarp();
    if (lane == 0) colk[k] = lkk;
    for (int j = k + 1 + lane; j < n; j += 32) {
      const double d = exact_dot_f(k, a + j, lda, a + k, lda);
      const double t = __ddiv_rn(__dsub_rn((double)a[(long long)j * lda + k], d), (double)lkk);
      colk[j] = __double2float_rn(t);
      dsum[j] = __dadd_rn(dsum[j], __dmul_rn(t, t));
    }
    __syncwarp();
  }
  for (int c = 1; c < n; ++c)
    for (int r = lane; r < c; r += 32) a[(long long)c * lda + r] = 0.0f;
  __syncwarp();
  return 0;
}

// Complex overload (Factorization.Cholesky.cs:195-249): t = (A(k,j) - DotConj(L(j,:), L(k,:)))
// / L(k,k); L(j,k) = conj(t); s += t.re^2 + t.im^2; L(j,j) = Complex(sqrt(A(j,j).re - s), 0).
__device__ int zpotrf_warp(zdouble* a, int n, long long lda, double* dsum) {
  const int lane = threadIdx.x & 31;
  for (int j = lane; j < n; j += 32) dsum[j] = 0.0;
  __syncwarp();
  for (int k = 0; k < n; ++k) {
    zdouble* colk = a + (long long)k * lda;
    const double s = __dsub_rn(colk[k].re, dsum[k]);
    if (!positive(s)) return k + 1;
    const zdouble lkk = zmake(__dsqrt_rn(s), 0.0);
    __syncwarp();
    if (lane == 0) colk[k] = lkk;
    for (int j = k + 1 + lane; j < n; j += 32) {
      const zdouble d = zdot<true>(k, a + j, lda, a + k, lda);
      const zdouble t = zdiv(zsub(a[(long long)j * lda + k], d), lkk);
      colk[j] = zconj(t);
      dsum[j] = __dadd_rn(dsum[j], __dadd_rn(__dmul_rn(t.re, t.re), __dmul_rn(t.im, t.im)));
    }
    __syncwarp();
  }
  for (int c = 1; c < n; ++c)
    for (int r = lane; r < c; r += 32) a[(long long)c * lda + r] = zmake(0.0, 0.0);
  __syncwarp();
  return 0;
}

__global__ void __launch_bounds__(32) spotrf_single_kernel(float* a, int n, int lda, int* out1,
                                                           double* dsum) {
  const int info = spotrf_warp(a, n, lda, dsum);
  if (threadIdx.x == 0) out1[0] = info;
}

__global__ void __launch_bounds__(32) zpotrf_single_kernel(zdouble* a, int n, int lda, int* out1,
                                                           double* dsum) {
  const int info = zpotrf_warp(a, n, lda, dsum);
  if (threadIdx.x == 0) out1[0] = info;
}

// Element types of the batched float / Complex Cholesky: the factorization, and the solve
// arithmetic of L y = b (Lower/NoTrans, dot form) and of L^T x = y (float, Lower/Trans) or
// L^H x = y (Complex, Lower/ConjTrans), both column sweeps over the rows of L.
struct SChol {
  using T = float;
  using Fwd = SSolve;
  using Bwd = SSolve;
  static __device__ __forceinline__ int factor(T* a, int n, long long lda, double* dsum) {
    return spotrf_warp(a, n, lda, dsum);
  }
};
struct ZChol {
  using T = zdouble;
  using Fwd = ZSolve<false>;
  using Bwd = ZSolve<true>;
  static __device__ __forceinline__ int factor(T* a, int n, long long lda, double* dsum) {
    return zpotrf_warp(a, n, lda, dsum);
  }
};

constexpr int SMEM_WARP_DOUBLES_T = SMEM_N + 2 * RHS_CHUNK * (SMEM_N + 1) + 2;

// Per-warp scratch, in doubles: dsum (n), staged right-hand sides (W * RHS_CHUNK * (n|1)) and
// their accumulators (the same), W = 1 (float: double sums) or 2 (Complex); shared memory for
// n <= SMEM_N, else the warp's slice of global scratch.
template <int WARPS, class C>
__global__ void __launch_bounds__(WARPS * 32) potrf_batched_t_kernel(BatchArgs p) {
  using T = typename C::T;
  using Acc = typename C::Fwd::Acc;
  constexpr int W = sizeof(Acc) / sizeof(double);
  extern __shared__ double sm_dyn[];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const long long gw = (long long)blockIdx.x * WARPS + warp;
  T* abase = reinterpret_cast<T*>(p.a);
  T* bbase = reinterpret_cast<T*>(p.b);
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(p.queue, 1);
    idx = __shfl_sync(FULL_MASK, idx, 0);
    if (idx >= p.count) break;
    const int mat = p.order[idx];
    const int n = p.n[mat];
    const long long lda = p.lda[mat];
    T* a = abase + p.a_off[mat];
    double* scr = (n <= SMEM_N) ? sm_dyn + warp * W * SMEM_WARP_DOUBLES_T
                                 : p.gscratch + gw * p.gscratch_stride;
    const int ldx = n | 1;
    const int info = p.solve_only ? 0 : C::factor(a, n, lda, scr);
    if (info == 0 && p.nrhs > 0) {
      T* b = bbase + p.b_off[mat];
      T* xs = (T*)(scr + n);
      Acc* acc = (Acc*)(scr + n + W * RHS_CHUNK * ldx);
      for (int r0 = 0; r0 < p.nrhs; r0 += RHS_CHUNK) {
        const int nr = p.nrhs - r0 < RHS_CHUNK ? p.nrhs - r0 : RHS_CHUNK;
        for (int e = lane; e < nr * n; e += 32) {
          const int r = e / n;
          const int i = e - r * n;
          xs[r * ldx + i] = b[(long long)(r0 + r) * n + i];
        }
        __syncwarp();
        warp_solve_dot<32, typename C::Fwd>(a, n, 1, lda, false, xs, ldx, acc, nr);
        warp_solve_sweep<32, typename C::Bwd>(a, n, 1, lda, xs, ldx, nr);
        for (int e = lane; e < nr * n; e += 32) {
          const int r = e / n;
          const int i = e - r * n;
          b[(long long)(r0 + r) * n + i] = xs[r * ldx + i];
        }
        __syncwarp();
      }
    }
    if (lane == 0 && !p.solve_only) p.info[mat] = info;
    __syncwarp();
  }
}

template <int WARPS, class C>
static size_t potrf_t_smem() {
  constexpr int W = sizeof(typename C::Fwd::Acc) / sizeof(double);
  return sizeof(double) * W * SMEM_WARP_DOUBLES_T * WARPS;
}

template <int WARPS, class C>
static cudaError_t launch_potrf_t_w(const BatchArgs& args, int ctas, cudaStream_t s) {
  potrf_batched_t_kernel<WARPS, C><<<ctas, WARPS * 32, potrf_t_smem<WARPS, C>(), s>>>(args);
  return cudaGetLastError();
}

// At most 8 warps per CTA; 16-warp plan shapes launch twice the CTAs (same warp count).
template <class C>
static cudaError_t launch_potrf_t(const BatchArgs& args, int ctas, int warps, cudaStream_t s) {
  if (warps > 8) {
    ctas *= warps / 8;
    warps = 8;
  }
  switch (warps) {
    case 1: return launch_potrf_t_w<1, C>(args, ctas, s);
    case 2: return launch_potrf_t_w<2, C>(args, ctas, s);
    case 4: return launch_potrf_t_w<4, C>(args, ctas, s);
    case 8: return launch_potrf_t_w<8, C>(args, ctas, s);
    default: return cudaErrorInvalidValue;
  }
}

template <class C>
static cudaError_t set_potrf_t_attrs() {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(potrf_batched_t_kernel<1, C>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)potrf_t_smem<1, C>())) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(potrf_batched_t_kernel<2, C>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)potrf_t_smem<2, C>())) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(potrf_batched_t_kernel<4, C>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)potrf_t_smem<4, C>())) != cudaSuccess)
    return e;
  return cudaFuncSetAttribute(potrf_batched_t_kernel<8, C>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)potrf_t_smem<8, C>());
}

// Float and Complex overloads of the GEVD front half (Factorization.GevdCore, MatFlat/
// Factorization.Gevd.cs:282-318 float, :378-422 Complex).  MatFlat solves every ROW of C in
// place at stride n (the Complex overload conjugates the row first and conjugates the solution
// back, :407-418), then every column.  The kernel runs both passes as row solves, one lane per
// row, so that a warp's loads of the rows' entries are coalesced:
//   D = conj(C)            the fill (for the real types C itself, which is symmetric)
//   D <- rows of D solved  MatFlat's row pass, before its conjugation back
//   E = D^H                row c of E is column c of MatFlat's C after the row pass
//   E <- rows of E solved  MatFlat's column pass
//   C = E^T
// Each row solve is SolveTriangular(Lower, NoTrans) in MatFlat's dot order (the stride does not
// change the arithmetic), with the rows of L staged in shared memory one ahead of use.  One warp
// per pair.  MFG_GEVD_LANES=0 selects the earlier form of the same passes, column solves of
// warp_solve_dot with the accumulators of a few columns in shared memory; MFG_GEVD_LANES=2 moves
// the Complex products to the integer pipes (ZSolveIM; measured slower at n=64, 138k against
// 153k pairs/s, with 116 registers a thread against 80).
constexpr int GEVD_T_WARPS = 8;

__device__ __forceinline__ float gevd_conj(float v) { return v; }
__device__ __forceinline__ zdouble gevd_conj(zdouble v) { return zconj(v); }

template <int W>
constexpr int gevd_rhs() {
  return 8 / W;
}
// Per-warp shared memory in doubles: the Cholesky sums, then the staged rows of L (lanes form)
// or the dot accumulators (warp_solve_dot form).
template <int W>
constexpr int gevd_t_warp_doubles() {
  return GRAD_MAX_N + W * gevd_rhs<W>() * GRAD_MAX_N;
}

// Copies src[k*stride] to dst[k] (shared memory) for k in [k0, k1) asynchronously, in 4-byte
// (float) or 8-byte (Complex: two per element) pieces, which the arrays' alignment allows.
template <class T>
__device__ __forceinline__ void stage_async_t(T* dst, const T* src, int k0, int k1,
                                              long long stride) {
  const int lane = threadIdx.x & 31;
  if constexpr (sizeof(T) == 4) {
    for (int k = k0 + lane; k < k1; k += 32) {
      const unsigned d = (unsigned)__cvta_generic_to_shared(dst + k);
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src + k * stride)
                   : "memory");
    }
  } else {
    constexpr int P = sizeof(T) / 8;
    for (int q = lane; q < (k1 - k0) * P; q += 32) {
      const int k = k0 + q / P;
      const int h = q - (q / P) * P;
      const unsigned d =
          (unsigned)__cvta_generic_to_shared(reinterpret_cast<double*>(dst + k) + h);
      const double* sp = reinterpret_cast<const double*>(src + k * stride) + h;
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(sp) : "memory");
    }
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// Every row of the n-by-n matrix M (leading dimension n) solved in place with the lower factor
// L (leading dimension ld): x_i = (x_i - Dot(i, L(i,:), x)) / L(i,i), one lane per row.
// vb: 2n elements of shared memory.
template <class Tr>
__device__ void gevd_rows_solve(const typename Tr::T* L, int n, long long ld, typename Tr::T* M,
                                typename Tr::T* vb) {
  using T = typename Tr::T;
  using Acc = typename Tr::Acc;
  const int lane = threadIdx.x & 31;
  for (int r0 = 0; r0 < n; r0 += 32) {
    const bool active = r0 + lane < n;
    T* x = M + r0 + (active ? lane : 0);
    stage_async_t(vb, L, 0, 1, ld);
    stage_wait();
    for (int i = 0; i < n; i++) {
      const T* li = vb + (i & 1) * n;
      if (i + 1 < n) stage_async_t(vb + ((i + 1) & 1) * n, L + i + 1, 0, i + 2, ld);
      if (active) {
        const T v = x[(long long)i * n];
        T out;
        if (i == 0) {
          out = Tr::fin0(v, li[0], false);
        } else {
          Acc s = Tr::zero();
          int k = 0;
          if (i & 1) {
            s = Tr::prod(li[0], x[0]);
            k = 1;
          }
          for (; k + 8 <= i; k += 8) {
            T l8[8], v8[8];
#pragma unroll
            for (int r = 0; r < 8; r++) {
              l8[r] = li[k + r];
              v8[r] = x[(long long)(k + r) * n];
            }
#pragma unroll
            for (int r = 0; r < 4; r++)
              s = Tr::pair(s, l8[2 * r], v8[2 * r], l8[2 * r + 1], v8[2 * r + 1]);
          }
          for (; k < i; k += 2)
            s = Tr::pair(s, li[k], x[(long long)k * n], li[k + 1], x[(long long)(k + 1) * n]);
          out = Tr::fin(v, s, li[i], false);
        }
        x[(long long)i * n] = out;
      }
      stage_wait();
    }
  }
}

// M <- M^H (CONJ) or M^T in place (n-by-n, leading dimension n).
template <bool CONJ, class T>
__device__ void gevd_transpose(T* M, int n) {
  const int lane = threadIdx.x & 31;
  auto cj = [](T v) { return CONJ ? gevd_conj(v) : v; };
  for (long long e = lane; e < (long long)n * n; e += 32) {
    const int j = (int)(e / n);
    const int i = (int)(e - (long long)j * n);
    if (i < j) {
      const T lo = M[(long long)i * n + j];
      const T up = M[e];
      M[e] = cj(lo);
      M[(long long)i * n + j] = cj(up);
    } else if (i == j && CONJ) {
      M[e] = cj(M[e]);
    }
  }
  __syncwarp();
}

template <class C, int MODE>
__global__ void __launch_bounds__(GEVD_T_WARPS * 32) gevd_front_batched_t_kernel(GevdArgs p) {
  using T = typename C::T;
  using Tr = typename C::Fwd;  // SolveTriangular(Lower, NoTrans): the dot form
  using TrRows = std::conditional_t<MODE == 2 && sizeof(T) == 16, ZSolveIM, Tr>;
  constexpr bool LANES = MODE != 0;
  using Acc = typename Tr::Acc;
  constexpr int W = sizeof(Acc) / sizeof(double);
  extern __shared__ double sm_gevd_t[];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  double* dsum = sm_gevd_t + warp * gevd_t_warp_doubles<W>();
  Acc* acc = reinterpret_cast<Acc*>(dsum + GRAD_MAX_N);
  T* vb = reinterpret_cast<T*>(dsum + GRAD_MAX_N);
  const T* abase = reinterpret_cast<const T*>(p.a);
  T* bbase = reinterpret_cast<T*>(p.b);
  T* cbase = reinterpret_cast<T*>(p.c);
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(p.queue, 1);
    idx = __shfl_sync(FULL_MASK, idx, 0);
    if (idx >= p.count) break;
    const int mat = p.order[idx];
    const int n = p.n[mat];
    const long long lda = p.lda[mat];
    const long long ldb = p.ldb[mat];
    const T* A = abase + p.a_off[mat];
    T* B = bbase + p.b_off[mat];
    T* Cm = cbase + p.c_off[mat];
    const int info = C::factor(B, n, ldb, dsum);
    if (info != 0) {
      if (lane == 0) p.info[mat] = info;
      __syncwarp();
      continue;
    }
    // MatFlat's C (Gevd.cs:393-406): C(i,k) = A(i,k) for i < k, conj(A(k,i)) for i > k, A(i,i)
    // on the diagonal.  Stored: D = conj(C) (lanes form) or C^H (warp_solve_dot form).
    for (long long e = lane; e < (long long)n * n; e += 32) {
      const int j = (int)(e / n);
      const int i = (int)(e - (long long)j * n);
      // element (i, j) of the stored matrix, from row r, column c of C, conjugated
      const int r = LANES ? i : j;
      const int c = LANES ? j : i;
      T v;
      if (r < c)
        v = gevd_conj(A[(long long)c * lda + r]);
      else if (r > c)
        v = A[(long long)r * lda + c];
      else
        v = gevd_conj(A[(long long)r * lda + r]);
      Cm[e] = v;
    }
    __syncwarp();
    if constexpr (LANES) {
      gevd_rows_solve<TrRows>(B, n, ldb, Cm, vb);
      gevd_transpose<true>(Cm, n);
      gevd_rows_solve<TrRows>(B, n, ldb, Cm, vb);
      gevd_transpose<false>(Cm, n);
    } else {
      for (int c0 = 0; c0 < n; c0 += gevd_rhs<W>()) {
        const int nr = min(gevd_rhs<W>(), n - c0);
        warp_solve_dot<32, Tr>(B, n, 1, ldb, false, Cm + (long long)c0 * n, n, acc, nr);
      }
      gevd_transpose<true>(Cm, n);   // back to rows: C(i,k) = conj(C^H(k,i))
      for (int c0 = 0; c0 < n; c0 += gevd_rhs<W>()) {
        const int nr = min(gevd_rhs<W>(), n - c0);
        warp_solve_dot<32, Tr>(B, n, 1, ldb, false, Cm + (long long)c0 * n, n, acc, nr);
      }
    }
    if (lane == 0) p.info[mat] = 0;
    __syncwarp();
  }
}

template <class C>
static size_t gevd_t_smem() {
  constexpr int W = sizeof(typename C::Fwd::Acc) / sizeof(double);
  return sizeof(double) * gevd_t_warp_doubles<W>() * GEVD_T_WARPS;
}

// MFG_GEVD_LANES: 0 column solves, 1 (default) row solves, 2 row solves with the Complex
// products on the integer pipes (float: the same kernel as 1).
static int gevd_mode() {
  static const int mode = [] {
    const char* v = std::getenv("MFG_GEVD_LANES");
    if (v && v[0] == '0') return 0;
    if (v && v[0] == '2') return 2;
    return 1;
  }();
  return mode;
}

template <class C, int MODE>
static cudaError_t gevd_t_launch(const GevdArgs& args, int ctas, cudaStream_t s) {
  gevd_front_batched_t_kernel<C, MODE><<<ctas, GEVD_T_WARPS * 32, gevd_t_smem<C>(), s>>>(args);
  return cudaGetLastError();
}

cudaError_t launch_gevd_front_batched_t(const GevdArgs& args, int elem, int ctas,
                                        cudaStream_t s) {
  const int mode = gevd_mode();
  if (elem == 1) return mode == 0 ? gevd_t_launch<SChol, 0>(args, ctas, s)
                                  : gevd_t_launch<SChol, 1>(args, ctas, s);
  return mode == 0   ? gevd_t_launch<ZChol, 0>(args, ctas, s)
         : mode == 1 ? gevd_t_launch<ZChol, 1>(args, ctas, s)
                     : gevd_t_launch<ZChol, 2>(args, ctas, s);
}

template <class C, int MODE>
static int gevd_t_blocks() {
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, gevd_front_batched_t_kernel<C, MODE>,
                                                    GEVD_T_WARPS * 32, gevd_t_smem<C>()) !=
      cudaSuccess)
    return 1;
  return b < 1 ? 1 : b;
}

// Resident CTAs per SM of the float / Complex kernel that the current mode launches.
int gevd_t_ctas_per_sm(int elem) {
  const int mode = gevd_mode();
  if (elem == 1) return mode == 0 ? gevd_t_blocks<SChol, 0>() : gevd_t_blocks<SChol, 1>();
  return mode == 0 ? gevd_t_blocks<ZChol, 0>()
                   : mode == 1 ? gevd_t_blocks<ZChol, 1>() : gevd_t_blocks<ZChol, 2>();
}

int gevd_t_warps_per_cta() { return GEVD_T_WARPS; }

cudaError_t init_potrf_t_attributes() {
  cudaError_t e = set_potrf_t_attrs<SChol>();
  if (e != cudaSuccess) return e;
  e = set_potrf_t_attrs<ZChol>();
  if (e != cudaSuccess) return e;
  const int ss = (int)gevd_t_smem<SChol>(), zs = (int)gevd_t_smem<ZChol>();
  const void* ks[5] = {(const void*)gevd_front_batched_t_kernel<SChol, 0>,
                       (const void*)gevd_front_batched_t_kernel<SChol, 1>,
                       (const void*)gevd_front_batched_t_kernel<ZChol, 0>,
                       (const void*)gevd_front_batched_t_kernel<ZChol, 1>,
                       (const void*)gevd_front_batched_t_kernel<ZChol, 2>};
  for (int i = 0; i < 5; i++)
    if ((e = cudaFuncSetAttribute(ks[i], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  i < 2 ? ss : zs)) != cudaSuccess)
      return e;
  return cudaSuccess;
}

cudaError_t launch_spotrf_batched(const BatchArgs& args, int ctas, int warps, cudaStream_t s) {
  return launch_potrf_t<SChol>(args, ctas, warps, s);
}
cudaError_t launch_zpotrf_batched(const BatchArgs& args, int ctas, int warps, cudaStream_t s) {
  return launch_potrf_t<ZChol>(args, ctas, warps, s);
}

cudaError_t launch_spotrf_single(float* a, int n, int lda, int* out1, double* scratch,
                                 cudaStream_t s) {
  spotrf_single_kernel<<<1, 32, 0, s>>>(a, n, lda, out1, scratch);
  return cudaGetLastError();
}

cudaError_t launch_zpotrf_single(double* a, int n, int lda, int* out1, double* scratch,
                                 cudaStream_t s) {
  zpotrf_single_kernel<<<1, 32, 0, s>>>((zdouble*)a, n, lda, out1, scratch);
  return cudaGetLastError();
}

}  // namespace mfg
