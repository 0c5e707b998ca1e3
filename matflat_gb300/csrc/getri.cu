// Batched Factorization.LuInverse (MatFlat/Factorization.LuInverse.cs:123-199): A^-1 from the LU
// factors and pivots of Factorization.Lu, bit-identical to MatFlat.
//
// MatFlat clears A, writes the columns of P^T (a[lda*piv[j] + j] = 1.0, :165-172), then solves
// every column with the unit lower factor (trsv Lower/NoTrans, dot form, against L with its
// diagonal set to 1.0: x_i = (x_i - Dot(i, L(i,:), x)) / 1.0, :174-182) and then with the upper
// factor (trsv Upper/NoTrans, column sweep: x_i /= U(i,i); x_k -= U(k,i) * x_i for k < i,
// :184-192 and Blas.SolveTriangular.cs:197-200, MulSub :397-421).
//
// GB300 mapping: one warp per matrix, one lane per right-hand side.  Lane l of chunk j solves the
// column c = piv[32j + l], whose right-hand side is the unit vector at row t = 32j + l.  Each lane
// runs MatFlat's sequential solve on its own column, so every FP64 instruction has 32 useful
// lanes and no shuffles; the factor entries are warp-uniform loads.  The columns live in shared
// memory (row stride 33: conflict-free for the per-lane sweeps and the transposed write-back).
//
// Zero skipping, exact: for k < t the lower solve leaves x_k = +0 (x_k = 0 - Dot(...) and any
// signed zero subtracted from +0 gives +0), so the terms L(i,k) * x_k with k < t are signed zeros
// as long as L is finite, and adding a signed zero to a partial sum changes at most the sign of a
// zero sum, which x_i = b_i - s then removes.  A chunk therefore starts its dots at k0 = 32j: an
// even-length dot pairs (k0, k0+1), ...; an odd-length one seeds the sum with the product at k0
// (MatFlat's pair (k0-1, k0) whose first product is a zero).  When L holds a NaN or an infinity
// (0 * inf = NaN must propagate) the matrix runs the full dots from k0 = 0, MatFlat's own order.
#include <cuda_runtime.h>

#include "mf_device.cuh"
#include "mf_kernels.h"
#include "mf_scalar.cuh"
#include "mf_solve.cuh"

namespace mfg {

constexpr int INV_WARPS = 6;  // 6 x 33.8 KB of staged columns per CTA, one CTA per SM
constexpr int INV_LDX = 33;     // row stride (doubles) of the staged columns
constexpr int INV_SMEM_N = 128; // orders whose staged columns fit in shared memory
constexpr int INV_SMEM_WARP = INV_LDX * INV_SMEM_N + 2 * INV_SMEM_N;  // doubles per warp
constexpr int INV_MAX_N = INV_SMEM_WARP / 2;  // largest order (two factor buffers in smem)

long long getri_scratch_doubles(int n) {
  long long d = (long long)n * n;                         // packed L rows + packed U columns
  if (n > INV_SMEM_N) d += (long long)INV_LDX * n;        // staged columns for large orders
  return (d + 31) / 32 * 32;
}

int getri_warps_per_cta() { return INV_WARPS; }

size_t getri_smem_bytes() { return sizeof(double) * INV_WARPS * INV_SMEM_WARP; }

int getri_max_n() { return INV_MAX_N; }

// Products of the solves: exact zeros are frequent here (the unit right-hand sides), so the
// integer-pipe product keeps them on the integer path.
template <int IM>
__device__ __forceinline__ double zmul_(double a, double b) {
  if constexpr (IM == 1) return imul_rn<true>(a, b);
  else return __dmul_rn(a, b);
}

// One matrix.  lp: packed rows of the strict lower factor (row i at i(i-1)/2, i entries);
// up: packed columns of U (column i at i(i+1)/2, i+1 entries, diagonal last).
template <int IM>
__device__ void getri_warp(double* a, int n, long long lda, const int* piv, double* lp,
                           double* xs, double* vb, int* info_out) {
  const int lane = threadIdx.x & 31;
  double* up = lp + (long long)n * (n - 1) / 2;

  // Singularity check before anything is written (LuInverse.cs:145-152): first zero diagonal.
  int bad = INT_MAX;
  for (int j = lane; j < n; j += 32)
    if (a[(long long)j * lda + j] == 0.0) bad = min(bad, j);
  for (int o = 16; o > 0; o >>= 1) bad = min(bad, __shfl_xor_sync(FULL_MASK, bad, o));
  if (bad != INT_MAX) {
    if (lane == 0) *info_out = bad + 1;
    return;
  }
  // piv must be a permutation of 0..n-1 (what Factorization.Lu returns); the staging area is the
  // bitmap.  Otherwise the matrix is left untouched and info = -1.
  unsigned* seen = reinterpret_cast<unsigned*>(xs);
  const int words = (n + 31) >> 5;
  for (int w = lane; w < words; w += 32) seen[w] = 0u;
  __syncwarp();
  int badp = 0;
  for (int t = lane; t < n; t += 32) {
    const int c = piv[t];
    if (c < 0 || c >= n) {
      badp = 1;
    } else if (atomicOr(&seen[c >> 5], 1u << (c & 31)) & (1u << (c & 31))) {
      badp = 1;
    }
  }
  if (__any_sync(FULL_MASK, badp)) {
    if (lane == 0) *info_out = -1;
    return;
  }

  // Repack the factors (coalesced reads of A's columns) and test L for non-finite entries.
  int nonfinite = 0;
  for (long long e = lane; e < (long long)n * n; e += 32) {
    const int j = (int)(e / n);
    const int r = (int)(e - (long long)j * n);
    const double v = a[(long long)j * lda + r];
    if (r > j) {
      lp[(long long)r * (r - 1) / 2 + j] = v;
      nonfinite |= ((dbits(v) >> 52) & 0x7FF) == 0x7FF;
    } else {
      up[(long long)j * (j + 1) / 2 + r] = v;
    }
  }
  nonfinite = __any_sync(FULL_MASK, nonfinite);
  __syncwarp();

  for (int j0 = 0; j0 < n; j0 += 32) {
    // Lanes past n (last chunk) repeat lane 0's column, so their operands take the same paths.
    const int t = j0 + lane < n ? j0 + lane : j0;
    const int k0 = nonfinite ? 0 : j0;
    double* x = xs + lane;
    for (int i = 0; i < n; i++) x[i * INV_LDX] = (i == t) ? 1.0 : 0.0;

    // Unit lower solve, dot form: x_i = x_i - Dot(i, L(i,:), x) (the division by 1.0 is exact).
    // Row i of L (entries k0..i-1) is read from shared memory while the next row streams in.
    // Blocks of 4 pairs: 8 independent products, then the sum's own chain in MatFlat's order.
    if (k0 + 1 < n) {
      stage_async(vb + ((k0 + 1) & 1) * n, lp + (long long)(k0 + 1) * k0 / 2, k0, k0 + 1);
      stage_wait();
    }
    for (int i = k0 + 1; i < n; i++) {
      const double* li = vb + (i & 1) * n;
      if (i + 1 < n) stage_async(vb + ((i + 1) & 1) * n, lp + (long long)(i + 1) * i / 2, k0, i + 1);
      double s = 0.0;
      int k = k0;
      if ((i - k0) & 1) {
        s = zmul_<IM>(li[k0], x[k0 * INV_LDX]);
        k = k0 + 1;
      }
      for (; k + 8 <= i; k += 8) {
        double l[8], v[8];
#pragma unroll
        for (int r = 0; r < 8; r++) {
          l[r] = li[k + r];
          v[r] = x[(k + r) * INV_LDX];
        }
        double pr[8];
        mul_block<IM, 8, true>(l, v, pr);
#pragma unroll
        for (int r = 0; r < 4; r++) s = __dadd_rn(s, __dadd_rn(pr[2 * r], pr[2 * r + 1]));
      }
      for (; k < i; k += 2) {
        const double q = __dadd_rn(zmul_<IM>(li[k], x[k * INV_LDX]),
                                   zmul_<IM>(li[k + 1], x[(k + 1) * INV_LDX]));
        s = __dadd_rn(s, q);
      }
      x[i * INV_LDX] = __dsub_rn(x[i * INV_LDX], s);
      stage_wait();
    }
    // Upper solve, column sweep: x_i /= U(i,i); x_k -= U(k,i) * x_i (k < i), column i of U from
    // shared memory while column i-1 streams in.  Blocks of 8 independent updates.
    stage_async(vb + ((n - 1) & 1) * n, up + (long long)(n - 1) * n / 2, 0, n);
    stage_wait();
    for (int i = n - 1; i >= 0; i--) {
      const double* ui = vb + (i & 1) * n;
      if (i > 0) stage_async(vb + ((i - 1) & 1) * n, up + (long long)(i - 1) * i / 2, 0, i);
      const double xi = __ddiv_rn(x[i * INV_LDX], ui[i]);
      x[i * INV_LDX] = xi;
      int k = 0;
      for (; k + 8 <= i; k += 8) {
        double u[8], v[8], pr[8];
#pragma unroll
        for (int r = 0; r < 8; r++) {
          u[r] = ui[k + r];
          v[r] = x[(k + r) * INV_LDX];
        }
        mul_block_s<IM, 8, true>(u, xi, pr);
#pragma unroll
        for (int r = 0; r < 8; r++) x[(k + r) * INV_LDX] = __dsub_rn(v[r], pr[r]);
      }
      for (; k < i; k++) x[k * INV_LDX] = __dsub_rn(x[k * INV_LDX], zmul_<IM>(ui[k], xi));
      stage_wait();
    }
    __syncwarp();
    // Column piv[t] of A^-1 is the staged column of lane t - j0; write it back coalesced.
    const int nc = min(32, n - j0);
    for (int l = 0; l < nc; l++) {
      double* col = a + (long long)piv[j0 + l] * lda;
      for (int i = lane; i < n; i += 32) col[i] = xs[i * INV_LDX + l];
    }
    __syncwarp();
  }
  if (lane == 0) *info_out = 0;
}

template <int IM>
__global__ void __launch_bounds__(INV_WARPS * 32) getri_batched_kernel(BatchArgs p) {
  extern __shared__ double sm_inv[];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const long long gw = (long long)blockIdx.x * INV_WARPS + warp;
  double* scr = p.gscratch + gw * p.gscratch_stride;
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(p.queue, 1);
    idx = __shfl_sync(FULL_MASK, idx, 0);
    if (idx >= p.count) break;
    const int mat = p.order[idx];
    const int n = p.n[mat];
    // Shared memory per warp: the staged columns (n <= 128), then two factor rows/columns.  For
    // larger n the staged columns live in global scratch and the smem holds the two buffers.
    double* wsm = sm_inv + warp * INV_SMEM_WARP;
    double* xs = n <= INV_SMEM_N ? wsm : scr + (long long)n * n;
    double* vb = n <= INV_SMEM_N ? wsm + INV_LDX * INV_SMEM_N : wsm;
    getri_warp<IM>(p.a + p.a_off[mat], n, p.lda[mat], p.piv + p.piv_off[mat], scr, xs, vb,
                   p.info + mat);
    __syncwarp();
  }
}

// ---- The float and Complex overloads (Factorization.LuInverse.cs:27-103, :219-295) -----------
// One warp per matrix, the single-matrix algorithm: the zero-diagonal and permutation checks of
// the double kernel, then the factors are copied to the warp's scratch (leading dimension n), A is
// set to the columns of P^T and solved RHS_CHUNK columns at a time, unit-lower (the LuInverse
// idiom; Complex divides by the explicit Complex(1, 0)) then upper, in MatFlat's order.
// Scratch per warp (getri_t_scratch_bytes): n*n elements, then the staged columns and their
// accumulators (the permutation check's bitmap reuses the staged columns).
template <class S>
__device__ __forceinline__ typename S::T inv_elem(double v);
template <>
__device__ __forceinline__ float inv_elem<SSolve>(double v) { return (float)v; }
template <>
__device__ __forceinline__ zdouble inv_elem<ZSolve<false>>(double v) { return zmake(v, 0.0); }

__device__ __forceinline__ bool inv_zero(float v) { return v == 0.0f; }
__device__ __forceinline__ bool inv_zero(zdouble v) { return v.re == 0.0 && v.im == 0.0; }

template <class S>
__global__ void __launch_bounds__(INV_WARPS * 32) getri_batched_t_kernel(BatchArgs p) {
  using T = typename S::T;
  using Acc = typename S::Acc;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const long long gw = (long long)blockIdx.x * INV_WARPS + warp;
  char* scr = reinterpret_cast<char*>(p.gscratch + gw * p.gscratch_stride);
  T* abase = reinterpret_cast<T*>(p.a);
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(p.queue, 1);
    idx = __shfl_sync(FULL_MASK, idx, 0);
    if (idx >= p.count) break;
    const int mat = p.order[idx];
    const int n = p.n[mat];
    const long long lda = p.lda[mat];
    T* a = abase + p.a_off[mat];
    const int* piv = p.piv + p.piv_off[mat];
    const int ldx = n | 1;
    T* work = reinterpret_cast<T*>(scr);
    Acc* acc = reinterpret_cast<Acc*>(scr + ((long long)n * n * sizeof(T) + 15) / 16 * 16);
    T* xs = reinterpret_cast<T*>(acc + RHS_CHUNK * ldx);
    // First zero diagonal entry (LuInverse.cs:145-152): nothing is written.
    int bad = INT_MAX;
    for (int j = lane; j < n; j += 32)
      if (inv_zero(a[(long long)j * lda + j])) bad = min(bad, j);
    for (int o = 16; o > 0; o >>= 1) bad = min(bad, __shfl_xor_sync(FULL_MASK, bad, o));
    if (bad != INT_MAX) {
      if (lane == 0) p.info[mat] = bad + 1;
      continue;
    }
    unsigned* seen = reinterpret_cast<unsigned*>(xs);
    for (int w = lane; w < ((n + 31) >> 5); w += 32) seen[w] = 0u;
    __syncwarp();
    int badp = 0;
    for (int t = lane; t < n; t += 32) {
      const int c = piv[t];
      if (c < 0 || c >= n)
        badp = 1;
      else if (atomicOr(&seen[c >> 5], 1u << (c & 31)) & (1u << (c & 31)))
        badp = 1;
    }
    if (__any_sync(FULL_MASK, badp)) {
      if (lane == 0) p.info[mat] = -1;
      continue;
    }
    for (long long e = lane; e < (long long)n * n; e += 32) {
      const int j = (int)(e / n);
      const int i = (int)(e - (long long)j * n);
      work[e] = a[(long long)j * lda + i];
    }
    __syncwarp();
    for (long long e = lane; e < (long long)n * n; e += 32) {
      const int j = (int)(e / n);
      const int i = (int)(e - (long long)j * n);
      a[(long long)j * lda + i] = inv_elem<S>(0.0);
    }
    __syncwarp();
    for (int j = lane; j < n; j += 32) a[lda * piv[j] + j] = inv_elem<S>(1.0);
    __syncwarp();
    for (int c0 = 0; c0 < n; c0 += RHS_CHUNK) {
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
    if (lane == 0) p.info[mat] = 0;
    __syncwarp();
  }
}

long long getri_t_scratch_bytes(int n, int elem) {
  const long long es = elem == 1 ? 4 : 16, as = elem == 1 ? 8 : 16;
  const long long ld = n | 1;
  const long long b = ((long long)n * n * es + 15) / 16 * 16 + RHS_CHUNK * ld * (as + es);
  return (b + 255) / 256 * 256;
}

cudaError_t launch_getri_batched_t(const BatchArgs& args, int elem, int ctas, cudaStream_t s) {
  if (elem == 1)
    getri_batched_t_kernel<SSolve><<<ctas, INV_WARPS * 32, 0, s>>>(args);
  else
    getri_batched_t_kernel<ZSolve<false>><<<ctas, INV_WARPS * 32, 0, s>>>(args);
  return cudaGetLastError();
}

cudaError_t init_getri_attributes() {
  cudaError_t e = cudaFuncSetAttribute(getri_batched_kernel<1>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)getri_smem_bytes());
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(getri_batched_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)getri_smem_bytes());
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(getri_batched_kernel<0>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)getri_smem_bytes());
}

int getri_ctas_per_sm() {
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, getri_batched_kernel<1>,
                                                    INV_WARPS * 32, getri_smem_bytes()) !=
      cudaSuccess)
    return 1;
  return blocks < 1 ? 1 : blocks;
}

cudaError_t launch_getri_batched(const BatchArgs& args, int ctas, cudaStream_t s) {
  if (args.hw_mul == 2)
    getri_batched_kernel<2><<<ctas, INV_WARPS * 32, getri_smem_bytes(), s>>>(args);
  else if (args.hw_mul)
    getri_batched_kernel<0><<<ctas, INV_WARPS * 32, getri_smem_bytes(), s>>>(args);
  else
    getri_batched_kernel<1><<<ctas, INV_WARPS * 32, getri_smem_bytes(), s>>>(args);
  return cudaGetLastError();
}

}  // namespace mfg
