// Mixed-precision batched LU solve with FP64 iterative refinement.
//
// For a batch of n-by-n systems A x = b (FP64 in HBM) the solver
//   1. rounds A to FP32 and factors it with partial pivoting, blocked right-looking with panel
//      width NB: a panel kernel (one CTA per matrix) factors the (n-k)-by-NB panel in shared
//      memory, applies its row interchanges to the rest of the matrix and forms
//      U12 = L11^-1 A12; the trailing update A22 -= L21 U12 is one strided-batched GEMM over the
//      whole batch on the tensor cores (TF32 or BF16 inputs, FP32 accumulation) or, in the FP32
//      mode, on the FP32 cores;
//   2. solves with the FP32 factors, then refines in FP64: r = b - A x with A in FP64,
//      d = (LU)^-1 r in FP32, x += d, until the normwise backward error
//      berr = |r|_inf / (|A|_inf |x|_inf + |b|_inf) reaches tol or stops halving (stall);
//   3. hands the systems that did not converge to the exact FP64 LU (MatFlat's arithmetic).
// The low-precision factorization is not MatFlat's arithmetic and makes no bit-exactness claim;
// the contract is the FP64 backward error, reported per system.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "mf_device.cuh"
#include "mf_kernels.h"

namespace mfg {

constexpr int MX_NB = 32;        // panel width
constexpr int MX_THREADS = 256;  // panel kernel CTA size

// Rounds the FP64 batch to FP32 (count * n * n elements).
__global__ void mx_round_kernel(const double* __restrict__ a, float* __restrict__ a32,
                                long long total) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x)
    a32[i] = (float)a[i];
}

// Panel step k for one matrix per CTA: factor rows [k, n) x columns [k, k+NB) with partial
// pivoting in shared memory, write ipiv (LAPACK convention: row k+j was swapped with ipiv[k+j]),
// apply the interchanges to the other columns, and overwrite A12 with U12 = L11^-1 A12.
__global__ void __launch_bounds__(MX_THREADS) mx_panel_kernel(float* a32, int n, int k, int* ipiv,
                                                              const int* active) {
  extern __shared__ float sp[];  // panel: (n-k) rows x NB columns, leading dimension ldp
  __shared__ float red_v[MX_THREADS / 32];
  __shared__ int red_i[MX_THREADS / 32];
  __shared__ int piv_s[MX_NB];
  const int mat = blockIdx.x;
  if (active && !active[mat]) return;
  float* a = a32 + (long long)mat * n * n;
  int* ip = ipiv + (long long)mat * n;
  const int tid = threadIdx.x;
  const int rows = n - k;
  const int ldp = rows;
  for (int e = tid; e < rows * MX_NB; e += MX_THREADS) {
    const int c = e / rows, r = e - c * rows;
    sp[c * ldp + r] = a[(long long)(k + c) * n + k + r];
  }
  __syncthreads();
  for (int j = 0; j < MX_NB; ++j) {
    // argmax |P(i, j)| over i in [j, rows): first index wins among equal magnitudes.
    float best = -1.0f;
    int bi = INT_MAX;
    for (int i = j + tid; i < rows; i += MX_THREADS) {
      const float v = fabsf(sp[j * ldp + i]);
      if (v > best) {
        best = v;
        bi = i;
      }
    }
    for (int off = 16; off > 0; off >>= 1) {
      const float ov = __shfl_xor_sync(FULL_MASK, best, off);
      const int oi = __shfl_xor_sync(FULL_MASK, bi, off);
      if (ov > best || (ov == best && oi < bi)) {
        best = ov;
        bi = oi;
      }
    }
    if ((tid & 31) == 0) {
      red_v[tid >> 5] = best;
      red_i[tid >> 5] = bi;
    }
    __syncthreads();
    if (tid == 0) {
      float bv = red_v[0];
      int b = red_i[0];
      for (int w = 1; w < MX_THREADS / 32; ++w)
        if (red_v[w] > bv || (red_v[w] == bv && red_i[w] < b)) {
          bv = red_v[w];
          b = red_i[w];
        }
      piv_s[j] = (b == INT_MAX) ? j : b;
    }
    __syncthreads();
    const int p = piv_s[j];
    if (p != j)
      for (int c = tid; c < MX_NB; c += MX_THREADS) {
        const float t = sp[c * ldp + j];
        sp[c * ldp + j] = sp[c * ldp + p];
        sp[c * ldp + p] = t;
      }
    __syncthreads();
    const float d = sp[j * ldp + j];
    if (d != 0.0f)
      for (int i = j + 1 + tid; i < rows; i += MX_THREADS) sp[j * ldp + i] /= d;
    __syncthreads();
    // Rank-1 update of the panel's remaining columns.
    const int w = MX_NB - j - 1;
    for (int e = tid; e < (rows - j - 1) * w; e += MX_THREADS) {
      const int c = j + 1 + e / (rows - j - 1);
      const int i = j + 1 + e % (rows - j - 1);
      sp[c * ldp + i] = fmaf(-sp[j * ldp + i], sp[c * ldp + j], sp[c * ldp + i]);
    }
    __syncthreads();
  }
  for (int e = tid; e < rows * MX_NB; e += MX_THREADS) {
    const int c = e / rows, r = e - c * rows;
    a[(long long)(k + c) * n + k + r] = sp[c * ldp + r];
  }
  for (int j = tid; j < MX_NB; j += MX_THREADS) ip[k + j] = k + piv_s[j];
  __syncthreads();
  // Interchanges on the columns left and right of the panel, in order.
  for (int c = tid; c < n; c += MX_THREADS) {
    if (c >= k && c < k + MX_NB) continue;
    float* col = a + (long long)c * n;
    for (int j = 0; j < MX_NB; ++j) {
      const int p = piv_s[j];
      if (p != j) {
        const float t = col[k + j];
        col[k + j] = col[k + p];
        col[k + p] = t;
      }
    }
  }
  __syncthreads();
  // U12 = L11^-1 A12 (unit lower), one column per thread, staged in shared memory after the panel
  // (us[i * MX_THREADS + tid]: conflict-free).  Column sweep: for every t, u[i] -= L(i,t) u[t]
  // for i > t, which is the same FMA sequence per entry as the dot form.  A fully unrolled
  // register version needed more than 255 registers and spilled.
  float* us = sp + rows * MX_NB + tid;
  for (int c = k + MX_NB + tid; c < n; c += MX_THREADS) {
    float* col = a + (long long)c * n + k;
    for (int i = 0; i < MX_NB; ++i) us[i * MX_THREADS] = col[i];
    for (int t = 0; t < MX_NB - 1; ++t) {
      const float ut = us[t * MX_THREADS];
      const float* lt = sp + t * ldp;
#pragma unroll 4
      for (int i = t + 1; i < MX_NB; ++i)
        us[i * MX_THREADS] = fmaf(-lt[i], ut, us[i * MX_THREADS]);
    }
    for (int i = 0; i < MX_NB; ++i) col[i] = us[i * MX_THREADS];
  }
}

// BF16 copies of L21 (rows [k+NB, n) x NB) and U12 (NB x columns [k+NB, n)) for the BF16 GEMM.
__global__ void mx_bf16_operands_kernel(const float* a32, int n, int k, __nv_bfloat16* l21,
                                        __nv_bfloat16* u12, const int* active) {
  const int mat = blockIdx.y;
  if (active && !active[mat]) return;
  const float* a = a32 + (long long)mat * n * n;
  const int m2 = n - k - MX_NB;
  __nv_bfloat16* l = l21 + (long long)mat * n * MX_NB;
  __nv_bfloat16* u = u12 + (long long)mat * n * MX_NB;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m2 * MX_NB;
       e += gridDim.x * blockDim.x) {
    const int c = e / m2, r = e - c * m2;
    l[(long long)c * m2 + r] = __float2bfloat16_rn(a[(long long)(k + c) * n + k + MX_NB + r]);
    const int uc = e / MX_NB, ur = e - uc * MX_NB;
    u[(long long)uc * MX_NB + ur] = __float2bfloat16_rn(a[(long long)(k + MX_NB + uc) * n + k + ur]);
  }
}

// Trailing update on the FP32 cores (the FP32 mode): A22 -= L21 U12, 64x64 tile per CTA, 4x4 per
// thread.  grid: (tiles, count).
__global__ void __launch_bounds__(256) mx_update_fp32_kernel(float* a32, int n, int k,
                                                             const int* active) {
  const int mat = blockIdx.y;
  if (active && !active[mat]) return;
  float* a = a32 + (long long)mat * n * n;
  const int o = k + MX_NB;
  const int m2 = n - o;
  const int tiles = (m2 + 63) / 64;
  const int ti = blockIdx.x % tiles, tj = blockIdx.x / tiles;
  if (tj >= tiles) return;
  __shared__ float ls[MX_NB][64 + 1];
  __shared__ float us[MX_NB][64 + 1];
  const int tid = threadIdx.x;
  for (int e = tid; e < MX_NB * 64; e += 256) {
    const int t = e / 64, r = e % 64;
    const int gi = o + ti * 64 + r, gj = o + tj * 64 + r;
    ls[t][r] = gi < n ? a[(long long)(k + t) * n + gi] : 0.0f;
    us[t][r] = gj < n ? a[(long long)gj * n + k + t] : 0.0f;
  }
  __syncthreads();
  const int tr = (tid % 16) * 4, tc = (tid / 16) * 4;
  float acc[4][4] = {};
#pragma unroll 8
  for (int t = 0; t < MX_NB; ++t) {
    float lv[4], uv[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      lv[q] = ls[t][tr + q];
      uv[q] = us[t][tc + q];
    }
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[p][q] = fmaf(lv[p], uv[q], acc[p][q]);
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int gj = o + tj * 64 + tc + q;
    if (gj >= n) continue;
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      const int gi = o + ti * 64 + tr + p;
      if (gi < n) a[(long long)gj * n + gi] -= acc[p][q];
    }
  }
}

// Solves (LU) y = v in FP32 for one matrix per warp: the interchanges, unit-lower forward sweep,
// upper backward sweep.  v: FP32 vector of n in shared memory of the warp.
__device__ void mx_lu_solve_warp(const float* lu, const int* ip, int n, float* v) {
  const int lane = threadIdx.x & 31;
  if (lane == 0)
    for (int i = 0; i < n; ++i) {
      const int p = ip[i];
      if (p != i) {
        const float t = v[i];
        v[i] = v[p];
        v[p] = t;
      }
    }
  __syncwarp();
  for (int t = 0; t < n; ++t) {
    const float yt = v[t];
    const float* col = lu + (long long)t * n;
    for (int i = t + 1 + lane; i < n; i += 32) v[i] = fmaf(-col[i], yt, v[i]);
    __syncwarp();
  }
  for (int t = n - 1; t >= 0; --t) {
    const float* col = lu + (long long)t * n;
    if (lane == 0) v[t] = v[t] / col[t];
    __syncwarp();
    const float xt = v[t];
    for (int i = lane; i < t; i += 32) v[i] = fmaf(-col[i], xt, v[i]);
    __syncwarp();
  }
}

// One refinement sweep per system, one CTA of MX_RT threads per system:
//   iter == -1: x = (LU)^-1 b                       (initial solve)
//   iter >= 0 : r = b - A x (FP64), berr; stop on convergence or stall, else x += (LU)^-1 r.
//   iter == -2: measure only: berr of x for the systems with state != 0 (FP64 fallback).
// state: 0 active, 1 converged, 2 stalled/diverged, 3 singular low-precision factor.
// The residual streams A (FP64) once per sweep with all MX_RT threads (thread t owns rows t,
// t + MX_RT, ...; coalesced column reads); warp 0 then runs the FP32 triangular solves.
constexpr int MX_RT = 256;       // refinement CTA size
constexpr int MX_RROWS = 4;      // rows per thread (n <= 1024)

__global__ void __launch_bounds__(MX_RT) mx_refine_kernel(
    const double* a, const double* b, double* x, const float* lu, const int* ipiv, int n,
    int count, int iter, double tol, double* berr, int* iters, int* state, double* anorm,
    int* active) {
  extern __shared__ double sx[];            // x (n doubles), then v (n floats)
  __shared__ double red[4][MX_RT / 32];
  __shared__ int verdict;
  float* v = reinterpret_cast<float*>(sx + n);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int mat = blockIdx.x;
  if (mat >= count) return;
  const double* A = a + (long long)mat * n * n;
  const double* B = b + (long long)mat * n;
  double* X = x + (long long)mat * n;
  const float* LU = lu + (long long)mat * n * n;
  const int* IP = ipiv + (long long)mat * n;
  const bool measure = iter == -2;
  if (iter == -1) {
    int sing = 0;
    for (int i = tid; i < n; i += MX_RT) {
      v[i] = (float)B[i];
      if (LU[(long long)i * n + i] == 0.0f) sing = 1;
    }
    sing = __syncthreads_or(sing);
    if (sing) {
      if (tid == 0) {
        state[mat] = 3;
        active[mat] = 0;
        berr[mat] = __longlong_as_double(0x7FF8000000000000LL);
        iters[mat] = 0;
      }
      return;
    }
    if (warp == 0) mx_lu_solve_warp(LU, IP, n, v);
    __syncthreads();
    for (int i = tid; i < n; i += MX_RT) X[i] = (double)v[i];
    if (tid == 0) {
      state[mat] = 0;
      iters[mat] = 0;
      berr[mat] = __longlong_as_double(0x7FF0000000000000LL);
    }
    return;
  }
  if (measure ? state[mat] == 0 : state[mat] != 0) return;
  for (int j = tid; j < n; j += MX_RT) sx[j] = X[j];
  __syncthreads();
  // r = b - A x, with |A|_inf accumulated on the first sweep.
  const bool rowsums = iter == 0 || measure;
  double r[MX_RROWS], rs[MX_RROWS];
#pragma unroll
  for (int q = 0; q < MX_RROWS; ++q) {
    const int i = tid + MX_RT * q;
    r[q] = i < n ? B[i] : 0.0;
    rs[q] = 0.0;
  }
#pragma unroll 4
  for (int j = 0; j < n; ++j) {
    const double xj = sx[j];
    const double* col = A + (long long)j * n;
#pragma unroll
    for (int q = 0; q < MX_RROWS; ++q) {
      const int i = tid + MX_RT * q;
      if (i < n) {
        const double aij = col[i];
        r[q] = fma(-aij, xj, r[q]);
        if (rowsums) rs[q] += fabs(aij);
      }
    }
  }
  double rn = 0.0, xn = 0.0, bn = 0.0, an = 0.0;
#pragma unroll
  for (int q = 0; q < MX_RROWS; ++q) {
    const int i = tid + MX_RT * q;
    if (i < n) {
      rn = fmax(rn, fabs(r[q]));
      xn = fmax(xn, fabs(sx[i]));
      bn = fmax(bn, fabs(B[i]));
      an = fmax(an, rs[q]);
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    rn = fmax(rn, __shfl_xor_sync(FULL_MASK, rn, off));
    xn = fmax(xn, __shfl_xor_sync(FULL_MASK, xn, off));
    bn = fmax(bn, __shfl_xor_sync(FULL_MASK, bn, off));
    an = fmax(an, __shfl_xor_sync(FULL_MASK, an, off));
  }
  if (lane == 0) {
    red[0][warp] = rn;
    red[1][warp] = xn;
    red[2][warp] = bn;
    red[3][warp] = an;
  }
  __syncthreads();
  if (tid == 0) {
    for (int w = 1; w < MX_RT / 32; ++w) {
      rn = fmax(rn, red[0][w]);
      xn = fmax(xn, red[1][w]);
      bn = fmax(bn, red[2][w]);
      an = fmax(an, red[3][w]);
    }
    if (iter == 0) anorm[mat] = an;
    const double An = rowsums ? an : anorm[mat];
    const double be = rn / (An * xn + bn);
    int st = 0;
    if (measure) {
      berr[mat] = be;
      st = -1;
    } else {
      const double prev = berr[mat];
      if (!(be == be)) st = 2;                 // NaN: diverged
      else if (be <= tol) st = 1;
      else if (iter >= 2 && be > 0.5 * prev) st = 2;
      berr[mat] = be;
      iters[mat] = iter;
      if (st != 0) {
        state[mat] = st;
        active[mat] = 0;
      }
    }
    verdict = st;
  }
  __syncthreads();
  if (verdict != 0) return;
#pragma unroll
  for (int q = 0; q < MX_RROWS; ++q) {
    const int i = tid + MX_RT * q;
    if (i < n) v[i] = (float)r[q];
  }
  __syncthreads();
  if (warp == 0) mx_lu_solve_warp(LU, IP, n, v);
  __syncthreads();
  for (int i = tid; i < n; i += MX_RT) X[i] = sx[i] + (double)v[i];
}

cudaError_t mx_round(const double* a, float* a32, long long total, cudaStream_t s) {
  mx_round_kernel<<<2048, 256, 0, s>>>(a, a32, total);
  return cudaGetLastError();
}

cudaError_t mx_panel(float* a32, int n, int k, int* ipiv, const int* active, int count,
                     cudaStream_t s) {
  const size_t smem = sizeof(float) * ((size_t)(n - k) * MX_NB + (size_t)MX_NB * MX_THREADS);
  mx_panel_kernel<<<count, MX_THREADS, smem, s>>>(a32, n, k, ipiv, active);
  return cudaGetLastError();
}

cudaError_t mx_panel_attr(int nmax) {
  return cudaFuncSetAttribute(
      mx_panel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
      (int)(sizeof(float) * ((size_t)nmax * MX_NB + (size_t)MX_NB * MX_THREADS)));
}

cudaError_t mx_update_fp32(float* a32, int n, int k, const int* active, int count,
                           cudaStream_t s) {
  const int m2 = n - k - MX_NB;
  if (m2 <= 0) return cudaSuccess;
  const int tiles = (m2 + 63) / 64;
  mx_update_fp32_kernel<<<dim3(tiles * tiles, count), 256, 0, s>>>(a32, n, k, active);
  return cudaGetLastError();
}

cudaError_t mx_bf16_operands(const float* a32, int n, int k, void* l21, void* u12,
                             const int* active, int count, cudaStream_t s) {
  const int m2 = n - k - MX_NB;
  if (m2 <= 0) return cudaSuccess;
  const int blocks = (m2 * MX_NB + 255) / 256;
  mx_bf16_operands_kernel<<<dim3(blocks, count), 256, 0, s>>>(
      a32, n, k, (__nv_bfloat16*)l21, (__nv_bfloat16*)u12, active);
  return cudaGetLastError();
}

cudaError_t mx_refine(const double* a, const double* b, double* x, const float* lu,
                      const int* ipiv, int n, int count, int iter, double tol, double* berr,
                      int* iters, int* state, double* anorm, int* active, cudaStream_t s) {
  const size_t smem = sizeof(double) * (size_t)n + sizeof(float) * (size_t)n;
  mx_refine_kernel<<<count, MX_RT, smem, s>>>(a, b, x, lu, ipiv, n, count, iter, tol, berr,
                                              iters, state, anorm, active);
  return cudaGetLastError();
}

int mx_panel_width() { return MX_NB; }

}  // namespace mfg
