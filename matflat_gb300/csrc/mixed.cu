// Mixed-precision batched LU solve with FP64 iterative refinement.
//
// For a batch of n-by-n systems A x = b (FP64 in HBM) the solver
//   1. rounds A to FP32 and factors it with partial pivoting, blocked right-looking with panel
//      width NB: a panel kernel (one CTA per matrix) factors the (n-k)-by-NB panel in shared
//      memory, applies its row interchanges to the rest of the matrix and forms
//      U12 = L11^-1 A12, and writes K-major copies of L21 and U12 in the low precision; the
//      trailing update A22 -= L21 U12 is one launch over the whole batch on the tensor cores
//      (mx_update_tc_kernel: TMA tile loads, tcgen05.mma kind::tf32 or kind::f16 with BF16
//      inputs, FP32 accumulators in Tensor Memory) or, in the FP32 mode, on the FP32 cores;
//   2. solves with the FP32 factors, then refines in FP64: r = b - A x with A in FP64,
//      d = (LU)^-1 r in FP32, x += d, until the normwise backward error
//      berr = |r|_inf / (|A|_inf |x|_inf + |b|_inf) reaches tol or stops halving (stall);
//   3. hands the systems that did not converge to the exact FP64 LU (MatFlat's arithmetic), all on
//      the device: the systems are gathered into a buffer the plan owns and factored by the
//      batched FP64 kernel over a device-side list, so a solve allocates nothing and never waits
//      on the host.
// The low-precision factorization is not MatFlat's arithmetic and makes no bit-exactness claim;
// the contract is the FP64 backward error, reported per system.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <mutex>

#include "mf_device.cuh"
#include "mf_kernels.h"
#include "mf_tc.cuh"

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
// Low-precision operand copies for the tensor-core update, K-major: row i of L21 (global row
// k+NB+i) at op_a[(mat*R + i)*NB ...], column j of U12 (global column k+NB+j) at
// op_b[(mat*R + j)*NB ...]; R rows per system.  opfmt 0: none (FP32 mode), 1: FP32 storage of
// the TF32-rounded value, 2: BF16, 3: split TF32 (high parts in op_a / op_b, low parts in
// op_a2 / op_b2).
__device__ __forceinline__ uint32_t tf32_rna(float v) {
  uint32_t t;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v));
  return t;
}

// opfmt 3 (split TF32): v = hi + lo with hi = tf32(v) in op and lo = tf32(v - hi) in op2, so that
// hi*hi + hi*lo + lo*hi on the tensor cores carries about FP32's precision.
__device__ __forceinline__ void mx_store_op(void* op, void* op2, long long idx, float v,
                                            int opfmt) {
  if (opfmt == 2) {
    reinterpret_cast<__nv_bfloat16*>(op)[idx] = __float2bfloat16_rn(v);
    return;
  }
  const uint32_t hi = tf32_rna(v);
  reinterpret_cast<uint32_t*>(op)[idx] = hi;
  if (opfmt == 3) reinterpret_cast<uint32_t*>(op2)[idx] = tf32_rna(v - __uint_as_float(hi));
}

__global__ void __launch_bounds__(MX_THREADS) mx_panel_kernel(float* a32, int n, int k, int* ipiv,
                                                              const int* active, void* op_a,
                                                              void* op_b, void* op_a2, void* op_b2,
                                                              int opfmt, int R) {
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
    // Scale the column and apply the rank-1 update to the panel's remaining columns, a whole row
    // per thread: the row's multiplier stays in a register, and row j (the U entries it reads)
    // is not changed by this step, so no barrier separates the two.
    const float d = sp[j * ldp + j];
    for (int i = j + 1 + tid; i < rows; i += MX_THREADS) {
      float l = sp[j * ldp + i];
      if (d != 0.0f) l /= d;
      sp[j * ldp + i] = l;
      for (int c = j + 1; c < MX_NB; ++c)
        sp[c * ldp + i] = fmaf(-l, sp[c * ldp + j], sp[c * ldp + i]);
    }
    __syncthreads();
  }
  for (int e = tid; e < rows * MX_NB; e += MX_THREADS) {
    const int c = e / rows, r = e - c * rows;
    a[(long long)(k + c) * n + k + r] = sp[c * ldp + r];
  }
  for (int j = tid; j < MX_NB; j += MX_THREADS) ip[k + j] = k + piv_s[j];
  if (opfmt != 0) {
    // L21, K-major: consecutive threads write consecutive K values of a row.
    const long long base = (long long)mat * R * MX_NB;
    for (int e = tid; e < (rows - MX_NB) * MX_NB; e += MX_THREADS) {
      const int i = e / MX_NB, c = e - i * MX_NB;
      mx_store_op(op_a, op_a2, base + e, sp[c * ldp + MX_NB + i], opfmt);
    }
  }
  // Interchanges on the columns left and right of the panel.  The panel's 32 swaps (row j with
  // row piv_s[j], in order) touch at most 64 rows; thread 0 composes them into one permutation of
  // those rows (new row dst[q] = old row src[q]), and each warp applies it to a column at a
  // time: all lanes gather their rows first, then scatter, so a column costs two rounds of
  // independent accesses instead of 32 dependent swaps.
  __shared__ int pm_src[2 * MX_NB], pm_dst[2 * MX_NB];
  __shared__ int pm_cnt;
  if (tid == 0) {
    int rows_t[2 * MX_NB], cur[2 * MX_NB];
    int nt = 0;
    for (int j = 0; j < MX_NB; ++j) {
      const int p = piv_s[j];
      if (p == j) continue;
      int qa = -1, qb = -1;
      for (int q = 0; q < nt; ++q) {
        if (rows_t[q] == j) qa = q;
        if (rows_t[q] == p) qb = q;
      }
      if (qa < 0) {
        rows_t[nt] = j;
        cur[nt] = j;
        qa = nt++;
      }
      if (qb < 0) {
        rows_t[nt] = p;
        cur[nt] = p;
        qb = nt++;
      }
      const int t = cur[qa];
      cur[qa] = cur[qb];
      cur[qb] = t;
    }
    int cnt = 0;
    for (int q = 0; q < nt; ++q)
      if (cur[q] != rows_t[q]) {
        pm_dst[cnt] = rows_t[q];
        pm_src[cnt] = cur[q];
        ++cnt;
      }
    pm_cnt = cnt;
  }
  __syncthreads();
  {
    const int lane = tid & 31, warp = tid >> 5, cnt = pm_cnt;
    const int s0 = lane < cnt ? pm_src[lane] : 0, d0 = lane < cnt ? pm_dst[lane] : 0;
    const int s1 = lane + 32 < cnt ? pm_src[lane + 32] : 0;
    const int d1 = lane + 32 < cnt ? pm_dst[lane + 32] : 0;
    // Eight columns per warp and round, so eight gathers are in flight at once (k is a multiple
    // of 32: a group of eight columns lies entirely inside or outside the panel).
    constexpr int CG = 8;
    for (int c0 = warp * CG; c0 < n && cnt > 0; c0 += (MX_THREADS / 32) * CG) {
      if (c0 >= k && c0 < k + MX_NB) continue;
      float v0[CG], v1[CG];
#pragma unroll
      for (int u = 0; u < CG; ++u) {
        const float* col = a + (long long)(c0 + u) * n + k;
        const bool ok = c0 + u < n;
        v0[u] = ok && lane < cnt ? col[s0] : 0.0f;
        v1[u] = ok && lane + 32 < cnt ? col[s1] : 0.0f;
      }
      __syncwarp();
#pragma unroll
      for (int u = 0; u < CG; ++u) {
        float* col = a + (long long)(c0 + u) * n + k;
        if (c0 + u >= n) continue;
        if (lane < cnt) col[d0] = v0[u];
        if (lane + 32 < cnt) col[d1] = v1[u];
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
    if (opfmt != 0) {
      const long long base = ((long long)mat * R + (c - k - MX_NB)) * MX_NB;
      for (int i = 0; i < MX_NB; ++i)
        mx_store_op(op_b, op_b2, base + i, us[i * MX_THREADS], opfmt);
    }
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

// Solves (LU) y = v in FP32 for one matrix: the interchanges, unit-lower forward sweep, upper
// backward sweep.  v: FP32 vector of n in shared memory.
// The whole CTA works (nt threads; n a multiple of 32), in blocks of 32 columns: warp 0 solves the
// block's 32 x 32 diagonal part with each lane holding one row in a register (the block's
// columns loaded up front), then every thread applies the block's 32 columns to its rows outside
// the block, column after column, with coalesced column loads.  Each entry of v receives its
// fused multiply-adds in column-sweep order (t ascending forward, descending backward), and the
// column loads are independent of one another: a solve is not one dependent global load per
// column, as a single warp sweeping the columns was (measured as half of a solve's time).
__device__ void mx_lu_solve_cta(const float* lu, const int* ip, int n, float* v) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nt = blockDim.x;
  if (tid == 0)
    for (int i = 0; i < n; ++i) {
      const int p = ip[i];
      if (p != i) {
        const float t = v[i];
        v[i] = v[p];
        v[p] = t;
      }
    }
  __syncthreads();
  // Forward, unit lower: v[i] -= L(i,t) v[t] for t < i, t ascending.
  for (int b0 = 0; b0 < n; b0 += 32) {
    if (warp == 0) {
      const int r = b0 + lane;
      float lr[32];
#pragma unroll
      for (int t = 0; t < 32; ++t) lr[t] = lu[(long long)(b0 + t) * n + r];
      float vr = v[r];
#pragma unroll
      for (int t = 0; t < 32; ++t) {
        const float yt = __shfl_sync(FULL_MASK, vr, t);
        if (lane > t) vr = fmaf(-lr[t], yt, vr);
      }
      v[r] = vr;
    }
    __syncthreads();
    for (int i = b0 + 32 + tid; i < n; i += nt) {
      float vi = v[i];
#pragma unroll 8
      for (int t = 0; t < 32; ++t) vi = fmaf(-lu[(long long)(b0 + t) * n + i], v[b0 + t], vi);
      v[i] = vi;
    }
    __syncthreads();
  }
  // Backward, upper: v[t] /= U(t,t); v[i] -= U(i,t) v[t] for i < t, t descending.
  for (int b0 = n - 32; b0 >= 0; b0 -= 32) {
    if (warp == 0) {
      const int r = b0 + lane;
      float ur[32];
#pragma unroll
      for (int t = 0; t < 32; ++t) ur[t] = lu[(long long)(b0 + t) * n + r];
      float vr = v[r];
#pragma unroll
      for (int t = 31; t >= 0; --t) {
        if (lane == t) vr = vr / ur[t];
        const float xt = __shfl_sync(FULL_MASK, vr, t);
        if (lane < t) vr = fmaf(-ur[t], xt, vr);
      }
      v[r] = vr;
    }
    __syncthreads();
    for (int i = tid; i < b0; i += nt) {
      float vi = v[i];
#pragma unroll 8
      for (int t = 31; t >= 0; --t) vi = fmaf(-lu[(long long)(b0 + t) * n + i], v[b0 + t], vi);
      v[i] = vi;
    }
    __syncthreads();
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
    mx_lu_solve_cta(LU, IP, n, v);
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
  mx_lu_solve_cta(LU, IP, n, v);
  for (int i = tid; i < n; i += MX_RT) X[i] = sx[i] + (double)v[i];
}

cudaError_t mx_round(const double* a, float* a32, long long total, cudaStream_t s) {
  mx_round_kernel<<<2048, 256, 0, s>>>(a, a32, total);
  return cudaGetLastError();
}

cudaError_t mx_panel(float* a32, int n, int k, int* ipiv, const int* active, int count,
                     void* op_a, void* op_b, void* op_a2, void* op_b2, int opfmt, int R,
                     cudaStream_t s) {
  const size_t smem = sizeof(float) * ((size_t)(n - k) * MX_NB + (size_t)MX_NB * MX_THREADS);
  mx_panel_kernel<<<count, MX_THREADS, smem, s>>>(a32, n, k, ipiv, active, op_a, op_b, op_a2,
                                                  op_b2, opfmt, R);
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

cudaError_t mx_refine(const double* a, const double* b, double* x, const float* lu,
                      const int* ipiv, int n, int count, int iter, double tol, double* berr,
                      int* iters, int* state, double* anorm, int* active, cudaStream_t s) {
  const size_t smem = sizeof(double) * (size_t)n + sizeof(float) * (size_t)n;
  mx_refine_kernel<<<count, MX_RT, smem, s>>>(a, b, x, lu, ipiv, n, count, iter, tol, berr,
                                              iters, state, anorm, active);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Trailing update on the tensor cores: A22 -= L21 U12 for every system, one CTA of 4 warps per
// 128 x 128 tile of A22 (grid: systems x tiles^2).  Thread 0 loads the tile's 128 rows of L21
// and 128 columns of U12 (K = NB = 32 low-precision values each, K-major) with two TMA copies,
// issues the tcgen05.mma steps (4 of K = 8 for TF32, 2 of K = 16 for BF16) into a 128-column FP32
// accumulator in Tensor Memory and commits them to an mbarrier; then each warp reads its 32 lanes
// (rows) of the accumulator with tcgen05.ld and subtracts them from A22 in global memory, one
// coalesced column segment per load.  Waits are bounded; a wait that runs out sets *status.
constexpr uint64_t MX_TC_WAIT_NS = 200000000ull;  // 0.2 s
constexpr int MX_TC_TILE = 128;

struct MxTcArgs {
  float* a32;
  int n, k, m2, tiles;
  int* status;
};

// MODE 0: TF32 (kind::tf32), 1: BF16 (kind::f16), 2: split TF32 (three kind::tf32 products per K
// step: lo*hi, hi*lo, hi*hi, from the high and low parts of both operands; tm_a2 / tm_b2 describe
// the low parts).
template <int MODE>
__global__ void __launch_bounds__(128) mx_update_tc_kernel(const __grid_constant__ CUtensorMap tm_a,
                                                          const __grid_constant__ CUtensorMap tm_b,
                                                          const __grid_constant__ CUtensorMap tm_a2,
                                                          const __grid_constant__ CUtensorMap tm_b2,
                                                          MxTcArgs p) {
  constexpr bool TF32 = MODE != 1;
  constexpr bool SPLIT = MODE == 2;
  constexpr int ROWB = TF32 ? 128 : 64;          // bytes of one operand row (32 values)
  constexpr int TILEB = MX_TC_TILE * ROWB;       // bytes of one operand tile
  constexpr uint32_t SBO = 8 * ROWB;             // 8-row swizzle atom
  constexpr uint32_t SWZ = TF32 ? 2 : 4;         // 128-byte / 64-byte swizzle
  constexpr int KSTEPS = TF32 ? 4 : 2;           // 32 bytes of K per tcgen05.mma
  constexpr uint32_t IDESC =
      tc::instr_desc(TF32 ? tc::FMT_TF32 : tc::FMT_BF16, MX_TC_TILE, MX_TC_TILE);
  extern __shared__ uint8_t mx_tc_smem[];
  uint8_t* base = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(mx_tc_smem) + 1023) & ~(uintptr_t)1023);
  uint8_t* sa = base;
  uint8_t* sb = base + TILEB;
  uint8_t* sa2 = base + 2 * TILEB;               // split mode only
  uint8_t* sb2 = base + 3 * TILEB;
  uint64_t* bar = reinterpret_cast<uint64_t*>(base + (SPLIT ? 4 : 2) * TILEB);
  uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 2);
  int* issued = reinterpret_cast<int*>(slot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int z = blockIdx.x;
  const int ti = blockIdx.y % p.tiles, tj = blockIdx.y / p.tiles;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar[0], 1);
    tc::mbar_init(&bar[1], 1);
    tc::mbar_fence_init();
    *issued = 0;
  }
  if (warp == 0) tc::tmem_alloc(slot, MX_TC_TILE);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *slot;
  if (threadIdx.x == 0) {
    tc::mbar_expect_tx(&bar[0], (SPLIT ? 4 : 2) * TILEB);
    tc::tma_load_3d(sa, &tm_a, &bar[0], 0, ti * MX_TC_TILE, z);
    tc::tma_load_3d(sb, &tm_b, &bar[0], 0, tj * MX_TC_TILE, z);
    if (SPLIT) {
      tc::tma_load_3d(sa2, &tm_a2, &bar[0], 0, ti * MX_TC_TILE, z);
      tc::tma_load_3d(sb2, &tm_b2, &bar[0], 0, tj * MX_TC_TILE, z);
    }
    if (tc::mbar_wait(&bar[0], 0, MX_TC_WAIT_NS)) {
      const uint64_t ad = tc::smem_desc(sa, SBO, SWZ);
      const uint64_t bd = tc::smem_desc(sb, SBO, SWZ);
      uint32_t acc = 0u;
      if (SPLIT) {
        const uint64_t ad2 = tc::smem_desc(sa2, SBO, SWZ);
        const uint64_t bd2 = tc::smem_desc(sb2, SBO, SWZ);
#pragma unroll
        for (int s = 0; s < KSTEPS; ++s) {   // the small products first
          tc::mma<true>(tmem, ad2 + 2 * s, bd + 2 * s, IDESC, acc);
          acc = 1u;
          tc::mma<true>(tmem, ad + 2 * s, bd2 + 2 * s, IDESC, acc);
        }
      }
#pragma unroll
      for (int s = 0; s < KSTEPS; ++s) {     // +32 bytes of K: +2 in the encoded start address
        tc::mma<TF32>(tmem, ad + 2 * s, bd + 2 * s, IDESC, acc);
        acc = 1u;
      }
      tc::mma_commit(&bar[1]);
      *issued = 1;
    } else {
      tc::mbar_wait(&bar[0], 0, MX_TC_WAIT_NS);   // let the copies land before leaving
      atomicExch(p.status, 1);
    }
  }
  __syncthreads();
  bool ready = false;
  if (*issued) {
    ready = tc::mbar_wait(&bar[1], 0, MX_TC_WAIT_NS);
    if (!ready) atomicExch(p.status, 2);
  }
  ready = __syncthreads_and(ready ? 1 : 0) != 0;
  tc::fence_after_sync();
  if (ready) {
    const int row = ti * MX_TC_TILE + warp * 32 + lane;
    float* c0 = p.a32 + (long long)z * p.n * p.n + (long long)(p.k + 32) * p.n + (p.k + 32);
    // All 32 loads of a column chunk are issued before any store (the compiler cannot reorder
    // loads above stores to the same array), so each thread keeps 32 reads in flight.
#pragma unroll 1
    for (int c = 0; c < MX_TC_TILE / 32; ++c) {
      uint32_t r[32];
      tc::tmem_load32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 32), r);
      const int col0 = tj * MX_TC_TILE + c * 32;
      if (row < p.m2) {
        float* dst = c0 + (long long)col0 * p.n + row;
        const int ncol = min(32, p.m2 - col0);
        float old[32];
#pragma unroll
        for (int q = 0; q < 32; ++q) old[q] = q < ncol ? dst[(long long)q * p.n] : 0.0f;
#pragma unroll
        for (int q = 0; q < 32; ++q)
          if (q < ncol) dst[(long long)q * p.n] = old[q] - __uint_as_float(r[q]);
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, MX_TC_TILE);
  }
}

// Shared memory of the update kernel: a 1024-byte alignment margin, the two operand tiles, two
// mbarriers, the TMEM address slot and a flag.
static size_t mx_tc_smem_bytes(int mode) {
  return 1024 + (mode == 2 ? 4 : 2) * MX_TC_TILE * (mode == 1 ? 64 : 128) + 64;
}

// Raises the shared-memory limit of the split mode (four 16 KB tiles); once per device.
cudaError_t mx_tc_attr() {
  return cudaFuncSetAttribute(mx_update_tc_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)mx_tc_smem_bytes(2));
}

// mode 0 TF32, 1 BF16, 2 split TF32 (tm[0..1] high parts, tm[2..3] low parts).
cudaError_t mx_update_tc(const CUtensorMap* tm, float* a32, int n, int k, int mode, int count,
                         int* status, cudaStream_t s) {
  const int m2 = n - k - MX_NB;
  if (m2 <= 0 || count == 0) return cudaSuccess;
  const int tiles = (m2 + MX_TC_TILE - 1) / MX_TC_TILE;
  MxTcArgs p{a32, n, k, m2, tiles, status};
  const dim3 grid((unsigned)count, (unsigned)(tiles * tiles));
  const size_t smem = mx_tc_smem_bytes(mode);
  if (mode == 0)
    mx_update_tc_kernel<0><<<grid, 128, smem, s>>>(tm[0], tm[1], tm[0], tm[1], p);
  else if (mode == 1)
    mx_update_tc_kernel<1><<<grid, 128, smem, s>>>(tm[0], tm[1], tm[0], tm[1], p);
  else
    mx_update_tc_kernel<2><<<grid, 128, smem, s>>>(tm[0], tm[1], tm[2], tm[3], p);
  return cudaGetLastError();
}

// Rows per system of the operand copies: the tiles read 128-row boxes, so the copies are padded
// to a multiple of 128 rows (rows past the system's trailing block are read but never stored).
int mx_op_rows(int n) { return (n + MX_TC_TILE - 1) / MX_TC_TILE * MX_TC_TILE; }

static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, []() {
    void* ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
  });
  return fn;
}

// TMA descriptors of the two operand copies: 3-D (K = 32 values, R rows, count systems), boxes of
// 32 x 128 x 1, 128-byte (TF32) or 64-byte (BF16) swizzle.
cudaError_t mx_make_tensor_maps(void* op_a, void* op_b, int n, int count, bool tf32,
                                CUtensorMap* tm_a, CUtensorMap* tm_b) {
  PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
  if (!encode) return cudaErrorNotSupported;
  const cuuint64_t es = tf32 ? 4 : 2;
  const int R = mx_op_rows(n);
  const cuuint64_t dims[3] = {(cuuint64_t)MX_NB, (cuuint64_t)R, (cuuint64_t)count};
  const cuuint64_t strides[2] = {MX_NB * es, (cuuint64_t)R * MX_NB * es};
  const cuuint32_t box[3] = {(cuuint32_t)MX_NB, (cuuint32_t)MX_TC_TILE, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUtensorMapDataType dt =
      tf32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
  const CUtensorMapSwizzle sw = tf32 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B;
  void* ops[2] = {op_a, op_b};
  CUtensorMap* maps[2] = {tm_a, tm_b};
  for (int i = 0; i < 2; ++i) {
    const CUresult r = encode(maps[i], dt, 3, ops[i], dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
  }
  return cudaSuccess;
}

// ---------------------------------------------------------------------------------------------
// The exact FP64 fallback, on the device.  Systems whose refinement did not converge
// (state != 1) are copied into the plan's fallback buffer (A) and into x (b, solved in place),
// and listed in `order` (count in *fb_count); the batched FP64 LU then runs over that list.
__global__ void mx_fb_gather_kernel(const double* a, const double* b, double* x, double* fa,
                                    const int* state, int n, int* order, int* fb_count) {
  const int i = blockIdx.x;
  if (state[i] == 1) return;
  if (threadIdx.x == 0) order[atomicAdd(fb_count, 1)] = i;
  const long long nn = (long long)n * n;
  const double* src = a + i * nn;
  double* dst = fa + i * nn;
  for (long long e = threadIdx.x; e < nn; e += blockDim.x) dst[e] = src[e];
  for (int e = threadIdx.x; e < n; e += blockDim.x) x[(long long)i * n + e] = b[(long long)i * n + e];
}

// info / state per system: 0 refined to the tolerance, 1 solved by the FP64 fallback, 2 the
// FP64 factor is singular.
__global__ void mx_fb_finish_kernel(int* state, int* info, const int* fb_info, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int v = state[i] == 1 ? 0 : (fb_info[i] != 0 ? 2 : 1);
  info[i] = v;
  state[i] = v;
}

cudaError_t mx_fb_gather(const double* a, const double* b, double* x, double* fa, const int* state,
                         int n, int count, int* order, int* fb_count, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  mx_fb_gather_kernel<<<count, 256, 0, s>>>(a, b, x, fa, state, n, order, fb_count);
  return cudaGetLastError();
}

cudaError_t mx_fb_finish(int* state, int* info, const int* fb_info, int count, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  mx_fb_finish_kernel<<<(count + 255) / 256, 256, 0, s>>>(state, info, fb_info, count);
  return cudaGetLastError();
}

int mx_panel_width() { return MX_NB; }

}  // namespace mfg
