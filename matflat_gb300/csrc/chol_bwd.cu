// Reverse mode of the Cholesky factor, its log-determinant and the solve (the adjoint of
// Factorization.Cholesky, MatFlat/Factorization.Cholesky.cs:114-168, followed by the two
// triangular solves of Blas.SolveTriangular, MatFlat/Blas.SolveTriangular.cs:162-242).
//
// Forward, per matrix: A = L L^T, logdet = 2 sum log L_ii, x = A^-1 b.  With A perturbed
// symmetrically, L^-1 dA L^-T = M + M^T for M = L^-1 dL lower triangular, so
//     dL = L Phi(L^-1 dA L^-T),   Phi(X) = lower triangle of X with the diagonal halved,
// and the pairing <Lbar, dL> = <L^-T Phi(L^T Lbar) L^-1, dA>.  The log-determinant adds
// logdet_bar * A^-1 (Phi of L^T * 2 logdet_bar diag(1/L_ii) is logdet_bar * I), and the solve adds
// -bbar x^T with bbar = A^-1 xbar.  The gradient returned is symmetric (d loss = <abar, dA> for
// symmetric dA):
//     S    = sym(Phi(L^T Lbar)) + logdet_bar I             (S_ij = X_ij / 2 below the diagonal,
//                                                          S_ii = X_ii / 2 + logdet_bar)
//     abar = sym(L^-T S L^-1) - sym(bbar x^T),   bbar = L^-T L^-1 xbar.
// MatFlat has no derivative, so no reference operation order binds this kernel: it uses fused
// multiply-adds and reciprocals of the diagonal, and its accuracy is checked against an FP64
// evaluation of the same formulas from the oracle's factor and against central differences.
//
// One CTA of 128 threads per matrix (n <= 128), the matrices in their global buffers:
//   1. S: thread i forms row i of X = L^T Lbar below the diagonal (dots of length n - i).
//   2. Y = S L^-1: thread r solves row r (y L = s_r, column sweep from the last column).
//   3. G = L^-T Y: thread c solves column c (L^T g = y_c, from the last row).
//   4. bbar (warp 0: the two triangular solves), then abar = sym(G) - sym(bbar x^T).
#include <cuda_runtime.h>

#include "mf_device.cuh"
#include "mf_kernels.h"

namespace mfg {

constexpr int BWD_THREADS = 128;
constexpr int BWD_MAX_N = 128;

__global__ void __launch_bounds__(BWD_THREADS) chol_backward_kernel(CholBwdArgs p) {
  __shared__ double rcp[BWD_MAX_N];
  __shared__ double bb[BWD_MAX_N];
  __shared__ double xv[BWD_MAX_N];
  __shared__ int next;
  const int tid = threadIdx.x;
  for (;;) {
    if (tid == 0) next = atomicAdd(p.queue, 1);
    __syncthreads();
    const int idx = next;
    __syncthreads();
    if (idx >= p.count) break;
    const int mat = p.order[idx];
    if (p.info && p.info[mat] != 0) continue;   // the recomputed factorization failed
    const int n = p.n[mat];
    const long long lda = p.lda[mat];
    const double* L = p.l + p.a_off[mat];
    const double* Lb = p.lbar ? p.lbar + p.a_off[mat] : nullptr;
    double* G = p.abar + p.a_off[mat];
    const double ldb = p.logdet_bar ? p.logdet_bar[mat] : 0.0;
    for (int i = tid; i < n; i += BWD_THREADS) rcp[i] = 1.0 / L[i * (lda + 1)];
    __syncthreads();

    // 1. S (both triangles of G).
    for (int i = tid; i < n; i += BWD_THREADS) {
      const double* li = L + i * lda;               // column i of L: L_ki, k >= i
      for (int j = 0; j <= i; ++j) {
        double xij = 0.0;
        if (Lb) {
          const double* lbj = Lb + j * lda;         // column j of Lbar
          for (int k = i; k < n; ++k) xij = fma(li[k], lbj[k], xij);
        }
        const double sij = 0.5 * xij + (i == j ? ldb : 0.0);
        G[i + j * lda] = sij;
        G[j + i * lda] = sij;
      }
    }
    __syncthreads();

    // 2. Y = S L^-1, row r per thread: y_j = (s_j - sum_{k>j} y_k L_kj) / L_jj.
    for (int r = tid; r < n; r += BWD_THREADS) {
      for (int j = n - 1; j >= 0; --j) {
        double acc = G[r + j * lda];
        const double* lj = L + j * lda;
        for (int k = j + 1; k < n; ++k) acc = fma(-G[r + k * lda], lj[k], acc);
        G[r + j * lda] = acc * rcp[j];
      }
    }
    __syncthreads();

    // 3. G = L^-T Y, column c per thread: g_i = (y_i - sum_{k>i} L_ki g_k) / L_ii.
    for (int c = tid; c < n; c += BWD_THREADS) {
      double* gc = G + c * lda;
      for (int i = n - 1; i >= 0; --i) {
        double acc = gc[i];
        const double* li = L + i * lda;
        for (int k = i + 1; k < n; ++k) acc = fma(-li[k], gc[k], acc);
        gc[i] = acc * rcp[i];
      }
    }
    __syncthreads();

    // 4. bbar = L^-T L^-1 xbar (warp 0), then the symmetric gradient.
    const bool sol = p.xbar != nullptr;
    if (sol && tid < 32) {
      const double* xb = p.xbar + p.b_off[mat];
      const double* xx = p.x + p.b_off[mat];
      for (int i = tid; i < n; i += 32) {
        bb[i] = xb[i];
        xv[i] = xx[i];
      }
      __syncwarp();
      for (int t = 0; t < n; ++t) {            // L z = xbar (column sweep)
        const double zt = bb[t] * rcp[t];
        __syncwarp();
        if (tid == 0) bb[t] = zt;
        const double* lt = L + t * lda;
        for (int i = t + 1 + tid; i < n; i += 32) bb[i] = fma(-lt[i], zt, bb[i]);
        __syncwarp();
      }
      for (int t = n - 1; t >= 0; --t) {       // L^T bbar = z (dot form, lanes split the dot)
        const double* lt = L + t * lda;
        double part = 0.0;
        for (int k = t + 1 + tid; k < n; k += 32) part = fma(lt[k], bb[k], part);
        for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(FULL_MASK, part, off);
        if (tid == 0) bb[t] = (bb[t] - part) * rcp[t];
        __syncwarp();
      }
      if (p.bbar)
        for (int i = tid; i < n; i += 32) p.bbar[p.b_off[mat] + i] = bb[i];
    } else if (!sol && p.bbar) {
      for (int i = tid; i < n; i += BWD_THREADS) p.bbar[p.b_off[mat] + i] = 0.0;   // no xbar
    }
    __syncthreads();
    for (int i = tid; i < n; i += BWD_THREADS) {
      for (int j = 0; j < i; ++j) {
        double g = 0.5 * (G[i + j * lda] + G[j + i * lda]);
        if (sol) g -= 0.5 * (bb[i] * xv[j] + xv[i] * bb[j]);
        G[i + j * lda] = g;
        G[j + i * lda] = g;
      }
      if (sol) G[i * (lda + 1)] -= bb[i] * xv[i];
    }
    __syncthreads();
  }
}

int chol_backward_max_n() { return BWD_MAX_N; }

cudaError_t launch_chol_backward(const CholBwdArgs& args, int ctas, cudaStream_t s) {
  chol_backward_kernel<<<ctas, BWD_THREADS, 0, s>>>(args);
  return cudaGetLastError();
}

}  // namespace mfg
