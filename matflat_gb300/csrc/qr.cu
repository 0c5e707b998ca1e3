// Householder QR in MatFlat's arithmetic and Mapack storage format:
//   Factorization.Qr                     (MatFlat/Factorization.Qr.cs:115-172 double, :32-89 float)
//   Factorization.QrOrthogonalFactor     (:357-413 double, :278-334 float)
//   Factorization.QrUpperTriangularFactor (:597-650 double, :518-571 float)
// and the batched least-squares solver built from them.
//
// For every column k MatFlat computes norm = sqrt(pairwise sum of squares) (Internals.Norm), and,
// if norm != 0, divides the column by it, adds 1 to the diagonal entry (no reflector sign choice)
// and updates every later column j with s = -Dot(v, a_j) / v[0]; a_j += s * v.  rdiag[k] = -norm.
// The float overload keeps float storage but sums its dots and norms in double.  Each column's
// dot is independent of the others, so one warp runs the column dots of a step across its lanes,
// then the rank-1 update across (row, column) pairs; every value is computed with MatFlat's own
// operations in MatFlat's order.
//
// Least squares: MatFlat has no QR solve.  The batched solver treats each right-hand side b as
// one more trailing column, so Q^T b is produced by the very same reflector updates, and then
// solves R x = (Q^T b)[0:n] with MatFlat's Upper/NoTrans column sweep (R = strict upper part of
// a, diagonal rdiag).  On exit b[0:n] = x and b[n:m] holds the residual components.
#include <cuda_runtime.h>

#include <type_traits>

#include "mf_device.cuh"
#include "mf_kernels.h"
#include "mf_scalar.cuh"
#include "mf_solve.cuh"

namespace mfg {

template <typename T>
struct QrArith;

// Pairs per software-pipelined block of the QR dot products (MFG_QR_DOT_BLOCK at build time):
// two pairs keep the double kernel within 128 registers without spills, so 16 warps fit per SM
// (5 % faster than four pairs on the 50,000-matrix batch).
#ifndef MFG_QR_DOT_BLOCK
#define MFG_QR_DOT_BLOCK 2
#endif
// Pairs per software-pipelined block of the fused column pass (double, float).  On the
// 50,000-matrix batch the double kernel measured 126.5 / 121.9 / 127.1 ms with 2 / 3 / 4 (151.0
// unpipelined), the float one 134.0 / 133.6 / 223.8 with 2 / 3 / 4 (134.5 unpipelined).
#ifndef MFG_QR_FUSE_BLOCK_D
#define MFG_QR_FUSE_BLOCK_D 3
#endif
#ifndef MFG_QR_FUSE_BLOCK_F
#define MFG_QR_FUSE_BLOCK_F 2
#endif

template <>
struct QrArith<double> {
  using R = double;  // type of the norm and of rdiag
  // Internals.Norm (Internals.cs:435-460): the Dot tree over x*x, then Math.Sqrt.
  static __device__ __forceinline__ double norm(int len, const double* x) {
    return __dsqrt_rn(exact_dot<1, MFG_QR_DOT_BLOCK>(len, x, 1, x, 1));
  }
  static __device__ __forceinline__ double dot(int len, const double* x, const double* y) {
    return exact_dot<1, MFG_QR_DOT_BLOCK>(len, x, 1, y, 1);
  }
  static __device__ __forceinline__ double div(double x, double y) { return __ddiv_rn(x, y); }
  static __device__ __forceinline__ double add1(double x) { return __dadd_rn(x, 1.0); }
  // s = -Dot(...) / colk[k]   (Qr.cs:163, :408)
  static __device__ __forceinline__ double coef(double d, double v0) { return __ddiv_rn(-d, v0); }
  // MulAdd: dst += x * s      (Internals.cs:49-73)
  // The product on the integer pipes (imul_rn: the same correctly rounded value as DMUL).
  static __device__ __forceinline__ double muladd(double dst, double x, double s) {
    return __dadd_rn(dst, imul_rn(x, s));
  }
  static __device__ __forceinline__ double mulsub(double dst, double x, double s) {
    return __dsub_rn(dst, __dmul_rn(x, s));
  }
  static __device__ __forceinline__ bool nz(double v) { return nonzero(v); }
  static __device__ __forceinline__ bool nzr(double v) { return nonzero(v); }
  static __device__ __forceinline__ double divn(double x, double norm) { return __ddiv_rn(x, norm); }
  // x[i] = x[i] / norm for i = first, first + step, ... < end: the quotients on the integer pipes
  // (idiv_column: the same bits as the FP64 division).
  static __device__ __forceinline__ void divcol(double* x, int first, int end, int step,
                                                double norm) {
    idiv_column(x, first, end, step, norm);
  }
  static __device__ __forceinline__ double neg_r(double norm) { return -norm; }
  // QrOrthogonalFactor's dot and update (Qr.cs:408-409)
  static __device__ __forceinline__ double qdot(int len, const double* a, const double* q) {
    return exact_dot<1, MFG_QR_DOT_BLOCK>(len, a, 1, q, 1);
  }
  static __device__ __forceinline__ double qmuladd(double q, double a, double s) {
    return __dadd_rn(q, __dmul_rn(a, s));
  }
  static __device__ __forceinline__ double rdiag_elem(double r) { return r; }
  // One term and one pair of Internals.Dot's tree (for loops that fuse the dot with an update).
  static __device__ __forceinline__ double prod(double x, double y) { return imul_rn(x, y); }
  static __device__ __forceinline__ double pair(double s, double x0, double y0, double x1,
                                                double y1) {
    return __dadd_rn(s, __dadd_rn(imul_rn(x0, y0), imul_rn(x1, y1)));
  }
};

template <>
struct QrArith<float> {
  using R = float;
  // (float)Internals.Norm(float*) (Qr.cs:68): double sum of widened squares, sqrt, to float.
  static __device__ __forceinline__ float norm(int len, const float* x) {
    return __double2float_rn(__dsqrt_rn(exact_dot_f(len, x, 1, x, 1)));
  }
  static __device__ __forceinline__ double dot(int len, const float* x, const float* y) {
    return exact_dot_f(len, x, 1, y, 1);
  }
  static __device__ __forceinline__ float div(float x, float y) { return __fdiv_rn(x, y); }
  static __device__ __forceinline__ float add1(float x) { return __fadd_rn(x, 1.0f); }
  // s = -(float)(Dot(...) / colk[k])   (Qr.cs:80, :329)
  static __device__ __forceinline__ float coef(double d, float v0) {
    return -__double2float_rn(__ddiv_rn(d, (double)v0));
  }
  static __device__ __forceinline__ float muladd(float dst, float x, float s) {
    return __fadd_rn(dst, __fmul_rn(x, s));
  }
  static __device__ __forceinline__ float mulsub(float dst, float x, float s) {
    return __fsub_rn(dst, __fmul_rn(x, s));
  }
  static __device__ __forceinline__ bool nz(float v) { return (__float_as_uint(v) << 1) != 0u; }
  static __device__ __forceinline__ bool nzr(float v) { return nz(v); }
  static __device__ __forceinline__ float divn(float x, float norm) { return __fdiv_rn(x, norm); }
  static __device__ __forceinline__ void divcol(float* x, int first, int end, int step,
                                                float norm) {
    for (int i = first; i < end; i += step) x[i] = __fdiv_rn(x[i], norm);
  }
  static __device__ __forceinline__ float neg_r(float norm) { return -norm; }
  static __device__ __forceinline__ double qdot(int len, const float* a, const float* q) {
    return exact_dot_f(len, a, 1, q, 1);
  }
  static __device__ __forceinline__ float qmuladd(float q, float a, float s) {
    return __fadd_rn(q, __fmul_rn(a, s));
  }
  static __device__ __forceinline__ float rdiag_elem(float r) { return r; }
  static __device__ __forceinline__ double prod(float x, float y) { return fmul_wide(x, y); }
  static __device__ __forceinline__ double pair(double s, float x0, float y0, float x1, float y1) {
    return __dadd_rn(s, __dadd_rn(fmul_wide(x0, y0), fmul_wide(x1, y1)));
  }
};

// Complex overload (Factorization.Qr.cs:198-255, :436-492, :677-730): the norm is real
// (Internals.Norm over re^2 + im^2, Internals.cs:489-514), the column is divided by
// Complex(norm, 0), the dots are DotConj, and QrOrthogonalFactor uses
// s = -DotConj(q_j, v) / v[0] with MulConjAdd (q += conj(s) * v).
template <>
struct QrArith<zdouble> {
  using R = double;
  static __device__ __forceinline__ double norm(int len, const zdouble* x) {
    double s;
    int i = 0;
    if (len & 1) {
      s = __dadd_rn(__dmul_rn(x[0].re, x[0].re), __dmul_rn(x[0].im, x[0].im));
      i = 1;
    } else {
      s = 0.0;
    }
    for (; i < len; i += 2) {
      // sum += x0.re*x0.re + x0.im*x0.im + x1.re*x1.re + x1.im*x1.im  (left to right)
      double t = __dadd_rn(__dmul_rn(x[i].re, x[i].re), __dmul_rn(x[i].im, x[i].im));
      t = __dadd_rn(t, __dmul_rn(x[i + 1].re, x[i + 1].re));
      t = __dadd_rn(t, __dmul_rn(x[i + 1].im, x[i + 1].im));
      s = __dadd_rn(s, t);
    }
    return __dsqrt_rn(s);
  }
  static __device__ __forceinline__ zdouble dot(int len, const zdouble* x, const zdouble* y) {
    return zdot<true>(len, x, 1, y, 1);
  }
  static __device__ __forceinline__ zdouble div(zdouble x, zdouble y) { return zdiv(x, y); }
  static __device__ __forceinline__ zdouble divn(zdouble x, double norm) {
    return zdiv(x, zmake(norm, 0.0));
  }
  static __device__ __forceinline__ void divcol(zdouble* x, int first, int end, int step,
                                                double norm) {
    for (int i = first; i < end; i += step) x[i] = zdiv(x[i], zmake(norm, 0.0));
  }
  static __device__ __forceinline__ zdouble add1(zdouble x) { return zadd(x, zmake(1.0, 0.0)); }
  static __device__ __forceinline__ zdouble coef(zdouble d, zdouble v0) { return zdiv(zneg(d), v0); }
  static __device__ __forceinline__ zdouble muladd(zdouble dst, zdouble x, zdouble s) {
    return zadd(dst, zmul(x, s));
  }
  static __device__ __forceinline__ bool nz(zdouble v) { return znonzero(v); }
  static __device__ __forceinline__ bool nzr(double v) { return nonzero(v); }
  static __device__ __forceinline__ double neg_r(double norm) { return -norm; }
  static __device__ __forceinline__ zdouble qdot(int len, const zdouble* a, const zdouble* q) {
    return zdot<true>(len, q, 1, a, 1);
  }
  static __device__ __forceinline__ zdouble qmuladd(zdouble q, zdouble a, zdouble s) {
    return zadd(q, zmulconj(s, a));
  }
  static __device__ __forceinline__ zdouble rdiag_elem(double r) { return zmake(r, 0.0); }
};

// The FMA form of the double QR (selected per plan, not MatFlat's bits): the same Householder
// algorithm and storage (no reflector sign choice, rdiag = -norm, the degenerate-reflector rules),
// with every dot and norm as fused multiply-adds in four chains, the updates as fused
// multiply-adds and the column scaled by the reciprocal of its norm.  Householder QR in any
// such arithmetic is backward stable: the computed R is the exact R of A + dA with
// ||dA|| <= c m n u ||A||.
struct QrArithFma {
  using R = double;
  static __device__ __forceinline__ double norm(int len, const double* x) {
    return __dsqrt_rn(fma_dot(len, x, 1, x, 1));
  }
  // The column dots in the order the fused column pass accumulates them (prod, then pair after
  // pair), so that solve-only calls apply the reflectors to right-hand sides with the fused
  // call's bits.
  static __device__ __forceinline__ double dot(int len, const double* x, const double* y) {
    double d = 0.0;
    int r = 0;
    if (len & 1) {
      d = __dmul_rn(x[0], y[0]);
      r = 1;
    }
#pragma unroll 4
    for (; r < len; r += 2) d = __fma_rn(x[r + 1], y[r + 1], __fma_rn(x[r], y[r], d));
    return d;
  }
  static __device__ __forceinline__ double div(double x, double y) { return __ddiv_rn(x, y); }
  static __device__ __forceinline__ double add1(double x) { return __dadd_rn(x, 1.0); }
  static __device__ __forceinline__ double coef(double d, double v0) { return __ddiv_rn(-d, v0); }
  static __device__ __forceinline__ double muladd(double dst, double x, double s) {
    return __fma_rn(x, s, dst);
  }
  static __device__ __forceinline__ double mulsub(double dst, double x, double s) {
    return __fma_rn(-x, s, dst);
  }
  static __device__ __forceinline__ bool nz(double v) { return nonzero(v); }
  static __device__ __forceinline__ bool nzr(double v) { return nonzero(v); }
  static __device__ __forceinline__ double divn(double x, double norm) { return __ddiv_rn(x, norm); }
  static __device__ __forceinline__ void divcol(double* x, int first, int end, int step,
                                                double norm) {
    const double r = __drcp_rn(norm);
    for (int i = first; i < end; i += step) x[i] = __dmul_rn(x[i], r);
  }
  static __device__ __forceinline__ double neg_r(double norm) { return -norm; }
  static __device__ __forceinline__ double prod(double x, double y) { return __dmul_rn(x, y); }
  static __device__ __forceinline__ double pair(double s, double x0, double y0, double x1,
                                                double y1) {
    return __fma_rn(x1, y1, __fma_rn(x0, y0, s));
  }
};

// Column j of the factored matrix, or right-hand side j - n when j >= n.
template <typename T>
__device__ __forceinline__ T* qr_col(T* a, long long lda, int n, T* b, long long ldb, int j) {
  return j < n ? a + (long long)j * lda : b + (long long)(j - n) * ldb;
}

// Factors the m-by-n matrix a (m >= n) in place, applying every reflector also to the nb columns
// of b (leading dimension ldb).  coefs: n - 1 + nb values of scratch.  G lanes work on the matrix
// (a whole warp for G = 32; 32/G matrices per warp otherwise): the norm is one sequential dot
// (every lane of the group evaluates it), the trailing-column dots are spread one per lane, and
// the rank-1 update over (row, column) pairs.
template <typename T, int G = 32, class A = QrArith<T>>
__device__ void qr_warp(T* a, int m, int n, long long lda, typename A::R* rdiag, T* b,
                        long long ldb, int nb, T* coefs) {
  using R = typename A::R;
  const int lane = group_lane<G>();
  const unsigned gm = group_mask<G>();
  for (int k = 0; k < n; ++k) {
    T* ck = a + (long long)k * lda;
    const int len = m - k;
    const R norm = A::norm(len, ck + k);  // every lane of the group, same value
    if (A::nzr(norm)) {
      A::divcol(ck, k + lane, m, G, norm);
      __syncwarp(gm);
      if (lane == 0) ck[k] = A::add1(ck[k]);
      __syncwarp(gm);
      const T v0 = ck[k];
      const int ncols = (n - k - 1) + nb;
      for (int c = lane; c < ncols; c += G) {
        const T* cj = qr_col(a, lda, n, b, ldb, k + 1 + c);
        coefs[c] = A::coef(A::dot(len, ck + k, cj + k), v0);
      }
      __syncwarp(gm);
      // Right-hand sides skip a degenerate reflector (v[0] == 0 means v == 0 and the reflector
      // is the identity), as QrOrthogonalFactor does for the columns of Q (Qr.cs:406); the
      // factored columns follow Qr itself, which does not skip.
      const int upd = A::nz(v0) ? ncols : (n - k - 1);
      const long long work = (long long)len * upd;
      for (long long e = lane; e < work; e += G) {
        const int c = (int)(e / len);
        const int r = k + (int)(e - (long long)c * len);
        T* cj = qr_col(a, lda, n, b, ldb, k + 1 + c);
        cj[r] = A::muladd(cj[r], ck[r], coefs[c]);
      }
    }
    __syncwarp(gm);
    if (lane == 0) rdiag[k] = A::neg_r(norm);
    __syncwarp(gm);
  }
}

// The same factorization with every trailing column visited once per step instead of twice: at
// step k a lane takes a trailing column, applies reflector k-1 to it (cj += v_{k-1} s) and, in the
// same pass, accumulates reflector k's dot Dot(m-k, v_k, cj) over the updated entries; column k
// itself is brought up to date first, because v_k is formed from it.  Each entry sees the same
// operations in the same order as in qr_warp (every update of a column precedes the next dot on
// it, and the dot's pairwise tree is unchanged), so the factors and rdiag are bit-identical.
// coefs: 2 (n + nb) values (the previous step's coefficients and the current ones).
template <typename T, int G = 32, class A = QrArith<T>>
__device__ void qr_warp_fused(T* a, int m, int n, long long lda, typename A::R* rdiag,
                              T* b, long long ldb, int nb, T* coefs) {
  using R = typename A::R;
  const int lane = group_lane<G>();
  const unsigned gm = group_mask<G>();
  T* pc = coefs;              // coefficients of reflector k-1 (index: column - k)
  T* nc = coefs + n + nb;     // coefficients of reflector k (index: column - k - 1)
  const T* pv = nullptr;      // reflector k-1 (column k-1 of a), or null
  bool pskip = false;         // reflector k-1 is degenerate (v0 == 0): right-hand sides skip it
  for (int k = 0; k < n; ++k) {
    T* ck = a + (long long)k * lda;
    if (pv) {
      const T s0 = pc[0];
      for (int r = k - 1 + lane; r < m; r += G) ck[r] = A::muladd(ck[r], pv[r], s0);
      __syncwarp(gm);
    }
    const int len = m - k;
    const R norm = A::norm(len, ck + k);  // every lane of the group, same value
    const bool has = A::nzr(norm);
    T v0{};
    if (has) {
      A::divcol(ck, k + lane, m, G, norm);
      __syncwarp(gm);
      if (lane == 0) ck[k] = A::add1(ck[k]);
      __syncwarp(gm);
      v0 = ck[k];
    }
    const int ncols = (n - k - 1) + nb;
    for (int c = lane; c < ncols; c += G) {
      const int j = k + 1 + c;
      T* cj = qr_col(a, lda, n, b, ldb, j);
      const bool upd = pv && !(j >= n && pskip);
      const T sp = upd ? pc[c + 1] : T{};
      if (upd) cj[k - 1] = A::muladd(cj[k - 1], pv[k - 1], sp);
      if (has) {
        // Dot(len, ck + k, cj + k) over the updated entries.
        int r = k;
        double d = 0.0;
        if (len & 1) {
          const T u = upd ? A::muladd(cj[r], pv[r], sp) : cj[r];
          cj[r] = u;
          d = A::prod(ck[r], u);
          ++r;
        }
        // Software-pipelined by blocks of QF pairs: the next block's loads are issued before the
        // current block's stores (the columns are distinct, but the compiler cannot know that).
        constexpr int QF = sizeof(T) == 8 ? MFG_QR_FUSE_BLOCK_D : MFG_QR_FUSE_BLOCK_F;
        const int pairs = (m - r) >> 1;
        const int blocks = pairs / QF;
        if (blocks > 0) {
          T cu[2 * QF], cv[2 * QF], cp[2 * QF];
#pragma unroll
          for (int u = 0; u < 2 * QF; ++u) {
            cu[u] = cj[r + u];
            cv[u] = ck[r + u];
            cp[u] = upd ? pv[r + u] : T{};
          }
          for (int blk = 0; blk < blocks; ++blk) {
            T nu[2 * QF], nv[2 * QF], np[2 * QF];
            const bool more = blk + 1 < blocks;
            if (more) {
#pragma unroll
              for (int u = 0; u < 2 * QF; ++u) {
                nu[u] = cj[r + 2 * QF + u];
                nv[u] = ck[r + 2 * QF + u];
                np[u] = upd ? pv[r + 2 * QF + u] : T{};
              }
            }
#pragma unroll
            for (int u = 0; u < 2 * QF; ++u) {
              if (upd) {
                cu[u] = A::muladd(cu[u], cp[u], sp);
                cj[r + u] = cu[u];
              }
            }
#pragma unroll
            for (int u = 0; u < QF; ++u)
              d = A::pair(d, cv[2 * u], cu[2 * u], cv[2 * u + 1], cu[2 * u + 1]);
            r += 2 * QF;
            if (more) {
#pragma unroll
              for (int u = 0; u < 2 * QF; ++u) {
                cu[u] = nu[u];
                cv[u] = nv[u];
                cp[u] = np[u];
              }
            }
          }
        }
        for (; r < m; r += 2) {
          T u0 = cj[r], u1 = cj[r + 1];
          if (upd) {
            u0 = A::muladd(u0, pv[r], sp);
            u1 = A::muladd(u1, pv[r + 1], sp);
            cj[r] = u0;
            cj[r + 1] = u1;
          }
          d = A::pair(d, ck[r], u0, ck[r + 1], u1);
        }
        nc[c] = A::coef(d, v0);
      } else if (upd) {
        for (int r = k; r < m; ++r) cj[r] = A::muladd(cj[r], pv[r], sp);
      }
    }
    __syncwarp(gm);
    if (lane == 0) rdiag[k] = A::neg_r(norm);
    __syncwarp(gm);
    pv = has ? ck : nullptr;
    pskip = has && !A::nz(v0);
    T* t = pc;
    pc = nc;
    nc = t;
  }
  // Reflector n-1 still owes its update to the right-hand sides.
  if (pv && !pskip) {
    for (int c = lane; c < nb; c += G) {
      T* cj = b + (long long)c * ldb;
      const T sp = pc[c];
      for (int r = n - 1; r < m; ++r) cj[r] = A::muladd(cj[r], pv[r], sp);
    }
  }
  __syncwarp(gm);
}

// Applies the stored reflectors of a factored matrix to the nb columns of b, in the order and
// arithmetic the factorization applies them (the right-hand-side branch of qr_warp): reflector k
// exists when rdiag[k] != 0 (the column norm was nonzero) and acts when v[0] != 0.
template <typename T, int G = 32, class A = QrArith<T>>
__device__ void qr_apply_warp(const T* a, int m, int n, long long lda,
                              const typename A::R* rdiag, T* b, long long ldb, int nb,
                              T* coefs) {
  const int lane = group_lane<G>();
  const unsigned gm = group_mask<G>();
  for (int k = 0; k < n; ++k) {
    const T* ck = a + (long long)k * lda;
    const T v0 = ck[k];
    if (A::nzr(rdiag[k]) && A::nz(v0)) {
      const int len = m - k;
      for (int c = lane; c < nb; c += G) {
        const T* bj = b + (long long)c * ldb;
        coefs[c] = A::coef(A::dot(len, ck + k, bj + k), v0);
      }
      __syncwarp(gm);
      const long long work = (long long)len * nb;
      for (long long e = lane; e < work; e += G) {
        const int c = (int)(e / len);
        const int r = k + (int)(e - (long long)c * len);
        T* bj = b + (long long)c * ldb;
        bj[r] = A::muladd(bj[r], ck[r], coefs[c]);
      }
    }
    __syncwarp(gm);
  }
}

// R x = y for the first n entries of every right-hand side (Blas.SolveTriangular Upper/NoTrans,
// MatFlat/Blas.SolveTriangular.cs:191-199, against QrUpperTriangularFactor's R).
template <typename T, int G = 32, class A = QrArith<T>>
__device__ void qr_rsolve_warp(const T* a, int n, long long lda, const T* rdiag, T* b,
                               long long ldb, int nb) {
  const int lane = group_lane<G>();
  const unsigned gm = group_mask<G>();
  for (int i = n - 1; i >= 0; --i) {
    for (int c = lane; c < nb; c += G) {
      T* x = b + (long long)c * ldb;
      x[i] = A::div(x[i], rdiag[i]);
    }
    __syncwarp(gm);
    const T* ai = a + (long long)i * lda;
    for (int e = lane; e < nb * i; e += G) {
      const int c = e / i;
      const int r = e - c * i;
      T* x = b + (long long)c * ldb;
      x[r] = A::mulsub(x[r], ai[r], x[i]);
    }
    __syncwarp(gm);
  }
}

// QrOrthogonalFactor: thin Q by backward accumulation of the reflectors.
template <typename T>
__device__ void qr_q_warp(const T* a, int m, int n, long long lda, T* q, long long ldq, T* coefs) {
  using A = QrArith<T>;
  const int lane = threadIdx.x & 31;
  for (int k = n - 1; k >= 0; --k) {
    T* qk = q + (long long)k * ldq;
    const T* ak = a + (long long)k * lda;
    for (int r = lane; r < m; r += 32) qk[r] = A::rdiag_elem((typename A::R)0);
    __syncwarp();
    if (lane == 0) qk[k] = A::rdiag_elem((typename A::R)1);
    __syncwarp();
    const T v0 = ak[k];
    if (A::nz(v0)) {
      const int len = m - k;
      const int ncols = n - k;
      for (int c = lane; c < ncols; c += 32) {
        const T* qj = q + (long long)(k + c) * ldq;
        coefs[c] = A::coef(A::qdot(len, ak + k, qj + k), v0);
      }
      __syncwarp();
      const long long work = (long long)len * ncols;
      for (long long e = lane; e < work; e += 32) {
        const int c = (int)(e / len);
        const int r = k + (int)(e - (long long)c * len);
        T* qj = q + (long long)(k + c) * ldq;
        qj[r] = A::qmuladd(qj[r], ak[r], coefs[c]);
      }
    }
    __syncwarp();
  }
}

constexpr int QR_SMEM_COEFS = 256;   // shared coefficients per warp (G = 32)
constexpr int QR_GROUP_COEFS = 136;  // shared coefficients per group (G < 32): 2 x (64 + 4)

int qr_smem_coefs(int group) { return group == 32 ? QR_SMEM_COEFS : QR_GROUP_COEFS; }

// Persistent batched QR (+ least squares): each group of G lanes takes the next matrix from the
// queue (a warp takes 32/G consecutive ones, which the plan orders to have equal n).
// Sixteen warps per SM are needed to hide the latency of the trailing-matrix streams: the
// register budget is capped accordingly (128 per thread).
// FMA (double only): the FMA form's arithmetic (QrArithFma) for the factorization, the
// reflector applications of solve-only calls and the triangular solve.
template <typename T, int WARPS, int G, bool SOLVE = false, bool FMA = false>
__global__ void __launch_bounds__(WARPS * 32, (16 / WARPS) > 0 ? 16 / WARPS : 1)
    qr_batched_kernel(QrBatchArgs<T> p) {
  using A = std::conditional_t<FMA, QrArithFma, QrArith<T>>;
  constexpr int GPW = 32 / G;
  constexpr int CO = G == 32 ? QR_SMEM_COEFS : QR_GROUP_COEFS;
  __shared__ T sm[WARPS][GPW][CO];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int g = lane / G;
  const long long gw = (long long)blockIdx.x * WARPS + warp;
  for (;;) {
    int idx0 = 0;
    if (lane == 0) idx0 = atomicAdd(p.queue, GPW);
    idx0 = __shfl_sync(FULL_MASK, idx0, 0);
    if (idx0 >= p.count) break;
    const int idx = idx0 + g;
    if (idx < p.count) {
      const int mat = p.order[idx];
      const int m = p.m[mat];
      const int n = p.n[mat];
      const long long lda = p.lda[mat];
      T* a = p.a + p.a_off[mat];
      T* rd = p.rdiag + p.rdiag_off[mat];
      T* b = p.nrhs > 0 ? p.b + p.b_off[mat] : nullptr;
      const int need = p.fused ? 2 * (n + p.nrhs) : n + p.nrhs;
      T* coefs = (need <= CO) ? &sm[warp][g][0]
                              : p.gscratch + (gw * GPW + g) * p.gscratch_stride;
      if constexpr (SOLVE)
        qr_apply_warp<T, G, A>(a, m, n, lda, rd, b, m, p.nrhs, coefs);
      else if (p.fused)
        qr_warp_fused<T, G, A>(a, m, n, lda, rd, b, m, p.nrhs, coefs);
      else
        qr_warp<T, G, A>(a, m, n, lda, rd, b, m, p.nrhs, coefs);
      if (p.nrhs > 0) qr_rsolve_warp<T, G, A>(a, n, lda, rd, b, m, p.nrhs);
    }
    __syncwarp();
  }
}

// Complex overload of the batched QR + least squares (Factorization.Qr Complex,
// MatFlat/Factorization.Qr.cs:198-255): one warp per matrix, the same column schedule as the
// double kernel in complex arithmetic (DotConj coefficients, Complex(norm, 0) divisions); rdiag
// is real.  The right-hand sides receive Q^H b from the same reflector updates, then R x = y with
// Complex SolveTriangular Upper/NoTrans arithmetic (x[i] /= Complex(rdiag[i], 0);
// x[r] -= R(r,i) * x[i]).  args carries the interleaved (re, im) arrays as doubles; offsets count
// complex elements; gscratch_stride counts doubles (2 per coefficient).
constexpr int QR_Z_SMEM_COEFS = 128;

__device__ void zqr_rsolve_warp(const zdouble* a, int n, long long lda, const double* rdiag,
                                zdouble* b, long long ldb, int nb) {
  const int lane = threadIdx.x & 31;
  for (int i = n - 1; i >= 0; --i) {
    const zdouble d = zmake(rdiag[i], 0.0);
    for (int c = lane; c < nb; c += 32) {
      zdouble* x = b + (long long)c * ldb;
      x[i] = zdiv(x[i], d);
    }
    __syncwarp();
    const zdouble* ai = a + (long long)i * lda;
    for (int e = lane; e < nb * i; e += 32) {
      const int c = e / i;
      const int r = e - c * i;
      zdouble* x = b + (long long)c * ldb;
      x[r] = zsub(x[r], zmul(ai[r], x[i]));
    }
    __syncwarp();
  }
}

template <int WARPS, bool SOLVE>
__global__ void __launch_bounds__(WARPS * 32) zqr_batched_kernel(QrBatchArgs<double> p) {
  __shared__ zdouble sm[WARPS][QR_Z_SMEM_COEFS];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const long long gw = (long long)blockIdx.x * WARPS + warp;
  zdouble* abase = reinterpret_cast<zdouble*>(p.a);
  zdouble* bbase = reinterpret_cast<zdouble*>(p.b);
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(p.queue, 1);
    idx = __shfl_sync(FULL_MASK, idx, 0);
    if (idx >= p.count) break;
    const int mat = p.order[idx];
    const int m = p.m[mat];
    const int n = p.n[mat];
    const long long lda = p.lda[mat];
    zdouble* a = abase + p.a_off[mat];
    double* rd = p.rdiag + p.rdiag_off[mat];
    zdouble* b = p.nrhs > 0 ? bbase + p.b_off[mat] : nullptr;
    zdouble* coefs = (n + p.nrhs <= QR_Z_SMEM_COEFS)
                         ? &sm[warp][0]
                         : reinterpret_cast<zdouble*>(p.gscratch + gw * p.gscratch_stride);
    if constexpr (SOLVE)
      qr_apply_warp<zdouble, 32>(a, m, n, lda, rd, b, m, p.nrhs, coefs);
    else
      qr_warp<zdouble, 32>(a, m, n, lda, rd, b, m, p.nrhs, coefs);
    if (p.nrhs > 0) zqr_rsolve_warp(a, n, lda, rd, b, m, p.nrhs);
    __syncwarp();
  }
}

template <bool SOLVE>
static cudaError_t launch_zqr_batched_s(const QrBatchArgs<double>& args, int ctas, int warps,
                                        cudaStream_t s) {
  if (warps > 8) {
    ctas *= warps / 8;
    warps = 8;
  }
  switch (warps) {
    case 1: zqr_batched_kernel<1, SOLVE><<<ctas, 32, 0, s>>>(args); break;
    case 2: zqr_batched_kernel<2, SOLVE><<<ctas, 64, 0, s>>>(args); break;
    case 4: zqr_batched_kernel<4, SOLVE><<<ctas, 128, 0, s>>>(args); break;
    case 8: zqr_batched_kernel<8, SOLVE><<<ctas, 256, 0, s>>>(args); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

int zqr_smem_coefs() { return QR_Z_SMEM_COEFS; }

cudaError_t launch_zqr_batched(const QrBatchArgs<double>& args, int ctas, int warps,
                               cudaStream_t s) {
  return args.solve_only ? launch_zqr_batched_s<true>(args, ctas, warps, s)
                         : launch_zqr_batched_s<false>(args, ctas, warps, s);
}

template <typename T>
__global__ void __launch_bounds__(32) qr_single_kernel(T* a, int m, int n, int lda,
                                                       typename QrArith<T>::R* rdiag, T* scratch) {
  qr_warp<T>(a, m, n, lda, rdiag, (T*)nullptr, 0, 0, scratch);
}

template <typename T>
__global__ void __launch_bounds__(32) qr_q_single_kernel(const T* a, int m, int n, int lda, T* q,
                                                         int ldq, T* scratch) {
  qr_q_warp<T>(a, m, n, lda, q, ldq, scratch);
}

// QrUpperTriangularFactor: R(0:i, i) = a(0:i, i); R(i,i) = rdiag[i]; R(i+1:n, i) = 0.
template <typename T>
__global__ void qr_r_single_kernel(const T* a, int n, int lda, T* r, int ldr,
                                   const typename QrArith<T>::R* rdiag) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)n * n) return;
  const int i = (int)(e / n);   // column
  const int row = (int)(e - (long long)i * n);
  T v;
  if (row < i) v = a[(long long)i * lda + row];
  else if (row == i) v = QrArith<T>::rdiag_elem(rdiag[i]);
  else v = QrArith<T>::rdiag_elem(0);
  r[(long long)i * ldr + row] = v;
}

template <typename T, bool SOLVE, bool FMA>
static cudaError_t launch_qr_batched_s(const QrBatchArgs<T>& args, int ctas, int warps,
                                       cudaStream_t s) {
  if (args.group == 16) {
    qr_batched_kernel<T, 4, 16, SOLVE, FMA><<<ctas, 128, 0, s>>>(args);
  } else if (args.group == 8) {
    qr_batched_kernel<T, 4, 8, SOLVE, FMA><<<ctas, 128, 0, s>>>(args);
  } else if (args.group == 4) {
    qr_batched_kernel<T, 4, 4, SOLVE, FMA><<<ctas, 128, 0, s>>>(args);
  } else {
    switch (warps) {
      case 1: qr_batched_kernel<T, 1, 32, SOLVE, FMA><<<ctas, 32, 0, s>>>(args); break;
      case 2: qr_batched_kernel<T, 2, 32, SOLVE, FMA><<<ctas, 64, 0, s>>>(args); break;
      case 4: qr_batched_kernel<T, 4, 32, SOLVE, FMA><<<ctas, 128, 0, s>>>(args); break;
      case 8: qr_batched_kernel<T, 8, 32, SOLVE, FMA><<<ctas, 256, 0, s>>>(args); break;
      case 16: qr_batched_kernel<T, 16, 32, SOLVE, FMA><<<ctas, 512, 0, s>>>(args); break;
      default: return cudaErrorInvalidValue;
    }
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_qr_batched(const QrBatchArgs<T>& args, int ctas, int warps, cudaStream_t s) {
  if constexpr (std::is_same<T, double>::value) {
    if (args.fma)
      return args.solve_only ? launch_qr_batched_s<T, true, true>(args, ctas, warps, s)
                             : launch_qr_batched_s<T, false, true>(args, ctas, warps, s);
  }
  return args.solve_only ? launch_qr_batched_s<T, true, false>(args, ctas, warps, s)
                         : launch_qr_batched_s<T, false, false>(args, ctas, warps, s);
}

template <typename T>
cudaError_t launch_qr_single(T* a, int m, int n, int lda, T* rdiag, T* scratch, cudaStream_t s) {
  qr_single_kernel<T><<<1, 32, 0, s>>>(a, m, n, lda, rdiag, scratch);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_qr_q_single(const T* a, int m, int n, int lda, T* q, int ldq, T* scratch,
                               cudaStream_t s) {
  qr_q_single_kernel<T><<<1, 32, 0, s>>>(a, m, n, lda, q, ldq, scratch);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_qr_r_single(const T* a, int n, int lda, T* r, int ldr, const T* rdiag,
                               cudaStream_t s) {
  const long long total = (long long)n * n;
  const int threads = 128;
  qr_r_single_kernel<T><<<(unsigned)((total + threads - 1) / threads), threads, 0, s>>>(
      a, n, lda, r, ldr, rdiag);
  return cudaGetLastError();
}

cudaError_t launch_zqr_single(double* a, int m, int n, int lda, double* rdiag, double* scratch,
                              cudaStream_t s) {
  qr_single_kernel<zdouble><<<1, 32, 0, s>>>((zdouble*)a, m, n, lda, rdiag, (zdouble*)scratch);
  return cudaGetLastError();
}

cudaError_t launch_zqr_q_single(const double* a, int m, int n, int lda, double* q, int ldq,
                                double* scratch, cudaStream_t s) {
  qr_q_single_kernel<zdouble><<<1, 32, 0, s>>>((const zdouble*)a, m, n, lda, (zdouble*)q, ldq,
                                               (zdouble*)scratch);
  return cudaGetLastError();
}

cudaError_t launch_zqr_r_single(const double* a, int n, int lda, double* r, int ldr,
                                const double* rdiag, cudaStream_t s) {
  const long long total = (long long)n * n;
  qr_r_single_kernel<zdouble><<<(unsigned)((total + 127) / 128), 128, 0, s>>>(
      (const zdouble*)a, n, lda, (zdouble*)r, ldr, rdiag);
  return cudaGetLastError();
}

template cudaError_t launch_qr_batched<double>(const QrBatchArgs<double>&, int, int, cudaStream_t);
template cudaError_t launch_qr_batched<float>(const QrBatchArgs<float>&, int, int, cudaStream_t);
template cudaError_t launch_qr_single<double>(double*, int, int, int, double*, double*,
                                              cudaStream_t);
template cudaError_t launch_qr_single<float>(float*, int, int, int, float*, float*, cudaStream_t);
template cudaError_t launch_qr_q_single<double>(const double*, int, int, int, double*, int,
                                                double*, cudaStream_t);
template cudaError_t launch_qr_q_single<float>(const float*, int, int, int, float*, int, float*,
                                               cudaStream_t);
template cudaError_t launch_qr_r_single<double>(const double*, int, int, double*, int,
                                                const double*, cudaStream_t);
template cudaError_t launch_qr_r_single<float>(const float*, int, int, float*, int, const float*,
                                               cudaStream_t);

}  // namespace mfg
