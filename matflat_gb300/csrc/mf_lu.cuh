// LU with partial pivoting in MatFlat's arithmetic (Factorization.LuCore,
// MatFlat/Factorization.Lu.cs:296-350) as warp-level and CTA-level routines, shared by the batched
// kernels of lu.cu (MatFlat's arithmetic), lu_fma.cu and lu_big.cu (the FMA form and its
// fallbacks).
//
// MatFlat is a left-looking "dot product" LU: for column j it computes every entry as
//     v(i,j) = A'(i,j) - Dot(min(i,j), L(i,0:), U(0:,j))         (Lu.cs:315-320)
// with Internals.Dot's pairwise tree, picks the pivot by a strict ">" scan over |v|
// (Lu.cs:323-330), swaps whole rows (Lu.cs:332-337) and divides the sub-diagonal by the pivot
// (Lu.cs:340-344).  Every entry's value depends only on its own dot, so the entries can be
// computed in any order that respects data dependencies.  The routines use the Crout order:
// step k finishes row k of U (U(k,j), j > k: dots of length k) and column k+1 of L (dots of
// length k+1), each dot evaluated with exactly MatFlat's tree, so factors and pivots are
// bit-identical.  To keep the lanes busy, the long prefix of every column-(k+1) dot (all pairs
// but the last) runs in the same round as the row-k dots; the last pair, which needs L(:,k) and
// U(k,k+1), is added afterwards:
//     Dot(k+1, x, y) = Dot(k-1, x, y) + (x[k-1]*y[k-1] + x[k]*y[k])      (k >= 1)
//     Dot(1, x, y)   = x[0]*y[0]
// A group of G lanes (8, 16 or 32) works on one matrix in place in its global buffer (L1/L2
// resident while it is being factored).
#pragma once

#include <cuda_runtime.h>

#include <climits>
#include <type_traits>

#include "mf_device.cuh"
#include "mf_kernels.h"
#include "mf_scalar.cuh"
#include "mf_solve.cuh"

namespace mfg {


// Finishes column c (rows [c, m)) once its dot sums are final, then pivots and scales it.
//   mode 0: column 0 (no dot: v = A - 0.0 = A, left as is)
//   mode 1: column 1 (sum = L(i,0) * U(0,1))
//   mode 2: column c >= 2 (sum = scol[i] + (L(i,c-2)*U(c-2,c) + L(i,c-1)*U(c-1,c)))
// Tr supplies the element type's arithmetic (double, float or Complex overload).
// G: lanes per matrix (8, 16 or 32): the matrix is worked on by a group of G consecutive lanes
// of the warp, the other groups of the warp work on other matrices of the same order.
//
// FMA (DTraitsFma): the FMA form's screen.  The form keeps MatFlat's pivot only where the choice
// cannot depend on rounding: every lane also keeps its second-largest key, and the column fails
// (*fail = true, nothing swapped or scaled, the caller redoes the matrix in MatFlat's arithmetic)
// when a candidate is not finite, the pivot is zero, or the runner-up is within 2^26 units in the
// last place (a relative margin of about 1.5e-8) of the pivot, ties included.  The margin is a
// screen, not a proof: FMA and MatFlat values of a candidate differ by rounding amplified by the
// conditioning of the leading block, far below it for the matrices of the benchmarks, and the
// oracle compares the pivots of whole batches.
constexpr unsigned long long LU_FMA_MARGIN_ULPS = 1ull << 26;

__device__ __forceinline__ bool finite_bits(double v) {
  return (dbits(v) & 0x7FF0000000000000ull) != 0x7FF0000000000000ull;
}

template <class Tr, int G = 32, bool IDIV = false, bool FMA = false>
__device__ __forceinline__ void lu_finish_column(typename Tr::T* a, int m, int n, long long lda,
                                                 int c, int mode,
                                                 const typename Tr::Acc* scol, int* piv,
                                                 int& sign, int& info, int* pivot = nullptr,
                                                 bool* fail = nullptr) {
  using T = typename Tr::T;
  using Acc = typename Tr::Acc;
  const int lane = group_lane<G>();
  const unsigned gm = group_mask<G>();
  T* cc = a + (long long)c * lda;
  unsigned long long bkey = 0ull;
  unsigned long long skey = 0ull;   // FMA: the lane's second-largest key
  bool bad = false;                 // FMA: a candidate that is not finite
  int bidx = INT_MAX;
  bool first_nan = false;
  if (mode == 0) {
    for (int i = c + lane; i < m; i += G) {
      const T v = cc[i];
      const unsigned long long key = Tr::key(v);
      if (key > bkey) {
        if constexpr (FMA) skey = bkey;
        bkey = key;
        bidx = i;
      } else if (FMA && key > skey) {
        skey = key;
      }
      if constexpr (FMA) bad |= !finite_bits(v);
      if (i == c) first_nan = Tr::nan0(v);
    }
  } else {
    const T* l1 = a + (long long)(c - 1) * lda;  // L(:, c-1)
    const T u1 = cc[c - 1];                       // U(c-1, c)
    const T* l2 = (mode == 2) ? a + (long long)(c - 2) * lda : l1;
    const T u2 = (mode == 2) ? cc[c - 2] : u1;    // U(c-2, c)
    for (int i = c + lane; i < m; i += G) {
      Acc s;
      if constexpr (IDIV) {
        // Double with integer-pipe arithmetic: the products on the integer pipes too.
        s = mode == 1 ? imul_rn(l1[i], u1)
                      : __dadd_rn(scol[i], __dadd_rn(imul_rn(l2[i], u2), imul_rn(l1[i], u1)));
      } else if (mode == 1) {
        s = Tr::prod(l1[i], u1);
      } else {
        s = Tr::pair(scol[i], l2[i], u2, l1[i], u1);
      }
      const T v = Tr::fin(cc[i], s);
      cc[i] = v;
      const unsigned long long key = Tr::key(v);
      if (key > bkey) {
        if constexpr (FMA) skey = bkey;
        bkey = key;
        bidx = i;
      } else if (FMA && key > skey) {
        skey = key;
      }
      if constexpr (FMA) bad |= !finite_bits(v);
      if (i == c) first_nan = Tr::nan0(v);
    }
  }
  int p = group_argmax<G>(bkey, bidx);
  if constexpr (FMA) {
    // The pivot's key and the largest key of the other rows, over the group.
    unsigned long long pk = bkey;
    unsigned long long q = bidx == p ? skey : bkey;
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) {
      const unsigned long long opk = __shfl_xor_sync(gm, pk, off);
      const unsigned long long oq = __shfl_xor_sync(gm, q, off);
      pk = opk > pk ? opk : pk;
      q = oq > q ? oq : q;
    }
    if (__any_sync(gm, bad || first_nan) || pk <= 1ull || pk - q < LU_FMA_MARGIN_ULPS) {
      *fail = true;   // the same outcome on every lane of the group
      return;
    }
  }
  // Row c is handled by the group's lane 0; a NaN there can never be displaced by the strict ">"
  // scan.
  if (__shfl_sync(gm, first_nan ? 1 : 0, 0, G)) p = c;
  if (pivot) *pivot = p;
  __syncwarp(gm);
  if (p != c && p < m) {
    for (int col = lane; col < n; col += G) {
      T* base = a + (long long)col * lda;
      const T t = base[c];
      base[c] = base[p];
      base[p] = t;
    }
    if (lane == 0) {
      const int t = piv[c];
      piv[c] = piv[p];
      piv[p] = t;
    }
    sign = -sign;
  }
  __syncwarp(gm);
  const T diag = cc[c];
  if (Tr::nz(diag)) {
    if constexpr (FMA) {
      const double r = __drcp_rn(diag);
      for (int i = c + 1 + lane; i < m; i += G) cc[i] = __dmul_rn(cc[i], r);
    } else if constexpr (IDIV) {
      // Quotients on the integer pipes (the same bits as the FP64 division): the reciprocal is
      // formed once per column.
      idiv_column(cc, c + 1 + lane, m, G, diag);
    } else {
      for (int i = c + 1 + lane; i < m; i += G) cc[i] = Tr::div(cc[i], diag);
    }
  } else if (info == 0) {
    info = c + 1;
  }
  __syncwarp(gm);
}

// Factors the m-by-n matrix a (leading dimension lda) in place; piv receives the permutation
// vector (m entries).  scol: m values of per-warp scratch (Tr::Acc).  Returns Lu's sign in `sign`
// and in `info` the first zero pivot (k+1), or 0.
//
// EARLY (square matrices; scol2: m more values): the lanes left idle in the last round of a step
// compute prefixes of the column after next.  Column c's prefix Dot(c-2, L(i,:), U(:,c)) reads
// U rows 0..c-3 only, which are final after step c-3, so it may run at step c-2 instead of c-1;
// the values are the same (the same dot, evaluated once).  At step k the rows [m - e, m) (e <= the
// idle lanes of the step's last round, rows >= k+2) get column k+2's prefix early; at step k+1
// column k+2's regular items cover the other rows, plus the row swapped into the early range by
// column k+1's pivot (its early value belonged to the row that moved out).  Columns alternate
// between the two prefix arrays (scol: even columns, scol2: odd).

// FMA (DTraitsFma): the FMA form; returns early with *fail set when a column fails the screen of
// lu_finish_column.
template <class Tr, int IM, int DB = DOT_BLOCK, int G = 32, bool EARLY = false, bool FMA = false>
__device__ void lu_warp(typename Tr::T* a, int m, int n, long long lda, int* piv,
                        typename Tr::Acc* scol, int& sign, int& info,
                        typename Tr::Acc* scol2 = nullptr, bool* fail = nullptr) {
  using T = typename Tr::T;
  using Acc = typename Tr::Acc;
  const int lane = group_lane<G>();
  const unsigned gm = group_mask<G>();
  for (int i = lane; i < m; i += G) piv[i] = i;
  sign = 1;
  info = 0;
  __syncwarp(gm);
  const int K = m < n ? m : n;
  constexpr bool IDIV = MFG_IDIV && IM != 0 && std::is_same<Tr, DTraits>::value;
  lu_finish_column<Tr, G, IDIV, FMA>(a, m, n, lda, 0, 0, scol, piv, sign, info, nullptr, fail);
  if constexpr (FMA) {
    if (*fail) return;
  }
  int e_prev = 0;        // rows [m - e_prev, m) got column k1's prefix at the previous step
  int p_prev = INT_MAX;  // the pivot row of column k (chosen at the end of the previous step)
  for (int k = 0; k < K; ++k) {
    const int k1 = k + 1;
    const int R = n - k1;                     // row-k dots: U(k, j), j in [k1, n)
    const T* rowk = a + k;                    // L(k, t) = rowk[t*lda]
    const T* colk1 = a + (long long)k1 * lda;
    Acc* pre1 = (EARLY && (k1 & 1)) ? scol2 : scol;   // column k1's prefixes
    // Regular prefix items of column k1: rows [k1, m - e_prev), plus the displaced row.
    const bool has_col = k1 < K && k >= 1;
    const int nreg0 = has_col ? max(0, m - e_prev - k1) : 0;
    const int disp = (has_col && EARLY && e_prev > 0 && p_prev >= m - e_prev && p_prev < m) ? 1
                                                                                            : 0;
    const int C = nreg0 + disp;
    int E = 0;
    if constexpr (EARLY) {
      if (k >= 2 && k + 2 < K) E = min(m - (k + 2), (G - (R + C) % G) % G);
    }
    Acc* pre2 = (k & 1) ? scol2 : scol;               // column k+2's prefixes (EARLY)
    const T* colk2 = a + (long long)(k + 2) * lda;
    for (int d = lane; d < R + C + E; d += G) {
      // One dot per item (a single call site keeps the register count of one dot loop): row
      // items U(k, idx) (length k), column k1's prefixes (k-1), column k+2's early prefixes (k).
      const bool isrow = d < R;
      const bool isreg = !isrow && d < R + C;
      const int c = d - R;
      const int idx = isrow ? k1 + d : isreg ? (c < nreg0 ? k1 + c : p_prev) : m - E + (c - C);
      const T* x = isrow ? rowk : a + idx;
      const T* y = isrow ? a + (long long)idx * lda : isreg ? colk1 : colk2;
      const int len = isreg ? k - 1 : k;
      const Acc s = Tr::template dot<IM, DB>(len, x, lda, y, 1);
      if (isrow) {
        T* dst = a + (long long)idx * lda + k;
        *dst = Tr::fin(*dst, s);
      } else {
        (isreg ? pre1 : pre2)[idx] = s;
      }
    }
    __syncwarp(gm);
    int pk = INT_MAX;
    if (k1 < K) {
      lu_finish_column<Tr, G, IDIV, FMA>(a, m, n, lda, k1, k1 == 1 ? 1 : 2, pre1, piv, sign,
                                         info, &pk, fail);
      if constexpr (FMA) {
        if (*fail) return;
      }
    }
    e_prev = E;
    p_prev = pk;
  }
  // MatFlat also visits columns j >= m when n > m, but nothing changes there (no pivot rows).
}

// Solves A x = b for nr right-hand sides from the factors of one square matrix:
// b' = P b (b'[i] = b[piv[i]]), then the unit-lower solve (dot form, LuInverse idiom), then the
// upper solve (column sweep).  b: column-major, leading dimension ldb, overwritten with x.
// S: the solve arithmetic of the element type (DSolve, SSolve or ZSolve<false>).
template <class S = DSolve, int G = 32>
__device__ void getrs_warp(const typename S::T* lu, int n, long long lda, const int* piv,
                           typename S::T* b, long long ldb, int nrhs, typename S::T* xs,
                           typename S::Acc* acc) {
  const int lane = group_lane<G>();
  const unsigned gm = group_mask<G>();
  const int ldx = n | 1;
  for (int r0 = 0; r0 < nrhs; r0 += RHS_CHUNK) {
    const int nr = nrhs - r0 < RHS_CHUNK ? nrhs - r0 : RHS_CHUNK;
    for (int e = lane; e < nr * n; e += G) {
      const int r = e / n;
      const int i = e - r * n;
      xs[r * ldx + i] = b[(long long)(r0 + r) * ldb + piv[i]];
    }
    __syncwarp(gm);
    warp_solve_dot<G, S>(lu, n, 1, lda, true, xs, ldx, acc, nr);
    warp_solve_sweep<G, S>(lu, n, lda, 1, xs, ldx, nr);
    for (int e = lane; e < nr * n; e += G) {
      const int r = e / n;
      const int i = e - r * n;
      b[(long long)(r0 + r) * ldb + i] = xs[r * ldx + i];
    }
    __syncwarp(gm);
  }
}

// A x = b for nr right-hand sides from the factors of one square matrix: b' = P b (b'[i] =
// b[piv[i]]), then L y = b' (unit lower) and U x = y, both as column sweeps with fused
// multiply-adds (column t of the factor is contiguous), U's diagonal applied as its reciprocal.
// rcp: n doubles of the group's scratch.  b: column-major, leading dimension ldb, overwritten.
// The solve of the FMA form (lu_fma.cu, lu_big.cu) for every matrix, fallbacks included.  Every
// right-hand side's arithmetic is independent of the others', so any split of them over calls
// or groups gives the same bits.  RCP: rcp already holds the reciprocals of U's diagonal.
template <int G, bool RCP = false>
__device__ void getrs_fma(const double* lu, int n, long long lda, const int* piv, double* b,
                          long long ldb, int nrhs, double* xs, double* rcp) {
  const int lane = group_lane<G>();
  const unsigned gm = group_mask<G>();
  const int ldx = n | 1;
  if (!RCP)
    for (int t = lane; t < n; t += G) rcp[t] = __drcp_rn(lu[(long long)t * lda + t]);
  __syncwarp(gm);
  for (int r0 = 0; r0 < nrhs; r0 += RHS_CHUNK) {
    const int nr = nrhs - r0 < RHS_CHUNK ? nrhs - r0 : RHS_CHUNK;
    for (int e = lane; e < nr * n; e += G) {
      const int r = e / n;
      const int i = e - r * n;
      xs[r * ldx + i] = b[(long long)(r0 + r) * ldb + piv[i]];
    }
    __syncwarp(gm);
    for (int t = 0; t + 1 < n; ++t) {
      const double* colt = lu + (long long)t * lda;
      double xt[RHS_CHUNK];
#pragma unroll
      for (int r = 0; r < RHS_CHUNK; ++r) xt[r] = r < nr ? xs[r * ldx + t] : 0.0;
      for (int i = t + 1 + lane; i < n; i += G) {
        const double l = colt[i];
#pragma unroll
        for (int r = 0; r < RHS_CHUNK; ++r)
          if (r < nr) xs[r * ldx + i] = __fma_rn(-l, xt[r], xs[r * ldx + i]);
      }
      __syncwarp(gm);
    }
    for (int t = n - 1; t >= 0; --t) {
      const double* colt = lu + (long long)t * lda;
      const double rt = rcp[t];
      double xt[RHS_CHUNK];
#pragma unroll
      for (int r = 0; r < RHS_CHUNK; ++r) xt[r] = r < nr ? __dmul_rn(xs[r * ldx + t], rt) : 0.0;
      __syncwarp(gm);
      if (lane == 0)
        for (int r = 0; r < nr; ++r) xs[r * ldx + t] = xt[r];
      for (int i = lane; i < t; i += G) {
        const double u = colt[i];
#pragma unroll
        for (int r = 0; r < RHS_CHUNK; ++r)
          if (r < nr) xs[r * ldx + i] = __fma_rn(-u, xt[r], xs[r * ldx + i]);
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

// ---------------------------------------------------------------------------------------------
// The same schedule with a whole CTA of W warps on one matrix, for large orders when there are too
// few matrices to give every SM several warps (and for the mixed solver's FP64 fallback): a step's
// 2(n-k-1) dots are spread over the CTA's threads, the pivot search is a warp argmax followed by a
// reduction over the W warps' candidates (larger key, then smaller row), and the swap and the
// scaling are spread over the threads.  Per-entry arithmetic is unchanged, so the bits are the same.
struct CtaRed {
  unsigned long long key[32];
  int idx[32];
  int nan0;
};

template <int W, bool IDIV = false>
__device__ void lu_cta_finish_column(double* a, int n, long long lda, int c, int mode,
                                     const double* scol, int* piv, int& sign, int& info,
                                     CtaRed* red, int* pivot = nullptr) {
  using Tr = DTraits;
  constexpr int T = W * 32;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  double* cc = a + (long long)c * lda;
  unsigned long long bkey = 0ull;
  int bidx = INT_MAX;
  if (mode == 0) {
    for (int i = c + tid; i < n; i += T) {
      const double v = cc[i];
      const unsigned long long key = Tr::key(v);
      if (key > bkey) {
        bkey = key;
        bidx = i;
      }
      if (i == c) red->nan0 = Tr::nan0(v) ? 1 : 0;
    }
  } else {
    const double* l1 = a + (long long)(c - 1) * lda;
    const double u1 = cc[c - 1];
    const double* l2 = (mode == 2) ? a + (long long)(c - 2) * lda : l1;
    const double u2 = (mode == 2) ? cc[c - 2] : u1;
    for (int i = c + tid; i < n; i += T) {
      const double s =
          IDIV ? (mode == 1 ? imul_rn(l1[i], u1)
                            : __dadd_rn(scol[i], __dadd_rn(imul_rn(l2[i], u2), imul_rn(l1[i], u1))))
               : (mode == 1 ? Tr::prod(l1[i], u1) : Tr::pair(scol[i], l2[i], u2, l1[i], u1));
      const double v = Tr::fin(cc[i], s);
      cc[i] = v;
      const unsigned long long key = Tr::key(v);
      if (key > bkey) {
        bkey = key;
        bidx = i;
      }
      if (i == c) red->nan0 = Tr::nan0(v) ? 1 : 0;
    }
  }
  const int wp = warp_argmax(bkey, bidx);
  unsigned long long wk = bkey;   // the warp's largest key, which belongs to row wp
  for (int off = 16; off > 0; off >>= 1) {
    const unsigned long long ok = __shfl_xor_sync(FULL_MASK, wk, off);
    if (ok > wk) wk = ok;
  }
  if (lane == 0) {
    red->key[warp] = wk;
    red->idx[warp] = wp;
  }
  __syncthreads();
  unsigned long long best = red->key[0];
  int p = red->idx[0];
  for (int w = 1; w < W; ++w) {
    const unsigned long long k2 = red->key[w];
    const int i2 = red->idx[w];
    if (k2 > best || (k2 == best && i2 < p)) {
      best = k2;
      p = i2;
    }
  }
  if (red->nan0) p = c;
  if (pivot) *pivot = p;
  if (p != c && p < n) {
    for (int col = tid; col < n; col += T) {
      double* base = a + (long long)col * lda;
      const double t = base[c];
      base[c] = base[p];
      base[p] = t;
    }
    if (tid == 0) {
      const int t = piv[c];
      piv[c] = piv[p];
      piv[p] = t;
    }
    sign = -sign;
  }
  __syncthreads();
  const double diag = cc[c];
  if (Tr::nz(diag)) {
    if constexpr (IDIV) {
      idiv_column(cc, c + 1 + tid, n, T, diag);
    } else {
      for (int i = c + 1 + tid; i < n; i += T) cc[i] = Tr::div(cc[i], diag);
    }
  } else if (info == 0) {
    info = c + 1;
  }
  __syncthreads();
}

template <int W, int IM, int DB>
__device__ void lu_cta(double* a, int n, long long lda, int* piv, double* scol, int& sign,
                       int& info, CtaRed* red) {
  using Tr = DTraits;
  constexpr int T = W * 32;
  const int tid = threadIdx.x;
  for (int i = tid; i < n; i += T) piv[i] = i;
  sign = 1;
  info = 0;
  __syncthreads();
  lu_cta_finish_column<W, MFG_IDIV && IM != 0>(a, n, lda, 0, 0, scol, piv, sign, info, red);
  for (int k = 0; k < n; ++k) {
    const int k1 = k + 1;
    const int R = n - k1;
    const int C = (k1 < n && k >= 1) ? n - k1 : 0;
    const double* rowk = a + k;
    const double* colk1 = a + (long long)k1 * lda;
    for (int d = tid; d < R + C; d += T) {
      const bool isrow = d < R;
      const int idx = isrow ? k1 + d : k1 + (d - R);
      const double* x = isrow ? rowk : a + idx;
      const double* y = isrow ? a + (long long)idx * lda : colk1;
      const int len = isrow ? k : k - 1;
      const double s = Tr::template dot<IM, DB>(len, x, lda, y, 1);
      if (isrow) {
        double* dst = a + (long long)idx * lda + k;
        *dst = Tr::fin(*dst, s);
      } else {
        scol[idx] = s;
      }
    }
    __syncthreads();
    if (k1 < n)
      lu_cta_finish_column<W, MFG_IDIV && IM != 0>(a, n, lda, k1, k1 == 1 ? 1 : 2, scol, piv, sign,
                                                   info, red);
  }
}

// lu_cta with the early prefixes of lu_warp<..., EARLY = true>: threads left idle in the last round
// of step k compute column k+2's prefixes for the bottom rows (the same dots, evaluated once, in the
// same tree), and the row swapped into that range by column k+1's pivot gets its prefix again at
// step k+1.  Column sums alternate between scol (even columns) and scol2 (odd columns).
template <int W, int IM, int DB>
__device__ void lu_cta_early(double* a, int n, long long lda, int* piv, double* scol,
                             double* scol2, int& sign, int& info, CtaRed* red) {
  using Tr = DTraits;
  constexpr int T = W * 32;
  constexpr bool IDIV = MFG_IDIV && IM != 0;
  const int tid = threadIdx.x;
  for (int i = tid; i < n; i += T) piv[i] = i;
  sign = 1;
  info = 0;
  __syncthreads();
  lu_cta_finish_column<W, IDIV>(a, n, lda, 0, 0, scol, piv, sign, info, red);
  int e_prev = 0;
  int p_prev = INT_MAX;
  for (int k = 0; k < n; ++k) {
    const int k1 = k + 1;
    const int R = n - k1;
    const double* rowk = a + k;
    const double* colk1 = a + (long long)k1 * lda;
    double* pre1 = (k1 & 1) ? scol2 : scol;
    const bool has_col = k1 < n && k >= 1;
    const int nreg0 = has_col ? max(0, n - e_prev - k1) : 0;
    const int disp = (has_col && e_prev > 0 && p_prev >= n - e_prev && p_prev < n) ? 1 : 0;
    const int C = nreg0 + disp;
    int E = 0;
    if (k >= 2 && k + 2 < n) E = min(n - (k + 2), (T - (R + C) % T) % T);
    double* pre2 = (k & 1) ? scol2 : scol;
    const double* colk2 = a + (long long)(k + 2) * lda;
    for (int d = tid; d < R + C + E; d += T) {
      const bool isrow = d < R;
      const bool isreg = !isrow && d < R + C;
      const int c = d - R;
      const int idx = isrow ? k1 + d : isreg ? (c < nreg0 ? k1 + c : p_prev) : n - E + (c - C);
      const double* x = isrow ? rowk : a + idx;
      const double* y = isrow ? a + (long long)idx * lda : isreg ? colk1 : colk2;
      const int len = isreg ? k - 1 : k;
      const double s = Tr::template dot<IM, DB>(len, x, lda, y, 1);
      if (isrow) {
        double* dst = a + (long long)idx * lda + k;
        *dst = Tr::fin(*dst, s);
      } else {
        (isreg ? pre1 : pre2)[idx] = s;
      }
    }
    __syncthreads();
    int pk = INT_MAX;
    if (k1 < n)
      lu_cta_finish_column<W, IDIV>(a, n, lda, k1, k1 == 1 ? 1 : 2, pre1, piv, sign, info, red,
                                    &pk);
    e_prev = E;
    p_prev = pk;
  }
}

// Per group of a size-bucketed task: the column sums of even and of odd columns (n <= SMEM_N),
// SMEM_N + 1 apart.
constexpr int GROUP_SMEM_DOUBLES = 2 * SMEM_N + 2;

}  // namespace mfg
