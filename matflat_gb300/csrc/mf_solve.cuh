// Warp-level triangular solves in MatFlat's operation order (Blas.SolveTriangular,
// MatFlat/Blas.SolveTriangular.cs:162-242).  One warp solves nr right-hand sides held in a
// scratch buffer xs (right-hand side r at xs[r*ldx + i]); acc is scratch of the same shape.
//
// MatFlat has two loop shapes:
//  - dot form (Lower/NoTrans :216-222, Upper/Trans :201-207):
//        x[i] = (x[i] - Dot(i, row_i, x)) / diag_i
//    The dot of row i has a fixed length i, so its MatFlat summation tree is known in advance:
//    its pairs end at t = i-1, i-3, ...; an odd row starts with its lone first product.  The warp
//    therefore accumulates every row's dot as soon as two more solution entries are final,
//    pair by pair, in exactly that tree, instead of running one dot per row at the end.
//  - column sweep (Upper/NoTrans :191-199, Lower/Trans :224-231):
//        x[i] /= diag_i;  x[r] -= a(r,i) * x[i]  for r < i        (i descending)
//    which is already parallel over r.
#pragma once

#include "mf_device.cuh"
#include "mf_scalar.cuh"

namespace mfg {

// Element arithmetic of the solves (Blas.SolveTriangular's double, float and Complex overloads).
//   prod/pair  the dot-form accumulation (Internals.Dot / DotConj tree, in the dot's type)
//   fin        x[i] = (x[i] - dot) / diag      (float: computed in double, then rounded)
//   fin0       the same for i = 0, where Dot(0) = 0.0 and x - 0.0 = x
//   sdiv/msub  the column sweep: x[i] /= diag; x[r] -= a(r,i) * x[i]
struct DSolve {
  using T = double;
  using Acc = double;
  static __device__ __forceinline__ Acc zero() { return 0.0; }
  static __device__ __forceinline__ Acc prod(T a, T x) { return __dmul_rn(a, x); }
  static __device__ __forceinline__ Acc pair(Acc s, T a0, T x0, T a1, T x1) {
    return __dadd_rn(s, __dadd_rn(__dmul_rn(a0, x0), __dmul_rn(a1, x1)));
  }
  static __device__ __forceinline__ T fin(T x, Acc s, T d, bool unit) {
    const T v = __dsub_rn(x, s);
    return unit ? v : __ddiv_rn(v, d);
  }
  static __device__ __forceinline__ T fin0(T x, T d, bool unit) { return unit ? x : __ddiv_rn(x, d); }
  static __device__ __forceinline__ T sdiv(T x, T d) { return __ddiv_rn(x, d); }
  static __device__ __forceinline__ T msub(T x, T a, T xi) { return __dsub_rn(x, __dmul_rn(a, xi)); }
};

// DSolve with the products on the integer pipes (imul_rn: the IEEE round-to-nearest product, bit
// for bit), which leaves the FP64 pipe the additions, subtractions and divisions.
struct DSolveIM : DSolve {
  static __device__ __forceinline__ Acc prod(T a, T x) { return imul_rn(a, x); }
  static __device__ __forceinline__ Acc pair(Acc s, T a0, T x0, T a1, T x1) {
    return __dadd_rn(s, __dadd_rn(imul_rn(a0, x0), imul_rn(a1, x1)));
  }
  static __device__ __forceinline__ T msub(T x, T a, T xi) { return __dsub_rn(x, imul_rn(a, xi)); }
};

struct SSolve {
  using T = float;
  using Acc = double;
  static __device__ __forceinline__ Acc zero() { return 0.0; }
  // Widened float products are exact in double: formed on the integer pipes (fmul_wide).
  static __device__ __forceinline__ Acc prod(T a, T x) { return fmul_wide(a, x); }
  static __device__ __forceinline__ Acc pair(Acc s, T a0, T x0, T a1, T x1) {
    return __dadd_rn(s, __dadd_rn(fmul_wide(a0, x0), fmul_wide(a1, x1)));
  }
  static __device__ __forceinline__ T fin(T x, Acc s, T d, bool unit) {
    const double v = __dsub_rn((double)x, s);
    return __double2float_rn(unit ? v : __ddiv_rn(v, (double)d));
  }
  static __device__ __forceinline__ T fin0(T x, T d, bool unit) {
    return unit ? x : __double2float_rn(__ddiv_rn((double)x, (double)d));
  }
  static __device__ __forceinline__ T sdiv(T x, T d) { return __fdiv_rn(x, d); }
  static __device__ __forceinline__ T msub(T x, T a, T xi) { return __fsub_rn(x, __fmul_rn(a, xi)); }
};

// CONJ: the ConjNoTrans / ConjTrans modes (DotConj, MulSubConj, division by conj(diag)).
template <bool CONJ>
struct ZSolve {
  using T = zdouble;
  using Acc = zdouble;
  static __device__ __forceinline__ zdouble m(zdouble a, zdouble x) {
    return CONJ ? zmulconj(a, x) : zmul(a, x);
  }
  static __device__ __forceinline__ zdouble dg(zdouble d) { return CONJ ? zconj(d) : d; }
  static __device__ __forceinline__ Acc zero() { return zmake(0.0, 0.0); }
  static __device__ __forceinline__ Acc prod(T a, T x) { return m(a, x); }
  static __device__ __forceinline__ Acc pair(Acc s, T a0, T x0, T a1, T x1) {
    return zadd(s, zadd(m(a0, x0), m(a1, x1)));
  }
  // A unit diagonal is still divided by: the LuInverse idiom stores Complex(1, 0) there, and
  // Complex division by (1, 0) is not the identity (a signed zero can flip, an infinite part
  // turns the other part into NaN).
  static __device__ __forceinline__ T fin(T x, Acc s, T d, bool unit) {
    const zdouble v = zsub(x, s);
    return zdiv(v, unit ? zmake(1.0, 0.0) : dg(d));
  }
  static __device__ __forceinline__ T fin0(T x, T d, bool unit) {
    return zdiv(x, unit ? zmake(1.0, 0.0) : dg(d));
  }
  static __device__ __forceinline__ T sdiv(T x, T d) { return zdiv(x, dg(d)); }
  static __device__ __forceinline__ T msub(T x, T a, T xi) { return zsub(x, m(a, xi)); }
};

// ZSolve<false> with the dot's four real products per multiply on the integer pipes (imul_rn,
// bit-identical to __dmul_rn), which leaves the FP64 pipe the additions only.
struct ZSolveIM : ZSolve<false> {
  static __device__ __forceinline__ zdouble m(zdouble a, zdouble x) {
    return {__dsub_rn(imul_rn(a.re, x.re), imul_rn(a.im, x.im)),
            __dadd_rn(imul_rn(a.im, x.re), imul_rn(a.re, x.im))};
  }
  static __device__ __forceinline__ Acc prod(T a, T x) { return m(a, x); }
  static __device__ __forceinline__ Acc pair(Acc s, T a0, T x0, T a1, T x1) {
    return zadd(s, zadd(m(a0, x0), m(a1, x1)));
  }
};

// Dot form.  Element (i, t), t < i, of the triangular operand is at a[i*si + t*st] and the
// diagonal at a[i*si + i*st].  With unit = true the diagonal is taken as one: MatFlat's
// unit-lower idiom divides by an explicit 1.0 (Factorization.LuInverse.cs:174-182), which is
// exact for double and float (the division is skipped) and done as a division for Complex.
template <int G = 32, class Tr = DSolve>
__device__ __forceinline__ void warp_solve_dot(const typename Tr::T* a, int n, long long si,
                                               long long st, bool unit, typename Tr::T* xs,
                                               int ldx, typename Tr::Acc* acc, int nr) {
  using T = typename Tr::T;
  const int lane = group_lane<G>();
  const unsigned gm = group_mask<G>();
  for (int e = lane; e < nr * n; e += G) {
    const int r = e / n;
    acc[r * ldx + (e - r * n)] = Tr::zero();
  }
  __syncwarp(gm);
  for (int t = 0; t < n; ++t) {
    // x[t] is final: its last pair was added at step t-1.
    for (int r = lane; r < nr; r += G) {
      const T v = xs[r * ldx + t];
      const T d = a[t * si + t * st];
      xs[r * ldx + t] = (t > 0) ? Tr::fin(v, acc[r * ldx + t], d, unit) : Tr::fin0(v, d, unit);
    }
    __syncwarp(gm);
    // Rows i = t+1, t+3, ... close a pair at t (or, at t = 0, take their lone first product).
    const int cnt = (n - t) >> 1;
    for (int e = lane; e < nr * cnt; e += G) {
      const int q = e / nr;
      const int r = e - q * nr;
      const int i = t + 1 + 2 * q;
      typename Tr::Acc* ap = acc + r * ldx + i;
      const T* ai = a + i * si;
      if (t == 0) {
        *ap = Tr::prod(ai[0], xs[r * ldx]);
      } else {
        *ap = Tr::pair(*ap, ai[(t - 1) * st], xs[r * ldx + t - 1], ai[t * st], xs[r * ldx + t]);
      }
    }
    __syncwarp(gm);
  }
}

// Column sweep.  Element (r, i), r < i, is at a[i*si + r*sr]; the diagonal at a[i*si + i*sr], or
// at diag[i] when diag is given (the R factor of QR keeps its diagonal apart, in rdiag).
template <int G = 32, class Tr = DSolve>
__device__ __forceinline__ void warp_solve_sweep(const typename Tr::T* a, int n, long long si,
                                                 long long sr, typename Tr::T* xs, int ldx,
                                                 int nr, const typename Tr::T* diag = nullptr) {
  using T = typename Tr::T;
  const int lane = group_lane<G>();
  const unsigned gm = group_mask<G>();
  for (int i = n - 1; i >= 0; --i) {
    const T* ai = a + i * si;
    const T d = diag ? diag[i] : ai[i * sr];
    for (int r = lane; r < nr; r += G) xs[r * ldx + i] = Tr::sdiv(xs[r * ldx + i], d);
    __syncwarp(gm);
    for (int e = lane; e < nr * i; e += G) {
      const int q = e / nr;
      const int r = e - q * nr;
      T* xp = xs + r * ldx + q;
      *xp = Tr::msub(*xp, ai[q * sr], xs[r * ldx + i]);
    }
    __syncwarp(gm);
  }
}

}  // namespace mfg
