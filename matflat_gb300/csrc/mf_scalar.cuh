// Exact scalar arithmetic of MatFlat's float and Complex overloads, on the GPU.
//
// Complex follows System.Numerics.Complex with every product and sum separately rounded:
//   (a+bi)(c+di) = (ac - bd) + (bc + ad)i,
//   division by Smith's algorithm (Smith, CACM 1962), which .NET's Complex uses,
//   Internals.MulConj(x, y) = conj(x) * y (MatFlat/Internals.cs:22-29),
//   Internals.MulConjConj(x, y) = conj(x) * conj(y) (:32-39),
//   Internals.FastMagnitude(x) = |re| + |im| (:16-19), the LU pivot measure.
// Float overloads keep float storage but accumulate dots in double (Internals.cs:149-176).
#pragma once

#include "mf_device.cuh"

namespace mfg {

struct zdouble {
  double re, im;
};

__device__ __forceinline__ zdouble zmake(double re, double im) { return zdouble{re, im}; }
__device__ __forceinline__ zdouble zadd(zdouble x, zdouble y) {
  return {__dadd_rn(x.re, y.re), __dadd_rn(x.im, y.im)};
}
__device__ __forceinline__ zdouble zsub(zdouble x, zdouble y) {
  return {__dsub_rn(x.re, y.re), __dsub_rn(x.im, y.im)};
}
__device__ __forceinline__ zdouble zmul(zdouble x, zdouble y) {
  return {__dsub_rn(__dmul_rn(x.re, y.re), __dmul_rn(x.im, y.im)),
          __dadd_rn(__dmul_rn(x.im, y.re), __dmul_rn(x.re, y.im))};
}
// conj(x) * y
__device__ __forceinline__ zdouble zmulconj(zdouble x, zdouble y) {
  const double a = x.re, b = -x.im, c = y.re, d = y.im;
  return {__dsub_rn(__dmul_rn(a, c), __dmul_rn(b, d)), __dadd_rn(__dmul_rn(a, d), __dmul_rn(b, c))};
}
// conj(x) * conj(y)
__device__ __forceinline__ zdouble zmulconjconj(zdouble x, zdouble y) {
  const double a = x.re, b = -x.im, c = y.re, d = -y.im;
  return {__dsub_rn(__dmul_rn(a, c), __dmul_rn(b, d)), __dadd_rn(__dmul_rn(a, d), __dmul_rn(b, c))};
}
__device__ __forceinline__ zdouble zconj(zdouble x) { return {x.re, -x.im}; }
__device__ __forceinline__ zdouble zneg(zdouble x) { return {-x.re, -x.im}; }
__device__ __forceinline__ double zfastmag(zdouble x) {
  return __dadd_rn(fabs(x.re), fabs(x.im));
}
__device__ __forceinline__ bool znonzero(zdouble x) { return nonzero(x.re) || nonzero(x.im); }

// Smith's algorithm, as System.Numerics.Complex.op_Division evaluates it.
__device__ __forceinline__ zdouble zdiv(zdouble x, zdouble y) {
  const double a = x.re, b = x.im, c = y.re, d = y.im;
  if (fabs(d) < fabs(c)) {
    const double doc = __ddiv_rn(d, c);
    const double den = __dadd_rn(c, __dmul_rn(d, doc));
    return {__ddiv_rn(__dadd_rn(a, __dmul_rn(b, doc)), den),
            __ddiv_rn(__dsub_rn(b, __dmul_rn(a, doc)), den)};
  } else {
    const double cod = __ddiv_rn(c, d);
    const double den = __dadd_rn(d, __dmul_rn(c, cod));
    return {__ddiv_rn(__dadd_rn(b, __dmul_rn(a, cod)), den),
            __ddiv_rn(__dadd_rn(-a, __dmul_rn(b, cod)), den)};
  }
}

// Internals.Dot (Complex, Internals.cs:294-321): same pairwise tree in complex arithmetic.
// CONJ = true gives Internals.DotConj (:352-379): sum of conj(x) * y.
template <bool CONJ>
__device__ __forceinline__ zdouble zdot(int len, const zdouble* x, long long incx,
                                        const zdouble* y, long long incy) {
  zdouble s = {0.0, 0.0};
  if (len & 1) {
    s = CONJ ? zmulconj(x[0], y[0]) : zmul(x[0], y[0]);
    x += incx;
    y += incy;
  }
  for (int p = 0; p < (len >> 1); ++p) {
    const zdouble p0 = CONJ ? zmulconj(x[0], y[0]) : zmul(x[0], y[0]);
    const zdouble p1 = CONJ ? zmulconj(x[incx], y[incy]) : zmul(x[incx], y[incy]);
    s = zadd(s, zadd(p0, p1));
    x += 2 * incx;
    y += 2 * incy;
  }
  return s;
}

__device__ __forceinline__ unsigned long long pivot_key_f(float v) {
  const unsigned b = __float_as_uint(v) & 0x7FFFFFFFu;
  return b > 0x7F800000u ? 0ull : (unsigned long long)b + 1ull;
}
__device__ __forceinline__ bool is_nan_f(float v) {
  return (__float_as_uint(v) & 0x7FFFFFFFu) > 0x7F800000u;
}
__device__ __forceinline__ bool nonzero_f(float v) { return (__float_as_uint(v) << 1) != 0u; }

// ---------------------------------------------------------------------------------------------
// Traits used by the generic LU (Factorization.LuCore, MatFlat/Factorization.Lu.cs:240-406).
//   Acc        type of a dot product's running sum
//   dot        Internals.Dot over (len, x strided, y strided)
//   pair       s + (x0*y0 + x1*y1) in the dot's arithmetic; prod: the lone first product
//   fin        colj[i] = work[i] - s  (the float overload subtracts (float)s in float)
//   key/nan0   pivot measure (|v| or FastMagnitude) as an orderable key / its NaN test
//   nz, div    the "diag != 0" test and DivInplace's true division

struct DTraits {
  using T = double;
  using Acc = double;
  template <int IM, int DB>
  static __device__ __forceinline__ Acc dot(int len, const T* x, long long incx, const T* y,
                                            long long incy) {
    return exact_dot<IM, DB>(len, x, incx, y, incy);
  }
  static __device__ __forceinline__ Acc prod(T x, T y) { return __dmul_rn(x, y); }
  static __device__ __forceinline__ Acc pair(Acc s, T x0, T y0, T x1, T y1) {
    return __dadd_rn(s, __dadd_rn(__dmul_rn(x0, y0), __dmul_rn(x1, y1)));
  }
  static __device__ __forceinline__ T fin(T a, Acc s) { return __dsub_rn(a, s); }
  static __device__ __forceinline__ unsigned long long key(T v) { return pivot_key(v); }
  static __device__ __forceinline__ bool nan0(T v) { return is_nan(v); }
  static __device__ __forceinline__ bool nz(T v) { return nonzero(v); }
  static __device__ __forceinline__ T div(T a, T d) { return __ddiv_rn(a, d); }
};

// The FMA form of the double LU (not MatFlat's bits): the same Crout schedule and pivot rule, with
// every dot as fused multiply-adds (any order; fma_dot's four chains, the last pair fused onto
// the prefix) and the column scaled by the reciprocal of the pivot.
struct DTraitsFma {
  using T = double;
  using Acc = double;
  // DB = 1: two chains (fma_dot2), else four (fma_dot).
  template <int IM, int DB>
  static __device__ __forceinline__ Acc dot(int len, const T* x, long long incx, const T* y,
                                            long long incy) {
    if constexpr (DB == 1) return fma_dot2(len, x, incx, y, incy);
    return fma_dot(len, x, incx, y, incy);
  }
  static __device__ __forceinline__ Acc prod(T x, T y) { return __dmul_rn(x, y); }
  static __device__ __forceinline__ Acc pair(Acc s, T x0, T y0, T x1, T y1) {
    return __fma_rn(x1, y1, __fma_rn(x0, y0, s));
  }
  static __device__ __forceinline__ T fin(T a, Acc s) { return __dsub_rn(a, s); }
  static __device__ __forceinline__ unsigned long long key(T v) { return pivot_key(v); }
  static __device__ __forceinline__ bool nan0(T v) { return is_nan(v); }
  static __device__ __forceinline__ bool nz(T v) { return nonzero(v); }
  static __device__ __forceinline__ T div(T a, T d) { return __ddiv_rn(a, d); }
};

struct STraits {
  using T = float;
  using Acc = double;
  template <int IM, int DB>
  static __device__ __forceinline__ Acc dot(int len, const T* x, long long incx, const T* y,
                                            long long incy) {
    return exact_dot_f(len, x, incx, y, incy);
  }
  static __device__ __forceinline__ Acc prod(T x, T y) { return fmul_wide(x, y); }
  static __device__ __forceinline__ Acc pair(Acc s, T x0, T y0, T x1, T y1) {
    return __dadd_rn(s, __dadd_rn(fmul_wide(x0, y0), fmul_wide(x1, y1)));
  }
  static __device__ __forceinline__ T fin(T a, Acc s) { return __fsub_rn(a, __double2float_rn(s)); }
  static __device__ __forceinline__ unsigned long long key(T v) { return pivot_key_f(v); }
  static __device__ __forceinline__ bool nan0(T v) { return is_nan_f(v); }
  static __device__ __forceinline__ bool nz(T v) { return nonzero_f(v); }
  static __device__ __forceinline__ T div(T a, T d) { return __fdiv_rn(a, d); }
};

struct ZTraits {
  using T = zdouble;
  using Acc = zdouble;
  template <int IM, int DB>
  static __device__ __forceinline__ Acc dot(int len, const T* x, long long incx, const T* y,
                                            long long incy) {
    return zdot<false>(len, x, incx, y, incy);
  }
  static __device__ __forceinline__ Acc prod(T x, T y) { return zmul(x, y); }
  static __device__ __forceinline__ Acc pair(Acc s, T x0, T y0, T x1, T y1) {
    return zadd(s, zadd(zmul(x0, y0), zmul(x1, y1)));
  }
  static __device__ __forceinline__ T fin(T a, Acc s) { return zsub(a, s); }
  static __device__ __forceinline__ unsigned long long key(T v) { return pivot_key(zfastmag(v)); }
  static __device__ __forceinline__ bool nan0(T v) { return is_nan(zfastmag(v)); }
  static __device__ __forceinline__ bool nz(T v) { return znonzero(v); }
  static __device__ __forceinline__ T div(T a, T d) { return zdiv(a, d); }
};

}  // namespace mfg
