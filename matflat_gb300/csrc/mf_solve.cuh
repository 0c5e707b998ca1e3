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

namespace mfg {

// Lanes of a group of G consecutive lanes (G = 32: the whole warp) and the group's sync mask.
template <int G>
__device__ __forceinline__ int group_lane() {
  return threadIdx.x & (G - 1);
}
template <int G>
__device__ __forceinline__ unsigned group_mask() {
  if constexpr (G == 32) {
    return FULL_MASK;
  } else {
    return ((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1));
  }
}

// Dot form.  Element (i, t), t < i, of the triangular operand is at a[i*si + t*st] and the
// diagonal at a[i*si + i*st].  With unit = true the division is skipped: MatFlat's unit-lower
// idiom divides by an explicit 1.0 (Factorization.LuInverse.cs:174-182), which is exact.
template <int G = 32>
__device__ __forceinline__ void warp_solve_dot(const double* a, int n, long long si, long long st,
                                               bool unit, double* xs, int ldx, double* acc,
                                               int nr) {
  const int lane = group_lane<G>();
  const unsigned gm = group_mask<G>();
  for (int e = lane; e < nr * n; e += G) {
    const int r = e / n;
    acc[r * ldx + (e - r * n)] = 0.0;
  }
  __syncwarp(gm);
  for (int t = 0; t < n; ++t) {
    // x[t] is final: its last pair was added at step t-1.
    for (int r = lane; r < nr; r += G) {
      double v = xs[r * ldx + t];
      if (t > 0) v = __dsub_rn(v, acc[r * ldx + t]);
      if (!unit) v = __ddiv_rn(v, a[t * si + t * st]);
      xs[r * ldx + t] = v;
    }
    __syncwarp(gm);
    // Rows i = t+1, t+3, ... close a pair at t (or, at t = 0, take their lone first product).
    const int cnt = (n - t) >> 1;
    for (int e = lane; e < nr * cnt; e += G) {
      const int q = e / nr;
      const int r = e - q * nr;
      const int i = t + 1 + 2 * q;
      double* ap = acc + r * ldx + i;
      const double* ai = a + i * si;
      if (t == 0) {
        *ap = __dmul_rn(ai[0], xs[r * ldx]);
      } else {
        const double q2 = __dadd_rn(__dmul_rn(ai[(t - 1) * st], xs[r * ldx + t - 1]),
                                    __dmul_rn(ai[t * st], xs[r * ldx + t]));
        *ap = __dadd_rn(*ap, q2);
      }
    }
    __syncwarp(gm);
  }
}

// Column sweep.  Element (r, i), r < i, is at a[i*si + r*sr]; the diagonal at a[i*si + i*sr], or
// at diag[i] when diag is given (the R factor of QR keeps its diagonal apart, in rdiag).
template <int G = 32>
__device__ __forceinline__ void warp_solve_sweep(const double* a, int n, long long si,
                                                 long long sr, double* xs, int ldx, int nr,
                                                 const double* diag = nullptr) {
  const int lane = group_lane<G>();
  const unsigned gm = group_mask<G>();
  for (int i = n - 1; i >= 0; --i) {
    const double* ai = a + i * si;
    const double d = diag ? diag[i] : ai[i * sr];
    for (int r = lane; r < nr; r += G) xs[r * ldx + i] = __ddiv_rn(xs[r * ldx + i], d);
    __syncwarp(gm);
    for (int e = lane; e < nr * i; e += G) {
      const int q = e / nr;
      const int r = e - q * nr;
      double* xp = xs + r * ldx + q;
      *xp = __dsub_rn(*xp, __dmul_rn(ai[q * sr], xs[r * ldx + i]));
    }
    __syncwarp(gm);
  }
}

}  // namespace mfg
