// Device-side building blocks shared by the factorization kernels.
//
// Numerical contract: MatFlat evaluates every product and every sum separately rounded and never
// fuses a multiply-add (RyuJIT does not contract), so every floating-point operation here is an
// explicit round-to-nearest intrinsic (__dmul_rn, __dadd_rn, __dsub_rn, __ddiv_rn, __dsqrt_rn).
// Those intrinsics are never contracted by nvcc, whatever -fmad says.
//
// Hardware note (measured on GB300): FP64 DFMA/DMUL/DADD issue at ~1.66 lane-ops per clock per
// SM, i.e. one warp-wide FP64 instruction every ~77 cycles per SM sub-partition, and inactive
// lanes are not skipped.  Integer, shuffle, shared-memory and load instructions are nearly free
// beside that, so the kernels are organised to keep the FP64 lanes busy, and compare and test
// floating-point values with integer instructions wherever that is exact.
#pragma once

#include <cstdint>
#include <climits>

namespace mfg {

constexpr unsigned FULL_MASK = 0xffffffffu;

// Same tree, float data widened to double (Internals.cs:236-263).  Products of two widened
// floats are exact in double.
// (double)x * (double)y on the integer pipes.  The product of two floats' 24-bit significands
// has at most 48 bits, so the widened product is exact in double: for normal x and y it is the
// integer product Mx * My (one 32x32->64 multiply) placed under the exponent
// ex + ey + t + 769 (t = 1 when the product reaches 2^47), with no rounding at all.  Zeros,
// subnormals, infinities and NaN take the FP64 multiply, which gives the same value for them.
__device__ __forceinline__ double fmul_wide(float x, float y) {
  const unsigned X = __float_as_uint(x), Y = __float_as_uint(y);
  const unsigned ex = (X >> 23) & 0xFFu, ey = (Y >> 23) & 0xFFu;
  if (ex - 1u >= 254u || ey - 1u >= 254u) return __dmul_rn((double)x, (double)y);
  const unsigned long long P =
      (unsigned long long)((X & 0x7FFFFFu) | 0x800000u) * ((Y & 0x7FFFFFu) | 0x800000u);
  const unsigned t = (unsigned)(P >> 47);
  const unsigned long long mant = (P << (6u - t)) & 0x000FFFFFFFFFFFFFull;
  const unsigned long long e = (unsigned long long)(ex + ey + t + 769u);
  return __longlong_as_double((long long)(((unsigned long long)((X ^ Y) & 0x80000000u) << 32) |
                                          (e << 52) | mant));
}

__device__ __forceinline__ double exact_dot_f(int len, const float* x, long long incx,
                                              const float* y, long long incy) {
  double s = 0.0;
  if (len & 1) {
    s = fmul_wide(x[0], y[0]);
    x += incx;
    y += incy;
  }
  const int pairs = len >> 1;
#pragma unroll 4
  for (int p = 0; p < pairs; ++p) {
    const double q = __dadd_rn(fmul_wide(x[0], y[0]), fmul_wide(x[incx], y[incy]));
    s = __dadd_rn(s, q);
    x += 2 * incx;
    y += 2 * incy;
  }
  return s;
}

__device__ __forceinline__ unsigned long long dbits(double v) {
  return (unsigned long long)__double_as_longlong(v);
}

// v != 0.0 (true for NaN), by integer test.
__device__ __forceinline__ bool nonzero(double v) { return (dbits(v) << 1) != 0ull; }

// v > 0.0 (false for NaN and for both zeros), by integer test.
__device__ __forceinline__ bool positive(double v) {
  const long long b = __double_as_longlong(v);
  return b > 0 && b <= 0x7FF0000000000000LL;
}

__device__ __forceinline__ bool is_nan(double v) {
  return (dbits(v) & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull;
}

// Pivot key.  MatFlat's scan (Factorization.Lu.cs:323-330) keeps p = j and moves to i only when
// |w_i| > |w_p|.  If w_j is NaN nothing ever beats it; otherwise the winner is the first index
// attaining the largest |w| among the non-NaN entries.  The key orders |w| by its bit pattern
// (monotone for non-NaN doubles) and maps NaN below every number; the caller handles a NaN w_j.
__device__ __forceinline__ unsigned long long pivot_key(double v) {
  const unsigned long long b = dbits(v) & 0x7FFFFFFFFFFFFFFFull;
  return b > 0x7FF0000000000000ull ? 0ull : b + 1ull;
}

// Warp-wide argmax over (key, index): the largest key wins, ties go to the smaller index.
__device__ __forceinline__ int warp_argmax(unsigned long long key, int idx) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const unsigned long long ok = __shfl_xor_sync(FULL_MASK, key, off);
    const int oi = __shfl_xor_sync(FULL_MASK, idx, off);
    if (ok > key || (ok == key && oi < idx)) {
      key = ok;
      idx = oi;
    }
  }
  return idx;
}

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

// The same argmax over the G consecutive lanes of a group (G = 8, 16 or 32); only the group's
// lanes take part, so other groups of the warp may be elsewhere.
template <int G>
__device__ __forceinline__ int group_argmax(unsigned long long key, int idx) {
  const unsigned gm = group_mask<G>();
#pragma unroll
  for (int off = G / 2; off > 0; off >>= 1) {
    const unsigned long long ok = __shfl_xor_sync(gm, key, off);
    const int oi = __shfl_xor_sync(gm, idx, off);
    if (ok > key || (ok == key && oi < idx)) {
      key = ok;
      idx = oi;
    }
  }
  return idx;
}

// Internals.Dot (MatFlat/Internals.cs:265-292): for an odd length the first product seeds the
// sum, then every following pair is added as sum = sum + (x_a*y_a + x_b*y_b); an even length
// starts from sum = 0.0.  x and y are strided.  Reproduced operation for operation.
//
// The operands usually come from L2, so the loop is software-pipelined: the loads of the next
// block of DOT_BLOCK pairs are issued before the arithmetic of the current block, which keeps
// 2*DOT_BLOCK loads per operand in flight while the (slow) FP64 pipe works.
constexpr int DOT_BLOCK = 4;

// The product used by the dot trees: the hardware DMUL (IM = false) or the integer-pipe product
// imul_rn (IM = true); both return the correctly rounded product, bit for bit.  exact_dot's IM is
// 0 (DMUL), 1 (integer path) or 2 (the first product of each pair on the integer path, the
// second on DMUL, splitting the work between the two pipes).
template <bool IM>
__device__ __forceinline__ double xmul(double a, double b);

// The pair loop of Internals.Dot continued from a running sum s: s = s + (x_0 y_0 + x_1 y_1),
// s = s + (x_2 y_2 + x_3 y_3), ... for `pairs` pairs.  A dot split at a pair boundary and
// evaluated in two calls (the second starting from the first's sum) gives the same bits as one
// call over the whole length.
template <int IM = 1, int DOT_BLOCK = mfg::DOT_BLOCK>
__device__ __forceinline__ double exact_dot_pairs(double s, int pairs, const double* x,
                                                  long long incx, const double* y,
                                                  long long incy) {
  const int blocks = pairs / DOT_BLOCK;
  if (blocks > 0) {
    double xa[2 * DOT_BLOCK], ya[2 * DOT_BLOCK];
#pragma unroll
    for (int u = 0; u < 2 * DOT_BLOCK; ++u) {
      xa[u] = x[u * incx];
      ya[u] = y[u * incy];
    }
    x += 2 * DOT_BLOCK * incx;
    y += 2 * DOT_BLOCK * incy;
    for (int blk = 0; blk < blocks; ++blk) {
      double xb[2 * DOT_BLOCK], yb[2 * DOT_BLOCK];
      const bool more = blk + 1 < blocks;
      if (more) {
#pragma unroll
        for (int u = 0; u < 2 * DOT_BLOCK; ++u) {
          xb[u] = x[u * incx];
          yb[u] = y[u * incy];
        }
        x += 2 * DOT_BLOCK * incx;
        y += 2 * DOT_BLOCK * incy;
      }
#pragma unroll
      for (int u = 0; u < DOT_BLOCK; ++u) {
        const double q = __dadd_rn(xmul<IM != 0>(xa[2 * u], ya[2 * u]),
                                   xmul<IM == 1>(xa[2 * u + 1], ya[2 * u + 1]));
        s = __dadd_rn(s, q);
      }
      if (more) {
#pragma unroll
        for (int u = 0; u < 2 * DOT_BLOCK; ++u) {
          xa[u] = xb[u];
          ya[u] = yb[u];
        }
      }
    }
  }
  for (int p = blocks * DOT_BLOCK; p < pairs; ++p) {
    const double q = __dadd_rn(xmul<IM != 0>(x[0], y[0]), xmul<IM == 1>(x[incx], y[incy]));
    s = __dadd_rn(s, q);
    x += 2 * incx;
    y += 2 * incy;
  }
  return s;
}

template <int IM = 1, int DOT_BLOCK = mfg::DOT_BLOCK>
__device__ __forceinline__ double exact_dot(int len, const double* x, long long incx,
                                            const double* y, long long incy) {
  double s = 0.0;
  if (len & 1) {
    s = xmul<IM != 0>(x[0], y[0]);
    x += incx;
    y += incy;
  }
  return exact_dot_pairs<IM, DOT_BLOCK>(s, len >> 1, x, incx, y, incy);
}

// Dot product with fused multiply-adds in four independent chains (the FMA form: any order is
// allowed, so the chains give the loop instruction-level parallelism); the next block's operands
// are loaded before the current block's multiply-adds.
__device__ __forceinline__ double fma_dot(int len, const double* x, long long incx, const double* y,
                                          long long incy) {
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  const int blocks = len >> 2;
  if (blocks > 0) {
    double xa[4], ya[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      xa[u] = x[u * incx];
      ya[u] = y[u * incy];
    }
    for (int blk = 0; blk < blocks; ++blk) {
      double xb[4], yb[4];
      const bool more = blk + 1 < blocks;
      if (more) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          xb[u] = x[(4 + u) * incx];
          yb[u] = y[(4 + u) * incy];
        }
      }
      s0 = __fma_rn(xa[0], ya[0], s0);
      s1 = __fma_rn(xa[1], ya[1], s1);
      s2 = __fma_rn(xa[2], ya[2], s2);
      s3 = __fma_rn(xa[3], ya[3], s3);
      x += 4 * incx;
      y += 4 * incy;
      if (more) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          xa[u] = xb[u];
          ya[u] = yb[u];
        }
      }
    }
  }
  for (int t = blocks * 4; t < len; ++t) {
    s0 = __fma_rn(x[0], y[0], s0);
    x += incx;
    y += incy;
  }
  return __dadd_rn(__dadd_rn(s0, s1), __dadd_rn(s2, s3));
}

// The same with two chains and blocks of two (fewer registers: for kernels that want warps more
// than instruction-level parallelism).
__device__ __forceinline__ double fma_dot2(int len, const double* x, long long incx,
                                           const double* y, long long incy) {
  double s0 = 0.0, s1 = 0.0;
  const int blocks = len >> 1;
  if (blocks > 0) {
    double x0 = x[0], x1 = x[incx], y0 = y[0], y1 = y[incy];
    for (int blk = 0; blk < blocks; ++blk) {
      const bool more = blk + 1 < blocks;
      double nx0 = 0.0, nx1 = 0.0, ny0 = 0.0, ny1 = 0.0;
      if (more) {
        nx0 = x[2 * incx];
        nx1 = x[3 * incx];
        ny0 = y[2 * incy];
        ny1 = y[3 * incy];
      }
      s0 = __fma_rn(x0, y0, s0);
      s1 = __fma_rn(x1, y1, s1);
      x += 2 * incx;
      y += 2 * incy;
      x0 = nx0;
      x1 = nx1;
      y0 = ny0;
      y1 = ny1;
    }
  }
  if (len & 1) s0 = __fma_rn(x[0], y[0], s0);
  return __dadd_rn(s0, s1);
}

// Copies src[k*stride] to dst[k] (shared memory) for k in [k0, k1) with asynchronous 8-byte
// copies, one element per lane per round (cp.async, completed by stage_wait): a warp stages the
// next row or column of a factor while it computes with the current one.
__device__ __forceinline__ void stage_async(double* dst, const double* src, int k0, int k1,
                                            long long stride = 1) {
  for (int k = k0 + (int)(threadIdx.x & 31); k < k1; k += 32) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst + k);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src + k * stride)
                 : "memory");
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
// Completes this lane's staged copies and makes every lane's copies visible to the warp.
__device__ __forceinline__ void stage_wait() {
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  __syncwarp();
}

}  // namespace mfg

#include "mf_imul.cuh"
