// Correctly rounded double-precision product on the integer pipes.
//
// Why: on GB300 the FP64 pipe issues one warp-wide DMUL/DADD every ~77 cycles per SM
// sub-partition (1/73 of the FP32 rate), while 32-bit integer multiply-add runs ~38x faster.
// MatFlat's exact operation order needs two separately rounded FP64 instructions per multiply-add
// (no FMA), so moving the multiplies to the integer pipes lets both pipes work at once.
//
// Method: IEEE 754 round-to-nearest-even multiplication from its definition.  For normal a, b
// with significands Ma, Mb in [2^52, 2^53), P = Ma*Mb is an exact 105/106-bit integer; the result
// significand is P's top 53 bits, rounded up when the next bit (round) is 1 and either any lower
// bit (sticky) is 1 or the kept significand is odd.  The exponent is ea + eb - 1023 (+1 when
// P >= 2^105); a carry out of the rounding is absorbed by adding the significand, implicit bit
// included, onto (exponent - 1) << 52.  Operands or results outside the normal range (zeros,
// subnormals, infinities, NaN, overflow, underflow) take the hardware __dmul_rn instead, so the
// function returns exactly __dmul_rn(a, b) for every input.  The low 64 bits of the 128-bit
// product are needed only to break a possible tie, so they are computed only then.
// ZEROS = true also keeps a zero times a normal number on the integer path (the result is the
// signed zero sign(a) ^ sign(b)), for kernels whose operands are often exact zeros: a warp whose
// lanes split between the two paths would otherwise issue the FP64 multiply as well.
#pragma once

#include "mf_device.cuh"

namespace mfg {

template <bool ZEROS = false>
__device__ __forceinline__ double imul_rn(double a, double b) {
  const unsigned long long A = dbits(a), B = dbits(b);
  const int ea = (int)((A >> 52) & 0x7FF);
  const int eb = (int)((B >> 52) & 0x7FF);
  const int e = ea + eb - 1023;
  const bool na = (unsigned)(ea - 1) < 2046u, nb = (unsigned)(eb - 1) < 2046u;
  bool zero = false;
  if (ZEROS) zero = ((A << 1) == 0ull && nb) || ((B << 1) == 0ull && na);
  // Fast path: ea, eb in [1, 2046] and e in [1, 2044] (so e + 1 + rounding carry <= 2046).
  if (!zero && (!na || !nb || (unsigned)(e - 1) >= 2044u)) return __dmul_rn(a, b);
  const unsigned long long ma = (A << 11) | 0x8000000000000000ull;  // Ma << 11
  const unsigned long long mb = (B << 11) | 0x8000000000000000ull;  // Mb << 11
  const unsigned long long hi = __umul64hi(ma, mb);                 // P >> 42
  const unsigned top = (unsigned)(hi >> 63);                         // P >= 2^105
  const unsigned sh = 10u + top;
  unsigned long long mant = hi >> sh;                                // 53 bits
  const unsigned long long below = hi & ((1ull << sh) - 1ull);       // round bit + high sticky
  const unsigned long long half = 1ull << (sh - 1u);
  bool up;
  if (below != half) {
    up = below > half;
  } else {
    // Round bit set and the sticky bits inside hi clear: the rest of P decides.
    const unsigned long long lo = ma * mb;                           // (P << 22) mod 2^64
    up = (lo != 0ull) || (mant & 1ull);
  }
  mant += up ? 1ull : 0ull;
  const unsigned long long sign = (A ^ B) & 0x8000000000000000ull;
  const unsigned long long r = sign | ((((unsigned long long)(e + (int)top - 1)) << 52) + mant);
  return __longlong_as_double((long long)(zero ? sign : r));
}

// Branch-free form of the fast path: returns the integer-path product and sets ok when it is the
// correctly rounded result (both operands normal and the result normal, or, with ZEROS, a zero
// times a normal number).  The tie test always computes the low product word, so a block of
// these products forms one basic block whose dependency chains the compiler interleaves.
template <bool ZEROS>
__device__ __forceinline__ double imul_nb(double a, double b, bool& ok) {
  const unsigned long long A = dbits(a), B = dbits(b);
  const int ea = (int)((A >> 52) & 0x7FF);
  const int eb = (int)((B >> 52) & 0x7FF);
  const int e = ea + eb - 1023;
  const bool na = (unsigned)(ea - 1) < 2046u, nb = (unsigned)(eb - 1) < 2046u;
  const bool zero = ZEROS && (((A << 1) == 0ull && nb) || ((B << 1) == 0ull && na));
  ok = zero || (na && nb && (unsigned)(e - 1) < 2044u);
  const unsigned long long ma = (A << 11) | 0x8000000000000000ull;
  const unsigned long long mb = (B << 11) | 0x8000000000000000ull;
  const unsigned long long hi = __umul64hi(ma, mb);
  const unsigned long long lo = ma * mb;
  const unsigned top = (unsigned)(hi >> 63);
  const unsigned sh = 10u + top;
  unsigned long long mant = hi >> sh;
  const unsigned long long below = hi & ((1ull << sh) - 1ull);
  const unsigned long long half = 1ull << (sh - 1u);
  const bool up = (below > half) || (below == half && (lo != 0ull || (mant & 1ull)));
  mant += up ? 1ull : 0ull;
  const unsigned long long sign = (A ^ B) & 0x8000000000000000ull;
  const unsigned long long r = sign | ((((unsigned long long)(e + (int)top - 1)) << 52) + mant);
  return __longlong_as_double((long long)(zero ? sign : r));
}

// p[r] = a[r] * b[r], correctly rounded, for R products: all on the integer path first, then one
// (rarely taken) branch that redoes the out-of-range ones with the hardware multiply.  IM = false
// uses the hardware multiply throughout.
template <bool IM, int R, bool ZEROS>
__device__ __forceinline__ void mul_block(const double* a, const double* b, double* p) {
  if constexpr (!IM) {
#pragma unroll
    for (int r = 0; r < R; r++) p[r] = __dmul_rn(a[r], b[r]);
  } else {
    unsigned bad = 0u;
#pragma unroll
    for (int r = 0; r < R; r++) {
      bool ok;
      p[r] = imul_nb<ZEROS>(a[r], b[r], ok);
      bad |= ok ? 0u : (1u << r);
    }
    if (bad) {
#pragma unroll
      for (int r = 0; r < R; r++)
        if ((bad >> r) & 1u) p[r] = __dmul_rn(a[r], b[r]);
    }
  }
}

// Same with one common factor: p[r] = a[r] * b.
template <bool IM, int R, bool ZEROS>
__device__ __forceinline__ void mul_block_s(const double* a, double b, double* p) {
  double bb[R];
#pragma unroll
  for (int r = 0; r < R; r++) bb[r] = b;
  mul_block<IM, R, ZEROS>(a, bb, p);
}

template <>
__device__ __forceinline__ double xmul<false>(double a, double b) {
  return __dmul_rn(a, b);
}
template <>
__device__ __forceinline__ double xmul<true>(double a, double b) {
  return imul_rn(a, b);
}

}  // namespace mfg
