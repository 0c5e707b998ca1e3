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
// function returns exactly __dmul_rn(a, b) for every input.
// ZEROS = true also keeps a zero times a normal number on the integer path (the result is the
// signed zero sign(a) ^ sign(b)), for kernels whose operands are often exact zeros: a warp whose
// lanes split between the two paths would otherwise issue the FP64 multiply as well.
#pragma once

#include "mf_device.cuh"

namespace mfg {

// The integer path for normal operands.  With 32-bit limbs M = m1 * 2^21 + m0 (m1: the top 32
// bits of the 53-bit significand, implicit bit included; m0: the low 21 bits),
//   P = Ma * Mb = H * 2^42 + C * 2^21 + L,  H = a1 b1,  C = a1 b0 + a0 b1,  L = a0 b0,
// and folding L and then C downwards gives P = T * 2^42 + s, T = H + ((C + (L >> 21)) >> 21)
// in [2^62, 2^64), s < 2^42 (only s != 0 matters: it is part of the sticky bit).  Normalising T
// to [2^63, 2^64) leaves the 53-bit significand above bit 11, the round bit at bit 10 and the
// rest of the sticky bits below it, so the rounding needs no tie special case.
__device__ __forceinline__ unsigned long long imul_bits(unsigned long long A, unsigned long long B,
                                                        int e) {
  const unsigned ah = (unsigned)(A >> 32), al = (unsigned)A;
  const unsigned bh = (unsigned)(B >> 32), bl = (unsigned)B;
  const unsigned a1 = __funnelshift_l(al, ah, 11) | 0x80000000u;
  const unsigned b1 = __funnelshift_l(bl, bh, 11) | 0x80000000u;
  const unsigned a0 = al & 0x1FFFFFu;
  const unsigned b0 = bl & 0x1FFFFFu;
  const unsigned long long hh = (unsigned long long)a1 * b1;
  const unsigned long long c = (unsigned long long)a1 * b0 + (unsigned long long)a0 * b1;
  const unsigned long long ll = (unsigned long long)a0 * b0;
  const unsigned long long x = c + (ll >> 21);
  const unsigned long long t = hh + (x >> 21);
  const unsigned low = ((unsigned)ll | (unsigned)x) & 0x1FFFFFu;
  const unsigned top = (unsigned)(t >> 63);
  const unsigned long long nrm = t << (top ^ 1u);
  unsigned long long mant = nrm >> 11;
  const unsigned nlo = (unsigned)nrm;
  const bool round = (nlo >> 10) & 1u;
  const bool sticky = ((nlo & 0x3FFu) | low) != 0u;
  mant += (round && (sticky || (mant & 1ull))) ? 1ull : 0ull;
  return ((A ^ B) & 0x8000000000000000ull) |
         ((((unsigned long long)(e + (int)top - 1)) << 52) + mant);
}

template <bool ZEROS = false>
__device__ __forceinline__ double imul_rn(double a, double b) {
  const unsigned long long A = dbits(a), B = dbits(b);
  const int ea = (int)((A >> 52) & 0x7FF);
  const int eb = (int)((B >> 52) & 0x7FF);
  const int e = ea + eb - 1023;
  const bool na = (unsigned)(ea - 1) < 2046u, nb = (unsigned)(eb - 1) < 2046u;
  bool zero = false;
  if (ZEROS) zero = ((A << 1) == 0ull && nb) || ((B << 1) == 0ull && na);
  // Integer path: ea, eb in [1, 2046] and e in [1, 2044] (so e + 1 + rounding carry <= 2046).
  if (!zero && (!na || !nb || (unsigned)(e - 1) >= 2044u)) return __dmul_rn(a, b);
  const unsigned long long r = imul_bits(A, B, e);
  return __longlong_as_double((long long)(zero ? (A ^ B) & 0x8000000000000000ull : r));
}

// Branch-free form: returns the integer-path product and sets ok when it is the correctly
// rounded result (both operands and the result normal, or, with ZEROS, a zero times a normal
// number), so a block of products forms one basic block.
template <bool ZEROS>
__device__ __forceinline__ double imul_nb(double a, double b, bool& ok) {
  const unsigned long long A = dbits(a), B = dbits(b);
  const int ea = (int)((A >> 52) & 0x7FF);
  const int eb = (int)((B >> 52) & 0x7FF);
  const int e = ea + eb - 1023;
  const bool na = (unsigned)(ea - 1) < 2046u, nb = (unsigned)(eb - 1) < 2046u;
  const bool zero = ZEROS && (((A << 1) == 0ull && nb) || ((B << 1) == 0ull && na));
  ok = zero || (na && nb && (unsigned)(e - 1) < 2044u);
  const unsigned long long r = imul_bits(A, B, e);
  return __longlong_as_double((long long)(zero ? (A ^ B) & 0x8000000000000000ull : r));
}

// p[r] = a[r] * b[r], correctly rounded, for R products: the integer-path ones first, then one
// (rarely taken) branch that redoes the out-of-range ones with the hardware multiply.  IM = 0
// uses the hardware multiply throughout, 1 the integer path, 2 the integer path for even r and
// the hardware multiply for odd r.
template <int IM, int R, bool ZEROS>
__device__ __forceinline__ void mul_block(const double* a, const double* b, double* p) {
  if constexpr (IM == 0) {
#pragma unroll
    for (int r = 0; r < R; r++) p[r] = __dmul_rn(a[r], b[r]);
  } else {
    unsigned bad = 0u;
#pragma unroll
    for (int r = 0; r < R; r++) {
      if (IM == 2 && (r & 1)) {
        p[r] = __dmul_rn(a[r], b[r]);
        continue;
      }
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
template <int IM, int R, bool ZEROS>
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
