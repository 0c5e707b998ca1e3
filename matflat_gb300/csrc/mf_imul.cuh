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

// The LU column scalings use the integer-pipe quotient below when MFG_IDIV is 1 (build flag; 0
// keeps the FP64 division).  Both give the same bits.  On the 100,000-matrix LU batch: 87.6 ms
// against 90.2 ms at the autotuner's shape (32 lanes per matrix, 28 warps per SM).  The Cholesky
// keeps the FP64 division: its integer-product kernel ran 55.6 ms against 52.7 ms with it.
#ifndef MFG_IDIV
#define MFG_IDIV 1
#endif

// Correctly rounded quotient a / b on the integer pipes, from the definition of IEEE division and
// an exact integer remainder (no FP64 instruction).  y must be the correctly rounded reciprocal of
// b (one __drcp_rn per divisor, shared by all the quotients of a column).
//
// For normal a, b with significands Ma, Mb in [2^52, 2^53): the result significand is
// q = RN(N / Mb), N = Ma * 2^s, s = 52 when Ma >= Mb (N / Mb in [2^52, 2^53)) and 53 otherwise,
// exponent ea - eb + 1023 - (s - 52).  With Y the significand of y (1/Mb = Y' * 2^-(104 + db),
// db = 0 when b is a power of two, else 1, and |Y - Y'| <= 1/2), Q0 = floor(Ma * Y / 2^(104 + db
// - s)) lies within 1 of N / Mb (relative error of Y at most 2^-53, N / Mb < 2^53), so after one
// correction step against the exact remainder R = N - Q0 * Mb (|R| < 2^55: computed modulo 2^64)
// Q0 = floor(N / Mb) and 0 <= R < Mb; the quotient rounds up when 2R > Mb (2R == Mb cannot occur
// for binary significands, and would round to even).  A carry to 2^53 is absorbed by adding the
// significand onto (exponent - 1) << 52.  Zeros, subnormals, infinities, NaN and out-of-range
// quotients take __ddiv_rn, so the function returns exactly __ddiv_rn(a, b) for every input; a zero
// dividend over a normal divisor gives the signed zero directly.
// The divisor's part of the quotient, formed once per divisor (column).
struct IDivisor {
  unsigned long long mb;   // significand of b, implicit bit included
  unsigned long long sgn;  // sign bit of b
  unsigned y1, y0;         // significand of y = 1/b in 32 + 21 bit limbs
  int eb;                  // biased exponent of b
  int sh;                  // 105 - db (db: 0 when b is a power of two): shift = sh - s
  bool ok;                 // b and y normal: the integer path applies
};

__device__ __forceinline__ IDivisor idiv_prepare(double b, double y) {
  const unsigned long long B = dbits(b), Yb = dbits(y);
  const unsigned long long M52 = (1ull << 52) - 1ull;
  IDivisor d;
  d.eb = (int)((B >> 52) & 0x7FF);
  const int ey = (int)((Yb >> 52) & 0x7FF);
  d.ok = (unsigned)(d.eb - 1) < 2046u && (unsigned)(ey - 1) < 2046u;
  d.mb = (B & M52) | (1ull << 52);
  d.sgn = B & 0x8000000000000000ull;
  const unsigned long long Y = (Yb & M52) | (1ull << 52);
  d.y1 = (unsigned)(Y >> 21);
  d.y0 = (unsigned)Y & 0x1FFFFFu;
  d.sh = (B & M52) != 0ull ? 105 : 104;
  return d;
}

// Branch-free form: the integer-path quotient, with ok = false where it does not apply (the caller
// then divides on the FP64 pipe).
__device__ __forceinline__ double idiv_nb(double a, const IDivisor& d, bool& ok) {
  const unsigned long long A = dbits(a);
  const unsigned long long M52 = (1ull << 52) - 1ull;
  const int ea = (int)((A >> 52) & 0x7FF);
  const unsigned long long Ma = (A & M52) | (1ull << 52);
  const unsigned long long Mb = d.mb;
  const bool ge = Ma >= Mb;
  const int eq = ea - d.eb + (ge ? 1023 : 1022);
  const bool zero = (A << 1) == 0ull;
  ok = d.ok && (zero || ((unsigned)(ea - 1) < 2046u && (unsigned)(eq - 1) < 2045u));
  const int s = ge ? 52 : 53;
  // floor(Ma * Y / 2^42) from 32/21-bit limbs (as in imul_bits), then the remaining shift.
  const unsigned a1 = (unsigned)(Ma >> 21), a0 = (unsigned)Ma & 0x1FFFFFu;
  const unsigned long long hh = (unsigned long long)a1 * d.y1;
  const unsigned long long c = (unsigned long long)a1 * d.y0 + (unsigned long long)a0 * d.y1;
  const unsigned long long ll = (unsigned long long)a0 * d.y0;
  const unsigned long long t = hh + ((c + (ll >> 21)) >> 21);
  unsigned long long q = t >> (d.sh - s - 42);
  long long r = (long long)((Ma << s) - q * Mb);
  if (r < 0) {
    q -= 1ull;
    r += (long long)Mb;
  } else if (r >= (long long)Mb) {
    q += 1ull;
    r -= (long long)Mb;
  }
  const unsigned long long r2 = (unsigned long long)r << 1;
  q += (r2 > Mb || (r2 == Mb && (q & 1ull))) ? 1ull : 0ull;
  const unsigned long long sg = (A & 0x8000000000000000ull) ^ d.sgn;
  return __longlong_as_double(
      (long long)(zero ? sg : (sg | ((((unsigned long long)(eq - 1)) << 52) + q))));
}

__device__ __forceinline__ double idiv_rn(double a, double b, const IDivisor& d) {
  bool ok;
  const double q = idiv_nb(a, d, ok);
  return ok ? q : __ddiv_rn(a, b);
}

__device__ __forceinline__ double idiv_rn(double a, double b, double y) {
  return idiv_rn(a, b, idiv_prepare(b, y));
}

// x[i] = x[i] / b for i = first, first + step, ... < end, the quotients on the integer pipes; the
// (rare) elements outside its range are divided on the FP64 pipe in a second pass, so the loop body
// stays one basic block.
__device__ __forceinline__ void idiv_column(double* x, int first, int end, int step, double b) {
  const IDivisor d = idiv_prepare(b, __drcp_rn(b));
  unsigned long long bad = 0ull;
  int it = 0;
  for (int i = first; i < end; i += step, ++it) {
    bool ok;
    const double q = idiv_nb(x[i], d, ok);
    if (ok) x[i] = q;
    else bad |= it < 64 ? 1ull << it : 0ull;
    if (!ok && it >= 64) x[i] = __ddiv_rn(x[i], b);
  }
  if (bad) {
    it = 0;
    for (int i = first; i < end && it < 64; i += step, ++it)
      if ((bad >> it) & 1ull) x[i] = __ddiv_rn(x[i], b);
  }
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
