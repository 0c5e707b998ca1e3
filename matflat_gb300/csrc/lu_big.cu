// The FMA form of the batched double LU + solve for orders above 128 (mfg_plan_set_form(
// MFG_FORM_FMA) on a getrf plan): one matrix per CTA, blocked right-looking, so that the bulk of
// the flops runs from shared-memory tiles instead of re-reading the matrix from L2/DRAM at every
// Crout step (the warp and CTA schedules of mf_lu.cuh / lu.cu are memory-bound at these orders).
// No counterpart in the reference, whose LU has one arithmetic; the pivots are MatFlat's
// (Factorization.LuCore, MatFlat/Factorization.Lu.cs:296-350).
//
// Per panel of BIG_NB columns [j0, j1):
//   1. the panel's columns one by one: pivot search with the FMA form's screen (the pivot's key
//      must beat the runner-up's by LU_FMA_MARGIN_ULPS, every candidate finite, the pivot not
//      zero), whole-row swap (MatFlat swaps whole rows, Lu.cs:332-337), scaling by the pivot's
//      reciprocal, rank-1 update of the panel's later columns;
//   2. per block of 64 trailing columns: U12 = L11^-1 A12 solved in shared memory (unit lower
//      32 x 32 L11 from shared memory), written back and kept on chip for
//   3. A22 -= L21 U12 in 64 x 64 tiles down the trailing rows, L21 staged in shared memory too,
//      4 x 4 fused multiply-adds per thread and k.
// A matrix whose screen fails at any column is restored from the copy the CTA took before
// factoring it and redone in MatFlat's arithmetic (lu_cta_early: the exact CTA schedule, MatFlat's
// bits).  The solves are getrs_fma's column sweeps for every matrix, so solve-only calls reproduce
// the fused call's bits.  The factors are backward stable, not MatFlat's bits.
#include <cuda_runtime.h>

#include "mf_lu.cuh"

namespace mfg {

constexpr int BIG_W = 8;               // warps per CTA
static_assert(2 * RHS_CHUNK >= BIG_W, "solve staging: BIG_W warps of n | 1 doubles per slice");
constexpr int BIG_T = BIG_W * 32;
constexpr int BIG_NB = 32;             // panel width
constexpr int BIG_TM = 64;             // trailing-update tile: BIG_TM x BIG_TM, 4 x 4 per thread

struct BigSmem {
  // L21 and U12 tiles, k-major, each row permuted so that the 4 rows (columns) a thread works on
  // are adjacent: tile row (column) rr = t + 16 u sits at 4 t + u (big_pos), read as two 16-byte
  // loads.
  double as[BIG_NB][BIG_TM];
  double bs[BIG_NB][BIG_TM + 2];
  double l11[BIG_NB][BIG_NB + 1];      // L11 of the panel, row-major
  double uj[BIG_NB];                   // row j of the panel after the swap
  unsigned long long pk[BIG_W];        // per warp: largest key, runner-up, its row, non-finite
  unsigned long long q[BIG_W];
  int pi[BIG_W];
  int bad[BIG_W];
  CtaRed red;
  int next;
};

// The thread's candidate (key, row) pairs of one column: largest key, runner-up, non-finite seen.
struct Cand {
  unsigned long long bk, sk;
  int bi;
  bool bad;
  __device__ __forceinline__ void reset() {
    bk = sk = 0ull;
    bi = INT_MAX;
    bad = false;
  }
  __device__ __forceinline__ void add(double v, int i) {
    const unsigned long long key = pivot_key(v);
    bad |= !finite_bits(v);
    if (key > bk) {
      sk = bk;
      bk = key;
      bi = i;
    } else if (key > sk) {
      sk = key;
    }
  }
};

// The CTA's pivot from every thread's candidates, with the screen: returns the pivot row, or -1
// when the column fails (the same answer on every thread).  Ties between rows fail the screen, so
// the tie rule of MatFlat's scan (the first row) never has to be reproduced.
__device__ __forceinline__ int big_pivot(const Cand& c, BigSmem& sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wp = warp_argmax(c.bk, c.bi);
  unsigned long long wk = c.bk;
  unsigned long long wq = c.bi == wp ? c.sk : c.bk;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const unsigned long long ok = __shfl_xor_sync(FULL_MASK, wk, off);
    const unsigned long long oq = __shfl_xor_sync(FULL_MASK, wq, off);
    wk = ok > wk ? ok : wk;
    wq = oq > wq ? oq : wq;
  }
  const bool wbad = __any_sync(FULL_MASK, c.bad);
  if (lane == 0) {
    sm.pk[warp] = wk;
    sm.q[warp] = wq;
    sm.pi[warp] = wp;
    sm.bad[warp] = wbad ? 1 : 0;
  }
  __syncthreads();
  unsigned long long pk = sm.pk[0];
  int p = sm.pi[0];
  int w0 = 0;
  int bad = sm.bad[0];
#pragma unroll
  for (int w = 1; w < BIG_W; ++w) {
    const unsigned long long k2 = sm.pk[w];
    const int i2 = sm.pi[w];
    bad |= sm.bad[w];
    if (k2 > pk || (k2 == pk && i2 < p)) {
      pk = k2;
      p = i2;
      w0 = w;
    }
  }
  unsigned long long q = 0ull;
#pragma unroll
  for (int w = 0; w < BIG_W; ++w) {
    const unsigned long long k2 = w == w0 ? sm.q[w] : sm.pk[w];
    q = k2 > q ? k2 : q;
  }
  if (bad || pk <= 1ull || pk - q < LU_FMA_MARGIN_ULPS) return -1;
  return p;
}

// Panel [j0, j1) of the n x n matrix a: returns false when a column fails the screen.
__device__ bool big_panel(double* a, int n, long long lda, int j0, int j1, int* piv, int& sign,
                          BigSmem& sm) {
  const int tid = threadIdx.x;
  Cand c;
  c.reset();
  {
    const double* cj = a + (long long)j0 * lda;
    for (int i = j0 + tid; i < n; i += BIG_T) c.add(cj[i], i);
  }
  for (int j = j0; j < j1; ++j) {
    const int p = big_pivot(c, sm);
    if (p < 0) return false;
    // Whole-row swap; the threads holding the panel's columns keep row j's new values.
    for (int col = tid; col < n; col += BIG_T) {
      double* base = a + (long long)col * lda;
      double v = base[j];
      if (p != j) {
        const double w = base[p];
        base[p] = v;
        base[j] = w;
        v = w;
      }
      if (col >= j && col < j1) sm.uj[col - j0] = v;
    }
    if (p != j) {
      if (tid == 0) {
        const int t = piv[j];
        piv[j] = piv[p];
        piv[p] = t;
      }
      sign = -sign;
    }
    __syncthreads();
    // Scaling, rank-1 update of the panel's later columns, candidates of column j + 1.
    const double r = __drcp_rn(sm.uj[j - j0]);
    double* cj = a + (long long)j * lda;
    c.reset();
    for (int i = j + 1 + tid; i < n; i += BIG_T) {
      const double l = __dmul_rn(cj[i], r);
      cj[i] = l;
      if (j + 1 < j1) {
        double* cc = cj + lda + i;
        const double v = __fma_rn(-l, sm.uj[j + 1 - j0], *cc);
        *cc = v;
        c.add(v, i);
      }
#pragma unroll 8
      for (int col = j + 2; col < j1; ++col) {
        double* cc = a + (long long)col * lda + i;
        *cc = __fma_rn(-l, sm.uj[col - j0], *cc);
      }
    }
    __syncthreads();
  }
  return true;
}

// Position of tile column (row) cc in a permuted shared row: 4 (cc mod 16) + cc / 16.
__device__ __forceinline__ int big_pos(int cc) { return 4 * (cc & 15) + (cc >> 4); }

// d = a b + d for one 8 x 8 x 4 double tile on the FP64 tensor pipe (mma.sync m8n8k4 f64): a is
// the lane's element A(lane / 4, lane % 4) of the 8 x 4 operand, b its element B(lane % 4,
// lane / 4) of the 4 x 8 operand, d its elements D(lane / 4, 2 (lane % 4) + {0, 1}).
__device__ __forceinline__ void dmma_8x8x4(double& d0, double& d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
               : "+d"(d0), "+d"(d1)
               : "d"(a), "d"(b));
}

// Fragment order of a k-major 32 x 64 tile for the tensor-pipe update: element (k, rr) (rr the
// tile row of L21, or the tile column of U12) sits where lane (rr mod 8) 4 + (k mod 4) of the
// warp reads it for k-step k / 4 and 8-wide block rr / 8, so a fragment is 32 consecutive doubles.
__device__ __forceinline__ int big_frag(int k, int rr) {
  return (((k >> 2) * 8 + (rr >> 3)) << 5) + ((rr & 7) << 2) + (k & 3);
}

// A22 -= L21 U12 on the FP64 tensor pipe for the BIG_TM columns from c0, down the trailing rows
// from j1 (mt tiles); bsf holds U12's block in fragment order.  Warp w computes tile rows
// 16 (w mod 4) + [0, 16) and columns 32 (w / 4) + [0, 32).
__device__ __forceinline__ void big_tiles_mma(double* a, int n, long long lda, int j0, int j1,
                                              int c0, int mt, double* asf, const double* bsf) {
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int wm = (warp & 3) * 2;      // the warp's first 8-row block of the tile
  const int wn = (warp >> 2) * 4;     // its first 8-column block
  const int fr = lane >> 2;           // the lane's row of an accumulator tile
  const int fc = (lane & 3) * 2;      // its first column
  for (int rb = 0; rb < mt; ++rb) {
    const int r0 = j1 + rb * BIG_TM;
    double acc[2][4][2];
#pragma unroll
    for (int mi = 0; mi < 2; ++mi) {
#pragma unroll
      for (int ni = 0; ni < 4; ++ni) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int i = r0 + (wm + mi) * 8 + fr, jj = c0 + (wn + ni) * 8 + fc + h;
          acc[mi][ni][h] = (i < n && jj < n) ? a[(long long)jj * lda + i] : 0.0;
        }
      }
    }
    for (int e = tid; e < BIG_NB * BIG_TM; e += BIG_T) {
      const int k = e / BIG_TM;
      const int rr = e - k * BIG_TM;
      const int i = r0 + rr;
      asf[big_frag(k, rr)] = i < n ? -a[(long long)(j0 + k) * lda + i] : 0.0;
    }
    __syncthreads();
#pragma unroll 2
    for (int ks = 0; ks < BIG_NB / 4; ++ks) {
      double af[2], bf[4];
#pragma unroll
      for (int mi = 0; mi < 2; ++mi) af[mi] = asf[((ks * 8 + wm + mi) << 5) + lane];
#pragma unroll
      for (int ni = 0; ni < 4; ++ni) bf[ni] = bsf[((ks * 8 + wn + ni) << 5) + lane];
#pragma unroll
      for (int mi = 0; mi < 2; ++mi) {
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
          dmma_8x8x4(acc[mi][ni][0], acc[mi][ni][1], af[mi], bf[ni]);
      }
    }
#pragma unroll
    for (int mi = 0; mi < 2; ++mi) {
#pragma unroll
      for (int ni = 0; ni < 4; ++ni) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int i = r0 + (wm + mi) * 8 + fr, jj = c0 + (wn + ni) * 8 + fc + h;
          if (i < n && jj < n) a[(long long)jj * lda + i] = acc[mi][ni][h];
        }
      }
    }
    __syncthreads();
  }
}

// A22 -= L21 U12 for the BIG_TM x BIG_TM tile at (r0, c0) with fused multiply-adds; U12's block
// is in sm.bs (big_pos order).  Each thread works on tile rows tx + 16 u, u < UR, and columns
// ty + 16 v, v < VR: UR (VR) = 2 covers the first 32 rows (columns), for an edge tile with no more
// valid ones, so that its padding costs no FP64 work.
template <int UR, int VR>
__device__ __forceinline__ void big_tile(double* a, int n, long long lda, int j0, int r0, int c0,
                                         BigSmem& sm) {
  static_assert((UR == 2 || UR == 4) && (VR == 2 || VR == 4), "2 or 4 rows / columns");
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  double acc[UR][VR];
#pragma unroll
  for (int u = 0; u < UR; ++u) {
#pragma unroll
    for (int v = 0; v < VR; ++v) {
      const int i = r0 + tx + 16 * u, jj = c0 + ty + 16 * v;
      acc[u][v] = (i < n && jj < n) ? a[(long long)jj * lda + i] : 0.0;
    }
  }
  constexpr int ROWS = 16 * UR;   // tile rows used
  for (int e = tid; e < BIG_NB * ROWS; e += BIG_T) {
    const int k = e / ROWS;
    const int rr = e - k * ROWS;
    const int i = r0 + rr;
    sm.as[k][big_pos(rr)] = i < n ? a[(long long)(j0 + k) * lda + i] : 0.0;
  }
  __syncthreads();
#pragma unroll 4
  for (int k = 0; k < BIG_NB; ++k) {
    double av[4], bv[4];
    const double2 a01 = *reinterpret_cast<const double2*>(&sm.as[k][4 * tx]);
    av[0] = a01.x, av[1] = a01.y;
    if constexpr (UR == 4) {
      const double2 a23 = *reinterpret_cast<const double2*>(&sm.as[k][4 * tx + 2]);
      av[2] = a23.x, av[3] = a23.y;
    }
    const double2 b01 = *reinterpret_cast<const double2*>(&sm.bs[k][4 * ty]);
    bv[0] = b01.x, bv[1] = b01.y;
    if constexpr (VR == 4) {
      const double2 b23 = *reinterpret_cast<const double2*>(&sm.bs[k][4 * ty + 2]);
      bv[2] = b23.x, bv[3] = b23.y;
    }
#pragma unroll
    for (int u = 0; u < UR; ++u) {
#pragma unroll
      for (int v = 0; v < VR; ++v) acc[u][v] = __fma_rn(-av[u], bv[v], acc[u][v]);
    }
  }
#pragma unroll
  for (int u = 0; u < UR; ++u) {
#pragma unroll
    for (int v = 0; v < VR; ++v) {
      const int i = r0 + tx + 16 * u, jj = c0 + ty + 16 * v;
      if (i < n && jj < n) a[(long long)jj * lda + i] = acc[u][v];
    }
  }
  __syncthreads();
}

// U12 = L11^-1 A12 and A22 -= L21 U12 for the rows and columns [j1, n), j1 = j0 + BIG_NB, one
// block of BIG_TM trailing columns at a time: the block's U12 rows are solved in shared memory
// (one column per thread of the first BIG_TM, from L11 in shared memory), written back, and kept
// in shared memory for the block's BIG_TM x BIG_TM update tiles down the trailing rows.
// MMA: the tiles on the FP64 tensor pipe (each warp 16 x 32 of the tile as 2 x 4 mma tiles of
// 8 x 8, operands in fragment order, big_frag); otherwise 4 x 4 fused multiply-adds per thread
// (operands in big_pos order, big_tile).
template <bool MMA>
__device__ void big_u12_update(double* a, int n, long long lda, int j0, BigSmem& sm) {
  const int tid = threadIdx.x;
  double* asf = &sm.as[0][0];
  double* bsf = &sm.bs[0][0];
  const int j1 = j0 + BIG_NB;
  const int mt = (n - j1 + BIG_TM - 1) / BIG_TM;
  for (int e = tid; e < BIG_NB * BIG_NB; e += BIG_T) {
    const int k = e / BIG_NB;
    const int r = e - k * BIG_NB;
    sm.l11[r][k] = a[(long long)(j0 + k) * lda + j0 + r];
  }
  for (int cb = 0; cb < mt; ++cb) {
    const int c0 = j1 + cb * BIG_TM;
    for (int e = tid; e < BIG_NB * BIG_TM; e += BIG_T) {
      const int cc = e / BIG_NB;
      const int k = e - cc * BIG_NB;
      const int jj = c0 + cc;
      const double v = jj < n ? a[(long long)jj * lda + j0 + k] : 0.0;
      if constexpr (MMA) bsf[big_frag(k, cc)] = v;
      else sm.bs[k][big_pos(cc)] = v;
    }
    __syncthreads();
    if (tid < BIG_TM) {
      // Thread tid solves the column stored at position tid (MMA: tile column tid).
      for (int r = 1; r < BIG_NB; ++r) {
        double* vr = MMA ? bsf + big_frag(r, tid) : &sm.bs[r][tid];
        double v = *vr;
#pragma unroll 8
        for (int k = 0; k < r; ++k)
          v = __fma_rn(-sm.l11[r][k], MMA ? bsf[big_frag(k, tid)] : sm.bs[k][tid], v);
        *vr = v;
      }
    }
    __syncthreads();
    for (int e = tid; e < BIG_NB * BIG_TM; e += BIG_T) {
      const int cc = e / BIG_NB;
      const int k = e - cc * BIG_NB;
      const int jj = c0 + cc;
      if (jj < n) a[(long long)jj * lda + j0 + k] = MMA ? bsf[big_frag(k, cc)] : sm.bs[k][big_pos(cc)];
    }
    if constexpr (MMA) {
      big_tiles_mma(a, n, lda, j0, j1, c0, mt, asf, bsf);
      continue;
    }
    // Edge tiles whose valid rows (columns) fit in 32 run 2 of each thread's 4 rows (columns).
    const int vr = n - c0 > 32 ? 4 : 2;
    for (int rb = 0; rb < mt; ++rb) {
      const int r0 = j1 + rb * BIG_TM;
      const int ur = n - r0 > 32 ? 4 : 2;
      if (ur == 4 && vr == 4) big_tile<4, 4>(a, n, lda, j0, r0, c0, sm);
      else if (ur == 4) big_tile<4, 2>(a, n, lda, j0, r0, c0, sm);
      else if (vr == 4) big_tile<2, 4>(a, n, lda, j0, r0, c0, sm);
      else big_tile<2, 2>(a, n, lda, j0, r0, c0, sm);
    }
  }
}

// The whole factorization in the FMA form; false when a column failed the screen (the matrix is
// then partly factored and must be restored).
template <bool MMA>
__device__ bool big_lu_fma(double* a, int n, long long lda, int* piv, int& sign, BigSmem& sm) {
  for (int i = threadIdx.x; i < n; i += BIG_T) piv[i] = i;
  sign = 1;
  __syncthreads();
  for (int j0 = 0; j0 < n; j0 += BIG_NB) {
    const int j1 = min(n, j0 + BIG_NB);
    if (!big_panel(a, n, lda, j0, j1, piv, sign, sm)) return false;
    if (j1 < n) big_u12_update<MMA>(a, n, lda, j0, sm);
  }
  return true;
}

// The redo of a matrix the screen rejected: restore it from the CTA's copy, factor it in MatFlat's
// arithmetic.  Out of line: rare, and inlined it would raise the main path's register count.
__device__ __noinline__ void big_fallback(double* a, int n, long long lda, const double* bk,
                                          int* piv, double* scol, int* sign, int* info,
                                          CtaRed* red) {
  __syncthreads();
  for (int j = 0; j < n; ++j)
    for (int i = threadIdx.x; i < n; i += BIG_T)
      a[(long long)j * lda + i] = __ldcs(bk + (long long)j * n + i);
  __syncthreads();
  int sg = 1, inf = 0;
  lu_cta_early<BIG_W, 1, 2>(a, n, lda, piv, scol, scol + n, sg, inf, red);
  *sign = sg;
  *info = inf;
}

// Work items: the plan's tasks (one matrix each, p.ntasks of them, taken from p.queue).  Per CTA:
// a copy of up to bstride doubles in p.fbackup and a slice of p.gscratch (warp_scratch_doubles(n)
// >= n + BIG_W (n | 1): the reciprocals and the warps' solve staging; the fallback's column
// sums).
// MINB: resident CTAs per SM the register allocation is bounded for (2: 128 registers, 3: 80).
template <int MINB, bool MMA>
__global__ void __launch_bounds__(BIG_T, MINB) getrf_big_fma_kernel(BatchArgs p,
                                                                   long long bstride) {
  __shared__ BigSmem sm;
  const int tid = threadIdx.x;
  double* slice = p.gscratch + (long long)blockIdx.x * p.gscratch_stride;
  double* bk = p.fbackup + (long long)blockIdx.x * bstride;
  for (;;) {
    if (tid == 0) sm.next = atomicAdd(p.queue, 1);
    __syncthreads();
    const int t = sm.next;
    __syncthreads();
    if (t >= p.ntasks) break;
    const int mat = p.order[p.task_first[t]];
    const int n = p.n[mat];
    const long long lda = p.lda[mat];
    double* a = p.a + p.a_off[mat];
    int* piv = p.piv + p.piv_off[mat];
    int sign = 1, info = 0;
    if (!p.solve_only) {
      for (int j = 0; j < n; ++j)
        for (int i = tid; i < n; i += BIG_T)
          __stcs(bk + (long long)j * n + i, a[(long long)j * lda + i]);
      __syncthreads();
      if (!big_lu_fma<MMA>(a, n, lda, piv, sign, sm)) {
        big_fallback(a, n, lda, bk, piv, slice, &sign, &info, &sm.red);
        if (tid == 0) atomicAdd(p.fcount, 1);
      }
      __syncthreads();
    }
    if (p.nrhs > 0) {
      // The reciprocals of U's diagonal once (slice[0, n)), then warp w solves right-hand sides
      // w, w + BIG_W, ... one at a time, staged in slice + n + w (n | 1).
      for (int i = tid; i < n; i += BIG_T) slice[i] = __drcp_rn(a[(long long)i * lda + i]);
      __syncthreads();
      const int warp = tid >> 5;
      double* xs = slice + n + (long long)warp * (n | 1);
      for (int r = warp; r < p.nrhs; r += BIG_W)
        getrs_fma<32, true>(a, n, lda, piv, p.b + p.b_off[mat] + (long long)r * n, n, 1, xs,
                            slice);
    }
    if (tid == 0 && !p.solve_only) {
      p.sign[mat] = sign;
      p.info[mat] = info;
    }
    __syncthreads();
  }
}

long long getrf_big_backup_doubles(int nmax) {
  return ((long long)nmax * nmax + 31) / 32 * 32;
}

cudaError_t launch_getrf_big_fma(const BatchArgs& args, int ctas, int nmax, int cps, bool mma,
                                 cudaStream_t s) {
  if (ctas < 1 || nmax < 1 || !args.fbackup || !args.fcount || !args.gscratch ||
      args.gscratch_stride < warp_scratch_doubles(nmax))
    return cudaErrorInvalidValue;
  const long long bs = getrf_big_backup_doubles(nmax);
  if (cps >= 3 && mma)
    getrf_big_fma_kernel<3, true><<<ctas, BIG_T, 0, s>>>(args, bs);
  else if (cps >= 3)
    getrf_big_fma_kernel<3, false><<<ctas, BIG_T, 0, s>>>(args, bs);
  else if (mma)
    getrf_big_fma_kernel<2, true><<<ctas, BIG_T, 0, s>>>(args, bs);
  else
    getrf_big_fma_kernel<2, false><<<ctas, BIG_T, 0, s>>>(args, bs);
  return cudaGetLastError();
}

}  // namespace mfg
