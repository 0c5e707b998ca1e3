// The FMA form of the batched double LU + solve (mfg_plan_set_form(MFG_FORM_FMA) on a getrf plan;
// no counterpart in the reference, whose LU has one arithmetic).
//
// MatFlat's LuCore (MatFlat/Factorization.Lu.cs:296-350) in the same Crout schedule as the exact
// kernels (mf_lu.cuh), with fused multiply-add dots and reciprocal column scaling
// (DTraitsFma), and a screen at every column that keeps MatFlat's pivot choice: a matrix whose
// pivot could depend on rounding (runner-up within about 1.5e-8 of the pivot, ties, zero pivots,
// NaN or infinite candidates) is restored from a copy taken before the factorization and redone in
// MatFlat's arithmetic by the same lanes (lu_finish_column's FMA screen).  The solves are column
// sweeps with fused multiply-adds and the reciprocal of U's diagonal, for every matrix (fallbacks
// included), so solve-only calls give the fused call's bits.  The factors are backward stable
// (|PA - LU| <= gamma_n |L| |U|), not MatFlat's bits.
#include <cuda_runtime.h>

#include "mf_lu.cuh"

namespace mfg {

// The fallback of a matrix the screen rejected: restore it from its copy and factor it in
// MatFlat's arithmetic (products on the FP64 pipe: the same bits as the integer-pipe form).  Kept
// out of line: it is rare, and inlined it would raise the register count of the FMA path.
template <int G>
__device__ __noinline__ void getrf_fma_fallback(double* a, int n, long long lda, const double* bk,
                                                int* piv, double* scr, double* scr2, int* sign,
                                                int* info) {
  const int gl = group_lane<G>();
  const unsigned gm = group_mask<G>();
  __syncwarp(gm);
  for (int j = 0; j < n; ++j)
    for (int i = gl; i < n; i += G) a[(long long)j * lda + i] = __ldcs(bk + (long long)j * n + i);
  __syncwarp(gm);
  int sg = 1, inf = 0;
  lu_warp<DTraits, 0, 2, G, true>(a, n, n, lda, piv, scr, sg, inf, scr2);
  *sign = sg;
  *info = inf;
}

// One task of the size-bucketed queue in the FMA form: the groups of G lanes each take one
// matrix of the task.  Scratch as in getrf_task (lu.cu); the copy for the fallback goes to the
// group's slice of args.fbackup (streaming stores: it is read again only by a fallback).
// FDB: 2 four-chain dots (fma_dot), 1 two-chain dots (fma_dot2, fewer registers).
template <int G, int FDB>
__device__ __forceinline__ void getrf_task_fma(const BatchArgs& p, int first, int cnt, double* ws,
                                               long long gw) {
  const int lane = threadIdx.x & 31;
  const int g = lane / G;
  if (g >= cnt) return;
  const int gl = lane & (G - 1);
  const unsigned gm = group_mask<G>();
  const int mat = p.order[first + g];
  const int n = p.n[mat];
  const long long lda = p.lda[mat];
  double* a = p.a + p.a_off[mat];
  int* piv = p.piv + p.piv_off[mat];
  double* scr;
  double* scr2;
  double* sol;
  if (n <= SMEM_N) {
    scr = ws + g * GROUP_SMEM_DOUBLES;
    scr2 = scr + SMEM_N + 1;
    sol = p.gsolve ? p.gsolve + (gw * GETRF_GROUPS + g) * GSOLVE_STRIDE : nullptr;
  } else {   // only 32-lane tasks hold orders above SMEM_N
    scr = p.gscratch + gw * p.gscratch_stride;
    scr2 = scr + n;
    sol = scr + 2 * n;
  }
  int sign = 1, info = 0;
  if (!p.solve_only) {
    double* bk = p.fbackup + gw * p.fbackup_stride + (long long)g * (p.fbackup_stride / (32 / G));
    for (int j = 0; j < n; ++j)
      for (int i = gl; i < n; i += G) __stcs(bk + (long long)j * n + i, a[(long long)j * lda + i]);
    __syncwarp(gm);
    bool fail = false;
    lu_warp<DTraitsFma, 1, FDB, G, true, true>(a, n, n, lda, piv, scr, sign, info, scr2, &fail);
    if (fail) {
      getrf_fma_fallback<G>(a, n, lda, bk, piv, scr, scr2, &sign, &info);
      if (gl == 0) atomicAdd(p.fcount, 1);
    }
  }
  if (p.nrhs > 0) getrs_fma<G>(a, n, lda, piv, p.b + p.b_off[mat], n, p.nrhs, sol, scr);
  if (gl == 0 && !p.solve_only) {
    p.sign[mat] = sign;
    p.info[mat] = info;
  }
}

template <int G, int FDB>
__device__ __forceinline__ void getrf_task_fma_loop(const BatchArgs& p, int warps) {
  extern __shared__ double sm_dyn[];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const long long gw = (long long)blockIdx.x * warps + warp;
  double* ws = sm_dyn + warp * (32 / G) * GROUP_SMEM_DOUBLES;
  for (;;) {
    int t = 0;
    if (lane == 0) t = atomicAdd(p.queue, 1);
    t = __shfl_sync(FULL_MASK, t, 0);
    if (t >= p.ntasks) break;
    getrf_task_fma<G, FDB>(p, p.task_first[t], p.task_gc[t] >> 8, ws, gw);
    __syncwarp();
  }
}

// Any number of warps per CTA (blockDim.x / 32), or 4 warps with the register allocation bounded
// for MINB resident CTAs per SM (5: 96 registers, 20 warps, no spills with two-chain dots).
template <int G, int FDB>
__global__ void __launch_bounds__(512, 1) getrf_task_fma_kernel(BatchArgs p) {
  getrf_task_fma_loop<G, FDB>(p, blockDim.x >> 5);
}
template <int G, int FDB, int MINB>
__global__ void __launch_bounds__(128, MINB) getrf_task_fma_kernel_occ(BatchArgs p) {
  getrf_task_fma_loop<G, FDB>(p, 4);
}

static size_t fma_smem_bytes(int warps, int g) {
  return sizeof(double) * (32 / g) * GROUP_SMEM_DOUBLES * warps;
}

template <int G, int FDB>
static void launch_fma_gd(const BatchArgs& args, int ctas, int warps, size_t smem,
                          cudaStream_t s) {
  if (warps == 4 && args.minb >= 7)
    getrf_task_fma_kernel_occ<G, FDB, 7><<<ctas, 128, smem, s>>>(args);
  else if (warps == 4 && args.minb == 6)
    getrf_task_fma_kernel_occ<G, FDB, 6><<<ctas, 128, smem, s>>>(args);
  else if (warps == 4 && args.minb == 5)
    getrf_task_fma_kernel_occ<G, FDB, 5><<<ctas, 128, smem, s>>>(args);
  else
    getrf_task_fma_kernel<G, FDB><<<ctas, warps * 32, smem, s>>>(args);
}

template <int G>
static cudaError_t launch_fma_g(const BatchArgs& args, int ctas, int warps, cudaStream_t s) {
  const size_t smem = fma_smem_bytes(warps, G);
  if (args.dot_block == 1)
    launch_fma_gd<G, 1>(args, ctas, warps, smem, s);
  else
    launch_fma_gd<G, 2>(args, ctas, warps, smem, s);
  return cudaGetLastError();
}

cudaError_t launch_getrf_tasks_fma(const BatchArgs& args, int ctas, int warps, int g,
                                   cudaStream_t s) {
  if (warps < 1 || warps > 16 || !args.fbackup || !args.fcount) return cudaErrorInvalidValue;
  if (g == 8) return launch_fma_g<8>(args, ctas, warps, s);
  if (g == 16) return launch_fma_g<16>(args, ctas, warps, s);
  return launch_fma_g<32>(args, ctas, warps, s);
}

template <int G, int FDB>
static cudaError_t set_fma_attr_gd() {
  const int smem = (int)fma_smem_bytes(16, G);
  cudaError_t e = cudaFuncSetAttribute(getrf_task_fma_kernel<G, FDB>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(getrf_task_fma_kernel_occ<G, FDB, 7>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(getrf_task_fma_kernel_occ<G, FDB, 6>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(getrf_task_fma_kernel_occ<G, FDB, 5>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  return e;
}

template <int G>
static cudaError_t set_fma_attr_g() {
  cudaError_t e = set_fma_attr_gd<G, 1>();
  if (e == cudaSuccess) e = set_fma_attr_gd<G, 2>();
  return e;
}

cudaError_t init_getrf_fma_attributes() {
  cudaError_t e = set_fma_attr_g<8>();
  if (e == cudaSuccess) e = set_fma_attr_g<16>();
  if (e == cudaSuccess) e = set_fma_attr_g<32>();
  return e;
}

}  // namespace mfg
