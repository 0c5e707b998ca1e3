// Batched LU + solve kernels in MatFlat's arithmetic (Factorization.LuCore,
// MatFlat/Factorization.Lu.cs:296-350; the warp-level routines are in mf_lu.cuh): the
// size-bucketed task kernels (G lanes per matrix, persistent, one launch per bucket), the
// one-matrix-per-warp and float / Complex kernels, the CTA-per-matrix kernel for large orders,
// the resident form (one matrix per CTA in shared memory), the single-matrix drop-ins and the
// allocation-free entry point.
#include <cuda_runtime.h>

#include <type_traits>

#include "mf_device.cuh"
#include "mf_kernels.h"
#include "mf_scalar.cuh"
#include "mf_solve.cuh"
#include "mf_lu.cuh"

namespace mfg {

constexpr int SMEM_WARP_DOUBLES = SMEM_N + 2 * RHS_CHUNK * (SMEM_N + 1) + 2;
// Per-warp shared memory when the solve is staged in global memory (BatchArgs::gsolve).
constexpr int SMEM_WARP_DOUBLES_G = SMEM_N + 2;

static size_t getrf_smem_bytes(const BatchArgs& args, int warps) {
  return sizeof(double) * (args.gsolve ? SMEM_WARP_DOUBLES_G : SMEM_WARP_DOUBLES) * warps;
}

template <int WARPS, int IM, int DB>
__global__ void __launch_bounds__(WARPS * 32) getrf_batched_kernel(BatchArgs p) {
  extern __shared__ double sm_dyn[];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const long long gw = (long long)blockIdx.x * WARPS + warp;
  const int count = p.dcount ? *p.dcount : p.count;
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(p.queue, 1);
    idx = __shfl_sync(FULL_MASK, idx, 0);
    if (idx >= count) break;
    const int mat = p.order[idx];
    const int n = p.n[mat];
    const long long lda = p.lda[mat];
    double* a = p.a + p.a_off[mat];
    int* piv = p.piv + p.piv_off[mat];
    const bool gs = p.gsolve != nullptr;
    double* scr = (n <= SMEM_N) ? sm_dyn + warp * (gs ? SMEM_WARP_DOUBLES_G : SMEM_WARP_DOUBLES)
                                 : p.gscratch + gw * p.gscratch_stride;
    // The solve's staging: after the column sums in the same buffer, or the warp's global slice.
    double* sol = (n <= SMEM_N && gs) ? p.gsolve + gw * GSOLVE_STRIDE : scr + n;
    const int ldx = n | 1;
    int sign = 1, info = 0;
    if (!p.solve_only) lu_warp<DTraits, IM, DB>(a, n, n, lda, piv, scr, sign, info);
    if (p.nrhs > 0)
      getrs_warp(a, n, lda, piv, p.b + p.b_off[mat], n, p.nrhs, sol, sol + RHS_CHUNK * ldx);
    if (lane == 0 && !p.solve_only) {
      p.sign[mat] = sign;
      p.info[mat] = info;
    }
    __syncwarp();
  }
}

// The float and Complex overloads of the batched LU + solve.  Same schedule as the double kernel;
// the per-warp scratch (column sums, staged right-hand sides and their accumulators) takes
// W = sizeof(Acc)/8 times the double kernel's doubles: 1 for float (float storage, double sums),
// 2 for Complex.  a and b are the typed arrays behind args.a / args.b; offsets count elements.
template <int WARPS, class Tr, class S>
__global__ void __launch_bounds__(WARPS * 32) getrf_batched_t_kernel(BatchArgs p) {
  using T = typename Tr::T;
  using Acc = typename Tr::Acc;
  constexpr int W = sizeof(Acc) / sizeof(double);
  extern __shared__ double sm_dyn[];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const long long gw = (long long)blockIdx.x * WARPS + warp;
  T* abase = reinterpret_cast<T*>(p.a);
  T* bbase = reinterpret_cast<T*>(p.b);
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(p.queue, 1);
    idx = __shfl_sync(FULL_MASK, idx, 0);
    if (idx >= p.count) break;
    const int mat = p.order[idx];
    const int n = p.n[mat];
    const long long lda = p.lda[mat];
    T* a = abase + p.a_off[mat];
    int* piv = p.piv + p.piv_off[mat];
    double* scr = (n <= SMEM_N) ? sm_dyn + warp * W * SMEM_WARP_DOUBLES
                                 : p.gscratch + gw * p.gscratch_stride;
    const int ldx = n | 1;
    int sign = 1, info = 0;
    if (!p.solve_only) lu_warp<Tr, 1, DOT_BLOCK>(a, n, n, lda, piv, (Acc*)scr, sign, info);
    if (p.nrhs > 0)
      getrs_warp<S>(a, n, lda, piv, bbase + p.b_off[mat], n, p.nrhs, (T*)(scr + W * n),
                    (Acc*)(scr + W * n + W * RHS_CHUNK * ldx));
    if (lane == 0 && !p.solve_only) {
      p.sign[mat] = sign;
      p.info[mat] = info;
    }
    __syncwarp();
  }
}

template <class Tr>
__global__ void __launch_bounds__(32) getrf_single_kernel(typename Tr::T* a, int m, int n, int lda,
                                                          int* piv, int* out2, void* scratch) {
  int sign, info;
  lu_warp<Tr, true>(a, m, n, lda, piv, (typename Tr::Acc*)scratch, sign, info);
  if (threadIdx.x == 0) {
    out2[0] = sign;
    out2[1] = info;
  }
}

// ---------------------------------------------------------------------------------------------
// Size-bucketed work.  The plan cuts the batch into tasks of up to 32/G matrices of one order,
// with G (lanes per matrix: 8, 16 or 32) chosen per size bucket, and queues the tasks; a warp takes
// one task at a time and its groups of G lanes each factor (and solve) one matrix of it, in exactly
// the schedule above.  Small G keeps the lanes busy when a step has few dots; groups of a task
// share the order, so they follow the same control flow.

template <int IM, int DB, int G>
__device__ __forceinline__ void getrf_task(const BatchArgs& p, int first, int cnt, double* ws,
                                           long long gw) {
  const int lane = threadIdx.x & 31;
  const int g = lane / G;
  if (g >= cnt) return;
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
  const int ldx = n | 1;
  int sign = 1, info = 0;
  if (!p.solve_only)
    lu_warp<DTraits, IM, DB, G, true>(a, n, n, lda, piv, scr, sign, info, scr2);
  if (p.nrhs > 0)
    getrs_warp<DSolveIM, G>(a, n, lda, piv, p.b + p.b_off[mat], n, p.nrhs, sol,
                            sol + RHS_CHUNK * ldx);
  if ((lane & (G - 1)) == 0 && !p.solve_only) {
    p.sign[mat] = sign;
    p.info[mat] = info;
  }
}

// One launch per lanes-per-matrix bucket: G is a template parameter, so each variant keeps the
// register count of its own schedule.  args.task_first / task_gc / ntasks / queue describe the
// bucket's tasks.
template <int WARPS, int IM, int DB, int G>
__device__ __forceinline__ void getrf_task_loop(const BatchArgs& p) {
  extern __shared__ double sm_dyn[];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const long long gw = (long long)blockIdx.x * WARPS + warp;
  double* ws = sm_dyn + warp * (32 / G) * GROUP_SMEM_DOUBLES;
  for (;;) {
    int t = 0;
    if (lane == 0) t = atomicAdd(p.queue, 1);
    t = __shfl_sync(FULL_MASK, t, 0);
    if (t >= p.ntasks) break;
    getrf_task<IM, DB, G>(p, p.task_first[t], p.task_gc[t] >> 8, ws, gw);
    __syncwarp();
  }
}

template <int WARPS, int IM, int DB, int G>
__global__ void __launch_bounds__(WARPS * 32) getrf_task_kernel(BatchArgs p) {
  getrf_task_loop<WARPS, IM, DB, G>(p);
}

// The same with the register allocation bounded for MINB resident CTAs of 4 warps per SM (28 or
// 32 warps): the plan launches it when its shape asks for that many, for 32 lanes per matrix (the
// 16- and 8-lane schedules spill under that bound and run slower).
template <int IM, int DB, int G, int MINB>
__global__ void __launch_bounds__(128, MINB) getrf_task_kernel_occ(BatchArgs p) {
  getrf_task_loop<4, IM, DB, G>(p);
}

// One matrix per CTA of CTA_WARPS warps, taken from `order` (count from p.count or *p.dcount;
// with p.task_first, work item t is order position task_first[t]).  Dynamic shared memory holds
// the column sums (nmax doubles) and, when it fits (smem_solve), the solve's staging
// (2 RHS_CHUNK (nmax | 1) doubles after them); otherwise the solve is staged in the CTA's slice of
// the global scratch, which plans holding orders above SMEM_N allocate.
constexpr int CTA_WARPS = 8;
constexpr size_t CTA_SMEM_MAX = 200 * 1024;

template <int IM, int DB>
__global__ void __launch_bounds__(CTA_WARPS * 32) getrf_cta_kernel(BatchArgs p, int nmax,
                                                                   int smem_solve) {
  extern __shared__ double sm_dyn[];
  __shared__ CtaRed red;
  __shared__ int next;
  const int tid = threadIdx.x;
  const int count = p.dcount ? *p.dcount : p.count;
  for (;;) {
    if (tid == 0) next = atomicAdd(p.queue, 1);
    __syncthreads();
    const int idx = next;
    __syncthreads();
    if (idx >= count) break;
    const int mat = p.order[p.task_first ? p.task_first[idx] : idx];
    const int n = p.n[mat];
    const long long lda = p.lda[mat];
    double* a = p.a + p.a_off[mat];
    int* piv = p.piv + p.piv_off[mat];
    int sign = 1, info = 0;
    if (!p.solve_only) lu_cta<CTA_WARPS, IM, DB>(a, n, lda, piv, sm_dyn, sign, info, &red);
    if (p.nrhs > 0 && tid < 32) {
      double* sol = smem_solve ? sm_dyn + nmax
                               : p.gscratch + (long long)blockIdx.x * p.gscratch_stride;
      getrs_warp<DSolveIM, 32>(a, n, lda, piv, p.b + p.b_off[mat], n, p.nrhs, sol,
                               sol + RHS_CHUNK * (n | 1));
    }
    if (tid == 0 && !p.solve_only) {
      p.sign[mat] = sign;
      p.info[mat] = info;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------------------
// Resident form: one matrix per CTA of W warps, held in shared memory for the whole factorization
// and solve.  The CTA copies the matrix in (asynchronous 8-byte copies, column by column into a
// leading dimension n | 1, odd, so that the row-k dots, whose lanes walk different columns, hit
// different banks), runs lu_cta_early on the copy, writes the factors back with coalesced stores
// and solves from the shared copy, the right-hand sides split over the warps.  Several CTAs share
// an SM, so the warps a step leaves idle are covered by the other CTAs' work, and every operand of
// the Crout dots comes from shared memory instead of L1/L2.  A matrix whose copy does not fit the
// CTA's shared memory (smem_doubles) is factored in place in global memory, as getrf_cta_kernel
// does.  Work items are the plan's tasks (one matrix each), `ntasks` of them.
//
// Shared memory per CTA: the copy (n (n|1) doubles), two column-sum vectors (2n), and per warp
// the staging of its right-hand sides (2 nrc (n|1), nrc = min(ceil(nrhs / W), RHS_CHUNK)).
__host__ __device__ inline long long blk_smem_doubles(int n, int nrhs, int w, bool resident) {
  const long long ld = n | 1;
  int nrc = (nrhs + w - 1) / w;
  if (nrc > RHS_CHUNK) nrc = RHS_CHUNK;
  return (resident ? (long long)n * ld : 0) + 2LL * n + (long long)w * 2 * nrc * ld;
}

template <int W, int IM, int DB>
__global__ void __launch_bounds__(W * 32) getrf_blk_kernel(BatchArgs p, int smem_doubles) {
  extern __shared__ double sm_dyn[];
  __shared__ CtaRed red;
  __shared__ int next;
  constexpr int T = W * 32;
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  for (;;) {
    if (tid == 0) next = atomicAdd(p.queue, 1);
    __syncthreads();
    const int t = next;
    __syncthreads();
    if (t >= p.ntasks) break;
    const int mat = p.order[p.task_first[t]];
    const int n = p.n[mat];
    const long long lda = p.lda[mat];
    double* a = p.a + p.a_off[mat];
    int* piv = p.piv + p.piv_off[mat];
    const int lds = n | 1;
    // Solve-only calls read the factors where they are.
    const bool res = !p.solve_only && blk_smem_doubles(n, p.nrhs, W, true) <= smem_doubles;
    double* m = res ? sm_dyn : a;
    const long long ldm = res ? (long long)lds : lda;
    double* scol = sm_dyn + (res ? (long long)n * lds : 0);
    double* scol2 = scol + n;
    double* stage = scol2 + n;
    const int ne = n * n;
    if (res) {
      for (int e = tid; e < ne; e += T) {
        const int j = e / n;
        const int i = e - j * n;
        const unsigned d = (unsigned)__cvta_generic_to_shared(m + (long long)j * lds + i);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d),
                     "l"(a + (long long)j * lda + i)
                     : "memory");
      }
      asm volatile("cp.async.commit_group;\n" ::: "memory");
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
      __syncthreads();
    }
    int sign = 1, info = 0;
    if (!p.solve_only) lu_cta_early<W, IM, DB>(m, n, ldm, piv, scol, scol2, sign, info, &red);
    if (res) {
      for (int e = tid; e < ne; e += T) {
        const int j = e / n;
        const int i = e - j * n;
        a[(long long)j * lda + i] = m[(long long)j * lds + i];
      }
    }
    if (p.nrhs > 0) {
      // Warp w solves right-hand sides [w q, min(nrhs, (w + 1) q)), q = ceil(nrhs / W).
      const int q = (p.nrhs + W - 1) / W;
      const int r0 = warp * q;
      const int nr = min(p.nrhs, r0 + q) - r0;
      int nrc = q < RHS_CHUNK ? q : RHS_CHUNK;
      double* xs = stage + (long long)warp * 2 * nrc * lds;
      if (nr > 0)
        getrs_warp<DSolveIM, 32>(m, n, ldm, piv, p.b + p.b_off[mat] + (long long)r0 * n, n, nr,
                                 xs, xs + (long long)nrc * lds);
    }
    if (tid == 0 && !p.solve_only) {
      p.sign[mat] = sign;
      p.info[mat] = info;
    }
    __syncthreads();
  }
}

constexpr int BLK_SMEM_MAX = 227 * 1024 - 1024;  // dynamic bytes, leaving room for the static part

template <int W>
static cudaError_t launch_getrf_blk_w(const BatchArgs& args, int ctas, int smem_bytes,
                                      cudaStream_t s) {
  const int sd = smem_bytes / (int)sizeof(double);
  if (args.hw_mul)
    getrf_blk_kernel<W, 0, 4><<<ctas, W * 32, smem_bytes, s>>>(args, sd);
  else if (args.dot_block == 2)
    getrf_blk_kernel<W, 1, 2><<<ctas, W * 32, smem_bytes, s>>>(args, sd);
  else
    getrf_blk_kernel<W, 1, 4><<<ctas, W * 32, smem_bytes, s>>>(args, sd);
  return cudaGetLastError();
}

template <int W>
static cudaError_t set_getrf_blk_attr() {
  cudaError_t e = cudaFuncSetAttribute(getrf_blk_kernel<W, 0, 4>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, BLK_SMEM_MAX);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(getrf_blk_kernel<W, 1, 2>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, BLK_SMEM_MAX);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(getrf_blk_kernel<W, 1, 4>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, BLK_SMEM_MAX);
  return e;
}

long long getrf_blk_smem_doubles(int n, int nrhs, int w, bool resident) {
  return blk_smem_doubles(n, nrhs, w, resident);
}

int getrf_blk_smem_max() { return BLK_SMEM_MAX; }

cudaError_t launch_getrf_blk(const BatchArgs& args, int ctas, int w, int smem_bytes,
                             cudaStream_t s) {
  if (smem_bytes > BLK_SMEM_MAX || smem_bytes < 0) return cudaErrorInvalidValue;
  switch (w) {
    case 2: return launch_getrf_blk_w<2>(args, ctas, smem_bytes, s);
    case 4: return launch_getrf_blk_w<4>(args, ctas, smem_bytes, s);
    case 8: return launch_getrf_blk_w<8>(args, ctas, smem_bytes, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_getrf_cta(const BatchArgs& args, int ctas, int nmax, cudaStream_t s) {
  const size_t with_solve =
      sizeof(double) * ((size_t)nmax + 2 * (size_t)RHS_CHUNK * (size_t)(nmax | 1));
  const int smem_solve = with_solve <= CTA_SMEM_MAX ? 1 : 0;
  // Without room for the solve in shared memory the staging needs the plan's global scratch.
  if (!smem_solve && args.nrhs > 0 && !args.gscratch) return cudaErrorInvalidValue;
  const size_t smem = smem_solve ? with_solve : sizeof(double) * (size_t)nmax;
  if (smem > CTA_SMEM_MAX) return cudaErrorInvalidValue;
  if (args.hw_mul)
    getrf_cta_kernel<0, 4><<<ctas, CTA_WARPS * 32, smem, s>>>(args, nmax, smem_solve);
  else
    getrf_cta_kernel<1, 2><<<ctas, CTA_WARPS * 32, smem, s>>>(args, nmax, smem_solve);
  return cudaGetLastError();
}

int getrf_cta_warps() { return CTA_WARPS; }

template <int WARPS>
static size_t getrf_task_smem_bytes(int g) {
  return sizeof(double) * (32 / g) * GROUP_SMEM_DOUBLES * WARPS;
}

template <int WARPS, int G>
static cudaError_t launch_getrf_task_g(const BatchArgs& args, int ctas, cudaStream_t s) {
  const size_t smem = getrf_task_smem_bytes<WARPS>(G);
  if (args.hw_mul)
    getrf_task_kernel<WARPS, 0, 4, G><<<ctas, WARPS * 32, smem, s>>>(args);
  else if (WARPS == 4 && G == 32 && args.dot_block == 2 && args.minb >= 8)
    getrf_task_kernel_occ<1, 2, G, 8><<<ctas, 128, smem, s>>>(args);
  else if (WARPS == 4 && G == 32 && args.dot_block == 2 && args.minb == 7)
    getrf_task_kernel_occ<1, 2, G, 7><<<ctas, 128, smem, s>>>(args);
  else if (args.dot_block == 2)
    getrf_task_kernel<WARPS, 1, 2, G><<<ctas, WARPS * 32, smem, s>>>(args);
  else
    getrf_task_kernel<WARPS, 1, 4, G><<<ctas, WARPS * 32, smem, s>>>(args);
  return cudaGetLastError();
}

template <int WARPS>
static cudaError_t launch_getrf_task_w(const BatchArgs& args, int ctas, int g, cudaStream_t s) {
  if (g == 8) return launch_getrf_task_g<WARPS, 8>(args, ctas, s);
  if (g == 16) return launch_getrf_task_g<WARPS, 16>(args, ctas, s);
  return launch_getrf_task_g<WARPS, 32>(args, ctas, s);
}

template <int WARPS, int G>
static cudaError_t set_getrf_task_attr_g() {
  const int smem = (int)getrf_task_smem_bytes<WARPS>(G);
  cudaError_t e = cudaFuncSetAttribute(getrf_task_kernel<WARPS, 0, 4, G>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(getrf_task_kernel<WARPS, 1, 2, G>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(getrf_task_kernel<WARPS, 1, 4, G>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (WARPS == 4 && G == 32 && e == cudaSuccess)
    e = cudaFuncSetAttribute(getrf_task_kernel_occ<1, 2, G, 8>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (WARPS == 4 && G == 32 && e == cudaSuccess)
    e = cudaFuncSetAttribute(getrf_task_kernel_occ<1, 2, G, 7>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  return e;
}

template <int WARPS>
static cudaError_t set_getrf_task_attr() {
  cudaError_t e = set_getrf_task_attr_g<WARPS, 8>();
  if (e == cudaSuccess) e = set_getrf_task_attr_g<WARPS, 16>();
  if (e == cudaSuccess) e = set_getrf_task_attr_g<WARPS, 32>();
  return e;
}

template <int WARPS>
static cudaError_t launch_getrf_w(const BatchArgs& args, int ctas, cudaStream_t s) {
  const size_t smem = getrf_smem_bytes(args, WARPS);
  if (args.hw_mul == 2)
    getrf_batched_kernel<WARPS, 2, 4><<<ctas, WARPS * 32, smem, s>>>(args);
  else if (args.hw_mul)
    getrf_batched_kernel<WARPS, 0, 4><<<ctas, WARPS * 32, smem, s>>>(args);
  else if (args.dot_block == 2)
    getrf_batched_kernel<WARPS, true, 2><<<ctas, WARPS * 32, smem, s>>>(args);
  else
    getrf_batched_kernel<WARPS, true, 4><<<ctas, WARPS * 32, smem, s>>>(args);
  return cudaGetLastError();
}

template <int WARPS>
static cudaError_t set_getrf_attr() {
  const size_t smem = sizeof(double) * SMEM_WARP_DOUBLES * WARPS;
  cudaError_t e = cudaFuncSetAttribute(getrf_batched_kernel<WARPS, true, 4>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(getrf_batched_kernel<WARPS, true, 2>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(getrf_batched_kernel<WARPS, 2, 4>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(getrf_batched_kernel<WARPS, false, 4>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

// Float / Complex overloads: at most 8 warps per CTA (a Complex warp keeps 18.6 KB of shared
// scratch); a plan shaped with 16 warps per CTA launches twice the CTAs of 8 warps, so the warp
// count, and with it the global-scratch slices, stay the same.
constexpr int GETRF_T_MAX_WARPS = 8;

template <int WARPS, class Tr, class S>
static cudaError_t launch_getrf_t_w(const BatchArgs& args, int ctas, cudaStream_t s) {
  constexpr int W = sizeof(typename Tr::Acc) / sizeof(double);
  const size_t smem = sizeof(double) * W * SMEM_WARP_DOUBLES * WARPS;
  getrf_batched_t_kernel<WARPS, Tr, S><<<ctas, WARPS * 32, smem, s>>>(args);
  return cudaGetLastError();
}

template <class Tr, class S>
static cudaError_t launch_getrf_t(const BatchArgs& args, int ctas, int warps, cudaStream_t s) {
  if (warps > GETRF_T_MAX_WARPS) {
    ctas *= warps / GETRF_T_MAX_WARPS;
    warps = GETRF_T_MAX_WARPS;
  }
  switch (warps) {
    case 1: return launch_getrf_t_w<1, Tr, S>(args, ctas, s);
    case 2: return launch_getrf_t_w<2, Tr, S>(args, ctas, s);
    case 4: return launch_getrf_t_w<4, Tr, S>(args, ctas, s);
    case 8: return launch_getrf_t_w<8, Tr, S>(args, ctas, s);
    default: return cudaErrorInvalidValue;
  }
}

template <int WARPS, class Tr, class S>
static cudaError_t set_getrf_t_attr() {
  constexpr int W = sizeof(typename Tr::Acc) / sizeof(double);
  const size_t smem = sizeof(double) * W * SMEM_WARP_DOUBLES * WARPS;
  return cudaFuncSetAttribute(getrf_batched_t_kernel<WARPS, Tr, S>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <class Tr, class S>
static cudaError_t set_getrf_t_attrs() {
  cudaError_t e;
  if ((e = set_getrf_t_attr<1, Tr, S>()) != cudaSuccess) return e;
  if ((e = set_getrf_t_attr<2, Tr, S>()) != cudaSuccess) return e;
  if ((e = set_getrf_t_attr<4, Tr, S>()) != cudaSuccess) return e;
  return set_getrf_t_attr<8, Tr, S>();
}

cudaError_t launch_sgetrf_batched(const BatchArgs& args, int ctas, int warps, cudaStream_t s) {
  return launch_getrf_t<STraits, SSolve>(args, ctas, warps, s);
}
cudaError_t launch_zgetrf_batched(const BatchArgs& args, int ctas, int warps, cudaStream_t s) {
  return launch_getrf_t<ZTraits, ZSolve<false>>(args, ctas, warps, s);
}

// Raises the dynamic shared-memory limit of every variant; called once per device, outside any
// stream capture.
cudaError_t init_getrf_attributes() {
  cudaError_t e;
  if ((e = set_getrf_t_attrs<STraits, SSolve>()) != cudaSuccess) return e;
  if ((e = set_getrf_t_attrs<ZTraits, ZSolve<false>>()) != cudaSuccess) return e;
  if ((e = set_getrf_attr<1>()) != cudaSuccess) return e;
  if ((e = set_getrf_attr<2>()) != cudaSuccess) return e;
  if ((e = set_getrf_attr<4>()) != cudaSuccess) return e;
  if ((e = set_getrf_attr<8>()) != cudaSuccess) return e;
  // The CTA-per-matrix kernel keeps the column sums (and, up to order ~2,800, the solve's
  // staging) in up to CTA_SMEM_MAX bytes of shared memory.
  if ((e = cudaFuncSetAttribute(getrf_cta_kernel<0, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)CTA_SMEM_MAX)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(getrf_cta_kernel<1, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)CTA_SMEM_MAX)) != cudaSuccess)
    return e;
  if ((e = set_getrf_task_attr<1>()) != cudaSuccess) return e;
  if ((e = set_getrf_task_attr<2>()) != cudaSuccess) return e;
  if ((e = set_getrf_task_attr<4>()) != cudaSuccess) return e;
  if ((e = set_getrf_task_attr<8>()) != cudaSuccess) return e;
  if ((e = set_getrf_task_attr<16>()) != cudaSuccess) return e;
  if ((e = set_getrf_blk_attr<2>()) != cudaSuccess) return e;
  if ((e = set_getrf_blk_attr<4>()) != cudaSuccess) return e;
  if ((e = set_getrf_blk_attr<8>()) != cudaSuccess) return e;
  return set_getrf_attr<16>();
}

cudaError_t launch_getrf_tasks(const BatchArgs& args, int ctas, int warps, int g, cudaStream_t s) {
  switch (warps) {
    case 1: return launch_getrf_task_w<1>(args, ctas, g, s);
    case 2: return launch_getrf_task_w<2>(args, ctas, g, s);
    case 4: return launch_getrf_task_w<4>(args, ctas, g, s);
    case 8: return launch_getrf_task_w<8>(args, ctas, g, s);
    case 16: return launch_getrf_task_w<16>(args, ctas, g, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_getrf_batched(const BatchArgs& args, int ctas, int warps, cudaStream_t s) {
  switch (warps) {
    case 1: return launch_getrf_w<1>(args, ctas, s);
    case 2: return launch_getrf_w<2>(args, ctas, s);
    case 4: return launch_getrf_w<4>(args, ctas, s);
    case 8: return launch_getrf_w<8>(args, ctas, s);
    case 16: return launch_getrf_w<16>(args, ctas, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_getrf_single(double* a, int m, int n, int lda, int* piv, int* out2,
                                double* scratch, cudaStream_t s) {
  getrf_single_kernel<DTraits><<<1, 32, 0, s>>>(a, m, n, lda, piv, out2, scratch);
  return cudaGetLastError();
}

cudaError_t launch_sgetrf_single(float* a, int m, int n, int lda, int* piv, int* out2,
                                 double* scratch, cudaStream_t s) {
  getrf_single_kernel<STraits><<<1, 32, 0, s>>>(a, m, n, lda, piv, out2, scratch);
  return cudaGetLastError();
}

cudaError_t launch_zgetrf_single(double* a, int m, int n, int lda, int* piv, int* out2,
                                 double* scratch, cudaStream_t s) {
  getrf_single_kernel<ZTraits><<<1, 32, 0, s>>>((zdouble*)a, m, n, lda, piv, out2, scratch);
  return cudaGetLastError();
}

}  // namespace mfg

namespace mfg {

// ---------------------------------------------------------------------------------------------
// Allocation-free variant for callers that must not allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: code that runs inside a CUDA stream capture
// owned by someone else, real-time or certified paths whose memory is budgeted once at start-up,
// and hosts that hand the library a fixed device arena.  For them the batched LU + solve has a
// second entry point that allocates nothing: the caller passes the matrices, pivots, right-hand
// sides and outputs (device pointers, one order n for the whole batch, fixed strides), and the
// kernel's scratch — the work-queue counter and, for n > 128, the per-warp column sums and staged
// right-hand sides — lives in the file-scope array below, which every GPU that loads the library
// holds until the process exits.
//
// Limits: n <= NOALLOC_MAX_N (256); for n > 128 at most NOALLOC_MAX_WARPS warps run, each with a
// NOALLOC_WARP_STRIDE-double slice (on a GPU with more SMs than NOALLOC_MAX_WARPS / 4 some SMs
// then get no work, so orders above 128 can run below the plan path's rate); the array is
// 11.4 MB.  Every call shares the array and keeps
// the previous call's contents, so the counter is cleared (cudaMemsetAsync) before each launch,
// and calls that overlap on the GPU (two streams, or two contexts on one device) race on it.
constexpr int NOALLOC_MAX_N = 256;
constexpr int NOALLOC_MAX_WARPS = 608;
constexpr long long NOALLOC_HEADER_DOUBLES = 32;  // 256 bytes: the work-queue counter
constexpr long long NOALLOC_WARP_STRIDE =
    ((NOALLOC_MAX_N + 2LL * RHS_CHUNK * (NOALLOC_MAX_N + 1) + 2) + 31) / 32 * 32;
constexpr long long NOALLOC_SCRATCH_DOUBLES =
    NOALLOC_HEADER_DOUBLES + (long long)NOALLOC_MAX_WARPS * NOALLOC_WARP_STRIDE;

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];

struct StridedArgs {
  double* a;
  long long stride_a;
  int* piv;
  long long stride_piv;
  double* b;
  long long stride_b;
  int* sign;
  int* info;
  int n;
  int lda;
  int nrhs;
  int count;
  double* scratch;  // device address of g_noalloc_scratch
};

template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32) getrf_strided_noalloc_kernel(StridedArgs p) {
  extern __shared__ double sm_dyn[];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const long long gw = (long long)blockIdx.x * WARPS + warp;
  int* queue = reinterpret_cast<int*>(p.scratch);
  const int n = p.n;
  const long long lda = p.lda;
  const int ldx = n | 1;
  double* scr = (n <= SMEM_N) ? sm_dyn + warp * SMEM_WARP_DOUBLES
                               : p.scratch + NOALLOC_HEADER_DOUBLES + gw * NOALLOC_WARP_STRIDE;
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(queue, 1);
    idx = __shfl_sync(FULL_MASK, idx, 0);
    if (idx >= p.count) break;
    double* a = p.a + (long long)idx * p.stride_a;
    int* piv = p.piv + (long long)idx * p.stride_piv;
    int sign, info;
    lu_warp<DTraits, true>(a, n, n, lda, piv, scr, sign, info);
    if (p.nrhs > 0)
      getrs_warp(a, n, lda, piv, p.b + (long long)idx * p.stride_b, n, p.nrhs, scr + n,
                 scr + n + RHS_CHUNK * ldx);
    if (lane == 0) {
      p.sign[idx] = sign;
      p.info[idx] = info;
    }
    __syncwarp();
  }
}

// Set-up: the device address of g_noalloc_scratch, looked up on every call with the context's
// device current (in host code the array's name is only a host-side stand-in, never a device
// address).  The look-up allocates nothing; the first one on a device may load this library's
// kernels onto it, so that first call should come before any stream capture.  Nothing is
// cached, so a failed look-up is simply retried by the next call and a cudaDeviceReset leaves
// no stale address behind.  The kernel's 37 KB of dynamic shared memory stay under the default
// 48 KB limit, so no function attribute has to be set.
static cudaError_t noalloc_scratch(int device, double** out) {
  int cur = -1;
  cudaError_t e = cudaGetDevice(&cur);
  if (e != cudaSuccess) return e;
  if (cur != device) return cudaErrorInvalidDevice;
  void* ptr = nullptr;
  e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess) return e;
  *out = (double*)ptr;
  return cudaSuccess;
}
static_assert(sizeof(double) * SMEM_WARP_DOUBLES * 4 <= 48 * 1024,
              "the allocation-free kernel must fit the default shared-memory limit");

int noalloc_max_n() { return NOALLOC_MAX_N; }

cudaError_t launch_getrf_strided_noalloc(double* a, int n, int lda, long long stride_a, int* piv,
                                         long long stride_piv, int nrhs, double* b,
                                         long long stride_b, int* sign, int* info, int count,
                                         int device, int sm_count, cudaStream_t s) {
  double* scratch = nullptr;
  cudaError_t e = noalloc_scratch(device, &scratch);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(scratch, 0, sizeof(double) * NOALLOC_HEADER_DOUBLES, s);
  if (e != cudaSuccess || count == 0) return e;
  constexpr int WARPS = 4;
  long long ctas = (long long)sm_count * (n <= SMEM_N ? 4 : 1);
  if (n > SMEM_N && ctas * WARPS > NOALLOC_MAX_WARPS) ctas = NOALLOC_MAX_WARPS / WARPS;
  const long long need = ((long long)count + WARPS - 1) / WARPS;
  if (ctas > need) ctas = need;
  if (ctas < 1) ctas = 1;
  StridedArgs p{a, stride_a, piv, stride_piv, b, stride_b, sign, info, n, lda, nrhs, count,
                scratch};
  const size_t smem = sizeof(double) * SMEM_WARP_DOUBLES * WARPS;
  getrf_strided_noalloc_kernel<WARPS><<<(unsigned)ctas, WARPS * 32, smem, s>>>(p);
  return cudaGetLastError();
}

}  // namespace mfg
