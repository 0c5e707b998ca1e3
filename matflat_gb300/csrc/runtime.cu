// Host runtime and C ABI (include/matflat_gpu.h): contexts, device workspace, batch plans with
// longest-first ordering, launch-shape selection and CUDA-graph replay.
//
// Argument validation mirrors MatFlat's checks, in MatFlat's order, and reports the 1-based
// position of the offending argument as a negative status (the context is argument 1).
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/matflat_gpu.h"
#include "mf_kernels.h"

using mfg::BatchArgs;

namespace {

constexpr const char* kVersion = "0.1.0";

// Owning device allocation (freed with its owner; movable, not copyable), so that every early
// return of a failing set-up releases what it had reserved.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : ptr(o.ptr), bytes(o.bytes) {
    o.ptr = nullptr;
    o.bytes = 0;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      ptr = o.ptr;
      bytes = o.bytes;
      o.ptr = nullptr;
      o.bytes = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  cudaError_t reserve(size_t want) {
    if (want <= bytes) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e == cudaSuccess) bytes = want;
    return e;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
  }
};

int env_int(const char* name, int dflt) {
  const char* v = std::getenv(name);
  if (!v || !*v) return dflt;
  return std::atoi(v);
}

std::once_flag g_attr_once[64];
cudaError_t g_attr_err[64];

}  // namespace

struct mfg_ctx {
  int device = 0;
  int sm_count = 0;
  int smem_per_sm = 0;   // shared memory per SM (bytes)
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  DevBuf work;
  std::string last_error;
  bool use_graphs = true;
  // Autotuner results: launch shape per (plan kind, size bucket), used by later plans.
  std::map<long long, std::array<int, 5>> tune;
};

// Makes the context's device current for the duration of an entry point and restores the
// caller's device afterwards, so a host thread that switched devices after mfg_create still
// launches on the context's device, stream and workspace.
struct DeviceScope {
  int prev = -1;
  explicit DeviceScope(const mfg_ctx* ctx) {
    if (!ctx) return;
    int cur = -1;
    if (cudaGetDevice(&cur) == cudaSuccess && cur != ctx->device &&
        cudaSetDevice(ctx->device) == cudaSuccess)
      prev = cur;
  }
  ~DeviceScope() {
    if (prev >= 0) cudaSetDevice(prev);
  }
  DeviceScope(const DeviceScope&) = delete;
  DeviceScope& operator=(const DeviceScope&) = delete;
};

struct mfg_plan {
  enum Kind { GETRF, POTRF, GEQRF, MIXED, GETRI, GEVD } kind;
  mfg_ctx* ctx = nullptr;
  int count = 0;
  int nrhs = 0;
  int max_n = 0;
  DevBuf meta;      // order | n | lda | a_off | piv_off | b_off | queue
  DevBuf scratch;   // per-warp scratch for n > SMEM_N
  DevBuf gsolve;    // GETRF: per-warp global staging of the solve (BatchArgs::gsolve)
  DevBuf fbackup;   // GETRF FMA form: per-warp copies of the matrices being factored
  long long fma_stride = 0;   // GETRF: doubles per warp the FMA form's copies need
  bool last_host = false;     // the last execution went through the host-buffer pipeline
  BatchArgs args{};
  mfg::QrBatchArgs<double> qd{};
  mfg::QrBatchArgs<float> qs{};
  mfg::GevdArgs gv{};  // GEVD: the front half of the generalized eigenproblem
  mfg::QrBatchArgs<double> qz{};  // GEQRF: the Complex overload (interleaved doubles)
  int qr_max_cols = 0;             // GEQRF: max over the batch of n + nrhs
  int qr_coef_need = 0;            // GEQRF: per-group coefficient count (fused: 2 (n + nrhs))
  const int* qr_order_work = nullptr;     // GEQRF: queue order for 32 lanes (longest first)
  const int* qr_order_grouped = nullptr;  // GEQRF: queue order for smaller groups (by n, then m)
  int qr_float = 0;  // GEQRF: which overload the next launch runs (0 double, 1 float, 2 Complex)
  int elem = 0;      // GETRF/POTRF/GETRI/GEVD: element type of the next launch (0 double, 1 float,
                     // 2 Complex)
  int ctas_t = 0;    // GEVD: the grid of the float / Complex kernel
  long long dstride = 0;  // GETRF/POTRF: the double kernels' per-group scratch stride
  int mx_n = 0;      // MIXED: order of every matrix
  DevBuf mx_work;    // MIXED: FP32 factors | ipiv | operand copies | per-system state | fallback
  mfg_plan* mx_fb = nullptr;  // MIXED: the exact FP64 LU plan of the fallback (all systems)
  // MIXED: TMA maps of the operand copies: TF32 A, B | BF16 A, B | split-TF32 low parts A, B
  alignas(64) CUtensorMap mx_tm[6];
  int ctas = 0;
  int warps = 0;
  // GETRF (double): size-bucketed tasks.  gsel picks the lanes-per-matrix table (-1: one matrix
  // per warp, no tasks); segment s holds the tasks of G = 32 >> s lanes per matrix.
  int gsel = -1;
  int seg_off[5] = {0, 0, 0, 0, 0};
  int seg_cnt[5] = {0, 0, 0, 0, 0};
  // POTRF (double): lanes-per-matrix table of the size buckets (0: one group size for the plan,
  // args.group); segment s of `order` holds the matrices of G = 32 >> s lanes.
  int csel = 0;
  int cta_nmax = 0;  // GETRF: largest order of the CTA-per-matrix segment (segment 3)
  int big_cps = 3;   // GETRF FMA form: CTAs per SM of the blocked kernel (2 or 3; MFG_LU_BIG_CPS)
  bool big_mma = false;  // ... and its trailing updates on the FP64 tensor pipe (MFG_LU_BIG_MMA)
  // GETRF (double): resident form (segment 4): orders in [blk_lo, SMEM_N] go to one CTA of blk_w
  // warps each, blk_cps CTAs per SM, the matrix in shared memory; blk_lo = 0: off.
  int blk_lo = 0;
  int blk_w = 4;
  int blk_cps = 2;
  int blk_nmax = 0;
  int* d_task_first = nullptr;
  int* d_task_gc = nullptr;
  std::vector<int> hn;  // GETRF/POTRF: the order of every matrix (host copy, for the autotuner)
  // Host copies of the layout (every batched kind), for the pipelined host-buffer calls: m (QR),
  // lda, ldb (GEVD), and the offsets of a, of the second array (piv / rdiag / B), of b and of C.
  std::vector<int> hm, hlda, hldb;
  std::vector<long long> haoff, hpivoff, hboff, hcoff;
  // The pipelined host-buffer path (built on the first host call of an operation): contiguous
  // chunks of the batch, each with its own plan, and device mirrors of the caller's arrays.
  struct PipeArray {
    int dir = 3;                     // 1: uploaded, 2: downloaded, 3: both
    size_t es = 8;                   // element size
    std::vector<size_t> beg, end;    // element range of every matrix
    std::vector<size_t> lo, hi;      // element range of every chunk
    DevBuf dev;
  };
  struct Pipe {
    int op = -1;
    std::vector<PipeArray> arr;
    std::vector<mfg_plan*> chunk;
    std::vector<int> c0, c1;
    cudaStream_t h2d = nullptr, d2h = nullptr;
    cudaStream_t comp[3] = {nullptr, nullptr, nullptr};  // with the context's stream: four
    std::vector<cudaEvent_t> in, done;
  } pipe;
  // CUDA graph of the last execution (keyed by the data pointers and the stream).
  cudaGraphExec_t exec = nullptr;
  const void* key[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
};

namespace {

void pipe_release(mfg_plan* p);
int plan_set_elem(mfg_plan* p, int elem);

int fail(mfg_ctx* ctx, int code, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    ctx->last_error = buf;
  }
  return code;
}

// A failed CUDA call: MFG_ERR_ALLOC when the device (or page-locked host memory) ran out,
// MFG_ERR_CUDA otherwise; the text names the call.
int cuda_fail(mfg_ctx* ctx, cudaError_t e, const char* what) {
  const int code = e == cudaErrorMemoryAllocation ? MFG_ERR_ALLOC : MFG_ERR_CUDA;
  return fail(ctx, code, "%s: %s", what, cudaGetErrorString(e));
}

#define MFG_CUDA(ctx, call)                                  \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
  } while (0)

cudaError_t init_device_attributes(int device) {
  const int slot = device & 63;
  std::call_once(g_attr_once[slot], [slot]() {
    cudaError_t e = mfg::init_getrf_attributes();
    if (e == cudaSuccess) e = mfg::init_getrf_fma_attributes();
    if (e == cudaSuccess) e = mfg::init_potrf_attributes();
    if (e == cudaSuccess) e = mfg::init_potrf_t_attributes();
    if (e == cudaSuccess) e = mfg::init_getri_attributes();
    if (e == cudaSuccess) e = mfg::init_grad_attributes();
    g_attr_err[slot] = e;
  });
  return g_attr_err[slot];
}

// Elements spanned by an m-by-n column-major matrix with leading dimension ld.
size_t span(long long m, long long n, long long ld) {
  if (m <= 0 || n <= 0) return 0;
  return (size_t)(ld * (n - 1) + m);
}

// Execution order of a batch.  Pure longest-first puts thousands of the largest matrices in
// flight at once, whose combined working set (up to 128 KB each) overflows the 129 MB L2 and turns
// every re-read of L and U into a DRAM access.  The "snake" order pairs the i-th largest with the
// i-th smallest matrix (L0 S0 L1 S1 ...), so the matrices in flight average out, and the
// mid-sized ones come last, which keeps the tail short.  MFG_ORDER=lpt selects longest-first.
std::vector<int> snake_order(int count, const int* n) {
  std::vector<int> sorted(count);
  std::iota(sorted.begin(), sorted.end(), 0);
  std::stable_sort(sorted.begin(), sorted.end(), [&](int x, int y) { return n[x] > n[y]; });
  const char* mode = std::getenv("MFG_ORDER");
  if (mode && std::strcmp(mode, "lpt") == 0) return sorted;
  if (mode && std::strcmp(mode, "shuffle") == 0) {
    // Deterministic shuffle of the first 95% of the work (so the matrices in flight have the
    // batch's average size), longest-first for the rest (a short tail).
    std::vector<int> out = sorted;
    double total = 0, acc = 0;
    for (int i = 0; i < count; i++) total += (double)n[i] * n[i] * n[i];
    int cut = count;
    for (int i = count - 1; i >= 0; i--) {
      acc += (double)n[sorted[i]] * n[sorted[i]] * n[sorted[i]];
      if (acc >= 0.05 * total) {
        cut = i;
        break;
      }
    }
    std::vector<int> head(sorted.begin(), sorted.begin() + cut), tail(sorted.begin() + cut,
                                                                      sorted.end());
    unsigned long long st = 0x9E3779B97F4A7C15ull;
    for (int i = (int)head.size() - 1; i > 0; i--) {
      st = st * 6364136223846793005ull + 1442695040888963407ull;
      const int j = (int)((st >> 33) % (unsigned long long)(i + 1));
      std::swap(head[i], head[j]);
    }
    out.assign(head.begin(), head.end());
    out.insert(out.end(), tail.begin(), tail.end());
    return out;
  }
  std::vector<int> out;
  out.reserve(count);
  int lo = 0, hi = count - 1;
  while (lo <= hi) {
    out.push_back(sorted[lo++]);
    if (lo <= hi) out.push_back(sorted[hi--]);
  }
  return out;
}

// Launch shape of a batched plan: WARPS warps per CTA and enough CTAs to hold `warps_per_sm`
// warps on every SM (persistent: each warp pulls matrices from the queue until it is empty).
void choose_shape(mfg_plan* p, int fixed_warps = 0) {
  const bool inv = p->kind == mfg_plan::GETRI;
  // LuInverse stages 32 columns per warp in shared memory: its CTA shape is fixed and the grid
  // holds as many CTAs as fit on an SM.
  const int warps = inv ? mfg::getri_warps_per_cta()
                        : fixed_warps ? fixed_warps : env_int("MFG_WARPS_PER_CTA", 4);
  p->warps = warps;
  long long ctas;
  if (inv) {
    ctas = (long long)p->ctx->sm_count * mfg::getri_ctas_per_sm();
  } else {
    // 24 warps per SM for the LU (its measured best on the 100,000-matrix batch), 16 otherwise.
    const int wps = env_int("MFG_WARPS_PER_SM", p->kind == mfg_plan::GETRF ? 24 : 16);
    ctas = (long long)p->ctx->sm_count * wps / warps;
  }
  // Never more warps than matrices.
  const long long need = ((long long)p->count + warps - 1) / warps;
  if (ctas > need) ctas = need;
  if (ctas < 1) ctas = 1;
  p->ctas = (int)ctas;
}

// Doubles per warp of the global solve staging of a getrf / potrf plan.
long long gsolve_stride(int kind) {
  return kind == mfg_plan::POTRF ? mfg::GSOLVE_STRIDE_C : mfg::GSOLVE_STRIDE * mfg::GETRF_GROUPS;
}

// Lanes per matrix of the LU's size buckets, by table: 0 all 32; 1 16 up to order 128; 2 8 up to
// order 48, 16 up to 128; 3 8 up to 128; 4 8 up to 32, 16 up to 96; 5 8 up to 24, 16 up to 64;
// 6 16 up to 48.  Orders above 128 always take 32 lanes (their vectors live in global scratch
// sized per warp).
int lu_lanes(int gsel, int n) {
  if (n > mfg::SMEM_N) return 32;
  switch (gsel) {
    case 1: return 16;
    case 2: return n <= 48 ? 8 : 16;
    case 3: return 8;
    case 4: return n <= 32 ? 8 : n <= 96 ? 16 : 32;
    case 5: return n <= 24 ? 8 : n <= 64 ? 16 : 32;
    case 6: return n <= 48 ? 16 : 32;
    default: return 32;
  }
}

// Lanes per matrix of the Cholesky's size buckets, by table: 1 4 up to order 16, 8 up to 32, 16
// up to 64, 32 above; 2 8 up to 32, 16 up to 64, 32 above.  A group of G lanes keeps its vectors
// in shared memory for orders up to 4G, which both tables respect.
int chol_lanes(int csel, int n) {
  if (csel == 1) return n <= 16 ? 4 : n <= 32 ? 8 : n <= 64 ? 16 : 32;
  if (csel == 2) return n <= 32 ? 8 : n <= 64 ? 16 : 32;
  return 32;
}

// Orders a POTRF plan's queue by size bucket for table csel: segments of 32, 16, 8 and 4 lanes
// per matrix, each in decreasing order of n (the groups of a warp take consecutive entries, so
// they get matrices of about the same order).  csel 0 restores the single queue.
int potrf_build_segments(mfg_plan* p, int csel) {
  mfg_ctx* ctx = p->ctx;
  const int count = p->count;
  std::vector<int> idx(count);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return p->hn[x] > p->hn[y]; });
  std::vector<int> order;
  order.reserve(count);
  for (int sg = 0; sg < 4; sg++) {
    p->seg_off[sg] = (int)order.size();
    for (int i : idx)
      if ((32 >> sg) == (csel > 0 ? chol_lanes(csel, p->hn[i]) : 32)) order.push_back(i);
    p->seg_cnt[sg] = (int)order.size() - p->seg_off[sg];
  }
  if (csel == 0) order = snake_order(count, p->hn.data());
  if (count > 0)
    MFG_CUDA(ctx, cudaMemcpy((void*)p->args.order, order.data(), sizeof(int) * count,
                             cudaMemcpyHostToDevice));
  p->csel = csel;
  if (p->exec) {
    cudaGraphExecDestroy(p->exec);
    p->exec = nullptr;
  }
  return MFG_OK;
}

// CTAs of a GETRF plan's CTA-per-matrix launch (segment 3): at most two per SM (the FMA form's
// blocked kernel: big_cps) and one per scratch slice.
long long getrf_cta_ctas(const mfg_plan* p) {
  const long long slices = (long long)p->ctas * p->warps;
  const long long cps = p->args.fma ? p->big_cps : 2;
  return std::max<long long>(
      1, std::min<long long>({(long long)p->seg_cnt[3], cps * p->ctx->sm_count, slices}));
}

// The FMA form's per-warp copies of a GETRF plan: fma_stride doubles for every warp its launches
// can run (waits for the stream when the buffer grows: it may be in use).  The fallback counter
// is the plan's work-counter slot 8, zeroed with the queues before every launch.
int fma_backup_reserve(mfg_plan* p) {
  if (p->kind != mfg_plan::GETRF || !p->args.fma) return MFG_OK;
  mfg_ctx* ctx = p->ctx;
  const long long stride = std::max<long long>(p->fma_stride, 32);
  size_t bytes = (size_t)stride * sizeof(double) * (size_t)p->ctas * (size_t)p->warps;
  if (p->seg_cnt[3] > 0)   // the blocked CTA kernel: one copy of the largest order per CTA
    bytes = std::max(bytes, (size_t)getrf_cta_ctas(p) * sizeof(double) *
                                (size_t)mfg::getrf_big_backup_doubles(p->cta_nmax));
  if (bytes > p->fbackup.bytes) {
    MFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    MFG_CUDA(ctx, p->fbackup.reserve(bytes));
  }
  p->args.fbackup = (double*)p->fbackup.ptr;
  p->args.fbackup_stride = stride;
  p->args.fcount = p->args.queue + 8;
  return MFG_OK;
}

// Sets a plan's arithmetic form: Cholesky (every overload's kernel that has one) and QR (double)
// take the flag; a GETRF plan in the FMA form also needs size-bucketed tasks (the one-matrix-per-
// warp queue has no FMA kernel) and its copies.
int plan_set_fma(mfg_plan* p, int on);

// Builds the tasks of a GETRF plan for table gsel: the matrices sorted by order, every run of one
// order cut into tasks of 32/G matrices, the tasks grouped by G, and inside each group put in
// "snake" order (largest, smallest, second largest, ...) so that the matrices in flight average
// out.  Uploads order / task_first / task_gc.
int getrf_build_tasks(mfg_plan* p, int gsel) {
  mfg_ctx* ctx = p->ctx;
  const int count = p->count;
  std::vector<int> idx(count);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return p->hn[x] > p->hn[y]; });
  struct Task { int first, cnt, g; };
  std::vector<Task> segs[5];
  // Orders above SMEM_N go to whole CTAs (segment 3) when there are too few of them to give every
  // SM eight warps (same bits either way).  The FMA form, whose bits depend on the schedule, sends
  // orders above BIG_FMA_MIN_N to its blocked CTA kernel whatever the count, so that host-buffer
  // chunks and device calls agree (the blocked kernel beats 32-lane warp tasks from about there,
  // 4 right-hand sides: 56.6 against 64.7 ms for 12,288 matrices of order 160, 62.6 against
  // 62.5 ms for 14,336 of order 152, 63.9 against 53.8 ms for 16,384 of order 136).
  // MFG_LU_CTA = 0 / 1 forces the warp / CTA form.
  constexpr int BIG_FMA_MIN_N = 152;
  long long big = 0;
  for (int i = 0; i < count; i++) big += p->hn[i] > mfg::SMEM_N ? 1 : 0;
  const int cta_env = env_int("MFG_LU_CTA", -1);
  const bool cta = cta_env >= 0 ? cta_env == 1 : big < 8LL * ctx->sm_count;
  const int cta_from = cta_env == 1 ? mfg::SMEM_N
                       : cta_env == 0 ? INT_MAX
                       : p->args.fma  ? BIG_FMA_MIN_N
                       : cta          ? mfg::SMEM_N
                                      : INT_MAX;
  for (int i = 0; i < count;) {
    int j = i;
    while (j < count && p->hn[idx[j]] == p->hn[idx[i]]) j++;
    const int nn = p->hn[idx[i]];
    if (nn > cta_from) {
      for (int k = i; k < j; k++) segs[3].push_back({k, 1, 0});
      i = j;
      continue;
    }
    if (p->blk_lo > 0 && nn >= p->blk_lo && nn <= mfg::SMEM_N) {
      for (int k = i; k < j; k++) segs[4].push_back({k, 1, 0});
      i = j;
      continue;
    }
    const int g = lu_lanes(gsel, nn);
    const int per = 32 / g;
    const int sg = g == 32 ? 0 : g == 16 ? 1 : 2;
    for (int k = i; k < j; k += per) segs[sg].push_back({k, std::min(per, j - k), g});
    i = j;
  }
  p->cta_nmax = 0;
  for (const Task& t : segs[3]) p->cta_nmax = std::max(p->cta_nmax, p->hn[idx[t.first]]);
  p->blk_nmax = 0;
  for (const Task& t : segs[4]) p->blk_nmax = std::max(p->blk_nmax, p->hn[idx[t.first]]);
  // The FMA form's copies: per warp, 32/G matrices of the bucket's largest order.
  p->fma_stride = 0;
  for (int sg = 0; sg < 3; sg++) {
    long long nm = 0;
    for (const Task& t : segs[sg]) nm = std::max<long long>(nm, p->hn[idx[t.first]]);
    p->fma_stride = std::max(p->fma_stride, (1LL << sg) * nm * nm);   // segment sg: 32 >> sg lanes
  }
  p->fma_stride = (p->fma_stride + 31) / 32 * 32;
  std::vector<int> order, first, gc;
  order.reserve(count);
  for (int sg = 0; sg < 5; sg++) {
    p->seg_off[sg] = (int)first.size();
    p->seg_cnt[sg] = (int)segs[sg].size();
    const auto& v = segs[sg];
    int lo = 0, hi = (int)v.size() - 1;
    while (lo <= hi) {
      for (int side = 0; side < 2 && lo <= hi; side++) {
        const Task& t = side == 0 ? v[lo++] : v[hi--];
        first.push_back((int)order.size());
        gc.push_back(t.g | (t.cnt << 8));
        for (int q = 0; q < t.cnt; q++) order.push_back(idx[t.first + q]);
      }
    }
  }
  p->gsel = gsel;
  if (p->args.fma) {
    const int rc = fma_backup_reserve(p);
    if (rc != MFG_OK) return rc;
  }
  if (count > 0) {
    MFG_CUDA(ctx, cudaMemcpy((void*)p->args.order, order.data(), sizeof(int) * count,
                             cudaMemcpyHostToDevice));
    MFG_CUDA(ctx, cudaMemcpy(p->d_task_first, first.data(), sizeof(int) * first.size(),
                             cudaMemcpyHostToDevice));
    MFG_CUDA(ctx, cudaMemcpy(p->d_task_gc, gc.data(), sizeof(int) * gc.size(),
                             cudaMemcpyHostToDevice));
  }
  p->args.task_first = p->d_task_first;
  p->args.task_gc = p->d_task_gc;
  p->args.ntasks = (int)first.size();
  if (p->exec) {
    cudaGraphExecDestroy(p->exec);
    p->exec = nullptr;
  }
  return MFG_OK;
}

// Re-shapes a getrf/potrf plan: warps per CTA (1, 2, 4, 8 or 16), warps per SM, lanes per
// matrix (potrf) and the multiply mode; grows the per-warp scratch when the new shape keeps more
// matrices in flight, and drops the cached graph.
int plan_reshape(mfg_plan* p, int warps, int wps, int group, int mul, int dot_block = 0) {
  mfg_ctx* ctx = p->ctx;
  long long ctas = (long long)ctx->sm_count * wps / warps;
  const long long need = ((long long)p->count + warps - 1) / warps;
  if (ctas > need) ctas = need;
  if (ctas < 1) ctas = 1;
  if (p->kind == mfg_plan::GETRF && group != p->gsel && group >= -1 && group <= 6) {
    if (group >= 0) {
      const int rc = getrf_build_tasks(p, group);
      if (rc != MFG_OK) return rc;
    } else {
      p->gsel = -1;
      p->args.task_first = nullptr;
      p->args.task_gc = nullptr;
      p->args.ntasks = 0;
    }
  }
  if (p->kind == mfg_plan::POTRF) {
    const int csel = group < 0 ? -group : 0;
    if (csel != p->csel) {
      const int rc = potrf_build_segments(p, csel);
      if (rc != MFG_OK) return rc;
    }
    if (group < 0) group = 32;
  }
  const int g = p->kind == mfg_plan::POTRF ? group : 32;
  const int smem_n = p->kind == mfg_plan::POTRF ? 4 * g : mfg::SMEM_N;
  long long stride = 0;
  if (p->max_n > smem_n) {
    stride = (mfg::warp_scratch_doubles(p->max_n) + 31) / 32 * 32;
    MFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // the scratch may be in use
    MFG_CUDA(ctx, p->scratch.reserve((size_t)stride * sizeof(double) * (size_t)ctas * warps *
                                     (size_t)(32 / g)));
  }
  p->warps = warps;
  p->ctas = (int)ctas;
  p->args.gscratch = (double*)p->scratch.ptr;
  p->args.gscratch_stride = stride;
  p->dstride = stride;
  p->elem = 0;
  if (p->args.gsolve) {
    MFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    MFG_CUDA(ctx, p->gsolve.reserve((size_t)gsolve_stride(p->kind) * sizeof(double) *
                                    (size_t)ctas * warps));
    p->args.gsolve = (double*)p->gsolve.ptr;
  }
  p->args.group = g;
  p->args.hw_mul = mul;
  if (dot_block > 0) p->args.dot_block = dot_block;
  if (p->exec) {
    cudaGraphExecDestroy(p->exec);
    p->exec = nullptr;
  }
  return fma_backup_reserve(p);
}

int plan_set_fma(mfg_plan* p, int on) {
  const bool changed = p->args.fma != (on ? 1 : 0);
  p->args.fma = on ? 1 : 0;
  p->qd.fma = p->args.fma;
  if (p->kind == mfg_plan::GETRF && (on || changed)) {
    // Tasks are needed in the FMA form, and the segment of orders above SMEM_N depends on the form.
    if (p->gsel < 0 || (changed && p->max_n > mfg::SMEM_N)) {
      const int rc = getrf_build_tasks(p, p->gsel < 0 ? 0 : p->gsel);
      if (rc != MFG_OK) return rc;
    }
    const int rc = fma_backup_reserve(p);
    if (rc != MFG_OK) return rc;
  }
  if (p->exec) {
    cudaGraphExecDestroy(p->exec);
    p->exec = nullptr;
  }
  return MFG_OK;
}

// Tuning-table key: plan kind, bucket of the largest order (16, 32, 64, 128, 256, more) and
// the batch size's power of two.
long long tune_key(int kind, int max_n, int count) {
  const int nb = max_n <= 16 ? 0 : max_n <= 32 ? 1 : max_n <= 64 ? 2 : max_n <= 128 ? 3
               : max_n <= 256 ? 4 : 5;
  int cb = 0;
  while (cb < 40 && (1LL << (cb + 1)) <= count) cb++;
  return (long long)kind * 10000 + nb * 100 + cb;
}

// A shape forced through the environment wins over the tuning table.
bool tune_env_override() {
  const char* names[] = {"MFG_WARPS_PER_CTA", "MFG_WARPS_PER_SM", "MFG_HW_MUL", "MFG_CHOL_GROUP",
                         "MFG_LU_GROUPS", "MFG_CHOL_TABLE"};
  for (const char* n : names) {
    const char* v = std::getenv(n);
    if (v && *v) return true;
  }
  return false;
}

// Dynamic shared memory of one resident-form CTA: an equal share of the SM's shared memory for
// blk_cps CTAs (less 2 KB each for the CTA's reservation and static variables), at least what the
// segment's largest order needs without its copy, at most what the kernel may be given.
int blk_smem_bytes(const mfg_plan* p) {
  const int cps = std::max(1, p->blk_cps);
  long long b = (long long)p->ctx->smem_per_sm / cps - 2048;
  b = b / 128 * 128;
  const long long floor_b =
      (long long)sizeof(double) * mfg::getrf_blk_smem_doubles(p->blk_nmax, p->nrhs, p->blk_w, false);
  if (b < floor_b) b = floor_b;
  if (b > mfg::getrf_blk_smem_max()) b = mfg::getrf_blk_smem_max();
  return (int)b;
}

int plan_launch(mfg_plan* p, cudaStream_t s) {
  mfg_ctx* ctx = p->ctx;
  int* queue = p->kind == mfg_plan::GEQRF  ? p->qd.queue
               : p->kind == mfg_plan::GEVD ? p->gv.queue
                                           : p->args.queue;
  // The task kernels stage their solves in the plan's gsolve slices (MFG_GSOLVE=0 plans have none
  // and keep the one-matrix-per-warp kernel).
  const bool tasks = p->kind == mfg_plan::GETRF && p->elem == 0 && p->gsel >= 0 &&
                     !p->args.dcount && (p->nrhs == 0 || p->args.gsolve != nullptr);
  const bool csegs = p->kind == mfg_plan::POTRF && p->elem == 0 && p->csel > 0;
  cudaError_t e = cudaMemsetAsync(queue, 0, (tasks || csegs ? 9 : 1) * sizeof(int), s);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemsetAsync(queue)");
  if (p->count == 0) return MFG_OK;
  if (tasks) {
    // One launch per lanes-per-matrix bucket (32, then 16, then 8 lanes), each persistent over
    // its own task queue.
    for (int sg = 0; sg < 5; sg++) {
      if (p->seg_cnt[sg] == 0) continue;
      BatchArgs a = p->args;
      a.task_first = p->d_task_first + p->seg_off[sg];
      a.task_gc = p->d_task_gc + p->seg_off[sg];
      a.ntasks = p->seg_cnt[sg];
      a.queue = p->args.queue + 1 + sg;
      if (sg == 4) {
        // Resident form: blk_cps CTAs of blk_w warps per SM, each with an equal share of the
        // SM's shared memory (at least what a matrix of the segment needs without its copy).
        int ctas = (int)std::min<long long>(a.ntasks, (long long)ctx->sm_count * p->blk_cps);
        if (ctas < 1) ctas = 1;
        e = mfg::launch_getrf_blk(a, ctas, p->blk_w, blk_smem_bytes(p), s);
      } else if (sg == 3) {
        // One matrix per CTA: the CTA kernel counts its work items in `count`; the FMA form
        // runs the blocked kernel.
        a.count = a.ntasks;
        const int ctas = (int)getrf_cta_ctas(p);
        e = p->args.fma ? mfg::launch_getrf_big_fma(a, ctas, p->cta_nmax, p->big_cps,
                                                    p->big_mma, s)
                        : mfg::launch_getrf_cta(a, ctas, p->cta_nmax, s);
      } else {
        const long long need = ((long long)a.ntasks + p->warps - 1) / p->warps;
        const int ctas = (int)std::max<long long>(1, std::min<long long>(p->ctas, need));
        a.minb = p->ctas / std::max(1, ctx->sm_count);
        e = p->args.fma ? mfg::launch_getrf_tasks_fma(a, ctas, p->warps, 32 >> sg, s)
                        : mfg::launch_getrf_tasks(a, ctas, p->warps, 32 >> sg, s);
      }
      if (e != cudaSuccess) return cuda_fail(ctx, e, "batched LU launch");
    }
    return MFG_OK;
  }
  if (p->kind == mfg_plan::GETRF && p->elem == 1)
    e = mfg::launch_sgetrf_batched(p->args, p->ctas, p->warps, s);
  else if (p->kind == mfg_plan::GETRF && p->elem == 2)
    e = mfg::launch_zgetrf_batched(p->args, p->ctas, p->warps, s);
  else if (p->kind == mfg_plan::GETRF)
    e = mfg::launch_getrf_batched(p->args, p->ctas, p->warps, s);
  else if (p->kind == mfg_plan::GETRI && p->elem != 0)
    e = mfg::launch_getri_batched_t(p->args, p->elem, p->ctas, s);
  else if (p->kind == mfg_plan::GETRI)
    e = mfg::launch_getri_batched(p->args, p->ctas, s);
  else if (p->kind == mfg_plan::GEVD && p->elem != 0)
    e = mfg::launch_gevd_front_batched_t(p->gv, p->elem, p->ctas_t, s);
  else if (p->kind == mfg_plan::GEVD)
    e = mfg::launch_gevd_front_batched(p->gv, p->ctas, s);
  else if (p->kind == mfg_plan::POTRF && p->elem == 1)
    e = mfg::launch_spotrf_batched(p->args, p->ctas, p->warps, s);
  else if (p->kind == mfg_plan::POTRF && p->elem == 2)
    e = mfg::launch_zpotrf_batched(p->args, p->ctas, p->warps, s);
  else if (csegs) {
    // One launch per lanes-per-matrix bucket, each over its segment of the queue.
    for (int sg = 0; sg < 4 && e == cudaSuccess; sg++) {
      if (p->seg_cnt[sg] == 0) continue;
      BatchArgs a = p->args;
      a.order = p->args.order + p->seg_off[sg];
      a.count = p->seg_cnt[sg];
      a.group = 32 >> sg;
      a.queue = p->args.queue + 1 + sg;
      const long long per = (long long)p->warps * (32 / a.group);
      const long long need = ((long long)a.count + per - 1) / per;
      const int ctas = (int)std::max<long long>(1, std::min<long long>(p->ctas, need));
      e = mfg::launch_potrf_batched(a, ctas, p->warps, s);
    }
  } else if (p->kind == mfg_plan::POTRF)
    e = mfg::launch_potrf_batched(p->args, p->ctas, p->warps, s);
  else if (p->qr_float == 2)
    e = mfg::launch_zqr_batched(p->qz, p->ctas, p->warps, s);
  else if (p->qr_float)
    e = mfg::launch_qr_batched<float>(p->qs, p->ctas, p->warps, s);
  else
    e = mfg::launch_qr_batched<double>(p->qd, p->ctas, p->warps, s);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batched kernel launch");
  return MFG_OK;
}

// Replays the plan's CUDA graph, capturing it first when the data pointers or the stream changed.
// The legacy default stream cannot be captured; on it the plan launches directly.
// GETRF plans add their element type to the key.
int plan_execute(mfg_plan* p, const void* k0, const void* k1, const void* k2, const void* k3,
                 const void* k4) {
  mfg_ctx* ctx = p->ctx;
  cudaStream_t s = ctx->stream;
  if (!ctx->use_graphs || s == nullptr || s == cudaStreamLegacy) return plan_launch(p, s);
  const void* key[7] = {k0, k1, k2, k3, k4, (const void*)s, (const void*)(intptr_t)p->elem};
  bool hit = p->exec != nullptr;
  for (int i = 0; i < 7 && hit; i++) hit = (key[i] == p->key[i]);
  if (!hit) {
    if (p->exec) {
      cudaGraphExecDestroy(p->exec);
      p->exec = nullptr;
    }
    cudaGraph_t g = nullptr;
    MFG_CUDA(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int rc = plan_launch(p, s);
    cudaError_t ee = cudaStreamEndCapture(s, &g);
    if (rc != MFG_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ee != cudaSuccess) return cuda_fail(ctx, ee, "cudaStreamEndCapture");
    ee = cudaGraphInstantiate(&p->exec, g, 0);
    cudaGraphDestroy(g);
    if (ee != cudaSuccess) {
      p->exec = nullptr;
      return cuda_fail(ctx, ee, "cudaGraphInstantiate");
    }
    for (int i = 0; i < 7; i++) p->key[i] = key[i];
  }
  MFG_CUDA(ctx, cudaGraphLaunch(p->exec, s));
  return MFG_OK;
}

// Common plan set-up: validation, longest-first order, descriptor upload, scratch.
int plan_create(mfg_ctx* ctx, mfg_plan** out, mfg_plan::Kind kind, int count, const int* n,
                const int* lda, const int64_t* a_off, const int64_t* piv_off, int nrhs,
                const int64_t* b_off) {
  if (!ctx) return -1;
  if (!out) return fail(ctx, -2, "plan output pointer is null");
  *out = nullptr;
  if (count < 0) return fail(ctx, -3, "count must be >= 0");
  if (count > 0 && !n) return fail(ctx, -4, "n is null");
  for (int i = 0; i < count; i++)
    if (n[i] < 1)
      return fail(ctx, -4, "n[%d] = %d: the order of the matrix must be >= 1", i, n[i]);
  if (lda)
    for (int i = 0; i < count; i++)
      if (lda[i] < n[i])
        return fail(ctx, -5, "lda[%d] = %d < n[%d] = %d", i, lda[i], i, n[i]);
  if (kind == mfg_plan::GETRI)
    for (int i = 0; i < count; i++)
      if (n[i] > mfg::getri_max_n())
        return fail(ctx, -4, "n[%d] = %d: the batched inverse supports orders up to %d", i, n[i],
                    mfg::getri_max_n());
  if (count > 0 && !a_off) return fail(ctx, -6, "a_off is null");
  for (int i = 0; i < count; i++)
    if (a_off[i] < 0) return fail(ctx, -6, "a_off[%d] < 0", i);
  int argi = 7;
  if (kind == mfg_plan::GETRF || kind == mfg_plan::GETRI) {
    if (count > 0 && !piv_off) return fail(ctx, -7, "piv_off is null");
    for (int i = 0; i < count; i++)
      if (piv_off[i] < 0) return fail(ctx, -7, "piv_off[%d] < 0", i);
    argi = 8;
  }
  if (nrhs < 0) return fail(ctx, -argi, "nrhs must be >= 0");
  if (nrhs > 0 && count > 0 && !b_off) return fail(ctx, -(argi + 1), "b_off is null");
  if (nrhs > 0)
    for (int i = 0; i < count; i++)
      if (b_off[i] < 0) return fail(ctx, -(argi + 1), "b_off[%d] < 0", i);

  mfg_plan* p = new mfg_plan();
  p->kind = kind;
  p->ctx = ctx;
  p->count = count;
  p->nrhs = nrhs;
  std::vector<int> order = snake_order(count, n);
  int max_n = 0;
  for (int i = 0; i < count; i++) max_n = std::max(max_n, n[i]);
  p->max_n = max_n;

  const size_t ints = (size_t)count;
  const size_t bytes_i = ((ints * sizeof(int) + 255) / 256) * 256;
  const size_t bytes_l = ((ints * sizeof(long long) + 255) / 256) * 256;
  const size_t total = 5 * bytes_i + 3 * bytes_l + 256;
  cudaError_t e = p->meta.reserve(total);
  if (e != cudaSuccess) {
    delete p;
    return cuda_fail(ctx, e, "cudaMalloc(plan descriptors)");
  }
  char* base = (char*)p->meta.ptr;
  int* d_order = (int*)base;
  int* d_n = (int*)(base + bytes_i);
  int* d_lda = (int*)(base + 2 * bytes_i);
  long long* d_aoff = (long long*)(base + 3 * bytes_i);
  long long* d_pivoff = (long long*)(base + 3 * bytes_i + bytes_l);
  long long* d_boff = (long long*)(base + 3 * bytes_i + 2 * bytes_l);
  int* d_queue = (int*)(base + 3 * bytes_i + 3 * bytes_l);   // work counters (one per bucket)
  p->d_task_first = (int*)(base + 3 * bytes_i + 3 * bytes_l + 256);
  p->d_task_gc = (int*)(base + 4 * bytes_i + 3 * bytes_l + 256);

  std::vector<char> host(total, 0);
  std::memcpy(host.data(), order.data(), ints * sizeof(int));
  std::memcpy(host.data() + bytes_i, n, ints * sizeof(int));
  if (lda)
    std::memcpy(host.data() + 2 * bytes_i, lda, ints * sizeof(int));
  else
    std::memcpy(host.data() + 2 * bytes_i, n, ints * sizeof(int));
  for (size_t i = 0; i < ints; i++) {
    ((long long*)(host.data() + 3 * bytes_i))[i] = a_off[i];
    ((long long*)(host.data() + 3 * bytes_i + bytes_l))[i] =
        (kind == mfg_plan::GETRF || kind == mfg_plan::GETRI) ? piv_off[i] : 0;
    ((long long*)(host.data() + 3 * bytes_i + 2 * bytes_l))[i] = nrhs > 0 ? b_off[i] : 0;
  }
  e = cudaMemcpy(p->meta.ptr, host.data(), total, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    delete p;
    return cuda_fail(ctx, e, "cudaMemcpy(plan descriptors)");
  }
  choose_shape(p);
  // Cholesky runs G lanes per matrix (32/G matrices per warp); small orders use small groups so
  // the per-column square root and the serial solve steps are shared by several matrices.
  int group = 32;
  if (kind == mfg_plan::POTRF) {
    group = env_int("MFG_CHOL_GROUP", max_n <= 16 ? 4 : max_n <= 32 ? 8 : max_n <= 64 ? 16 : 32);
    if (group != 4 && group != 8 && group != 16 && group != 32) group = 32;
  }
  const int smem_n = kind == mfg_plan::POTRF ? 4 * group : mfg::SMEM_N;
  long long stride = 0;
  if (kind == mfg_plan::GETRI) {
    // The inverse keeps a packed copy of the factors per warp (A is overwritten column by column).
    stride = mfg::getri_scratch_doubles(max_n);
    const size_t sbytes = (size_t)stride * sizeof(double) * (size_t)p->ctas * p->warps;
    e = p->scratch.reserve(sbytes);
    if (e != cudaSuccess) {
      delete p;
      return cuda_fail(ctx, e, "cudaMalloc(plan scratch)");
    }
  } else if (max_n > smem_n) {
    stride = (mfg::warp_scratch_doubles(max_n) + 31) / 32 * 32;
    const size_t sbytes = (size_t)stride * sizeof(double) * (size_t)p->ctas * p->warps *
                          (size_t)(32 / group);
    e = p->scratch.reserve(sbytes);
    if (e != cudaSuccess) {
      delete p;
      return cuda_fail(ctx, e, "cudaMalloc(plan scratch)");
    }
  }
  BatchArgs& a = p->args;
  a.order = d_order;
  a.n = d_n;
  a.lda = d_lda;
  a.a_off = d_aoff;
  a.piv_off = d_pivoff;
  a.b_off = d_boff;
  a.count = count;
  a.nrhs = nrhs;
  a.queue = d_queue;
  a.gscratch = (double*)p->scratch.ptr;
  a.gscratch_stride = stride;
  p->dstride = stride;
  // LuInverse's per-lane solves multiply on the FP64 pipe by default: measured faster there than
  // the integer-pipe product, whose long dependency chains one or two warps per scheduler cannot
  // hide.
  a.hw_mul = kind == mfg_plan::GETRI ? env_int("MFG_INV_HW_MUL", 1) : env_int("MFG_HW_MUL", 0);
  // Split dots (whole-warp groups with integer-pipe products): 54.8 vs 56.6 ms on the
  // 100,000-matrix Cholesky batch.
  a.split = kind == mfg_plan::POTRF ? env_int("MFG_CHOL_SPLIT", 1) : 0;
  a.gsolve = nullptr;
  if ((kind == mfg_plan::GETRF || kind == mfg_plan::POTRF) && nrhs > 0 &&
      env_int("MFG_GSOLVE", 1)) {
    e = p->gsolve.reserve((size_t)gsolve_stride(kind) * sizeof(double) * (size_t)p->ctas *
                          p->warps);
    if (e != cudaSuccess) {
      delete p;
      return cuda_fail(ctx, e, "cudaMalloc(plan solve staging)");
    }
    a.gsolve = (double*)p->gsolve.ptr;
  }
  a.group = group;
  a.dot_block = env_int("MFG_DOT_BLOCK", 4);
  p->hn.assign(n, n + count);
  p->hlda.resize(count);
  p->haoff.assign(a_off, a_off + count);
  p->hpivoff.assign(count, 0);
  p->hboff.assign(count, 0);
  for (int i = 0; i < count; i++) {
    p->hlda[i] = lda ? lda[i] : n[i];
    if (kind == mfg_plan::GETRF || kind == mfg_plan::GETRI) p->hpivoff[i] = piv_off[i];
    if (nrhs > 0) p->hboff[i] = b_off[i];
  }
  if (kind == mfg_plan::GETRF) {
    // Size-bucketed tasks (lanes per matrix by order); MFG_LU_GROUPS picks the table, -1 the
    // one-matrix-per-warp queue.
    const int gsel = env_int("MFG_LU_GROUPS", 2);
    // Resident form: MFG_LU_BLK = "lo,w,cps" (smallest order, warps per CTA, CTAs per SM).
    if (const char* v = std::getenv("MFG_LU_BLK")) {
      int lo = 0, w = 4, cps = 2;
      if (std::sscanf(v, "%d,%d,%d", &lo, &w, &cps) >= 1) {
        p->blk_lo = lo;
        p->blk_w = (w == 2 || w == 4 || w == 8) ? w : 4;
        p->blk_cps = std::max(1, std::min(cps, 16));
      }
    }
    // The FMA form's blocked kernel for orders above SMEM_N: CTAs per SM (2 or 3).
    p->big_cps = env_int("MFG_LU_BIG_CPS", 3) == 2 ? 2 : 3;
    p->big_mma = env_int("MFG_LU_BIG_MMA", 0) != 0;
    if (gsel >= 0) {
      const int rc = getrf_build_tasks(p, gsel);
      if (rc != MFG_OK) {
        delete p;
        return rc;
      }
    }
  }
  if (kind == mfg_plan::POTRF) {
    const int csel = env_int("MFG_CHOL_TABLE", 0);
    if (csel == 1 || csel == 2) {
      const int rc = potrf_build_segments(p, csel);
      if (rc != MFG_OK) {
        delete p;
        return rc;
      }
    }
  }
  if (kind == mfg_plan::GETRF || kind == mfg_plan::POTRF) {
    if (!tune_env_override()) {
      auto it = ctx->tune.find(tune_key((int)kind, max_n, count));
      if (it != ctx->tune.end()) {
        const auto& c = it->second;
        const int rc = plan_reshape(p, c[0], c[1], c[2], c[3], c[4]);
        if (rc != MFG_OK) {
          delete p;
          return rc;
        }
      }
    }
  }
  *out = p;
  return MFG_OK;
}


// Plan of the batched GEVD front half: pair i is A (order n[i], leading dimension lda[i]) at
// a_off[i], B (ldb[i]) at b_off[i], and C (leading dimension n[i]) at c_off[i].
int plan_create_gevd(mfg_ctx* ctx, mfg_plan** out, int count, const int* n, const int* lda,
                     const int64_t* a_off, const int* ldb, const int64_t* b_off,
                     const int64_t* c_off) {
  if (!ctx) return -1;
  if (!out) return fail(ctx, -2, "plan output pointer is null");
  *out = nullptr;
  if (count < 0) return fail(ctx, -3, "count must be >= 0");
  if (count > 0 && !n) return fail(ctx, -4, "n is null");
  for (int i = 0; i < count; i++) {
    if (n[i] < 1)
      return fail(ctx, -4, "n[%d] = %d: The order of the matrix must be greater than or equal "
                           "to one.", i, n[i]);
    if (n[i] > mfg::gevd_max_n())
      return fail(ctx, -4, "n[%d] = %d: the batched GEVD front half supports orders up to %d", i,
                  n[i], mfg::gevd_max_n());
    if (lda && lda[i] < n[i])
      return fail(ctx, -5, "lda[%d]: The leading dimension must be greater than or equal to the "
                           "order of the matrix.", i);
    if (ldb && ldb[i] < n[i])
      return fail(ctx, -7, "ldb[%d]: The leading dimension must be greater than or equal to the "
                           "order of the matrix.", i);
  }
  if (count > 0 && !a_off) return fail(ctx, -6, "a_off is null");
  if (count > 0 && !b_off) return fail(ctx, -8, "b_off is null");
  if (count > 0 && !c_off) return fail(ctx, -9, "c_off is null");
  for (int i = 0; i < count; i++) {
    if (a_off[i] < 0) return fail(ctx, -6, "a_off[%d] < 0", i);
    if (b_off[i] < 0) return fail(ctx, -8, "b_off[%d] < 0", i);
    if (c_off[i] < 0) return fail(ctx, -9, "c_off[%d] < 0", i);
  }
  mfg_plan* p = new mfg_plan();
  p->kind = mfg_plan::GEVD;
  p->ctx = ctx;
  p->count = count;
  std::vector<int> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return n[x] > n[y]; });
  const size_t ints = (size_t)count;
  const size_t bi = ((ints * sizeof(int) + 255) / 256) * 256;
  const size_t bl = ((ints * sizeof(long long) + 255) / 256) * 256;
  const size_t total = 4 * bi + 3 * bl + 256;
  cudaError_t e = p->meta.reserve(total);
  if (e != cudaSuccess) {
    delete p;
    return cuda_fail(ctx, e, "cudaMalloc(plan descriptors)");
  }
  std::vector<char> host(total, 0);
  std::memcpy(host.data(), order.data(), ints * sizeof(int));
  std::memcpy(host.data() + bi, n, ints * sizeof(int));
  std::memcpy(host.data() + 2 * bi, lda ? lda : n, ints * sizeof(int));
  std::memcpy(host.data() + 3 * bi, ldb ? ldb : n, ints * sizeof(int));
  for (size_t i = 0; i < ints; i++) {
    ((long long*)(host.data() + 4 * bi))[i] = a_off[i];
    ((long long*)(host.data() + 4 * bi + bl))[i] = b_off[i];
    ((long long*)(host.data() + 4 * bi + 2 * bl))[i] = c_off[i];
  }
  e = cudaMemcpy(p->meta.ptr, host.data(), total, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    delete p;
    return cuda_fail(ctx, e, "cudaMemcpy(plan descriptors)");
  }
  // Same shape as the gradient kernel: one CTA of six warps per SM (shared-memory bound).
  p->warps = mfg::grad_warps_per_cta();
  long long ctas = (long long)ctx->sm_count * mfg::grad_ctas_per_sm();
  ctas = std::min<long long>(ctas, ((long long)count + p->warps - 1) / p->warps);
  p->ctas = (int)std::max<long long>(1, ctas);
  char* base = (char*)p->meta.ptr;
  mfg::GevdArgs& g = p->gv;
  g.order = (const int*)base;
  g.n = (const int*)(base + bi);
  g.lda = (const int*)(base + 2 * bi);
  g.ldb = (const int*)(base + 3 * bi);
  g.a_off = (const long long*)(base + 4 * bi);
  g.b_off = (const long long*)(base + 4 * bi + bl);
  g.c_off = (const long long*)(base + 4 * bi + 2 * bl);
  g.count = count;
  g.queue = (int*)(base + 4 * bi + 3 * bl);
  p->hn.assign(n, n + count);
  p->hlda.resize(count);
  p->hldb.resize(count);
  for (int i = 0; i < count; i++) {
    p->hlda[i] = lda ? lda[i] : n[i];
    p->hldb[i] = ldb ? ldb[i] : n[i];
  }
  p->haoff.assign(a_off, a_off + count);
  p->hboff.assign(b_off, b_off + count);
  p->hcoff.assign(c_off, c_off + count);
  *out = p;
  return MFG_OK;
}

int max_n_of(const int* n, int count) {
  int mx = 0;
  for (int i = 0; i < count; i++) mx = std::max(mx, n[i]);
  return mx;
}

// Tuning-table key of a QR plan: the buckets of its largest n (16, 32, 64, more) and largest m
// (128, 256, 512, more) and the batch size's power of two.
long long qr_tune_key(int max_n, int max_m, int count) {
  const int nb = max_n <= 16 ? 0 : max_n <= 32 ? 1 : max_n <= 64 ? 2 : 3;
  const int mb = max_m <= 128 ? 0 : max_m <= 256 ? 1 : max_m <= 512 ? 2 : 3;
  int cb = 0;
  while (cb < 40 && (1LL << (cb + 1)) <= count) cb++;
  return (long long)mfg_plan::GEQRF * 10000 + nb * 1000 + mb * 100 + cb;
}

// Re-shapes a QR plan: lanes per matrix (4, 8, 16 or 32, both real overloads) and warps per SM;
// picks the matching queue order, grows the coefficient scratch, drops the cached graph.
int qr_reshape(mfg_plan* p, int group, int wps) {
  mfg_ctx* ctx = p->ctx;
  if (group != 4 && group != 8 && group != 16 && group != 32) return MFG_OK;
  const int warps = group == 32 ? env_int("MFG_WARPS_PER_CTA", 4) : 4;
  long long ctas = (long long)ctx->sm_count * wps / warps;
  const long long per = group == 32 ? 1 : 32 / group;
  const long long need = ((long long)p->count + warps * per - 1) / (warps * per);
  if (ctas > need) ctas = need;
  if (ctas < 1) ctas = 1;
  long long stride = 0;
  if (p->qr_coef_need > mfg::qr_smem_coefs(group)) {
    stride = (p->qr_coef_need + 31) / 32 * 32;
    MFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));   // the scratch may be in use
    MFG_CUDA(ctx, p->scratch.reserve((size_t)stride * sizeof(double) * (size_t)ctas * warps *
                                     (size_t)(32 / group)));
  }
  p->warps = warps;
  p->ctas = (int)ctas;
  p->qd.group = p->qs.group = group;
  p->qd.order = p->qs.order = group < 32 ? p->qr_order_grouped : p->qr_order_work;
  p->qd.gscratch_stride = p->qs.gscratch_stride = stride;
  p->qd.gscratch = (double*)p->scratch.ptr;
  p->qs.gscratch = (float*)p->scratch.ptr;
  if (p->exec) {
    cudaGraphExecDestroy(p->exec);
    p->exec = nullptr;
  }
  return MFG_OK;
}

int plan_create_qr(mfg_ctx* ctx, mfg_plan** out, int count, const int* m, const int* n,
                   const int* lda, const int64_t* a_off, const int64_t* rdiag_off, int nrhs,
                   const int64_t* b_off) {
  if (!ctx) return -1;
  if (!out) return fail(ctx, -2, "plan output pointer is null");
  *out = nullptr;
  if (count < 0) return fail(ctx, -3, "count must be >= 0");
  if (count > 0 && (!m || !n)) return fail(ctx, !m ? -4 : -5, "m or n is null");
  for (int i = 0; i < count; i++) {
    if (m[i] < 1) return fail(ctx, -4, "m[%d] = %d: must be >= 1", i, m[i]);
    if (n[i] < 1) return fail(ctx, -5, "n[%d] = %d: must be >= 1", i, n[i]);
    if (n[i] > m[i])
      return fail(ctx, -5,
                  "The number of rows must be greater than or equal to the number of columns.");
  }
  if (lda)
    for (int i = 0; i < count; i++)
      if (lda[i] < m[i]) return fail(ctx, -6, "lda[%d] = %d < m[%d] = %d", i, lda[i], i, m[i]);
  if (count > 0 && !a_off) return fail(ctx, -7, "a_off is null");
  if (count > 0 && !rdiag_off) return fail(ctx, -8, "rdiag_off is null");
  if (nrhs < 0) return fail(ctx, -9, "nrhs must be >= 0");
  if (nrhs > 0 && count > 0 && !b_off) return fail(ctx, -10, "b_off is null");
  for (int i = 0; i < count; i++) {
    if (a_off[i] < 0) return fail(ctx, -7, "a_off[%d] < 0", i);
    if (rdiag_off[i] < 0) return fail(ctx, -8, "rdiag_off[%d] < 0", i);
    if (nrhs > 0 && b_off[i] < 0) return fail(ctx, -10, "b_off[%d] < 0", i);
  }
  mfg_plan* p = new mfg_plan();
  p->kind = mfg_plan::GEQRF;
  p->ctx = ctx;
  p->count = count;
  p->nrhs = nrhs;
  std::vector<int> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::vector<double> work(count);
  int max_cols = 0;
  for (int i = 0; i < count; i++) {
    work[i] = 2.0 * m[i] * (double)n[i] * n[i] - 2.0 / 3.0 * (double)n[i] * n[i] * n[i];
    max_cols = std::max(max_cols, n[i] + nrhs);
  }
  // Lanes per matrix: 8 for both overloads (four matrices per warp).  On the 50,000-matrix
  // batch (m 64..512, n 16..64) the double kernel measured 194 / 175 / 166 / 263 ms with 32 / 16
  // / 8 / 4 lanes and the float one 180 / 154 / 210 ms with 16 / 8 / 4: the column dots (one per
  // lane, n - k of them) fill small groups better, and four times the matrices in flight hide
  // more of the trailing-matrix streams; 4 lanes leave too few lanes for the rank-1 updates.
  // MFG_QR_GROUP = 32, 16, 8 or 4 overrides both.
  int group_d = 8, group_s = 8;
  const int genv = env_int("MFG_QR_GROUP", 0);
  if (genv == 4 || genv == 8 || genv == 16 || genv == 32) group_d = group_s = genv;
  const int group = std::min(group_d, group_s);
  // One queue order per group size: a whole warp per matrix takes them longest first (by work);
  // groups of fewer lanes take decreasing n, then decreasing m, so the matrices that share a
  // warp have the same n and similar m and run in lockstep.
  std::vector<int> order_g = order;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return work[x] > work[y]; });
  std::stable_sort(order_g.begin(), order_g.end(),
                   [&](int x, int y) { return n[x] != n[y] ? n[x] > n[y] : m[x] > m[y]; });
  const size_t ints = (size_t)count;
  const size_t bi = ((ints * sizeof(int) + 255) / 256) * 256;
  const size_t bl = ((ints * sizeof(long long) + 255) / 256) * 256;
  const size_t total = 5 * bi + 3 * bl + 256;
  cudaError_t e = p->meta.reserve(total);
  if (e != cudaSuccess) {
    delete p;
    return cuda_fail(ctx, e, "cudaMalloc(plan descriptors)");
  }
  std::vector<char> host(total, 0);
  std::memcpy(host.data(), order.data(), ints * sizeof(int));
  std::memcpy(host.data() + bi, m, ints * sizeof(int));
  std::memcpy(host.data() + 2 * bi, n, ints * sizeof(int));
  std::memcpy(host.data() + 3 * bi, lda ? lda : m, ints * sizeof(int));
  for (size_t i = 0; i < ints; i++) {
    ((long long*)(host.data() + 4 * bi))[i] = a_off[i];
    ((long long*)(host.data() + 4 * bi + bl))[i] = rdiag_off[i];
    ((long long*)(host.data() + 4 * bi + 2 * bl))[i] = nrhs > 0 ? b_off[i] : 0;
  }
  std::memcpy(host.data() + 4 * bi + 3 * bl + 256, order_g.data(), ints * sizeof(int));
  e = cudaMemcpy(p->meta.ptr, host.data(), total, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    delete p;
    return cuda_fail(ctx, e, "cudaMemcpy(plan descriptors)");
  }
  choose_shape(p, group == 32 ? 0 : 4);
  // The fused variant (one pass per trailing column and step; default, measured 9 % faster in
  // FP64 and 13 % in FP32 on the 50,000-matrix batch) keeps two steps' coefficients.
  const int fused = env_int("MFG_QR_FUSED", 1) ? 1 : 0;
  const int coef_need = fused ? 2 * max_cols : max_cols;
  long long stride = 0;
  if (coef_need > mfg::qr_smem_coefs(group)) {
    stride = (coef_need + 31) / 32 * 32;
    e = p->scratch.reserve((size_t)stride * sizeof(double) * (size_t)p->ctas * p->warps *
                           (size_t)(32 / group));
    if (e != cudaSuccess) {
      delete p;
      return cuda_fail(ctx, e, "cudaMalloc(plan scratch)");
    }
  }
  char* base = (char*)p->meta.ptr;
  auto fill = [&](auto& q) {
    q.order = (const int*)base;
    q.m = (const int*)(base + bi);
    q.n = (const int*)(base + 2 * bi);
    q.lda = (const int*)(base + 3 * bi);
    q.a_off = (const long long*)(base + 4 * bi);
    q.rdiag_off = (const long long*)(base + 4 * bi + bl);
    q.b_off = (const long long*)(base + 4 * bi + 2 * bl);
    q.count = count;
    q.nrhs = nrhs;
    q.queue = (int*)(base + 4 * bi + 3 * bl);
    q.gscratch_stride = stride;
  };
  fill(p->qd);
  fill(p->qs);
  fill(p->qz);
  p->qd.fused = p->qs.fused = fused;
  p->qz.fused = 0;
  p->qd.group = group_d;
  p->qs.group = group_s;
  p->qz.group = 32;
  p->qz.gscratch_stride = 0;
  p->qr_max_cols = max_cols;
  const int* order_grouped = (const int*)(base + 4 * bi + 3 * bl + 256);
  p->qr_order_work = (const int*)base;
  p->qr_order_grouped = order_grouped;
  p->qr_coef_need = coef_need;
  if (group_d < 32) p->qd.order = order_grouped;
  if (group_s < 32) p->qs.order = order_grouped;
  p->qd.gscratch = (double*)p->scratch.ptr;
  p->qs.gscratch = (float*)p->scratch.ptr;
  p->hm.assign(m, m + count);
  p->hn.assign(n, n + count);
  p->hlda.resize(count);
  p->haoff.assign(a_off, a_off + count);
  p->hpivoff.assign(rdiag_off, rdiag_off + count);
  p->hboff.assign(count, 0);
  for (int i = 0; i < count; i++) {
    p->hlda[i] = lda ? lda[i] : m[i];
    if (nrhs > 0) p->hboff[i] = b_off[i];
  }
  if (genv == 0 && !tune_env_override()) {
    int max_m = 0;
    for (int i = 0; i < count; i++) max_m = std::max(max_m, m[i]);
    auto it = ctx->tune.find(qr_tune_key(max_n_of(n, count), max_m, count));
    if (it != ctx->tune.end()) {
      const int rc = qr_reshape(p, it->second[2], it->second[1]);
      if (rc != MFG_OK) {
        delete p;
        return rc;
      }
    }
  }
  *out = p;
  return MFG_OK;
}

// Single-matrix staging: device workspace carve-up helper.
struct Carve {
  char* base;
  size_t off = 0;
  explicit Carve(void* b) : base((char*)b) {}
  template <typename T>
  T* take(size_t count) {
    T* r = (T*)(base + off);
    off += ((count * sizeof(T) + 255) / 256) * 256;
    return r;
  }
  static size_t bytes_for(size_t count, size_t elem) { return ((count * elem + 255) / 256) * 256; }
  size_t used() const { return off; }
};

}  // namespace

extern "C" {

MFG_API const char* mfg_version(void) { return kVersion; }

MFG_API int mfg_create(mfg_ctx** ctx) {
  if (!ctx) return -1;
  *ctx = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return MFG_ERR_NO_DEVICE;
  mfg_ctx* c = new mfg_ctx();
  cudaGetDevice(&c->device);
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device);
  cudaDeviceGetAttribute(&c->smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c->device);
  e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return MFG_ERR_NO_DEVICE;
  }
  c->stream = c->own_stream;
  c->use_graphs = env_int("MFG_GRAPHS", 1) != 0;
  e = init_device_attributes(c->device);
  if (e != cudaSuccess) {
    cudaStreamDestroy(c->own_stream);
    delete c;
    return MFG_ERR_NO_DEVICE;
  }
  *ctx = c;
  return MFG_OK;
}

MFG_API int mfg_destroy(mfg_ctx* ctx) {
  if (!ctx) return -1;
  DeviceScope device_scope_(ctx);
  cudaStreamSynchronize(ctx->stream);
  ctx->work.release();
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return MFG_OK;
}

MFG_API int mfg_set_stream(mfg_ctx* ctx, void* stream) {
  DeviceScope device_scope_(ctx);
  if (!ctx) return -1;
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  return MFG_OK;
}

MFG_API int mfg_synchronize(mfg_ctx* ctx) {
  DeviceScope device_scope_(ctx);
  if (!ctx) return -1;
  MFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MFG_OK;
}

MFG_API int mfg_get_device(mfg_ctx* ctx, int* device) {
  if (!ctx) return -1;
  if (!device) return fail(ctx, -2, "device is null");
  *device = ctx->device;
  return MFG_OK;
}

MFG_API const char* mfg_last_error(mfg_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

// ------------------------------------------------------------------------------------------
// Single-matrix drop-ins.

MFG_API int mfg_dgetrf(mfg_ctx* ctx, int m, int n, double* a, int lda, int* piv, int* sign) {
  DeviceScope device_scope_(ctx);
  if (!ctx) return -1;
  // Factorization.Lu argument checks (Factorization.Lu.cs:124-147).
  if (m <= 0) return fail(ctx, -2, "The number of rows must be greater than or equal to one.");
  if (n <= 0) return fail(ctx, -3, "The number of columns must be greater than or equal to one.");
  if (!a) return fail(ctx, -4, "a is null");
  if (lda < m)
    return fail(ctx, -5,
                "The leading dimension must be greater than or equal to the number of rows.");
  if (!piv) return fail(ctx, -6, "piv is null");
  const int big = std::max(m, n);
  const size_t na = span(m, n, lda);
  const size_t need = Carve::bytes_for(na, 8) + Carve::bytes_for(mfg::warp_scratch_doubles(big), 8) +
                      Carve::bytes_for(m, 4) + Carve::bytes_for(2, 4);
  MFG_CUDA(ctx, ctx->work.reserve(need));
  Carve cv(ctx->work.ptr);
  double* d_a = cv.take<double>(na);
  double* d_s = cv.take<double>(mfg::warp_scratch_doubles(big));
  int* d_piv = cv.take<int>(m);
  int* d_out = cv.take<int>(2);
  cudaStream_t s = ctx->stream;
  MFG_CUDA(ctx, cudaMemcpy2DAsync(d_a, (size_t)lda * 8, a, (size_t)lda * 8, (size_t)m * 8, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, mfg::launch_getrf_single(d_a, m, n, lda, d_piv, d_out, d_s, s));
  int out[2];
  MFG_CUDA(ctx, cudaMemcpy2DAsync(a, (size_t)lda * 8, d_a, (size_t)lda * 8, (size_t)m * 8, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaMemcpyAsync(piv, d_piv, sizeof(int) * m, cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaMemcpyAsync(out, d_out, sizeof(out), cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaStreamSynchronize(s));
  if (sign) *sign = out[0];
  return MFG_OK;
}

MFG_API int mfg_dpotrf(mfg_ctx* ctx, int n, double* a, int lda, int* info) {
  DeviceScope device_scope_(ctx);
  if (!ctx) return -1;
  // Factorization.Cholesky argument checks (Factorization.Cholesky.cs:116-129).
  if (n <= 0) return fail(ctx, -2, "The order of the matrix must be greater than or equal to one.");
  if (!a) return fail(ctx, -3, "a is null");
  if (lda < n)
    return fail(ctx, -4,
                "The leading dimension must be greater than or equal to the order of the matrix.");
  const size_t na = span(n, n, lda);
  const size_t need = Carve::bytes_for(na, 8) + Carve::bytes_for(mfg::warp_scratch_doubles(n), 8) +
                      Carve::bytes_for(1, 4);
  MFG_CUDA(ctx, ctx->work.reserve(need));
  Carve cv(ctx->work.ptr);
  double* d_a = cv.take<double>(na);
  double* d_s = cv.take<double>(mfg::warp_scratch_doubles(n));
  int* d_out = cv.take<int>(1);
  cudaStream_t s = ctx->stream;
  MFG_CUDA(ctx, cudaMemcpy2DAsync(d_a, (size_t)lda * 8, a, (size_t)lda * 8, (size_t)n * 8, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, mfg::launch_potrf_single(d_a, n, lda, d_out, d_s, s));
  int out = 0;
  MFG_CUDA(ctx, cudaMemcpy2DAsync(a, (size_t)lda * 8, d_a, (size_t)lda * 8, (size_t)n * 8, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaMemcpyAsync(&out, d_out, sizeof(int), cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaStreamSynchronize(s));
  if (info) *info = out;
  return MFG_OK;
}

MFG_API int mfg_dtrsv(mfg_ctx* ctx, int uplo, int trans, int n, const double* a, int lda,
                      double* x, int incx) {
  DeviceScope device_scope_(ctx);
  if (!ctx) return -1;
  // Blas.SolveTriangular argument checks (Blas.SolveTriangular.cs:164-187, enums :189-241).
  if (n <= 0) return fail(ctx, -4, "The order of the matrix must be greater than or equal to one.");
  if (!a) return fail(ctx, -5, "a is null");
  if (lda < n)
    return fail(ctx, -6,
                "The leading dimension must be greater than or equal to the number of rows.");
  if (!x) return fail(ctx, -7, "x is null");
  if (incx <= 0) return fail(ctx, -8, "The value must be greater than or equal to one.");
  if (uplo != MFG_UPPER && uplo != MFG_LOWER) return fail(ctx, -2, "Invalid enum value.");
  if (trans != MFG_NOTRANS && trans != MFG_TRANS) return fail(ctx, -3, "Invalid enum value.");
  const size_t na = span(n, n, lda);
  const size_t nx = (size_t)(n - 1) * incx + 1;
  const size_t need = Carve::bytes_for(na, 8) + Carve::bytes_for(nx, 8) +
                      Carve::bytes_for(2 * (size_t)(n | 1), 8);
  MFG_CUDA(ctx, ctx->work.reserve(need));
  Carve cv(ctx->work.ptr);
  double* d_a = cv.take<double>(na);
  double* d_x = cv.take<double>(nx);
  double* d_s = cv.take<double>(2 * (size_t)(n | 1));
  cudaStream_t s = ctx->stream;
  MFG_CUDA(ctx, cudaMemcpy2DAsync(d_a, (size_t)lda * 8, a, (size_t)lda * 8, (size_t)n * 8, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaMemcpyAsync(d_x, x, nx * 8, cudaMemcpyDefault, s));
  MFG_CUDA(ctx, mfg::launch_trsv_single(uplo, trans, n, d_a, lda, d_x, incx, d_s, s));
  MFG_CUDA(ctx, cudaMemcpyAsync(x, d_x, nx * 8, cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaStreamSynchronize(s));
  return MFG_OK;
}

MFG_API int mfg_dgemm(mfg_ctx* ctx, int transa, int transb, int m, int n, int k, const double* a,
                      int lda, const double* b, int ldb, double* c, int ldc) {
  DeviceScope device_scope_(ctx);
  if (!ctx) return -1;
  // Blas.MulMatMat argument checks (Blas.MulMatMat.cs:228-304).
  if (m <= 0) return fail(ctx, -4, "The value must be greater than or equal to one.");
  if (n <= 0) return fail(ctx, -5, "The value must be greater than or equal to one.");
  if (k <= 0) return fail(ctx, -6, "The value must be greater than or equal to one.");
  if (!a) return fail(ctx, -7, "a is null");
  if (transa == MFG_NOTRANS) {
    if (lda < m)
      return fail(ctx, -8,
                  "The leading dimension must be greater than or equal to the number of rows.");
  } else if (transa == MFG_TRANS) {
    if (lda < k)
      return fail(ctx, -8,
                  "The leading dimension must be greater than or equal to the number of rows.");
  } else {
    return fail(ctx, -2, "Invalid enum value.");
  }
  if (!b) return fail(ctx, -9, "b is null");
  if (transb == MFG_NOTRANS) {
    if (ldb < k)
      return fail(ctx, -10,
                  "The leading dimension must be greater than or equal to the number of rows.");
  } else if (transb == MFG_TRANS) {
    if (ldb < n)
      return fail(ctx, -10,
                  "The leading dimension must be greater than or equal to the number of rows.");
  } else {
    return fail(ctx, -3, "Invalid enum value.");
  }
  if (!c) return fail(ctx, -11, "c is null");
  if (ldc < m)
    return fail(ctx, -12,
                "The leading dimension must be greater than or equal to the number of rows.");
  if ((const double*)c == a || (const double*)c == b)
    return fail(ctx, MFG_ERR_INPLACE, "In-place operation is not supported.");
  const int ar = transa == MFG_NOTRANS ? m : k, ac = transa == MFG_NOTRANS ? k : m;
  const int br = transb == MFG_NOTRANS ? k : n, bc = transb == MFG_NOTRANS ? n : k;
  const size_t na = span(ar, ac, lda), nb = span(br, bc, ldb), nc = span(m, n, ldc);
  const size_t need = Carve::bytes_for(na, 8) + Carve::bytes_for(nb, 8) + Carve::bytes_for(nc, 8);
  MFG_CUDA(ctx, ctx->work.reserve(need));
  Carve cv(ctx->work.ptr);
  double* d_a = cv.take<double>(na);
  double* d_b = cv.take<double>(nb);
  double* d_c = cv.take<double>(nc);
  cudaStream_t s = ctx->stream;
  MFG_CUDA(ctx, cudaMemcpy2DAsync(d_a, (size_t)lda * 8, a, (size_t)lda * 8, (size_t)ar * 8, ac,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaMemcpy2DAsync(d_b, (size_t)ldb * 8, b, (size_t)ldb * 8, (size_t)br * 8, bc,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, mfg::launch_gemm_single(transa, transb, m, n, k, d_a, lda, d_b, ldb, d_c, ldc, s));
  MFG_CUDA(ctx, cudaMemcpy2DAsync(c, (size_t)ldc * 8, d_c, (size_t)ldc * 8, (size_t)m * 8, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaStreamSynchronize(s));
  return MFG_OK;
}

}  // extern "C"

// Factorization.LuInverse, all three overloads (elem 0 double, 1 float, 2 Complex as interleaved
// doubles): argument checks in MatFlat's order (Factorization.LuInverse.cs:125-143), then the
// singularity test before anything is written (:145-152), on host copies of the diagonal and the
// pivots (a and piv may be device arrays).
static int getri_single_any(mfg_ctx* ctx, int elem, int n, void* a, int lda, const int* piv,
                            int* info) {
  if (!ctx) return -1;
  if (n <= 0) return fail(ctx, -2, "The order of the matrix must be greater than or equal to one.");
  if (!a) return fail(ctx, -3, "a is null");
  if (lda < n)
    return fail(ctx, -4,
                "The leading dimension must be greater than or equal to the order of the matrix.");
  if (!piv) return fail(ctx, -5, "piv is null");
  const size_t es = elem == 1 ? 4 : elem == 2 ? 16 : 8;
  std::vector<char> diag((size_t)n * es);
  std::vector<int> hpiv(n);
  MFG_CUDA(ctx, cudaMemcpy2D(diag.data(), es, a, (size_t)(lda + 1) * es, es, n,
                             cudaMemcpyDefault));
  MFG_CUDA(ctx, cudaMemcpy(hpiv.data(), piv, sizeof(int) * n, cudaMemcpyDefault));
  for (int j = 0; j < n; j++) {
    bool zero;
    if (elem == 1) {
      zero = ((const float*)diag.data())[j] == 0.0f;
    } else if (elem == 2) {
      const double* z = (const double*)diag.data() + 2 * j;
      zero = z[0] == 0.0 && z[1] == 0.0;
    } else {
      zero = ((const double*)diag.data())[j] == 0.0;
    }
    if (zero) {
      if (info) *info = 1;
      return MFG_OK;
    }
  }
  for (int j = 0; j < n; j++)
    if (hpiv[j] < 0 || hpiv[j] >= n)
      return fail(ctx, -5, "piv[%d] = %d is out of range", j, hpiv[j]);
  const int warps = 8;
  const size_t na = span(n, n, lda);
  const size_t nwork = (size_t)n * n;
  const size_t sbytes = (size_t)warps * (size_t)mfg::getri_single_scratch_bytes_per_warp(n, elem);
  const size_t need = Carve::bytes_for(na, es) + Carve::bytes_for(nwork, es) +
                      Carve::bytes_for(sbytes, 1) + Carve::bytes_for(n, 4);
  MFG_CUDA(ctx, ctx->work.reserve(need));
  Carve cv(ctx->work.ptr);
  char* d_a = cv.take<char>(na * es);
  char* d_w = cv.take<char>(nwork * es);
  char* d_s = cv.take<char>(sbytes);
  int* d_piv = cv.take<int>(n);
  cudaStream_t s = ctx->stream;
  MFG_CUDA(ctx, cudaMemcpy2DAsync(d_a, (size_t)lda * es, a, (size_t)lda * es, (size_t)n * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaMemcpyAsync(d_piv, piv, sizeof(int) * n, cudaMemcpyDefault, s));
  if (elem == 1)
    MFG_CUDA(ctx, mfg::launch_sgetri_single((float*)d_a, n, lda, d_piv, (float*)d_w, d_s, warps,
                                            s));
  else if (elem == 2)
    MFG_CUDA(ctx, mfg::launch_zgetri_single((double*)d_a, n, lda, d_piv, (double*)d_w, d_s,
                                            warps, s));
  else
    MFG_CUDA(ctx, mfg::launch_getri_single((double*)d_a, n, lda, d_piv, (double*)d_w,
                                           (double*)d_s, warps, s));
  MFG_CUDA(ctx, cudaMemcpy2DAsync(a, (size_t)lda * es, d_a, (size_t)lda * es, (size_t)n * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaStreamSynchronize(s));
  if (info) *info = 0;
  return MFG_OK;
}

extern "C" {

MFG_API int mfg_dgetri(mfg_ctx* ctx, int n, double* a, int lda, const int* piv, int* info) {
  DeviceScope device_scope_(ctx);
  return getri_single_any(ctx, 0, n, a, lda, piv, info);
}
MFG_API int mfg_sgetri(mfg_ctx* ctx, int n, float* a, int lda, const int* piv, int* info) {
  DeviceScope device_scope_(ctx);
  return getri_single_any(ctx, 1, n, a, lda, piv, info);
}
MFG_API int mfg_zgetri(mfg_ctx* ctx, int n, double* a, int lda, const int* piv, int* info) {
  DeviceScope device_scope_(ctx);
  return getri_single_any(ctx, 2, n, a, lda, piv, info);
}


// ------------------------------------------------------------------------------------------
// QR drop-ins (Factorization.Qr / QrOrthogonalFactor / QrUpperTriangularFactor), both precisions.

}  // extern "C"

template <typename T>
static int qr_single(mfg_ctx* ctx, int m, int n, T* a, int lda, T* rdiag) {
  if (!ctx) return -1;
  // Factorization.Qr argument checks (Factorization.Qr.cs:117-145).
  if (m <= 0) return fail(ctx, -2, "The number of rows must be greater than or equal to one.");
  if (n <= 0) return fail(ctx, -3, "The number of columns must be greater than or equal to one.");
  if (!a) return fail(ctx, -4, "a is null");
  if (lda < m)
    return fail(ctx, -5,
                "The leading dimension must be greater than or equal to the number of rows.");
  if (!rdiag) return fail(ctx, -6, "rdiag is null");
  if (n > m)
    return fail(ctx, -3,
                "The number of rows must be greater than or equal to the number of columns.");
  const size_t na = span(m, n, lda);
  const size_t need = Carve::bytes_for(na, sizeof(T)) + Carve::bytes_for(n, sizeof(T)) +
                      Carve::bytes_for(n + 1, sizeof(T));
  MFG_CUDA(ctx, ctx->work.reserve(need));
  Carve cv(ctx->work.ptr);
  T* d_a = cv.take<T>(na);
  T* d_r = cv.take<T>(n);
  T* d_s = cv.take<T>(n + 1);
  cudaStream_t s = ctx->stream;
  const size_t es = sizeof(T);
  MFG_CUDA(ctx, cudaMemcpy2DAsync(d_a, (size_t)lda * es, a, (size_t)lda * es, (size_t)m * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, mfg::launch_qr_single<T>(d_a, m, n, lda, d_r, d_s, s));
  MFG_CUDA(ctx, cudaMemcpy2DAsync(a, (size_t)lda * es, d_a, (size_t)lda * es, (size_t)m * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaMemcpyAsync(rdiag, d_r, n * es, cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaStreamSynchronize(s));
  return MFG_OK;
}

template <typename T>
static int qr_q_single(mfg_ctx* ctx, int m, int n, const T* a, int lda, T* q, int ldq) {
  if (!ctx) return -1;
  // QrOrthogonalFactor argument checks (Factorization.Qr.cs:359-392).
  if (m <= 0) return fail(ctx, -2, "The number of rows must be greater than or equal to one.");
  if (n <= 0) return fail(ctx, -3, "The number of columns must be greater than or equal to one.");
  if (!a) return fail(ctx, -4, "a is null");
  if (lda < m)
    return fail(ctx, -5,
                "The leading dimension must be greater than or equal to the number of rows.");
  if (!q) return fail(ctx, -6, "q is null");
  if (ldq < m)
    return fail(ctx, -7,
                "The leading dimension must be greater than or equal to the number of rows.");
  if (n > m)
    return fail(ctx, -3,
                "The number of rows must be greater than or equal to the number of columns.");
  const size_t na = span(m, n, lda), nq = span(m, n, ldq);
  const size_t need = Carve::bytes_for(na, sizeof(T)) + Carve::bytes_for(nq, sizeof(T)) +
                      Carve::bytes_for(n + 1, sizeof(T));
  MFG_CUDA(ctx, ctx->work.reserve(need));
  Carve cv(ctx->work.ptr);
  T* d_a = cv.take<T>(na);
  T* d_q = cv.take<T>(nq);
  T* d_s = cv.take<T>(n + 1);
  cudaStream_t s = ctx->stream;
  const size_t es = sizeof(T);
  MFG_CUDA(ctx, cudaMemcpy2DAsync(d_a, (size_t)lda * es, a, (size_t)lda * es, (size_t)m * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, mfg::launch_qr_q_single<T>(d_a, m, n, lda, d_q, ldq, d_s, s));
  MFG_CUDA(ctx, cudaMemcpy2DAsync(q, (size_t)ldq * es, d_q, (size_t)ldq * es, (size_t)m * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaStreamSynchronize(s));
  return MFG_OK;
}

template <typename T>
static int qr_r_single(mfg_ctx* ctx, int m, int n, const T* a, int lda, T* r, int ldr,
                       const T* rdiag) {
  if (!ctx) return -1;
  // QrUpperTriangularFactor argument checks (Factorization.Qr.cs:599-632).
  if (m <= 0) return fail(ctx, -2, "The number of rows must be greater than or equal to one.");
  if (n <= 0) return fail(ctx, -3, "The number of columns must be greater than or equal to one.");
  if (!a) return fail(ctx, -4, "a is null");
  if (lda < m)
    return fail(ctx, -5,
                "The leading dimension must be greater than or equal to the number of rows.");
  if (!r) return fail(ctx, -6, "r is null");
  if (ldr < n)
    return fail(ctx, -7,
                "The leading dimension must be greater than or equal to the number of rows.");
  if (n > m)
    return fail(ctx, -3,
                "The number of rows must be greater than or equal to the number of columns.");
  if (!rdiag) return fail(ctx, -8, "rdiag is null");
  const size_t na = span(n, n, lda), nr = span(n, n, ldr);
  const size_t need = Carve::bytes_for(na, sizeof(T)) + Carve::bytes_for(nr, sizeof(T)) +
                      Carve::bytes_for(n, sizeof(T));
  MFG_CUDA(ctx, ctx->work.reserve(need));
  Carve cv(ctx->work.ptr);
  T* d_a = cv.take<T>(na);
  T* d_r = cv.take<T>(nr);
  T* d_d = cv.take<T>(n);
  cudaStream_t s = ctx->stream;
  const size_t es = sizeof(T);
  MFG_CUDA(ctx, cudaMemcpy2DAsync(d_a, (size_t)lda * es, a, (size_t)lda * es, (size_t)n * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaMemcpyAsync(d_d, rdiag, n * es, cudaMemcpyDefault, s));
  MFG_CUDA(ctx, mfg::launch_qr_r_single<T>(d_a, n, lda, d_r, ldr, d_d, s));
  MFG_CUDA(ctx, cudaMemcpy2DAsync(r, (size_t)ldr * es, d_r, (size_t)ldr * es, (size_t)n * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaStreamSynchronize(s));
  return MFG_OK;
}

extern "C" {

MFG_API int mfg_dgeqrf(mfg_ctx* ctx, int m, int n, double* a, int lda, double* rdiag) {
  DeviceScope device_scope_(ctx);
  return qr_single<double>(ctx, m, n, a, lda, rdiag);
}
MFG_API int mfg_sgeqrf(mfg_ctx* ctx, int m, int n, float* a, int lda, float* rdiag) {
  DeviceScope device_scope_(ctx);
  return qr_single<float>(ctx, m, n, a, lda, rdiag);
}
MFG_API int mfg_dorgqr(mfg_ctx* ctx, int m, int n, const double* a, int lda, double* q, int ldq) {
  DeviceScope device_scope_(ctx);
  return qr_q_single<double>(ctx, m, n, a, lda, q, ldq);
}
MFG_API int mfg_sorgqr(mfg_ctx* ctx, int m, int n, const float* a, int lda, float* q, int ldq) {
  DeviceScope device_scope_(ctx);
  return qr_q_single<float>(ctx, m, n, a, lda, q, ldq);
}
MFG_API int mfg_dqr_r(mfg_ctx* ctx, int m, int n, const double* a, int lda, double* r, int ldr,
                      const double* rdiag) {
  DeviceScope device_scope_(ctx);
  return qr_r_single<double>(ctx, m, n, a, lda, r, ldr, rdiag);
}
MFG_API int mfg_sqr_r(mfg_ctx* ctx, int m, int n, const float* a, int lda, float* r, int ldr,
                      const float* rdiag) {
  DeviceScope device_scope_(ctx);
  return qr_r_single<float>(ctx, m, n, a, lda, r, ldr, rdiag);
}

MFG_API int mfg_plan_geqrf_batched(mfg_ctx* ctx, mfg_plan** plan, int count, const int* m,
                                   const int* n, const int* lda, const int64_t* a_off,
                                   const int64_t* rdiag_off, int nrhs, const int64_t* b_off) {
  DeviceScope device_scope_(ctx);
  return plan_create_qr(ctx, plan, count, m, n, lda, a_off, rdiag_off, nrhs, b_off);
}

MFG_API int mfg_dgeqrf_batched(mfg_plan* plan, double* a, double* rdiag, double* b) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::GEQRF) return fail(ctx, -1, "plan is not a geqrf plan");
  if (plan->count > 0) {
    if (!a) return fail(ctx, -2, "a is null");
    if (!rdiag) return fail(ctx, -3, "rdiag is null");
    if (plan->nrhs > 0 && !b) return fail(ctx, -4, "b is null");
  }
  plan->qr_float = 0;
  plan->qd.a = a;
  plan->qd.rdiag = rdiag;
  plan->qd.b = b;
  plan->qd.solve_only = 0;
  return plan_execute(plan, a, rdiag, b, (const void*)1, nullptr);
}

MFG_API int mfg_sgeqrf_batched(mfg_plan* plan, float* a, float* rdiag, float* b) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::GEQRF) return fail(ctx, -1, "plan is not a geqrf plan");
  if (plan->count > 0) {
    if (!a) return fail(ctx, -2, "a is null");
    if (!rdiag) return fail(ctx, -3, "rdiag is null");
    if (plan->nrhs > 0 && !b) return fail(ctx, -4, "b is null");
  }
  plan->qr_float = 1;
  plan->qs.a = a;
  plan->qs.rdiag = rdiag;
  plan->qs.b = b;
  plan->qs.solve_only = 0;
  return plan_execute(plan, a, rdiag, b, (const void*)2, nullptr);
}

}  // extern "C"

// The Complex overload keeps 2 doubles per reflector coefficient: matrices whose n + nrhs
// coefficients do not fit in shared memory use global scratch, grown on first use (after the
// stream drains: it may be in use; the other overloads follow the new address).
static int zqr_prepare(mfg_plan* p) {
  mfg_ctx* ctx = p->ctx;
  long long stride = 0;
  if (p->qr_max_cols > mfg::zqr_smem_coefs()) {
    stride = 2LL * ((p->qr_max_cols + 31) / 32 * 32);
    const size_t need = (size_t)stride * sizeof(double) * (size_t)p->ctas * (size_t)p->warps;
    if (need > p->scratch.bytes) {
      MFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      MFG_CUDA(ctx, p->scratch.reserve(need));
      p->qd.gscratch = (double*)p->scratch.ptr;
      p->qs.gscratch = (float*)p->scratch.ptr;
      if (p->exec) {
        cudaGraphExecDestroy(p->exec);
        p->exec = nullptr;
      }
    }
  }
  p->qz.gscratch = (double*)p->scratch.ptr;
  p->qz.gscratch_stride = stride;
  return MFG_OK;
}

extern "C" {

MFG_API int mfg_zgeqrf_batched(mfg_plan* plan, double* a, double* rdiag, double* b) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::GEQRF) return fail(ctx, -1, "plan is not a geqrf plan");
  if (plan->count > 0) {
    if (!a) return fail(ctx, -2, "a is null");
    if (!rdiag) return fail(ctx, -3, "rdiag is null");
    if (plan->nrhs > 0 && !b) return fail(ctx, -4, "b is null");
  }
  const int rc = zqr_prepare(plan);
  if (rc != MFG_OK) return rc;
  plan->qr_float = 2;
  plan->qz.a = a;
  plan->qz.rdiag = rdiag;
  plan->qz.b = b;
  plan->qz.solve_only = 0;
  return plan_execute(plan, a, rdiag, b, (const void*)4, nullptr);
}

MFG_API int mfg_zgeqrs_batched(mfg_plan* plan, const double* a, const double* rdiag, double* b) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::GEQRF) return fail(ctx, -1, "plan is not a geqrf plan");
  if (plan->nrhs < 1) return fail(ctx, -1, "the plan has no right-hand sides (nrhs = 0)");
  if (plan->count > 0) {
    if (!a) return fail(ctx, -2, "a is null");
    if (!rdiag) return fail(ctx, -3, "rdiag is null");
    if (!b) return fail(ctx, -4, "b is null");
  }
  const int rc = zqr_prepare(plan);
  if (rc != MFG_OK) return rc;
  plan->qr_float = 2;
  plan->qz.a = const_cast<double*>(a);
  plan->qz.rdiag = const_cast<double*>(rdiag);
  plan->qz.b = b;
  plan->qz.solve_only = 1;
  return plan_execute(plan, a, rdiag, b, (const void*)4, (const void*)3);
}

}  // extern "C"

// Least-squares solve with an existing factorization (the plan's nrhs right-hand sides).
template <typename T>
static int geqrs_batched(mfg_plan* plan, const T* a, const T* rdiag, T* b, int single) {
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::GEQRF) return fail(ctx, -1, "plan is not a geqrf plan");
  if (plan->nrhs < 1) return fail(ctx, -1, "the plan has no right-hand sides (nrhs = 0)");
  if (plan->count > 0) {
    if (!a) return fail(ctx, -2, "a is null");
    if (!rdiag) return fail(ctx, -3, "rdiag is null");
    if (!b) return fail(ctx, -4, "b is null");
  }
  plan->qr_float = single;
  mfg::QrBatchArgs<T>& q = *reinterpret_cast<mfg::QrBatchArgs<T>*>(single ? (void*)&plan->qs
                                                                           : (void*)&plan->qd);
  q.a = const_cast<T*>(a);
  q.rdiag = const_cast<T*>(rdiag);
  q.b = b;
  q.solve_only = 1;
  return plan_execute(plan, a, rdiag, b, (const void*)(intptr_t)(single ? 2 : 1), (const void*)3);
}

extern "C" {

MFG_API int mfg_dgeqrs_batched(mfg_plan* plan, const double* a, const double* rdiag, double* b) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return geqrs_batched<double>(plan, a, rdiag, b, 0);
}

MFG_API int mfg_sgeqrs_batched(mfg_plan* plan, const float* a, const float* rdiag, float* b) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return geqrs_batched<float>(plan, a, rdiag, b, 1);
}


// ------------------------------------------------------------------------------------------
// Float and Complex overloads of the single-matrix drop-ins.  Complex arrays are interleaved
// (re, im) doubles, the layout of System.Numerics.Complex; es is the element size in bytes.

}  // extern "C"

namespace {

int getrf_t(mfg_ctx* ctx, int m, int n, void* a, int lda, int* piv, int* sign, size_t es,
            cudaError_t (*launch)(void*, int, int, int, int*, int*, double*, cudaStream_t)) {
  if (!ctx) return -1;
  if (m <= 0) return fail(ctx, -2, "The number of rows must be greater than or equal to one.");
  if (n <= 0) return fail(ctx, -3, "The number of columns must be greater than or equal to one.");
  if (!a) return fail(ctx, -4, "a is null");
  if (lda < m)
    return fail(ctx, -5,
                "The leading dimension must be greater than or equal to the number of rows.");
  if (!piv) return fail(ctx, -6, "piv is null");
  const size_t na = span(m, n, lda);
  const size_t need = Carve::bytes_for(na, es) + Carve::bytes_for(2 * (size_t)m + 2, 8) +
                      Carve::bytes_for(m, 4) + Carve::bytes_for(2, 4);
  MFG_CUDA(ctx, ctx->work.reserve(need));
  Carve cv(ctx->work.ptr);
  char* d_a = cv.take<char>(na * es);
  double* d_s = cv.take<double>(2 * (size_t)m + 2);
  int* d_piv = cv.take<int>(m);
  int* d_out = cv.take<int>(2);
  cudaStream_t s = ctx->stream;
  MFG_CUDA(ctx, cudaMemcpy2DAsync(d_a, (size_t)lda * es, a, (size_t)lda * es, (size_t)m * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, launch(d_a, m, n, lda, d_piv, d_out, d_s, s));
  int out[2];
  MFG_CUDA(ctx, cudaMemcpy2DAsync(a, (size_t)lda * es, d_a, (size_t)lda * es, (size_t)m * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaMemcpyAsync(piv, d_piv, sizeof(int) * m, cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaMemcpyAsync(out, d_out, sizeof(out), cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaStreamSynchronize(s));
  if (sign) *sign = out[0];
  return MFG_OK;
}

int potrf_t(mfg_ctx* ctx, int n, void* a, int lda, int* info, size_t es,
            cudaError_t (*launch)(void*, int, int, int*, double*, cudaStream_t)) {
  if (!ctx) return -1;
  if (n <= 0) return fail(ctx, -2, "The order of the matrix must be greater than or equal to one.");
  if (!a) return fail(ctx, -3, "a is null");
  if (lda < n)
    return fail(ctx, -4,
                "The leading dimension must be greater than or equal to the order of the matrix.");
  const size_t na = span(n, n, lda);
  const size_t need = Carve::bytes_for(na, es) + Carve::bytes_for(n, 8) + Carve::bytes_for(1, 4);
  MFG_CUDA(ctx, ctx->work.reserve(need));
  Carve cv(ctx->work.ptr);
  char* d_a = cv.take<char>(na * es);
  double* d_s = cv.take<double>(n);
  int* d_out = cv.take<int>(1);
  cudaStream_t s = ctx->stream;
  MFG_CUDA(ctx, cudaMemcpy2DAsync(d_a, (size_t)lda * es, a, (size_t)lda * es, (size_t)n * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, launch(d_a, n, lda, d_out, d_s, s));
  int out = 0;
  MFG_CUDA(ctx, cudaMemcpy2DAsync(a, (size_t)lda * es, d_a, (size_t)lda * es, (size_t)n * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaMemcpyAsync(&out, d_out, sizeof(int), cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaStreamSynchronize(s));
  if (info) *info = out;
  return MFG_OK;
}

int trsv_t(mfg_ctx* ctx, int uplo, int trans, int n, const void* a, int lda, void* x, int incx,
           size_t es, bool complex_modes,
           cudaError_t (*launch)(int, int, int, const void*, int, void*, int, double*,
                                 cudaStream_t)) {
  if (!ctx) return -1;
  if (n <= 0) return fail(ctx, -4, "The order of the matrix must be greater than or equal to one.");
  if (!a) return fail(ctx, -5, "a is null");
  if (lda < n)
    return fail(ctx, -6,
                "The leading dimension must be greater than or equal to the number of rows.");
  if (!x) return fail(ctx, -7, "x is null");
  if (incx <= 0) return fail(ctx, -8, "The value must be greater than or equal to one.");
  if (uplo != MFG_UPPER && uplo != MFG_LOWER) return fail(ctx, -2, "Invalid enum value.");
  const bool okt = trans == MFG_NOTRANS || trans == MFG_TRANS ||
                   (complex_modes && (trans == MFG_CONJTRANS || trans == MFG_CONJNOTRANS));
  if (!okt) return fail(ctx, -3, "Invalid enum value.");
  const size_t na = span(n, n, lda);
  const size_t nx = (size_t)(n - 1) * incx + 1;
  const size_t nscr = 4 * (size_t)(n | 1);
  const size_t need = Carve::bytes_for(na, es) + Carve::bytes_for(nx, es) + Carve::bytes_for(nscr, 8);
  MFG_CUDA(ctx, ctx->work.reserve(need));
  Carve cv(ctx->work.ptr);
  char* d_a = cv.take<char>(na * es);
  char* d_x = cv.take<char>(nx * es);
  double* d_s = cv.take<double>(nscr);
  cudaStream_t s = ctx->stream;
  MFG_CUDA(ctx, cudaMemcpy2DAsync(d_a, (size_t)lda * es, a, (size_t)lda * es, (size_t)n * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaMemcpyAsync(d_x, x, nx * es, cudaMemcpyDefault, s));
  MFG_CUDA(ctx, launch(uplo, trans, n, d_a, lda, d_x, incx, d_s, s));
  MFG_CUDA(ctx, cudaMemcpyAsync(x, d_x, nx * es, cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaStreamSynchronize(s));
  return MFG_OK;
}

int gemm_t(mfg_ctx* ctx, int transa, int transb, int m, int n, int k, const void* a, int lda,
           const void* b, int ldb, void* c, int ldc, size_t es, bool complex_modes,
           cudaError_t (*launch)(int, int, int, int, int, const void*, int, const void*, int,
                                 void*, int, cudaStream_t)) {
  if (!ctx) return -1;
  if (m <= 0) return fail(ctx, -4, "The value must be greater than or equal to one.");
  if (n <= 0) return fail(ctx, -5, "The value must be greater than or equal to one.");
  if (k <= 0) return fail(ctx, -6, "The value must be greater than or equal to one.");
  if (!a) return fail(ctx, -7, "a is null");
  auto valid = [&](int t) {
    return t == MFG_NOTRANS || t == MFG_TRANS ||
           (complex_modes && (t == MFG_CONJTRANS || t == MFG_CONJNOTRANS));
  };
  auto is_t = [](int t) { return t == MFG_TRANS || t == MFG_CONJTRANS; };
  if (!valid(transa)) return fail(ctx, -2, "Invalid enum value.");
  if (lda < (is_t(transa) ? k : m))
    return fail(ctx, -8, "The leading dimension must be greater than or equal to the number of rows.");
  if (!b) return fail(ctx, -9, "b is null");
  if (!valid(transb)) return fail(ctx, -3, "Invalid enum value.");
  if (ldb < (is_t(transb) ? n : k))
    return fail(ctx, -10, "The leading dimension must be greater than or equal to the number of rows.");
  if (!c) return fail(ctx, -11, "c is null");
  if (ldc < m)
    return fail(ctx, -12, "The leading dimension must be greater than or equal to the number of rows.");
  if (c == a || c == b) return fail(ctx, MFG_ERR_INPLACE, "In-place operation is not supported.");
  const int ar = is_t(transa) ? k : m, ac = is_t(transa) ? m : k;
  const int br = is_t(transb) ? n : k, bc = is_t(transb) ? k : n;
  const size_t na = span(ar, ac, lda), nb = span(br, bc, ldb), nc = span(m, n, ldc);
  const size_t need = Carve::bytes_for(na, es) + Carve::bytes_for(nb, es) + Carve::bytes_for(nc, es);
  MFG_CUDA(ctx, ctx->work.reserve(need));
  Carve cv(ctx->work.ptr);
  char* d_a = cv.take<char>(na * es);
  char* d_b = cv.take<char>(nb * es);
  char* d_c = cv.take<char>(nc * es);
  cudaStream_t s = ctx->stream;
  MFG_CUDA(ctx, cudaMemcpy2DAsync(d_a, (size_t)lda * es, a, (size_t)lda * es, (size_t)ar * es, ac,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaMemcpy2DAsync(d_b, (size_t)ldb * es, b, (size_t)ldb * es, (size_t)br * es, bc,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, launch(transa, transb, m, n, k, d_a, lda, d_b, ldb, d_c, ldc, s));
  MFG_CUDA(ctx, cudaMemcpy2DAsync(c, (size_t)ldc * es, d_c, (size_t)ldc * es, (size_t)m * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaStreamSynchronize(s));
  return MFG_OK;
}

// Launch adapters from the typeless helpers to the typed kernels.
cudaError_t sgetrf_l(void* a, int m, int n, int lda, int* piv, int* o, double* s, cudaStream_t st) {
  return mfg::launch_sgetrf_single((float*)a, m, n, lda, piv, o, s, st);
}
cudaError_t zgetrf_l(void* a, int m, int n, int lda, int* piv, int* o, double* s, cudaStream_t st) {
  return mfg::launch_zgetrf_single((double*)a, m, n, lda, piv, o, s, st);
}
cudaError_t spotrf_l(void* a, int n, int lda, int* o, double* s, cudaStream_t st) {
  return mfg::launch_spotrf_single((float*)a, n, lda, o, s, st);
}
cudaError_t zpotrf_l(void* a, int n, int lda, int* o, double* s, cudaStream_t st) {
  return mfg::launch_zpotrf_single((double*)a, n, lda, o, s, st);
}
cudaError_t strsv_l(int u, int t, int n, const void* a, int lda, void* x, int incx, double* s,
                    cudaStream_t st) {
  return mfg::launch_strsv_single(u, t, n, (const float*)a, lda, (float*)x, incx, s, st);
}
cudaError_t ztrsv_l(int u, int t, int n, const void* a, int lda, void* x, int incx, double* s,
                    cudaStream_t st) {
  return mfg::launch_ztrsv_single(u, t, n, (const double*)a, lda, (double*)x, incx, s, st);
}
cudaError_t sgemm_l(int ta, int tb, int m, int n, int k, const void* a, int lda, const void* b,
                    int ldb, void* c, int ldc, cudaStream_t st) {
  return mfg::launch_sgemm_single(ta, tb, m, n, k, (const float*)a, lda, (const float*)b, ldb,
                                  (float*)c, ldc, st);
}
cudaError_t zgemm_l(int ta, int tb, int m, int n, int k, const void* a, int lda, const void* b,
                    int ldb, void* c, int ldc, cudaStream_t st) {
  return mfg::launch_zgemm_single(ta, tb, m, n, k, (const double*)a, lda, (const double*)b, ldb,
                                  (double*)c, ldc, st);
}

}  // namespace

extern "C" {

MFG_API int mfg_sgetrf(mfg_ctx* ctx, int m, int n, float* a, int lda, int* piv, int* sign) {
  DeviceScope device_scope_(ctx);
  return getrf_t(ctx, m, n, a, lda, piv, sign, sizeof(float), sgetrf_l);
}
MFG_API int mfg_zgetrf(mfg_ctx* ctx, int m, int n, double* a, int lda, int* piv, int* sign) {
  DeviceScope device_scope_(ctx);
  return getrf_t(ctx, m, n, a, lda, piv, sign, 2 * sizeof(double), zgetrf_l);
}
MFG_API int mfg_spotrf(mfg_ctx* ctx, int n, float* a, int lda, int* info) {
  DeviceScope device_scope_(ctx);
  return potrf_t(ctx, n, a, lda, info, sizeof(float), spotrf_l);
}
MFG_API int mfg_zpotrf(mfg_ctx* ctx, int n, double* a, int lda, int* info) {
  DeviceScope device_scope_(ctx);
  return potrf_t(ctx, n, a, lda, info, 2 * sizeof(double), zpotrf_l);
}
MFG_API int mfg_strsv(mfg_ctx* ctx, int uplo, int trans, int n, const float* a, int lda, float* x,
                      int incx) {
  DeviceScope device_scope_(ctx);
  return trsv_t(ctx, uplo, trans, n, a, lda, x, incx, sizeof(float), false, strsv_l);
}
MFG_API int mfg_ztrsv(mfg_ctx* ctx, int uplo, int trans, int n, const double* a, int lda,
                      double* x, int incx) {
  DeviceScope device_scope_(ctx);
  return trsv_t(ctx, uplo, trans, n, a, lda, x, incx, 2 * sizeof(double), true, ztrsv_l);
}
MFG_API int mfg_sgemm(mfg_ctx* ctx, int transa, int transb, int m, int n, int k, const float* a,
                      int lda, const float* b, int ldb, float* c, int ldc) {
  DeviceScope device_scope_(ctx);
  return gemm_t(ctx, transa, transb, m, n, k, a, lda, b, ldb, c, ldc, sizeof(float), false,
                sgemm_l);
}
MFG_API int mfg_zgemm(mfg_ctx* ctx, int transa, int transb, int m, int n, int k, const double* a,
                      int lda, const double* b, int ldb, double* c, int ldc) {
  DeviceScope device_scope_(ctx);
  return gemm_t(ctx, transa, transb, m, n, k, a, lda, b, ldb, c, ldc, 2 * sizeof(double), true,
                zgemm_l);
}

}  // extern "C"

namespace {

// Complex QR staging (the QR template above is keyed on float/double; Complex uses these).
int zqr_single(mfg_ctx* ctx, int m, int n, double* a, int lda, double* rdiag) {
  if (!ctx) return -1;
  if (m <= 0) return fail(ctx, -2, "The number of rows must be greater than or equal to one.");
  if (n <= 0) return fail(ctx, -3, "The number of columns must be greater than or equal to one.");
  if (!a) return fail(ctx, -4, "a is null");
  if (lda < m)
    return fail(ctx, -5,
                "The leading dimension must be greater than or equal to the number of rows.");
  if (!rdiag) return fail(ctx, -6, "rdiag is null");
  if (n > m)
    return fail(ctx, -3,
                "The number of rows must be greater than or equal to the number of columns.");
  const size_t es = 16;
  const size_t na = span(m, n, lda);
  const size_t need = Carve::bytes_for(na, es) + Carve::bytes_for(n, 8) +
                      Carve::bytes_for(2 * (size_t)(n + 1), 8);
  MFG_CUDA(ctx, ctx->work.reserve(need));
  Carve cv(ctx->work.ptr);
  double* d_a = cv.take<double>(2 * na);
  double* d_r = cv.take<double>(n);
  double* d_s = cv.take<double>(2 * (size_t)(n + 1));
  cudaStream_t s = ctx->stream;
  MFG_CUDA(ctx, cudaMemcpy2DAsync(d_a, (size_t)lda * es, a, (size_t)lda * es, (size_t)m * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, mfg::launch_zqr_single(d_a, m, n, lda, d_r, d_s, s));
  MFG_CUDA(ctx, cudaMemcpy2DAsync(a, (size_t)lda * es, d_a, (size_t)lda * es, (size_t)m * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaMemcpyAsync(rdiag, d_r, n * 8, cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaStreamSynchronize(s));
  return MFG_OK;
}

int zqr_q_single(mfg_ctx* ctx, int m, int n, const double* a, int lda, double* q, int ldq) {
  if (!ctx) return -1;
  if (m <= 0) return fail(ctx, -2, "The number of rows must be greater than or equal to one.");
  if (n <= 0) return fail(ctx, -3, "The number of columns must be greater than or equal to one.");
  if (!a) return fail(ctx, -4, "a is null");
  if (lda < m)
    return fail(ctx, -5,
                "The leading dimension must be greater than or equal to the number of rows.");
  if (!q) return fail(ctx, -6, "q is null");
  if (ldq < m)
    return fail(ctx, -7,
                "The leading dimension must be greater than or equal to the number of rows.");
  if (n > m)
    return fail(ctx, -3,
                "The number of rows must be greater than or equal to the number of columns.");
  const size_t es = 16;
  const size_t na = span(m, n, lda), nq = span(m, n, ldq);
  const size_t need = Carve::bytes_for(na, es) + Carve::bytes_for(nq, es) +
                      Carve::bytes_for(2 * (size_t)(n + 1), 8);
  MFG_CUDA(ctx, ctx->work.reserve(need));
  Carve cv(ctx->work.ptr);
  double* d_a = cv.take<double>(2 * na);
  double* d_q = cv.take<double>(2 * nq);
  double* d_s = cv.take<double>(2 * (size_t)(n + 1));
  cudaStream_t s = ctx->stream;
  MFG_CUDA(ctx, cudaMemcpy2DAsync(d_a, (size_t)lda * es, a, (size_t)lda * es, (size_t)m * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, mfg::launch_zqr_q_single(d_a, m, n, lda, d_q, ldq, d_s, s));
  MFG_CUDA(ctx, cudaMemcpy2DAsync(q, (size_t)ldq * es, d_q, (size_t)ldq * es, (size_t)m * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaStreamSynchronize(s));
  return MFG_OK;
}

int zqr_r_single(mfg_ctx* ctx, int m, int n, const double* a, int lda, double* r, int ldr,
                 const double* rdiag) {
  if (!ctx) return -1;
  if (m <= 0) return fail(ctx, -2, "The number of rows must be greater than or equal to one.");
  if (n <= 0) return fail(ctx, -3, "The number of columns must be greater than or equal to one.");
  if (!a) return fail(ctx, -4, "a is null");
  if (lda < m)
    return fail(ctx, -5,
                "The leading dimension must be greater than or equal to the number of rows.");
  if (!r) return fail(ctx, -6, "r is null");
  if (ldr < n)
    return fail(ctx, -7,
                "The leading dimension must be greater than or equal to the number of rows.");
  if (n > m)
    return fail(ctx, -3,
                "The number of rows must be greater than or equal to the number of columns.");
  if (!rdiag) return fail(ctx, -8, "rdiag is null");
  const size_t es = 16;
  const size_t na = span(n, n, lda), nr = span(n, n, ldr);
  const size_t need = Carve::bytes_for(na, es) + Carve::bytes_for(nr, es) + Carve::bytes_for(n, 8);
  MFG_CUDA(ctx, ctx->work.reserve(need));
  Carve cv(ctx->work.ptr);
  double* d_a = cv.take<double>(2 * na);
  double* d_r = cv.take<double>(2 * nr);
  double* d_d = cv.take<double>(n);
  cudaStream_t s = ctx->stream;
  MFG_CUDA(ctx, cudaMemcpy2DAsync(d_a, (size_t)lda * es, a, (size_t)lda * es, (size_t)n * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaMemcpyAsync(d_d, rdiag, n * 8, cudaMemcpyDefault, s));
  MFG_CUDA(ctx, mfg::launch_zqr_r_single(d_a, n, lda, d_r, ldr, d_d, s));
  MFG_CUDA(ctx, cudaMemcpy2DAsync(r, (size_t)ldr * es, d_r, (size_t)ldr * es, (size_t)n * es, n,
                                  cudaMemcpyDefault, s));
  MFG_CUDA(ctx, cudaStreamSynchronize(s));
  return MFG_OK;
}

}  // namespace

extern "C" {

MFG_API int mfg_zgeqrf(mfg_ctx* ctx, int m, int n, double* a, int lda, double* rdiag) {
  DeviceScope device_scope_(ctx);
  return zqr_single(ctx, m, n, a, lda, rdiag);
}
MFG_API int mfg_zorgqr(mfg_ctx* ctx, int m, int n, const double* a, int lda, double* q, int ldq) {
  DeviceScope device_scope_(ctx);
  return zqr_q_single(ctx, m, n, a, lda, q, ldq);
}
MFG_API int mfg_zqr_r(mfg_ctx* ctx, int m, int n, const double* a, int lda, double* r, int ldr,
                      const double* rdiag) {
  DeviceScope device_scope_(ctx);
  return zqr_r_single(ctx, m, n, a, lda, r, ldr, rdiag);
}

// ------------------------------------------------------------------------------------------
// Batched plans.

MFG_API int mfg_plan_getrf_batched(mfg_ctx* ctx, mfg_plan** plan, int count, const int* n,
                                   const int* lda, const int64_t* a_off, const int64_t* piv_off,
                                   int nrhs, const int64_t* b_off) {
  DeviceScope device_scope_(ctx);
  return plan_create(ctx, plan, mfg_plan::GETRF, count, n, lda, a_off, piv_off, nrhs, b_off);
}

MFG_API int mfg_plan_potrf_batched(mfg_ctx* ctx, mfg_plan** plan, int count, const int* n,
                                   const int* lda, const int64_t* a_off, int nrhs,
                                   const int64_t* b_off) {
  DeviceScope device_scope_(ctx);
  return plan_create(ctx, plan, mfg_plan::POTRF, count, n, lda, a_off, nullptr, nrhs, b_off);
}

MFG_API int mfg_plan_getri_batched(mfg_ctx* ctx, mfg_plan** plan, int count, const int* n,
                                   const int* lda, const int64_t* a_off, const int64_t* piv_off) {
  DeviceScope device_scope_(ctx);
  return plan_create(ctx, plan, mfg_plan::GETRI, count, n, lda, a_off, piv_off, 0, nullptr);
}

}  // extern "C"

static int getri_batched_any(mfg_plan* plan, int elem, void* a, const int* piv, int* info) {
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::GETRI) return fail(ctx, -1, "plan is not a getri plan");
  if (plan->count > 0) {
    if (!a) return fail(ctx, -2, "a is null");
    if (!piv) return fail(ctx, -3, "piv is null");
    if (!info) return fail(ctx, -4, "info is null");
  }
  const int rc = plan_set_elem(plan, elem);
  if (rc != MFG_OK) return rc;
  plan->args.a = (double*)a;
  plan->args.piv = const_cast<int*>(piv);
  plan->args.b = nullptr;
  plan->args.sign = nullptr;
  plan->args.info = info;
  return plan_execute(plan, a, piv, info, nullptr, nullptr);
}

extern "C" {

MFG_API int mfg_sgetri_batched(mfg_plan* plan, float* a, const int* piv, int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return getri_batched_any(plan, 1, a, piv, info);
}
MFG_API int mfg_zgetri_batched(mfg_plan* plan, double* a, const int* piv, int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return getri_batched_any(plan, 2, a, piv, info);
}

MFG_API int mfg_dgetri_batched(mfg_plan* plan, double* a, const int* piv, int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::GETRI) return fail(ctx, -1, "plan is not a getri plan");
  if (plan->count > 0) {
    if (!a) return fail(ctx, -2, "a is null");
    if (!piv) return fail(ctx, -3, "piv is null");
    if (!info) return fail(ctx, -4, "info is null");
  }
  const int rc = plan_set_elem(plan, 0);
  if (rc != MFG_OK) return rc;
  plan->args.a = a;
  plan->args.piv = const_cast<int*>(piv);
  plan->args.b = nullptr;
  plan->args.sign = nullptr;
  plan->args.info = info;
  return plan_execute(plan, a, piv, info, nullptr, nullptr);
}

MFG_API int mfg_dgemv_strided_batched(mfg_ctx* ctx, int trans, int m, int n, const double* a,
                                      int lda, int64_t stride_a, const double* x, int incx,
                                      int64_t stride_x, double* y, int incy, int64_t stride_y,
                                      int count) {
  DeviceScope device_scope_(ctx);
  if (!ctx) return -1;
  // Blas.MulMatVec's checks (Blas.MulMatVec.cs:140-183).
  if (m <= 0) return fail(ctx, -3, "The number of rows must be greater than or equal to one.");
  if (n <= 0) return fail(ctx, -4, "The number of columns must be greater than or equal to one.");
  if (!a) return fail(ctx, -5, "a is null");
  if (lda < m)
    return fail(ctx, -6,
                "The leading dimension must be greater than or equal to the number of rows.");
  if (!x) return fail(ctx, -8, "x is null");
  if (incx <= 0) return fail(ctx, -9, "The value must be greater than or equal to one.");
  if (!y) return fail(ctx, -11, "y is null");
  if (incy <= 0) return fail(ctx, -12, "The value must be greater than or equal to one.");
  if ((const void*)a == (const void*)y || (const void*)x == (const void*)y)
    return fail(ctx, MFG_ERR_INPLACE, "In-place operation is not supported.");
  if (trans != MFG_NOTRANS && trans != MFG_TRANS) return fail(ctx, -2, "Invalid enum value.");
  if (count < 0) return fail(ctx, -14, "count must be >= 0");
  MFG_CUDA(ctx, mfg::launch_gemv_strided(trans, m, n, a, lda, stride_a, x, incx, stride_x, y,
                                         incy, stride_y, count, ctx->stream));
  return MFG_OK;
}

MFG_API int mfg_ddot_strided_batched(mfg_ctx* ctx, int n, const double* x, int incx,
                                     int64_t stride_x, const double* y, int incy,
                                     int64_t stride_y, double* result, int count) {
  DeviceScope device_scope_(ctx);
  if (!ctx) return -1;
  if (n <= 0) return fail(ctx, -2, "The length of the vector must be greater than or equal to one.");
  if (!x) return fail(ctx, -3, "x is null");
  if (incx <= 0) return fail(ctx, -4, "The value must be greater than or equal to one.");
  if (!y) return fail(ctx, -6, "y is null");
  if (incy <= 0) return fail(ctx, -7, "The value must be greater than or equal to one.");
  if (!result) return fail(ctx, -9, "result is null");
  if (count < 0) return fail(ctx, -10, "count must be >= 0");
  MFG_CUDA(ctx, mfg::launch_dot_strided(n, x, incx, stride_x, y, incy, stride_y, result, count,
                                        0, ctx->stream));
  return MFG_OK;
}

MFG_API int mfg_dnrm2_strided_batched(mfg_ctx* ctx, int n, const double* x, int incx,
                                      int64_t stride_x, double* result, int count) {
  DeviceScope device_scope_(ctx);
  if (!ctx) return -1;
  if (n <= 0) return fail(ctx, -2, "The length of the vector must be greater than or equal to one.");
  if (!x) return fail(ctx, -3, "x is null");
  if (incx <= 0) return fail(ctx, -4, "The value must be greater than or equal to one.");
  if (!result) return fail(ctx, -6, "result is null");
  if (count < 0) return fail(ctx, -7, "count must be >= 0");
  MFG_CUDA(ctx, mfg::launch_dot_strided(n, x, incx, stride_x, x, incx, stride_x, result, count,
                                        1, ctx->stream));
  return MFG_OK;
}

MFG_API int mfg_dger_strided_batched(mfg_ctx* ctx, int m, int n, const double* x, int incx,
                                     int64_t stride_x, const double* y, int incy,
                                     int64_t stride_y, double* a, int lda, int64_t stride_a,
                                     int count) {
  DeviceScope device_scope_(ctx);
  if (!ctx) return -1;
  if (m <= 0) return fail(ctx, -2, "The number of rows must be greater than or equal to one.");
  if (n <= 0) return fail(ctx, -3, "The number of columns must be greater than or equal to one.");
  if (!x) return fail(ctx, -4, "x is null");
  if (incx <= 0) return fail(ctx, -5, "The value must be greater than or equal to one.");
  if (!y) return fail(ctx, -7, "y is null");
  if (incy <= 0) return fail(ctx, -8, "The value must be greater than or equal to one.");
  if (!a) return fail(ctx, -10, "a is null");
  if (lda < m)
    return fail(ctx, -11,
                "The leading dimension must be greater than or equal to the number of rows.");
  if (count < 0) return fail(ctx, -13, "count must be >= 0");
  MFG_CUDA(ctx, mfg::launch_ger_strided(m, n, x, incx, stride_x, y, incy, stride_y, a, lda,
                                        stride_a, count, ctx->stream));
  return MFG_OK;
}

}  // extern "C"

// The float and Complex strided batches: MatFlat's argument checks, as for the double ones.
static int gemv_strided_any(mfg_ctx* ctx, int elem, int trans, int m, int n, const void* a,
                            int lda, int64_t sa, const void* x, int incx, int64_t sx, void* y,
                            int incy, int64_t sy, int count) {
  if (!ctx) return -1;
  if (m <= 0) return fail(ctx, -3, "The number of rows must be greater than or equal to one.");
  if (n <= 0) return fail(ctx, -4, "The number of columns must be greater than or equal to one.");
  if (!a) return fail(ctx, -5, "a is null");
  if (lda < m)
    return fail(ctx, -6,
                "The leading dimension must be greater than or equal to the number of rows.");
  if (!x) return fail(ctx, -8, "x is null");
  if (incx <= 0) return fail(ctx, -9, "The value must be greater than or equal to one.");
  if (!y) return fail(ctx, -11, "y is null");
  if (incy <= 0) return fail(ctx, -12, "The value must be greater than or equal to one.");
  if (a == (const void*)y || x == (const void*)y)
    return fail(ctx, MFG_ERR_INPLACE, "In-place operation is not supported.");
  const bool ok = trans == MFG_NOTRANS || trans == MFG_TRANS ||
                  (elem == 2 && (trans == MFG_CONJTRANS || trans == MFG_CONJNOTRANS));
  if (!ok) return fail(ctx, -2, "Invalid enum value.");
  if (count < 0) return fail(ctx, -14, "count must be >= 0");
  MFG_CUDA(ctx, mfg::launch_gemv_strided_t(elem, trans, m, n, a, lda, sa, x, incx, sx, y, incy,
                                           sy, count, ctx->stream));
  return MFG_OK;
}

static int dot_strided_any(mfg_ctx* ctx, int elem, int mode, int n, const void* x, int incx,
                           int64_t sx, const void* y, int incy, int64_t sy, void* result,
                           int count) {
  if (!ctx) return -1;
  if (n <= 0) return fail(ctx, -2, "The length of the vector must be greater than or equal to one.");
  if (!x) return fail(ctx, -3, "x is null");
  if (incx <= 0) return fail(ctx, -4, "The value must be greater than or equal to one.");
  if (mode != 1) {
    if (!y) return fail(ctx, -6, "y is null");
    if (incy <= 0) return fail(ctx, -7, "The value must be greater than or equal to one.");
    if (!result) return fail(ctx, -9, "result is null");
    if (count < 0) return fail(ctx, -10, "count must be >= 0");
  } else {
    if (!result) return fail(ctx, -6, "result is null");
    if (count < 0) return fail(ctx, -7, "count must be >= 0");
  }
  MFG_CUDA(ctx, mfg::launch_dot_strided_t(elem, n, x, incx, sx, mode == 1 ? x : y,
                                          mode == 1 ? incx : incy, mode == 1 ? sx : sy, result,
                                          count, mode, ctx->stream));
  return MFG_OK;
}

static int ger_strided_any(mfg_ctx* ctx, int elem, int conj, int m, int n, const void* x,
                           int incx, int64_t sx, const void* y, int incy, int64_t sy, void* a,
                           int lda, int64_t sa, int count) {
  if (!ctx) return -1;
  if (m <= 0) return fail(ctx, -2, "The number of rows must be greater than or equal to one.");
  if (n <= 0) return fail(ctx, -3, "The number of columns must be greater than or equal to one.");
  if (!x) return fail(ctx, -4, "x is null");
  if (incx <= 0) return fail(ctx, -5, "The value must be greater than or equal to one.");
  if (!y) return fail(ctx, -7, "y is null");
  if (incy <= 0) return fail(ctx, -8, "The value must be greater than or equal to one.");
  if (!a) return fail(ctx, -10, "a is null");
  if (lda < m)
    return fail(ctx, -11,
                "The leading dimension must be greater than or equal to the number of rows.");
  if (count < 0) return fail(ctx, -13, "count must be >= 0");
  MFG_CUDA(ctx, mfg::launch_ger_strided_t(elem, m, n, x, incx, sx, y, incy, sy, a, lda, sa,
                                          count, conj, ctx->stream));
  return MFG_OK;
}

extern "C" {

MFG_API int mfg_sgemv_strided_batched(mfg_ctx* ctx, int trans, int m, int n, const float* a,
                                      int lda, int64_t stride_a, const float* x, int incx,
                                      int64_t stride_x, float* y, int incy, int64_t stride_y,
                                      int count) {
  DeviceScope device_scope_(ctx);
  return gemv_strided_any(ctx, 1, trans, m, n, a, lda, stride_a, x, incx, stride_x, y, incy,
                          stride_y, count);
}
MFG_API int mfg_zgemv_strided_batched(mfg_ctx* ctx, int trans, int m, int n, const double* a,
                                      int lda, int64_t stride_a, const double* x, int incx,
                                      int64_t stride_x, double* y, int incy, int64_t stride_y,
                                      int count) {
  DeviceScope device_scope_(ctx);
  return gemv_strided_any(ctx, 2, trans, m, n, a, lda, stride_a, x, incx, stride_x, y, incy,
                          stride_y, count);
}
MFG_API int mfg_sdot_strided_batched(mfg_ctx* ctx, int n, const float* x, int incx,
                                     int64_t stride_x, const float* y, int incy,
                                     int64_t stride_y, float* result, int count) {
  DeviceScope device_scope_(ctx);
  return dot_strided_any(ctx, 1, 0, n, x, incx, stride_x, y, incy, stride_y, result, count);
}
MFG_API int mfg_zdot_strided_batched(mfg_ctx* ctx, int n, const double* x, int incx,
                                     int64_t stride_x, const double* y, int incy,
                                     int64_t stride_y, double* result, int count) {
  DeviceScope device_scope_(ctx);
  return dot_strided_any(ctx, 2, 0, n, x, incx, stride_x, y, incy, stride_y, result, count);
}
MFG_API int mfg_zdotc_strided_batched(mfg_ctx* ctx, int n, const double* x, int incx,
                                      int64_t stride_x, const double* y, int incy,
                                      int64_t stride_y, double* result, int count) {
  DeviceScope device_scope_(ctx);
  return dot_strided_any(ctx, 2, 2, n, x, incx, stride_x, y, incy, stride_y, result, count);
}
MFG_API int mfg_snrm2_strided_batched(mfg_ctx* ctx, int n, const float* x, int incx,
                                      int64_t stride_x, float* result, int count) {
  DeviceScope device_scope_(ctx);
  return dot_strided_any(ctx, 1, 1, n, x, incx, stride_x, nullptr, 0, 0, result, count);
}
MFG_API int mfg_dznrm2_strided_batched(mfg_ctx* ctx, int n, const double* x, int incx,
                                       int64_t stride_x, double* result, int count) {
  DeviceScope device_scope_(ctx);
  return dot_strided_any(ctx, 2, 1, n, x, incx, stride_x, nullptr, 0, 0, result, count);
}
MFG_API int mfg_sger_strided_batched(mfg_ctx* ctx, int m, int n, const float* x, int incx,
                                     int64_t stride_x, const float* y, int incy,
                                     int64_t stride_y, float* a, int lda, int64_t stride_a,
                                     int count) {
  DeviceScope device_scope_(ctx);
  return ger_strided_any(ctx, 1, 0, m, n, x, incx, stride_x, y, incy, stride_y, a, lda,
                         stride_a, count);
}
MFG_API int mfg_zger_strided_batched(mfg_ctx* ctx, int m, int n, const double* x, int incx,
                                     int64_t stride_x, const double* y, int incy,
                                     int64_t stride_y, double* a, int lda, int64_t stride_a,
                                     int count) {
  DeviceScope device_scope_(ctx);
  return ger_strided_any(ctx, 2, 0, m, n, x, incx, stride_x, y, incy, stride_y, a, lda,
                         stride_a, count);
}
MFG_API int mfg_zgerc_strided_batched(mfg_ctx* ctx, int m, int n, const double* x, int incx,
                                      int64_t stride_x, const double* y, int incy,
                                      int64_t stride_y, double* a, int lda, int64_t stride_a,
                                      int count) {
  DeviceScope device_scope_(ctx);
  return ger_strided_any(ctx, 2, 1, m, n, x, incx, stride_x, y, incy, stride_y, a, lda,
                         stride_a, count);
}

MFG_API int mfg_plan_gevd_front_batched(mfg_ctx* ctx, mfg_plan** plan, int count, const int* n,
                                        const int* lda, const int64_t* a_off, const int* ldb,
                                        const int64_t* b_off, const int64_t* c_off) {
  DeviceScope device_scope_(ctx);
  return plan_create_gevd(ctx, plan, count, n, lda, a_off, ldb, b_off, c_off);
}

}  // extern "C"

static int gevd_front_any(mfg_plan* plan, int elem, const void* a, void* b, void* c, int* info) {
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::GEVD) return fail(ctx, -1, "plan is not a gevd plan");
  if (plan->count > 0) {
    if (!a) return fail(ctx, -2, "a is null");
    if (!b) return fail(ctx, -3, "b is null");
    if (!c) return fail(ctx, -4, "c is null");
    if (!info) return fail(ctx, -5, "info is null");
  }
  const int rc = plan_set_elem(plan, elem);
  if (rc != MFG_OK) return rc;
  plan->gv.a = (const double*)a;
  plan->gv.b = (double*)b;
  plan->gv.c = (double*)c;
  plan->gv.info = info;
  return plan_execute(plan, a, b, c, info, nullptr);
}

extern "C" {

MFG_API int mfg_dgevd_front_batched(mfg_plan* plan, const double* a, double* b, double* c,
                                    int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return gevd_front_any(plan, 0, a, b, c, info);
}
MFG_API int mfg_sgevd_front_batched(mfg_plan* plan, const float* a, float* b, float* c,
                                    int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return gevd_front_any(plan, 1, a, b, c, info);
}
MFG_API int mfg_zgevd_front_batched(mfg_plan* plan, const double* a, double* b, double* c,
                                    int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return gevd_front_any(plan, 2, a, b, c, info);
}

}  // extern "C"

namespace {

// QR plans: times lanes per matrix (4, 8, 16, 32) and warps per SM on a sample of up to 50,000
// matrices spread evenly over the batch (so it keeps the plan's (m, n) mix), with the FP64
// kernel, and installs the fastest for both real overloads; the tuning table keeps it under the
// plan's (m, n) size bucket for later plans.
int qr_autotune(mfg_plan* plan, int* config) {
  mfg_ctx* ctx = plan->ctx;
  cudaStream_t s = ctx->stream;
  // Groups of fewer lanes hold 2-8 matrices per warp: the sample must keep every warp of the
  // launch busy for many matrices, or the trial favours 32 lanes (it did with 8,000 matrices).
  const int cap = 50000;
  const int step = (plan->count + cap - 1) / cap;
  std::vector<int> sm, sn;
  for (int i = 0; i < plan->count; i += step) {
    sm.push_back(plan->hm[i]);
    sn.push_back(plan->hn[i]);
  }
  const int cnt = (int)sm.size();
  const int nrhs = plan->nrhs;
  std::vector<int64_t> aoff(cnt), roff(cnt), boff(cnt);
  long long at = 0, rt = 0, bt = 0;
  int max_m = 0, max_n = 0;
  for (int i = 0; i < cnt; i++) {
    aoff[i] = at;
    at += (long long)sm[i] * sn[i];
    roff[i] = rt;
    rt += sn[i];
    boff[i] = bt;
    bt += (long long)sm[i] * nrhs;
  }
  for (int i = 0; i < plan->count; i++) {
    max_m = std::max(max_m, plan->hm[i]);
    max_n = std::max(max_n, plan->hn[i]);
  }
  mfg_plan* tp = nullptr;
  int rc = plan_create_qr(ctx, &tp, cnt, sm.data(), sn.data(), nullptr, aoff.data(), roff.data(),
                          nrhs, nrhs > 0 ? boff.data() : nullptr);
  if (rc != MFG_OK) return rc;
  DevBuf buf;
  const size_t need = Carve::bytes_for(at, 8) * 2 + Carve::bytes_for(bt + 1, 8) * 2 +
                      Carve::bytes_for(rt, 8);
  cudaError_t ce = buf.reserve(need);
  if (ce != cudaSuccess) {
    mfg_plan_destroy(tp);
    return cuda_fail(ctx, ce, "cudaMalloc(autotune batch)");
  }
  Carve cv(buf.ptr);
  double* a = cv.take<double>(at);
  double* a0 = cv.take<double>(at);
  double* b = cv.take<double>(bt + 1);
  double* b0 = cv.take<double>(bt + 1);
  double* rd = cv.take<double>(rt);
  tp->qd.a = a;
  tp->qd.b = nrhs > 0 ? b : nullptr;
  tp->qd.rdiag = rd;
  tp->qd.solve_only = 0;
  tp->qr_float = 0;
  tp->qd.fma = plan->qd.fma;
  std::vector<std::array<int, 5>> cands;
  for (int g : {4, 8, 16, 32})
    for (int wps : {8, 12, 16, 24}) cands.push_back({4, wps, g, 0, 0});
  std::array<int, 5> best = cands[0];
  float best_ms = 3.0e38f;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  ce = mfg::launch_tune_fill_qr(tp->qd, s);
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(a0, a, sizeof(double) * at, cudaMemcpyDeviceToDevice, s);
  if (ce == cudaSuccess)
    ce = cudaMemcpyAsync(b0, b, sizeof(double) * (bt + 1), cudaMemcpyDeviceToDevice, s);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e0);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
  for (size_t c = 0; ce == cudaSuccess && rc == MFG_OK && c < cands.size(); c++) {
    const auto& k = cands[c];
    rc = qr_reshape(tp, k[2], k[1]);
    float tmin = 3.0e38f;
    for (int rep = 0; rc == MFG_OK && ce == cudaSuccess && rep < 2; rep++) {
      ce = cudaMemcpyAsync(a, a0, sizeof(double) * at, cudaMemcpyDeviceToDevice, s);
      if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(b, b0, sizeof(double) * (bt + 1), cudaMemcpyDeviceToDevice, s);
      if (ce == cudaSuccess) ce = cudaEventRecord(e0, s);
      if (ce == cudaSuccess) rc = plan_launch(tp, s);
      if (rc == MFG_OK && ce == cudaSuccess) ce = cudaEventRecord(e1, s);
      if (rc == MFG_OK && ce == cudaSuccess) ce = cudaEventSynchronize(e1);
      float ms = 0.0f;
      if (rc == MFG_OK && ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
      if (rc == MFG_OK && ce == cudaSuccess) tmin = std::min(tmin, ms);
    }
    if (tmin < best_ms) {
      best_ms = tmin;
      best = k;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaStreamSynchronize(s);
  buf.release();
  mfg_plan_destroy(tp);
  if (rc != MFG_OK) return rc;
  if (ce != cudaSuccess) return cuda_fail(ctx, ce, "autotune");
  pipe_release(plan);
  rc = qr_reshape(plan, best[2], best[1]);
  if (rc != MFG_OK) return rc;
  best[0] = plan->warps;
  ctx->tune[qr_tune_key(max_n, max_m, plan->count)] = best;
  if (config)
    for (int i = 0; i < 5; i++) config[i] = best[i];
  return MFG_OK;
}

}  // namespace

extern "C" {

MFG_API int mfg_plan_set_form(mfg_plan* plan, int form) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::POTRF && plan->kind != mfg_plan::GEQRF &&
      plan->kind != mfg_plan::GETRF)
    return fail(ctx, MFG_ERR_UNSUPPORTED, "set_form: getrf, potrf and geqrf plans only");
  if (form != MFG_FORM_EXACT && form != MFG_FORM_FMA)
    return fail(ctx, -2, "form must be MFG_FORM_EXACT or MFG_FORM_FMA");
  pipe_release(plan);  // host-buffer chunk plans are rebuilt with the form on next use
  return plan_set_fma(plan, form == MFG_FORM_FMA ? 1 : 0);
}

MFG_API int mfg_plan_form_fallbacks(mfg_plan* plan, long long* count) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (!count) return fail(ctx, -2, "count is null");
  *count = 0;
  if (plan->kind != mfg_plan::GETRF || plan->count == 0) return MFG_OK;
  // Host-buffer calls return when their streams are done; device calls run on the context's.
  MFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  std::vector<mfg_plan*> plans;
  if (plan->last_host)
    plans = plan->pipe.chunk;
  else
    plans.push_back(plan);
  for (mfg_plan* q : plans) {
    int v = 0;
    MFG_CUDA(ctx, cudaMemcpy(&v, q->args.queue + 8, sizeof(int), cudaMemcpyDeviceToHost));
    *count += v;
  }
  return MFG_OK;
}

MFG_API int mfg_plan_autotune(mfg_plan* plan, int* config) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind == mfg_plan::GEQRF) return plan->count > 0 ? qr_autotune(plan, config) : MFG_OK;
  if (plan->kind != mfg_plan::GETRF && plan->kind != mfg_plan::POTRF)
    return fail(ctx, MFG_ERR_UNSUPPORTED, "autotune: getrf, potrf and geqrf plans only");
  if (plan->count == 0) return MFG_OK;
  cudaStream_t s = ctx->stream;
  // A sample of up to 100,000 matrices spread evenly over the batch keeps its size mix, and
  // keeps enough tasks per warp for the tables that put several matrices in a warp.
  const int cap = 100000;
  const int step = (plan->count + cap - 1) / cap;
  std::vector<int> sn;
  for (int i = 0; i < plan->count; i += step) sn.push_back(plan->hn[i]);
  const int cnt = (int)sn.size();
  const int nrhs = plan->nrhs;
  std::vector<int64_t> aoff(cnt), poff(cnt), boff(cnt);
  long long at = 0, pt = 0, bt = 0;
  for (int i = 0; i < cnt; i++) {
    aoff[i] = at;
    at += (long long)sn[i] * sn[i];
    poff[i] = pt;
    pt += sn[i];
    boff[i] = bt;
    bt += (long long)sn[i] * nrhs;
  }
  mfg_plan* tp = nullptr;
  int rc = plan_create(ctx, &tp, plan->kind, cnt, sn.data(), nullptr, aoff.data(), poff.data(),
                       nrhs, nrhs > 0 ? boff.data() : nullptr);
  if (rc != MFG_OK) return rc;
  DevBuf buf;
  const size_t need = Carve::bytes_for(at, 8) * 2 + Carve::bytes_for(bt + 1, 8) * 2 +
                      Carve::bytes_for(pt, 4) + 2 * Carve::bytes_for(cnt, 4);
  cudaError_t ce = buf.reserve(need);
  if (ce != cudaSuccess) {
    mfg_plan_destroy(tp);
    return cuda_fail(ctx, ce, "cudaMalloc(autotune batch)");
  }
  Carve cv(buf.ptr);
  double* a = cv.take<double>(at);
  double* a0 = cv.take<double>(at);
  double* b = cv.take<double>(bt + 1);
  double* b0 = cv.take<double>(bt + 1);
  int* piv = cv.take<int>(pt);
  int* sign = cv.take<int>(cnt);
  int* info = cv.take<int>(cnt);
  tp->args.a = a;
  tp->args.b = nrhs > 0 ? b : nullptr;
  tp->args.piv = plan->kind == mfg_plan::GETRF ? piv : nullptr;
  tp->args.sign = plan->kind == mfg_plan::GETRF ? sign : nullptr;
  tp->args.info = info;
  tp->args.solve_only = 0;
  if (plan->args.fma) {
    rc = plan_set_fma(tp, 1);
    if (rc != MFG_OK) {
      mfg_plan_destroy(tp);
      return rc;
    }
  }
  std::vector<std::array<int, 5>> cands;
  if (plan->kind == mfg_plan::GETRF) {
    // Slot 2 is the lanes-per-matrix table of the size buckets (lu_lanes; -1: one matrix per
    // warp).  Two-pair dot blocks need ~72 registers (up to 28 warps/SM), four-pair ~100.  Tables
    // with 16 or 8 lanes per matrix keep 2 or 4 matrices in flight per warp, so they are tried at
    // fewer warps per SM.
    // Measured on the 100,000-matrix batch (n 8..128): 16 lanes per matrix at n = 128 is slower
    // than 32 (two matrices per warp double the footprint in flight), 8 lanes pays off at small
    // orders; the tables are tried at 20-28 warps per SM, where they are fastest.
    if (plan->args.fma) {
      // The FMA form (no integer-pipe products) is fastest with fewer warps in flight and
      // two-chain dots (slot 4 = 1): 65.5 ms at 16 warps/SM against 70.7 with four chains and
      // 82.5 at 28 warps/SM on the 100,000-matrix batch.
      // Tables 5 and 6 (16 lanes for the small orders): 62.1 / 61.6 ms at 16 warps/SM.
      for (int gsel : {0, 4, 5, 6})
        for (int wps : {8, 12, 16, 20})
          for (int db : {1, 2}) cands.push_back({4, wps, gsel, 0, db});
    } else {
      // Measured on the 100,000-matrix batch: table 0 at 28 warps/SM 81.4 ms, 24: 83.6, 32:
      // 82.6; table 6 at 28: 80.6, table 5: 81.2; table 4 at 28: 85.4; table 2 at 24: 90.9; one
      // matrix per warp (-1) at 24: 90.4.
      for (int gsel : {0, 2, 4, 5, 6})
        for (int wps : {24, 28, 32}) cands.push_back({4, wps, gsel, 0, 2});
    }
  } else {
    // The integer-product variants need ~100 registers (up to 20 warps/SM), the FP64-pipe ones
    // ~128 (16 warps/SM).
    // The FMA form has no multiply pipe to choose.
    for (int g : {4, 8, 16, 32}) {
      for (int wps : {8, 16})
        for (int mul : {0, 1})
          if (mul == 0 || !plan->args.fma) cands.push_back({4, wps, g, mul, 4});
      cands.push_back({4, 20, g, 0, 4});
      if (plan->args.fma) cands.push_back({4, 24, g, 0, 4});
    }
    // Lanes per matrix by size bucket (slot 2 = -table, chol_lanes); the FMA form also with
    // two-chain dots (slot 4 = 1).
    for (int t : {1, 2})
      for (int wps : {12, 16, 20}) {
        cands.push_back({4, wps, -t, 0, 4});
        if (plan->args.fma) cands.push_back({4, wps, -t, 0, 1});
      }
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  std::array<int, 5> best = cands[0];
  float best_ms = 3.0e38f;
  ce = mfg::launch_tune_fill(tp->args, plan->kind == mfg_plan::POTRF ? 1 : 0, s);
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(a0, a, sizeof(double) * at, cudaMemcpyDeviceToDevice, s);
  if (ce == cudaSuccess)
    ce = cudaMemcpyAsync(b0, b, sizeof(double) * (bt + 1), cudaMemcpyDeviceToDevice, s);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e0);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
  for (size_t c = 0; ce == cudaSuccess && rc == MFG_OK && c < cands.size(); c++) {
    const auto& k = cands[c];
    // The LU's FMA form runs on the size-bucketed tasks only.
    if (plan->kind == mfg_plan::GETRF && plan->args.fma && k[2] < 0) continue;
    rc = plan_reshape(tp, k[0], k[1], k[2], k[3], k[4]);
    float tmin = 3.0e38f;
    // Three trials per shape (the minimum): two left the choice to noise between shapes a few
    // per cent apart.
    for (int rep = 0; rc == MFG_OK && ce == cudaSuccess && rep < 3; rep++) {
      ce = cudaMemcpyAsync(a, a0, sizeof(double) * at, cudaMemcpyDeviceToDevice, s);
      if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(b, b0, sizeof(double) * (bt + 1), cudaMemcpyDeviceToDevice, s);
      if (ce == cudaSuccess) ce = cudaEventRecord(e0, s);
      if (ce == cudaSuccess) rc = plan_launch(tp, s);
      if (rc == MFG_OK && ce == cudaSuccess) ce = cudaEventRecord(e1, s);
      if (rc == MFG_OK && ce == cudaSuccess) ce = cudaEventSynchronize(e1);
      float ms = 0.0f;
      if (rc == MFG_OK && ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
      if (rc == MFG_OK && ce == cudaSuccess) tmin = std::min(tmin, ms);
    }
    if (tmin < best_ms) {
      best_ms = tmin;
      best = k;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaStreamSynchronize(s);
  buf.release();
  mfg_plan_destroy(tp);
  if (rc != MFG_OK) return rc;
  if (ce != cudaSuccess) return cuda_fail(ctx, ce, "autotune");
  pipe_release(plan);  // host-buffer chunk plans are rebuilt with the new shape on next use
  rc = plan_reshape(plan, best[0], best[1], best[2], best[3], best[4]);
  if (rc != MFG_OK) return rc;
  // Plans in the FMA form record their shape under a key of their own.
  ctx->tune[tune_key((int)plan->kind + (plan->args.fma ? 100 : 0), plan->max_n, plan->count)] =
      best;
  if (config)
    for (int i = 0; i < 5; i++) config[i] = best[i];
  return MFG_OK;
}

MFG_API int mfg_plan_destroy(mfg_plan* plan) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  if (plan->exec) cudaGraphExecDestroy(plan->exec);
  cudaStreamSynchronize(plan->ctx->stream);
  pipe_release(plan);
  plan->meta.release();
  plan->scratch.release();
  plan->gsolve.release();
  if (plan->mx_fb) mfg_plan_destroy(plan->mx_fb);
  plan->mx_work.release();
  delete plan;
  return MFG_OK;
}

}  // extern "C"

namespace {

// Points a GETRF or POTRF plan at the element type of the next launch.  The double kernels use
// the scratch stride the plan was shaped with; the float / Complex kernels run one warp per matrix
// and keep the per-warp vectors of orders above SMEM_N in global scratch, Complex twice the
// doubles of float, so their first launch may grow the scratch (after the stream drains: it may
// be in use).  A changed scratch address or stride drops the cached graph.
int plan_set_elem(mfg_plan* p, int elem) {
  mfg_ctx* ctx = p->ctx;
  p->elem = elem;
  if (p->kind == mfg_plan::GEVD) {
    // The float / Complex kernel keeps its accumulators in shared memory: only its grid differs.
    if (elem != 0 && p->ctas_t == 0) {
      const long long w = mfg::gevd_t_warps_per_cta();
      const long long ctas = std::min<long long>(
          (long long)ctx->sm_count * std::min(mfg::gevd_t_ctas_per_sm(1), mfg::gevd_t_ctas_per_sm(2)),
          ((long long)p->count + w - 1) / w);
      p->ctas_t = (int)std::max<long long>(1, ctas);
    }
    return MFG_OK;
  }
  long long stride = p->dstride;
  if (elem != 0 && p->kind == mfg_plan::GETRI) {
    // The float / Complex inverse keeps a copy of the factors per warp in global scratch.
    stride = mfg::getri_t_scratch_bytes(p->max_n, elem) / (long long)sizeof(double);
    const size_t need = (size_t)stride * sizeof(double) * (size_t)p->ctas * (size_t)p->warps;
    if (need > p->scratch.bytes) {
      MFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      MFG_CUDA(ctx, p->scratch.reserve(need));
    }
  } else if (elem != 0) {
    stride = 0;
    if (p->max_n > mfg::SMEM_N) {
      const long long base = (mfg::warp_scratch_doubles(p->max_n) + 31) / 32 * 32;
      stride = elem == 2 ? 2 * base : base;
      const size_t need = (size_t)stride * sizeof(double) * (size_t)p->ctas * (size_t)p->warps;
      if (need > p->scratch.bytes) {
        MFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        MFG_CUDA(ctx, p->scratch.reserve(need));
      }
    }
  }
  if (p->args.gscratch != (double*)p->scratch.ptr || p->args.gscratch_stride != stride) {
    p->args.gscratch = (double*)p->scratch.ptr;
    p->args.gscratch_stride = stride;
    if (p->exec) {
      cudaGraphExecDestroy(p->exec);
      p->exec = nullptr;
    }
  }
  return MFG_OK;
}

int getrf_batched_any(mfg_plan* plan, int elem, void* a, int* piv, void* b, int* sign,
                      int* info) {
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::GETRF) return fail(ctx, -1, "plan is not a getrf plan");
  plan->last_host = false;
  if (plan->count > 0) {
    if (!a) return fail(ctx, -2, "a is null");
    if (!piv) return fail(ctx, -3, "piv is null");
    if (plan->nrhs > 0 && !b) return fail(ctx, -4, "b is null");
    if (!sign) return fail(ctx, -5, "sign is null");
    if (!info) return fail(ctx, -6, "info is null");
  }
  const int rc = plan_set_elem(plan, elem);
  if (rc != MFG_OK) return rc;
  plan->args.a = (double*)a;
  plan->args.piv = piv;
  plan->args.b = (double*)b;
  plan->args.sign = sign;
  plan->args.info = info;
  plan->args.solve_only = 0;
  return plan_execute(plan, a, piv, b, sign, info);
}

int getrs_batched_any(mfg_plan* plan, int elem, const void* a, const int* piv, void* b) {
  if (!plan) return -1;
  plan->last_host = false;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::GETRF) return fail(ctx, -1, "plan is not a getrf plan");
  if (plan->nrhs < 1) return fail(ctx, -1, "the plan has no right-hand sides (nrhs = 0)");
  if (plan->count > 0) {
    if (!a) return fail(ctx, -2, "a is null");
    if (!piv) return fail(ctx, -3, "piv is null");
    if (!b) return fail(ctx, -4, "b is null");
  }
  const int rc = plan_set_elem(plan, elem);
  if (rc != MFG_OK) return rc;
  plan->args.a = (double*)const_cast<void*>(a);
  plan->args.piv = const_cast<int*>(piv);
  plan->args.b = (double*)b;
  plan->args.sign = nullptr;
  plan->args.info = nullptr;
  plan->args.solve_only = 1;
  return plan_execute(plan, a, piv, b, nullptr, (const void*)3);
}

}  // namespace

extern "C" {

MFG_API int mfg_sgetrf_batched(mfg_plan* plan, float* a, int* piv, float* b, int* sign,
                               int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return getrf_batched_any(plan, 1, a, piv, b, sign, info);
}
MFG_API int mfg_zgetrf_batched(mfg_plan* plan, double* a, int* piv, double* b, int* sign,
                               int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return getrf_batched_any(plan, 2, a, piv, b, sign, info);
}
MFG_API int mfg_sgetrs_batched(mfg_plan* plan, const float* a, const int* piv, float* b) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return getrs_batched_any(plan, 1, a, piv, b);
}
MFG_API int mfg_zgetrs_batched(mfg_plan* plan, const double* a, const int* piv, double* b) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return getrs_batched_any(plan, 2, a, piv, b);
}

MFG_API int mfg_dgetrf_batched(mfg_plan* plan, double* a, int* piv, double* b, int* sign,
                               int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return getrf_batched_any(plan, 0, a, piv, b, sign, info);
}

MFG_API int mfg_dgetrs_batched(mfg_plan* plan, const double* a, const int* piv, double* b) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return getrs_batched_any(plan, 0, a, piv, b);
}

}  // extern "C"

namespace {

// ---- Pipelined host-buffer calls --------------------------------------------------------------
// A host call cuts the batch into contiguous chunks of about equal work, each with its own plan
// whose offsets address device mirrors of the caller's arrays (laid out exactly like the host
// arrays).  Chunk c's upload (stream h2d), kernel (one of two compute streams) and download
// (stream d2h) overlap with the neighbouring chunks', so the copies hide behind the compute.
enum PipeOp {
  OP_GETRF, OP_POTRF, OP_GRAD, OP_GETRI, OP_GEQRF_D, OP_GEQRF_S, OP_GEVD,
  OP_GETRF_S, OP_GETRF_Z, OP_POTRF_S, OP_POTRF_Z, OP_GEQRF_Z, OP_GEVD_S, OP_GEVD_Z
};

// Element type of an operation's factor arrays: 0 double, 1 float, 2 Complex.
int pipe_elem(int op) {
  switch (op) {
    case OP_GETRF_S: case OP_POTRF_S: case OP_GEQRF_S: case OP_GEVD_S: return 1;
    case OP_GETRF_Z: case OP_POTRF_Z: case OP_GEQRF_Z: case OP_GEVD_Z: return 2;
    default: return 0;
  }
}
bool pipe_qr(int op) { return op == OP_GEQRF_D || op == OP_GEQRF_S || op == OP_GEQRF_Z; }

void pipe_release(mfg_plan* p) {
  auto& pp = p->pipe;
  for (mfg_plan* c : pp.chunk) mfg_plan_destroy(c);
  pp.chunk.clear();
  for (cudaEvent_t e : pp.in) cudaEventDestroy(e);
  for (cudaEvent_t e : pp.done) cudaEventDestroy(e);
  pp.in.clear();
  pp.done.clear();
  for (cudaStream_t* st : {&pp.h2d, &pp.d2h, &pp.comp[0], &pp.comp[1], &pp.comp[2]})
    if (*st) {
      cudaStreamSynchronize(*st);
      cudaStreamDestroy(*st);
      *st = nullptr;
    }
  for (auto& a : pp.arr) a.dev.release();
  pp.arr.clear();
  pp.op = -1;
}

// The arrays an operation moves: per matrix i, the element range of each array.
void pipe_arrays(mfg_plan* p, int op, int keep_factor) {
  auto& arr = p->pipe.arr;
  const int count = p->count, nrhs = p->nrhs;
  const bool qr = pipe_qr(op);
  const int elem = pipe_elem(op);
  const size_t es = elem == 1 ? 4 : elem == 2 ? 16 : 8;  // factor and right-hand-side elements
  const size_t rs = elem == 1 ? 4 : 8;                    // QR's rdiag (real for Complex)
  auto add = [&](int dir, size_t esz, auto beg, auto len) {
    mfg_plan::PipeArray a;
    a.dir = dir;
    a.es = esz;
    a.beg.resize(count);
    a.end.resize(count);
    for (int i = 0; i < count; i++) {
      a.beg[i] = beg(i);
      a.end[i] = a.beg[i] + len(i);
    }
    arr.push_back(std::move(a));
  };
  auto rows = [&](int i) { return qr ? p->hm[i] : p->hn[i]; };
  auto aspan = [&](int i) { return span(rows(i), p->hn[i], p->hlda[i]); };
  auto self = [](int i) { return (size_t)i; };
  auto one = [](int) { return (size_t)1; };
  switch (op) {
    case OP_GETRF:
    case OP_GETRF_S:
    case OP_GETRF_Z:  // a, b, piv, sign, info
      add(3, es, [&](int i) { return (size_t)p->haoff[i]; }, aspan);
      add(3, es, [&](int i) { return (size_t)p->hboff[i]; },
          [&](int i) { return (size_t)p->hn[i] * nrhs; });
      add(2, 4, [&](int i) { return (size_t)p->hpivoff[i]; }, [&](int i) { return (size_t)p->hn[i]; });
      add(2, 4, self, one);
      add(2, 4, self, one);
      break;
    case OP_POTRF:
    case OP_POTRF_S:
    case OP_POTRF_Z:  // a, b, info
      add(3, es, [&](int i) { return (size_t)p->haoff[i]; }, aspan);
      add(3, es, [&](int i) { return (size_t)p->hboff[i]; },
          [&](int i) { return (size_t)p->hn[i] * nrhs; });
      add(2, 4, self, one);
      break;
    case OP_GRAD:  // k, y, loss, grad, info
      add(keep_factor ? 3 : 1, 8, [&](int i) { return (size_t)p->haoff[i]; }, aspan);
      add(3, 8, [&](int i) { return (size_t)p->hboff[i]; }, [&](int i) { return (size_t)p->hn[i]; });
      add(2, 8, self, one);
      add(2, 8, [&](int i) { return (size_t)p->haoff[i]; }, aspan);
      add(2, 4, self, one);
      break;
    case OP_GETRI:  // a, piv, info
      add(3, 8, [&](int i) { return (size_t)p->haoff[i]; }, aspan);
      add(1, 4, [&](int i) { return (size_t)p->hpivoff[i]; }, [&](int i) { return (size_t)p->hn[i]; });
      add(2, 4, self, one);
      break;
    case OP_GEQRF_D:
    case OP_GEQRF_S:
    case OP_GEQRF_Z:  // a, rdiag, b
      add(3, es, [&](int i) { return (size_t)p->haoff[i]; }, aspan);
      add(2, rs, [&](int i) { return (size_t)p->hpivoff[i]; }, [&](int i) { return (size_t)p->hn[i]; });
      add(3, es, [&](int i) { return (size_t)p->hboff[i]; },
          [&](int i) { return (size_t)p->hm[i] * nrhs; });
      break;
    case OP_GEVD:
    case OP_GEVD_S:
    case OP_GEVD_Z:  // a, b, c, info
      add(1, es, [&](int i) { return (size_t)p->haoff[i]; }, aspan);
      add(3, es, [&](int i) { return (size_t)p->hboff[i]; },
          [&](int i) { return span(p->hn[i], p->hn[i], p->hldb[i]); });
      add(2, es, [&](int i) { return (size_t)p->hcoff[i]; },
          [&](int i) { return (size_t)p->hn[i] * p->hn[i]; });
      add(2, 4, self, one);
      break;
  }
}

int pipe_build(mfg_plan* p, int op, int keep_factor) {
  mfg_ctx* ctx = p->ctx;
  pipe_release(p);
  auto& pp = p->pipe;
  const int count = p->count;
  const bool qr = pipe_qr(op);
  pipe_arrays(p, op, keep_factor);
  // Chunks of about equal work (n^3, or m n^2 for QR), each about two full rounds of the GPU's
  // resident warps (shorter chunks leave SMs idle in their tails), at least four for batches of
  // 8,192 matrices or more and two from 2,048 (so that copies overlap compute), at most sixteen;
  // the sweep over the seven benchmark batches is in the profiles.
  long long per_wave;
  if (op == OP_GRAD)
    per_wave = (long long)ctx->sm_count * mfg::grad_ctas_per_sm() * mfg::grad_warps_per_cta();
  else if (op == OP_GEQRF_D)
    per_wave = (long long)p->ctas * p->warps * (32 / p->qd.group);
  else if (op == OP_GEQRF_Z)
    per_wave = (long long)p->ctas * p->warps;
  else if (op == OP_GEQRF_S)
    per_wave = (long long)p->ctas * p->warps * (32 / p->qs.group);
  else if (p->kind == mfg_plan::POTRF)
    per_wave = (long long)p->ctas * p->warps * (32 / p->args.group);
  else
    per_wave = (long long)p->ctas * p->warps;
  // QR chunks hold about four rounds and at least two chunks are used: its per-matrix work
  // spans a 128x range, so shorter chunks end in long tails (the 50,000-matrix batch measured
  // 236 / 236 / 216 / 210 / 181 / 145 / 119 thousand matrices/s with 1 / 2 / 3 / 4 / 8 / 12 / 16
  // chunks at 8 lanes per matrix).
  int K = (int)std::min<long long>(16, count / std::max<long long>(1, (qr ? 4 : 2) * per_wave));
  if (count >= 8192)
    K = std::max(K, qr ? 2 : 4);
  else if (count >= 2048)
    K = std::max(K, 2);
  K = env_int("MFG_PIPE_CHUNKS", std::max(K, 1));
  if (K < 1) K = 1;
  auto work = [&](int i) {
    const double n = p->hn[i];
    return qr ? (double)p->hm[i] * n * n : n * n * n;
  };
  double total = 0;
  for (int i = 0; i < count; i++) total += work(i);
  std::vector<int> cut{0};
  double acc = 0;
  for (int i = 0; i < count && (int)cut.size() < K; i++) {
    acc += work(i);
    if (acc >= total * cut.size() / K && i + 1 < count) cut.push_back(i + 1);
  }
  cut.push_back(count);
  auto chunk_ranges = [&]() {
    const int nc = (int)cut.size() - 1;
    for (auto& a : pp.arr) {
      a.lo.assign(nc, SIZE_MAX);
      a.hi.assign(nc, 0);
      for (int c = 0; c < nc; c++)
        for (int i = cut[c]; i < cut[c + 1]; i++)
          if (a.end[i] > a.beg[i]) {
            a.lo[c] = std::min(a.lo[c], a.beg[i]);
            a.hi[c] = std::max(a.hi[c], a.end[i]);
          }
      for (int c = 0; c < nc; c++)
        if (a.lo[c] == SIZE_MAX) a.lo[c] = a.hi[c] = 0;
    }
  };
  chunk_ranges();
  // Overlapping chunk ranges would let one chunk's upload overwrite another's data.
  bool overlap = false;
  for (auto& a : pp.arr)
    for (size_t c = 0; c < a.lo.size() && !overlap; c++)
      for (size_t d = c + 1; d < a.lo.size() && !overlap; d++)
        overlap = a.lo[c] < a.hi[d] && a.lo[d] < a.hi[c];
  if (overlap) {
    cut = {0, count};
    chunk_ranges();
  }
  for (auto& a : pp.arr) {
    size_t hi = 1;
    for (size_t v : a.hi) hi = std::max(hi, v);
    MFG_CUDA(ctx, a.dev.reserve(a.es * hi));
  }
  MFG_CUDA(ctx, cudaStreamCreateWithFlags(&pp.h2d, cudaStreamNonBlocking));
  MFG_CUDA(ctx, cudaStreamCreateWithFlags(&pp.d2h, cudaStreamNonBlocking));
  for (auto& st : pp.comp) MFG_CUDA(ctx, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  const int nrhs = p->nrhs;
  for (size_t c = 0; c + 1 < cut.size(); c++) {
    const int c0 = cut[c], cnt = cut[c + 1] - cut[c];
    mfg_plan* sub = nullptr;
    auto at = [c0](const std::vector<long long>& v) {
      return v.empty() ? (const int64_t*)nullptr : (const int64_t*)v.data() + c0;
    };
    const int64_t* aoff = at(p->haoff);
    const int64_t* poff = at(p->hpivoff);
    const int64_t* boff = at(p->hboff);
    int rc;
    if (qr)
      rc = plan_create_qr(ctx, &sub, cnt, p->hm.data() + c0, p->hn.data() + c0,
                          p->hlda.data() + c0, aoff, poff, nrhs, nrhs > 0 ? boff : nullptr);
    else if (p->kind == mfg_plan::GEVD)
      rc = plan_create_gevd(ctx, &sub, cnt, p->hn.data() + c0, p->hlda.data() + c0, aoff,
                            p->hldb.data() + c0, boff, at(p->hcoff));
    else
      rc = plan_create(ctx, &sub, p->kind, cnt, p->hn.data() + c0, p->hlda.data() + c0, aoff,
                       poff, nrhs, nrhs > 0 ? boff : nullptr);
    if (rc != MFG_OK) return rc;
    pp.chunk.push_back(sub);
    if (p->kind == mfg_plan::GETRF || p->kind == mfg_plan::POTRF) {
      // Same launch shape as the parent plan (which the autotuner may have chosen), then the
      // element type's scratch.
      // The lanes table (GETRF) or the Cholesky's size-bucket table travel in plan_reshape's
      // group argument, as the autotuner passes them.  LU chunks take 32 lanes for every order
      // (table 0, one launch per chunk): with a two-bucket table each chunk's second launch
      // lengthens the pipeline (e2e 1.10 against 1.13 M matrices/s on the 100,000-matrix batch,
      // 1.37 against 1.46 M in the FMA form).
      const int group = p->kind == mfg_plan::GETRF ? (p->gsel >= 0 ? 0 : -1)
                        : p->csel > 0               ? -p->csel
                                                    : p->args.group;
      rc = plan_reshape(sub, p->warps, std::max(1, p->ctas * p->warps / ctx->sm_count), group,
                        p->args.hw_mul, p->args.dot_block);
      if (rc == MFG_OK) rc = plan_set_elem(sub, pipe_elem(op));
      if (rc == MFG_OK && p->args.fma) rc = plan_set_fma(sub, 1);
      if (rc != MFG_OK) return rc;
    }
    if (p->kind == mfg_plan::GEVD) {
      rc = plan_set_elem(sub, pipe_elem(op));
      if (rc != MFG_OK) return rc;
    }
    if (op == OP_GEQRF_D || op == OP_GEQRF_S) {
      // The parent's (possibly autotuned) lanes per matrix and warps per SM, and its form.
      rc = qr_reshape(sub, p->qd.group, std::max(1, p->ctas * p->warps / ctx->sm_count));
      if (rc != MFG_OK) return rc;
      sub->qd.fma = p->qd.fma;
    }
    if (op == OP_GEQRF_Z) {
      rc = zqr_prepare(sub);
      if (rc != MFG_OK) return rc;
    }
    pp.c0.push_back(c0);
    pp.c1.push_back(c0 + cnt);
    cudaEvent_t e1, e2;
    MFG_CUDA(ctx, cudaEventCreateWithFlags(&e1, cudaEventDisableTiming));
    MFG_CUDA(ctx, cudaEventCreateWithFlags(&e2, cudaEventDisableTiming));
    pp.in.push_back(e1);
    pp.done.push_back(e2);
  }
  pp.op = op;
  return MFG_OK;
}

// Runs operation op on the caller's host arrays (in the order pipe_arrays lists them).
int pipe_run_body(mfg_plan* p, int op, int keep_factor, std::initializer_list<void*> host) {
  mfg_ctx* ctx = p->ctx;
  auto& pp = p->pipe;
  if (pp.op != op) {
    // op % 100 is the operation; the hundreds distinguish variants with other array sets.
    const int rc = pipe_build(p, op % 100, keep_factor);
    if (rc != MFG_OK) {
      pipe_release(p);
      return rc;
    }
    pp.op = op;
  }
  std::vector<char*> h;
  for (void* v : host) h.push_back((char*)v);
  auto dev = [&](int k) { return (char*)pp.arr[k].dev.ptr; };
  for (size_t c = 0; c < pp.chunk.size(); c++) {
    for (size_t k = 0; k < pp.arr.size(); k++) {
      const auto& a = pp.arr[k];
      if ((a.dir & 1) && h[k] && a.hi[c] > a.lo[c])
        MFG_CUDA(ctx, cudaMemcpyAsync(dev((int)k) + a.lo[c] * a.es, h[k] + a.lo[c] * a.es,
                                      (a.hi[c] - a.lo[c]) * a.es, cudaMemcpyDefault, pp.h2d));
    }
    MFG_CUDA(ctx, cudaEventRecord(pp.in[c], pp.h2d));
    // Four compute streams in turn: the kernels of the next chunks fill the SMs that a chunk's
    // last matrices leave idle.
    cudaStream_t sc = (c & 3) ? pp.comp[(c & 3) - 1] : ctx->stream;
    MFG_CUDA(ctx, cudaStreamWaitEvent(sc, pp.in[c], 0));
    mfg_plan* sub = pp.chunk[c];
    const int c0 = pp.c0[c];
    int rc = MFG_OK;
    switch (op % 100) {
      case OP_GETRF:
      case OP_GETRF_S:
      case OP_GETRF_Z:
        sub->args.a = (double*)dev(0);
        sub->args.b = p->nrhs > 0 ? (double*)dev(1) : nullptr;
        sub->args.piv = (int*)dev(2);
        sub->args.sign = (int*)dev(3) + c0;
        sub->args.info = (int*)dev(4) + c0;
        sub->args.solve_only = 0;
        rc = plan_launch(sub, sc);
        break;
      case OP_POTRF:
      case OP_POTRF_S:
      case OP_POTRF_Z:
        sub->args.a = (double*)dev(0);
        sub->args.b = p->nrhs > 0 ? (double*)dev(1) : nullptr;
        sub->args.info = (int*)dev(2) + c0;
        sub->args.solve_only = 0;
        rc = plan_launch(sub, sc);
        break;
      case OP_GRAD: {
        BatchArgs a = sub->args;
        a.a = (double*)dev(0);
        a.b = (double*)dev(1);
        a.info = (int*)dev(4) + c0;
        MFG_CUDA(ctx, cudaMemsetAsync(a.queue, 0, sizeof(int), sc));
        const int wpc = mfg::grad_warps_per_cta();
        const long long ctas = std::min<long long>(
            (long long)ctx->sm_count * mfg::grad_ctas_per_sm(), ((long long)sub->count + wpc - 1) / wpc);
        MFG_CUDA(ctx, mfg::launch_chol_grad_batched(a, (double*)dev(2) + c0, (double*)dev(3),
                                                    keep_factor ? 1 : 0,
                                                    (int)std::max<long long>(1, ctas), sc));
        break;
      }
      case OP_GETRI:
        sub->args.a = (double*)dev(0);
        sub->args.piv = (int*)dev(1);
        sub->args.info = (int*)dev(2) + c0;
        rc = plan_launch(sub, sc);
        break;
      case OP_GEQRF_D:
        sub->qr_float = 0;
        sub->qd.a = (double*)dev(0);
        sub->qd.rdiag = (double*)dev(1);
        sub->qd.b = p->nrhs > 0 ? (double*)dev(2) : nullptr;
        sub->qd.solve_only = 0;
        rc = plan_launch(sub, sc);
        break;
      case OP_GEQRF_S:
        sub->qr_float = 1;
        sub->qs.a = (float*)dev(0);
        sub->qs.rdiag = (float*)dev(1);
        sub->qs.b = p->nrhs > 0 ? (float*)dev(2) : nullptr;
        sub->qs.solve_only = 0;
        rc = plan_launch(sub, sc);
        break;
      case OP_GEQRF_Z:
        sub->qr_float = 2;
        sub->qz.a = (double*)dev(0);
        sub->qz.rdiag = (double*)dev(1);
        sub->qz.b = p->nrhs > 0 ? (double*)dev(2) : nullptr;
        sub->qz.solve_only = 0;
        rc = plan_launch(sub, sc);
        break;
      case OP_GEVD:
      case OP_GEVD_S:
      case OP_GEVD_Z:
        sub->gv.a = (const double*)dev(0);
        sub->gv.b = (double*)dev(1);
        sub->gv.c = (double*)dev(2);
        sub->gv.info = (int*)dev(3) + c0;
        rc = plan_launch(sub, sc);
        break;
    }
    if (rc != MFG_OK) return rc;
    MFG_CUDA(ctx, cudaEventRecord(pp.done[c], sc));
    MFG_CUDA(ctx, cudaStreamWaitEvent(pp.d2h, pp.done[c], 0));
    for (size_t k = 0; k < pp.arr.size(); k++) {
      const auto& a = pp.arr[k];
      if ((a.dir & 2) && h[k] && a.hi[c] > a.lo[c])
        MFG_CUDA(ctx, cudaMemcpyAsync(h[k] + a.lo[c] * a.es, dev((int)k) + a.lo[c] * a.es,
                                      (a.hi[c] - a.lo[c]) * a.es, cudaMemcpyDefault, pp.d2h));
    }
  }
  MFG_CUDA(ctx, cudaStreamSynchronize(pp.d2h));
  return MFG_OK;
}

// A host-buffer call returns only when none of its copies can still touch the caller's arrays:
// on a failure part-way through, the copies and kernels queued for earlier chunks are drained
// first (their own errors are ignored; the first failure is the one reported).
int pipe_run(mfg_plan* p, int op, int keep_factor, std::initializer_list<void*> host) {
  p->last_host = true;
  const int rc = pipe_run_body(p, op, keep_factor, host);
  if (rc != MFG_OK) {
    auto& pp = p->pipe;
    for (cudaStream_t st : {pp.h2d, pp.comp[0], pp.comp[1], pp.comp[2], p->ctx->stream, pp.d2h})
      if (st) cudaStreamSynchronize(st);
  }
  return rc;
}

}  // namespace

extern "C" {

MFG_API int mfg_dgetrf_batched_host(mfg_plan* plan, double* a, int* piv, double* b, int* sign,
                                    int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::GETRF) return fail(ctx, -1, "plan is not a getrf plan");
  if (plan->count == 0) return MFG_OK;
  if (!a) return fail(ctx, -2, "a is null");
  if (!piv) return fail(ctx, -3, "piv is null");
  if (plan->nrhs > 0 && !b) return fail(ctx, -4, "b is null");
  if (!sign) return fail(ctx, -5, "sign is null");
  if (!info) return fail(ctx, -6, "info is null");
  return pipe_run(plan, OP_GETRF, 0, {a, b, piv, sign, info});
}

static int getrf_host_any(mfg_plan* plan, int op, void* a, int* piv, void* b, int* sign,
                          int* info) {
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::GETRF) return fail(ctx, -1, "plan is not a getrf plan");
  if (plan->count == 0) return MFG_OK;
  if (!a) return fail(ctx, -2, "a is null");
  if (!piv) return fail(ctx, -3, "piv is null");
  if (plan->nrhs > 0 && !b) return fail(ctx, -4, "b is null");
  if (!sign) return fail(ctx, -5, "sign is null");
  if (!info) return fail(ctx, -6, "info is null");
  return pipe_run(plan, op, 0, {a, b, piv, sign, info});
}

static int potrf_host_any(mfg_plan* plan, int op, void* a, void* b, int* info) {
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::POTRF) return fail(ctx, -1, "plan is not a potrf plan");
  if (plan->count == 0) return MFG_OK;
  if (!a) return fail(ctx, -2, "a is null");
  if (plan->nrhs > 0 && !b) return fail(ctx, -3, "b is null");
  if (!info) return fail(ctx, -4, "info is null");
  return pipe_run(plan, op, 0, {a, b, info});
}

MFG_API int mfg_sgetrf_batched_host(mfg_plan* plan, float* a, int* piv, float* b, int* sign,
                                    int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return getrf_host_any(plan, OP_GETRF_S, a, piv, b, sign, info);
}
MFG_API int mfg_zgetrf_batched_host(mfg_plan* plan, double* a, int* piv, double* b, int* sign,
                                    int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return getrf_host_any(plan, OP_GETRF_Z, a, piv, b, sign, info);
}
MFG_API int mfg_spotrf_batched_host(mfg_plan* plan, float* a, float* b, int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return potrf_host_any(plan, OP_POTRF_S, a, b, info);
}
MFG_API int mfg_zpotrf_batched_host(mfg_plan* plan, double* a, double* b, int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return potrf_host_any(plan, OP_POTRF_Z, a, b, info);
}
MFG_API int mfg_zgeqrf_batched_host(mfg_plan* plan, double* a, double* rdiag, double* b) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::GEQRF) return fail(ctx, -1, "plan is not a geqrf plan");
  if (plan->count == 0) return MFG_OK;
  if (!a) return fail(ctx, -2, "a is null");
  if (!rdiag) return fail(ctx, -3, "rdiag is null");
  if (plan->nrhs > 0 && !b) return fail(ctx, -4, "b is null");
  return pipe_run(plan, OP_GEQRF_Z, 0, {a, rdiag, b});
}

MFG_API int mfg_dpotrf_batched_host(mfg_plan* plan, double* a, double* b, int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::POTRF) return fail(ctx, -1, "plan is not a potrf plan");
  if (plan->count == 0) return MFG_OK;
  if (!a) return fail(ctx, -2, "a is null");
  if (plan->nrhs > 0 && !b) return fail(ctx, -3, "b is null");
  if (!info) return fail(ctx, -4, "info is null");
  return pipe_run(plan, OP_POTRF, 0, {a, b, info});
}

MFG_API int mfg_dpotrf_logdet_solve_grad_batched_host(mfg_plan* plan, double* k, double* y,
                                                     double* loss, double* grad, int* info,
                                                     int keep_factor) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::POTRF) return fail(ctx, -1, "plan is not a potrf plan");
  if (plan->nrhs != 1) return fail(ctx, -1, "the plan must have nrhs = 1 (the vector y)");
  if (plan->max_n > 128)
    return fail(ctx, MFG_ERR_UNSUPPORTED, "matrix order %d > 128 is not supported here",
                plan->max_n);
  if (plan->count == 0) return MFG_OK;
  if (!k) return fail(ctx, -2, "k is null");
  if (!y) return fail(ctx, -3, "y is null");
  if (!loss) return fail(ctx, -4, "loss is null");
  if (!grad) return fail(ctx, -5, "grad is null");
  if (!info) return fail(ctx, -6, "info is null");
  if ((void*)grad == (void*)k) return fail(ctx, -5, "grad must not alias k");
  // keep_factor changes which arrays come back, hence its own pipe variant.
  return pipe_run(plan, OP_GRAD + (keep_factor ? 0 : 100), keep_factor ? 1 : 0,
                  {k, y, loss, grad, info});
}

MFG_API int mfg_dgetri_batched_host(mfg_plan* plan, double* a, const int* piv, int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::GETRI) return fail(ctx, -1, "plan is not a getri plan");
  if (plan->count == 0) return MFG_OK;
  if (!a) return fail(ctx, -2, "a is null");
  if (!piv) return fail(ctx, -3, "piv is null");
  if (!info) return fail(ctx, -4, "info is null");
  return pipe_run(plan, OP_GETRI, 0, {a, const_cast<int*>(piv), info});
}

MFG_API int mfg_dgeqrf_batched_host(mfg_plan* plan, double* a, double* rdiag, double* b) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::GEQRF) return fail(ctx, -1, "plan is not a geqrf plan");
  if (plan->count == 0) return MFG_OK;
  if (!a) return fail(ctx, -2, "a is null");
  if (!rdiag) return fail(ctx, -3, "rdiag is null");
  if (plan->nrhs > 0 && !b) return fail(ctx, -4, "b is null");
  return pipe_run(plan, OP_GEQRF_D, 0, {a, rdiag, b});
}

MFG_API int mfg_sgeqrf_batched_host(mfg_plan* plan, float* a, float* rdiag, float* b) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::GEQRF) return fail(ctx, -1, "plan is not a geqrf plan");
  if (plan->count == 0) return MFG_OK;
  if (!a) return fail(ctx, -2, "a is null");
  if (!rdiag) return fail(ctx, -3, "rdiag is null");
  if (plan->nrhs > 0 && !b) return fail(ctx, -4, "b is null");
  return pipe_run(plan, OP_GEQRF_S, 0, {a, rdiag, b});
}

}  // extern "C"

static int gevd_front_host_any(mfg_plan* plan, int op, const void* a, void* b, void* c,
                               int* info) {
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::GEVD) return fail(ctx, -1, "plan is not a gevd plan");
  if (plan->count == 0) return MFG_OK;
  if (!a) return fail(ctx, -2, "a is null");
  if (!b) return fail(ctx, -3, "b is null");
  if (!c) return fail(ctx, -4, "c is null");
  if (!info) return fail(ctx, -5, "info is null");
  return pipe_run(plan, op, 0, {const_cast<void*>(a), b, c, info});
}

extern "C" {

MFG_API int mfg_dgevd_front_batched_host(mfg_plan* plan, const double* a, double* b, double* c,
                                         int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return gevd_front_host_any(plan, OP_GEVD, a, b, c, info);
}
MFG_API int mfg_sgevd_front_batched_host(mfg_plan* plan, const float* a, float* b, float* c,
                                         int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return gevd_front_host_any(plan, OP_GEVD_S, a, b, c, info);
}
MFG_API int mfg_zgevd_front_batched_host(mfg_plan* plan, const double* a, double* b, double* c,
                                         int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return gevd_front_host_any(plan, OP_GEVD_Z, a, b, c, info);
}

}  // extern "C"

namespace {

int potrf_batched_any(mfg_plan* plan, int elem, void* a, void* b, int* info) {
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::POTRF) return fail(ctx, -1, "plan is not a potrf plan");
  if (plan->count > 0) {
    if (!a) return fail(ctx, -2, "a is null");
    if (plan->nrhs > 0 && !b) return fail(ctx, -3, "b is null");
    if (!info) return fail(ctx, -4, "info is null");
  }
  const int rc = plan_set_elem(plan, elem);
  if (rc != MFG_OK) return rc;
  plan->args.a = (double*)a;
  plan->args.piv = nullptr;
  plan->args.b = (double*)b;
  plan->args.sign = nullptr;
  plan->args.info = info;
  plan->args.solve_only = 0;
  return plan_execute(plan, a, b, info, nullptr, nullptr);
}

int potrs_batched_any(mfg_plan* plan, int elem, const void* a, void* b) {
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::POTRF) return fail(ctx, -1, "plan is not a potrf plan");
  if (plan->nrhs < 1) return fail(ctx, -1, "the plan has no right-hand sides (nrhs = 0)");
  if (plan->count > 0) {
    if (!a) return fail(ctx, -2, "a is null");
    if (!b) return fail(ctx, -3, "b is null");
  }
  const int rc = plan_set_elem(plan, elem);
  if (rc != MFG_OK) return rc;
  plan->args.a = (double*)const_cast<void*>(a);
  plan->args.piv = nullptr;
  plan->args.b = (double*)b;
  plan->args.sign = nullptr;
  plan->args.info = nullptr;
  plan->args.solve_only = 1;
  return plan_execute(plan, a, b, nullptr, (const void*)3, nullptr);
}

}  // namespace

extern "C" {

MFG_API int mfg_spotrf_batched(mfg_plan* plan, float* a, float* b, int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return potrf_batched_any(plan, 1, a, b, info);
}
MFG_API int mfg_zpotrf_batched(mfg_plan* plan, double* a, double* b, int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return potrf_batched_any(plan, 2, a, b, info);
}
MFG_API int mfg_spotrs_batched(mfg_plan* plan, const float* a, float* b) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return potrs_batched_any(plan, 1, a, b);
}
MFG_API int mfg_zpotrs_batched(mfg_plan* plan, const double* a, double* b) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  return potrs_batched_any(plan, 2, a, b);
}

MFG_API int mfg_dpotrf_batched(mfg_plan* plan, double* a, double* b, int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::POTRF) return fail(ctx, -1, "plan is not a potrf plan");
  if (plan->count > 0) {
    if (!a) return fail(ctx, -2, "a is null");
    if (plan->nrhs > 0 && !b) return fail(ctx, -3, "b is null");
    if (!info) return fail(ctx, -4, "info is null");
  }
  const int rc = plan_set_elem(plan, 0);
  if (rc != MFG_OK) return rc;
  plan->args.a = a;
  plan->args.piv = nullptr;
  plan->args.b = b;
  plan->args.sign = nullptr;
  plan->args.info = info;
  plan->args.solve_only = 0;
  return plan_execute(plan, a, b, info, nullptr, nullptr);
}

MFG_API int mfg_dpotrs_batched(mfg_plan* plan, const double* a, double* b) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::POTRF) return fail(ctx, -1, "plan is not a potrf plan");
  if (plan->nrhs < 1) return fail(ctx, -1, "the plan has no right-hand sides (nrhs = 0)");
  if (plan->count > 0) {
    if (!a) return fail(ctx, -2, "a is null");
    if (!b) return fail(ctx, -3, "b is null");
  }
  const int rc = plan_set_elem(plan, 0);
  if (rc != MFG_OK) return rc;
  plan->args.a = const_cast<double*>(a);
  plan->args.piv = nullptr;
  plan->args.b = b;
  plan->args.sign = nullptr;
  plan->args.info = nullptr;
  plan->args.solve_only = 1;
  return plan_execute(plan, a, b, nullptr, (const void*)3, nullptr);
}

MFG_API int mfg_selftest_dmul(mfg_ctx* ctx, const double* a, const double* b, double* out,
                              int64_t n) {
  DeviceScope device_scope_(ctx);
  if (!ctx) return -1;
  if (n < 0) return fail(ctx, -5, "n must be >= 0");
  if (n > 0 && (!a || !b || !out)) return fail(ctx, !a ? -2 : (!b ? -3 : -4), "null pointer");
  MFG_CUDA(ctx, mfg::launch_selftest_mul(a, b, out, n, ctx->stream));
  return MFG_OK;
}

MFG_API int mfg_selftest_ddiv(mfg_ctx* ctx, const double* a, const double* b, double* out,
                              int64_t n) {
  DeviceScope device_scope_(ctx);
  if (!ctx) return -1;
  if (n < 0) return fail(ctx, -5, "n must be >= 0");
  if (n > 0 && (!a || !b || !out)) return fail(ctx, !a ? -2 : (!b ? -3 : -4), "null pointer");
  MFG_CUDA(ctx, mfg::launch_selftest_div(a, b, out, n, ctx->stream));
  return MFG_OK;
}

MFG_API int mfg_dgetrf_strided_batched_noalloc(mfg_ctx* ctx, int n, int count, double* a,
                                              int lda, int64_t stride_a, int* piv,
                                              int64_t stride_piv, int nrhs, double* b,
                                              int64_t stride_b, int* sign, int* info) {
  DeviceScope device_scope_(ctx);
  if (!ctx) return -1;
  if (n < 1) return fail(ctx, -2, "n must be >= 1");
  if (n > mfg::noalloc_max_n())
    return fail(ctx, MFG_ERR_UNSUPPORTED,
                "n = %d exceeds the allocation-free limit of %d (use the plan entry points)", n,
                mfg::noalloc_max_n());
  if (count < 0) return fail(ctx, -3, "count must be >= 0");
  if (count > 0 && !a) return fail(ctx, -4, "a is null");
  if (lda < n) return fail(ctx, -5, "lda = %d < n = %d", lda, n);
  if (count > 1 && stride_a < (int64_t)lda * n) return fail(ctx, -6, "stride_a too small");
  if (count > 0 && !piv) return fail(ctx, -7, "piv is null");
  if (count > 1 && stride_piv < n) return fail(ctx, -8, "stride_piv too small");
  if (nrhs < 0) return fail(ctx, -9, "nrhs must be >= 0");
  if (nrhs > 0 && count > 0 && !b) return fail(ctx, -10, "b is null");
  if (nrhs > 0 && count > 1 && stride_b < (int64_t)n * nrhs)
    return fail(ctx, -11, "stride_b too small");
  if (count > 0 && !sign) return fail(ctx, -12, "sign is null");
  if (count > 0 && !info) return fail(ctx, -13, "info is null");
  MFG_CUDA(ctx, mfg::launch_getrf_strided_noalloc(a, n, lda, stride_a, piv, stride_piv, nrhs, b,
                                                  stride_b, sign, info, count, ctx->device,
                                                  ctx->sm_count, ctx->stream));
  return MFG_OK;
}

MFG_API int mfg_dpotrf_logdet_solve_grad_batched(mfg_plan* plan, double* k, double* y,
                                                double* loss, double* grad, int* info,
                                                int keep_factor) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::POTRF) return fail(ctx, -1, "plan is not a potrf plan");
  if (plan->nrhs != 1) return fail(ctx, -1, "the plan must have nrhs = 1 (the vector y)");
  if (plan->max_n > 128)
    return fail(ctx, MFG_ERR_UNSUPPORTED, "matrix order %d > 128 is not supported here",
                plan->max_n);
  if (plan->count > 0) {
    if (!k) return fail(ctx, -2, "k is null");
    if (!y) return fail(ctx, -3, "y is null");
    if (!loss) return fail(ctx, -4, "loss is null");
    if (!grad) return fail(ctx, -5, "grad is null");
    if (!info) return fail(ctx, -6, "info is null");
    if ((void*)grad == (void*)k) return fail(ctx, -5, "grad must not alias k");
  }
  cudaStream_t s = ctx->stream;
  MFG_CUDA(ctx, cudaMemsetAsync(plan->args.queue, 0, sizeof(int), s));
  if (plan->count == 0) return MFG_OK;
  BatchArgs a = plan->args;
  a.a = k;
  a.b = y;
  a.info = info;
  const int wpc = mfg::grad_warps_per_cta();
  const long long ctas = std::min<long long>((long long)ctx->sm_count * mfg::grad_ctas_per_sm(),
                                             ((long long)plan->count + wpc - 1) / wpc);
  MFG_CUDA(ctx, mfg::launch_chol_grad_batched(a, loss, grad, keep_factor ? 1 : 0,
                                              (int)std::max<long long>(1, ctas), s));
  return MFG_OK;
}


MFG_API int mfg_dpotrf_backward_batched(mfg_plan* plan, double* a, const double* lbar,
                                        const double* logdet_bar, const double* x,
                                        const double* xbar, double* abar, double* bbar,
                                        int* info, int recompute) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::POTRF) return fail(ctx, -1, "plan is not a potrf plan");
  if (plan->max_n > mfg::chol_backward_max_n())
    return fail(ctx, MFG_ERR_UNSUPPORTED, "matrix order %d > %d is not supported here",
                plan->max_n, mfg::chol_backward_max_n());
  if (plan->count == 0) return MFG_OK;
  if (!a) return fail(ctx, -2, "a is null");
  if (xbar && !x) return fail(ctx, -5, "x is null (needed with xbar)");
  if (xbar && plan->nrhs < 1)
    return fail(ctx, -6, "xbar needs a plan with right-hand-side offsets (nrhs >= 1)");
  if (!abar) return fail(ctx, -7, "abar is null");
  if ((const void*)abar == (const void*)a || (const void*)abar == (const void*)lbar)
    return fail(ctx, -7, "abar must not alias a or lbar");
  if (!info) return fail(ctx, -9, "info is null");
  cudaStream_t s = ctx->stream;
  if (recompute) {
    // L = Cholesky(A) in place, MatFlat's arithmetic (the plan's forward kernel, no solve).
    BatchArgs f = plan->args;
    f.a = a;
    f.b = nullptr;
    f.nrhs = 0;
    f.info = info;
    f.solve_only = 0;
    MFG_CUDA(ctx, cudaMemsetAsync(f.queue, 0, sizeof(int), s));
    MFG_CUDA(ctx, mfg::launch_potrf_batched(f, plan->ctas, plan->warps, s));
  } else {
    MFG_CUDA(ctx, cudaMemsetAsync(info, 0, sizeof(int) * plan->count, s));
  }
  mfg::CholBwdArgs b{};
  b.order = plan->args.order;
  b.n = plan->args.n;
  b.lda = plan->args.lda;
  b.a_off = plan->args.a_off;
  b.b_off = plan->args.b_off;
  b.l = a;
  b.lbar = lbar;
  b.logdet_bar = logdet_bar;
  b.x = xbar ? x : nullptr;
  b.xbar = xbar;
  b.abar = abar;
  b.bbar = plan->nrhs > 0 ? bbar : nullptr;
  b.info = info;
  b.count = plan->count;
  b.queue = plan->args.queue;
  MFG_CUDA(ctx, cudaMemsetAsync(b.queue, 0, sizeof(int), s));
  // CTAs of 128 threads per SM: the kernel's 48 registers let 10 fit, and the reverse pass
  // (latency-bound per-thread sweeps) gains with every one: 4,096 x n=128 in the FMA form, 37.2 /
  // 32.5 / 30.7 / 29.5 / 28.5 ms with 2 / 4 / 6 / 8 / 10.  MFG_BWD_CTAS_PER_SM overrides.
  const int cps = std::max(1, std::min(10, env_int("MFG_BWD_CTAS_PER_SM", 10)));
  const int ctas = (int)std::min<long long>((long long)ctx->sm_count * cps, plan->count);
  MFG_CUDA(ctx, mfg::launch_chol_backward(b, std::max(1, ctas), s));
  return MFG_OK;
}

// ------------------------------------------------------------------------------------------
// Mixed-precision LU solve with FP64 iterative refinement.

}  // extern "C"

namespace {
// Workspace layout of a mixed plan (one allocation at plan creation; nothing is allocated by a
// solve).
struct MixedLayout {
  float* a32;
  int* ipiv;
  void* op_a;
  void* op_b;
  void* op_a2;      // split TF32: the low parts
  void* op_b2;
  double* anorm;
  int* state;
  int* active;
  int* status;      // set by a bounded device-side wait that gave up
  double* fb_a;     // fallback: copies of the systems that did not converge
  int* fb_piv;
  int* fb_sign;
  int* fb_info;
  int* fb_order;
  int* fb_count;
};

MixedLayout mixed_layout(void* base, int count, int n, size_t* bytes) {
  Carve cv(base);
  const size_t nn = (size_t)n * n * count;
  const size_t ops = (size_t)mfg::mx_op_rows(n) * mfg::mx_panel_width() * count;
  MixedLayout L;
  L.a32 = cv.take<float>(nn);
  L.ipiv = cv.take<int>((size_t)n * count);
  L.op_a = cv.take<float>(ops);
  L.op_b = cv.take<float>(ops);
  L.op_a2 = cv.take<float>(ops);
  L.op_b2 = cv.take<float>(ops);
  L.anorm = cv.take<double>(count);
  L.state = cv.take<int>(count);
  L.active = cv.take<int>(count);
  L.status = cv.take<int>(64);
  L.fb_a = cv.take<double>(nn);
  L.fb_piv = cv.take<int>((size_t)n * count);
  L.fb_sign = cv.take<int>(count);
  L.fb_info = cv.take<int>(count);
  L.fb_order = cv.take<int>(count);
  L.fb_count = cv.take<int>(64);
  if (bytes) *bytes = cv.used();
  return L;
}

int mixed_plan_setup(mfg_ctx* ctx, mfg_plan* p) {
  const int n = p->mx_n, count = p->count;
  size_t bytes = 0;
  mixed_layout(nullptr, count, n, &bytes);
  MFG_CUDA(ctx, p->mx_work.reserve(bytes + 256));
  MFG_CUDA(ctx, cudaMemset(p->mx_work.ptr, 0, bytes + 256));
  MFG_CUDA(ctx, p->meta.reserve(256));
  MFG_CUDA(ctx, mfg::mx_panel_attr(1024));
  p->args.queue = (int*)p->meta.ptr;
  const MixedLayout L = mixed_layout(p->mx_work.ptr, count, n, nullptr);
  if (count > 0) {
    MFG_CUDA(ctx, mfg::mx_make_tensor_maps(L.op_a, L.op_b, n, count, true, &p->mx_tm[0],
                                           &p->mx_tm[1]));
    MFG_CUDA(ctx, mfg::mx_make_tensor_maps(L.op_a, L.op_b, n, count, false, &p->mx_tm[2],
                                           &p->mx_tm[3]));
    MFG_CUDA(ctx, mfg::mx_make_tensor_maps(L.op_a2, L.op_b2, n, count, true, &p->mx_tm[4],
                                           &p->mx_tm[5]));
    MFG_CUDA(ctx, mfg::mx_tc_attr());
    // The fallback's exact FP64 LU over every system slot (only the listed ones run).
    std::vector<int> nn(count, n);
    std::vector<int64_t> aoff(count), poff(count);
    for (int q = 0; q < count; q++) {
      aoff[q] = (int64_t)q * n * n;
      poff[q] = (int64_t)q * n;
    }
    const int rc = plan_create(ctx, &p->mx_fb, mfg_plan::GETRF, count, nn.data(), nullptr,
                               aoff.data(), poff.data(), 1, poff.data());
    if (rc != MFG_OK) return rc;
  }
  return MFG_OK;
}
}  // namespace

extern "C" {

MFG_API int mfg_plan_gesv_mixed_batched(mfg_ctx* ctx, mfg_plan** plan, int count, int n) {
  DeviceScope device_scope_(ctx);
  if (!ctx) return -1;
  if (!plan) return fail(ctx, -2, "plan output pointer is null");
  *plan = nullptr;
  if (count < 0) return fail(ctx, -3, "count must be >= 0");
  const int nb = mfg::mx_panel_width();
  if (n < nb || n > 1024 || n % nb != 0)
    return fail(ctx, -4, "n = %d: the mixed solver takes multiples of %d up to 1024", n, nb);
  mfg_plan* p = new mfg_plan();
  p->kind = mfg_plan::MIXED;
  p->ctx = ctx;
  p->count = count;
  p->nrhs = 1;
  p->mx_n = n;
  p->max_n = n;
  const int rc = mixed_plan_setup(ctx, p);
  if (rc != MFG_OK) {
    mfg_plan_destroy(p);
    return rc;
  }
  *plan = p;
  return MFG_OK;
}

MFG_API int mfg_dgesv_mixed_batched(mfg_plan* plan, const double* a, const double* b, double* x,
                                    int lowp, int max_iter, double tol, double* berr,
                                    int* iters, int* info) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  if (plan->kind != mfg_plan::MIXED) return fail(ctx, -1, "plan is not a mixed-precision plan");
  if (plan->count == 0) return MFG_OK;
  if (!a) return fail(ctx, -2, "a is null");
  if (!b) return fail(ctx, -3, "b is null");
  if (!x) return fail(ctx, -4, "x is null");
  if (lowp != MFG_LOWP_FP32 && lowp != MFG_LOWP_TF32 && lowp != MFG_LOWP_BF16 &&
      lowp != MFG_LOWP_TF32X3)
    return fail(ctx, -5, "unknown low precision %d", lowp);
  if (max_iter < 0) return fail(ctx, -6, "max_iter must be >= 0");
  if (!(tol > 0)) return fail(ctx, -7, "tol must be > 0");
  if (!berr) return fail(ctx, -8, "berr is null");
  if (!iters) return fail(ctx, -9, "iters is null");
  if (!info) return fail(ctx, -10, "info is null");
  const int n = plan->mx_n, count = plan->count, nb = mfg::mx_panel_width();
  cudaStream_t s = ctx->stream;
  const MixedLayout L = mixed_layout(plan->mx_work.ptr, count, n, nullptr);
  const int opfmt = lowp == MFG_LOWP_TF32 ? 1 : lowp == MFG_LOWP_BF16 ? 2
                  : lowp == MFG_LOWP_TF32X3 ? 3 : 0;
  // TMA maps of the mode: high parts (or the only parts) first, then the split mode's low parts.
  const CUtensorMap tm[4] = {plan->mx_tm[opfmt == 2 ? 2 : 0], plan->mx_tm[opfmt == 2 ? 3 : 1],
                             plan->mx_tm[4], plan->mx_tm[5]};
  const int R = mfg::mx_op_rows(n);
  MFG_CUDA(ctx, mfg::mx_round(a, L.a32, (long long)n * n * count, s));
  for (int k = 0; k < n; k += nb) {
    MFG_CUDA(ctx, mfg::mx_panel(L.a32, n, k, L.ipiv, nullptr, count, L.op_a, L.op_b, L.op_a2,
                                L.op_b2, opfmt, R, s));
    if (n - k - nb <= 0) continue;
    if (opfmt == 0) {
      MFG_CUDA(ctx, mfg::mx_update_fp32(L.a32, n, k, nullptr, count, s));
    } else {
      MFG_CUDA(ctx, mfg::mx_update_tc(tm, L.a32, n, k, opfmt == 1 ? 0 : opfmt == 2 ? 1 : 2, count,
                                      L.status, s));
    }
  }
  MFG_CUDA(ctx, cudaMemsetAsync(L.active, 0xFF, sizeof(int) * count, s));
  MFG_CUDA(ctx, mfg::mx_refine(a, b, x, L.a32, L.ipiv, n, count, -1, tol, berr, iters, L.state,
                               L.anorm, L.active, s));
  for (int it = 0; it <= max_iter; ++it)
    MFG_CUDA(ctx, mfg::mx_refine(a, b, x, L.a32, L.ipiv, n, count, it, tol, berr, iters, L.state,
                                 L.anorm, L.active, s));
  // Systems that did not converge (stalled, diverged, out of iterations, singular low-precision
  // factor) are solved again with the exact FP64 LU, entirely on the device.
  MFG_CUDA(ctx, cudaMemsetAsync(L.fb_count, 0, sizeof(int), s));
  MFG_CUDA(ctx, mfg::mx_fb_gather(a, b, x, L.fb_a, L.state, n, count, L.fb_order, L.fb_count, s));
  // The listed systems, one per CTA (a few systems would otherwise leave most SMs idle).
  mfg_plan* fp = plan->mx_fb;
  BatchArgs fa = fp->args;
  fa.a = L.fb_a;
  fa.piv = L.fb_piv;
  fa.b = x;
  fa.sign = L.fb_sign;
  fa.info = L.fb_info;
  fa.solve_only = 0;
  fa.order = L.fb_order;
  fa.dcount = L.fb_count;
  fa.task_first = nullptr;
  MFG_CUDA(ctx, cudaMemsetAsync(fa.queue, 0, sizeof(int), s));
  const long long slices = (long long)fp->ctas * fp->warps;
  const int fctas = (int)std::max<long long>(
      1, std::min<long long>({(long long)count, 2LL * ctx->sm_count, slices}));
  MFG_CUDA(ctx, mfg::launch_getrf_cta(fa, fctas, n, s));
  MFG_CUDA(ctx, mfg::mx_fb_finish(L.state, info, L.fb_info, count, s));
  // Backward error of the FP64 solutions: one measuring sweep (no correction) over them.
  MFG_CUDA(ctx, mfg::mx_refine(a, b, x, L.a32, L.ipiv, n, count, -2, tol, berr, iters, L.state,
                               L.anorm, L.active, s));
  return MFG_OK;
}

MFG_API int mfg_plan_status(mfg_plan* plan) {
  DeviceScope device_scope_(plan ? plan->ctx : nullptr);
  if (!plan) return -1;
  mfg_ctx* ctx = plan->ctx;
  MFG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  MFG_CUDA(ctx, cudaGetLastError());
  if (plan->kind == mfg_plan::MIXED && plan->count > 0) {
    const MixedLayout L = mixed_layout(plan->mx_work.ptr, plan->count, plan->mx_n, nullptr);
    int st = 0;
    MFG_CUDA(ctx, cudaMemcpy(&st, L.status, sizeof(int), cudaMemcpyDeviceToHost));
    if (st != 0) {
      MFG_CUDA(ctx, cudaMemset(L.status, 0, sizeof(int)));
      return fail(ctx, MFG_ERR_TIMEOUT,
                  "a bounded device-side wait of the tensor-core update gave up (%s); the "
                  "solutions of that execution are not valid",
                  st == 1 ? "operand tiles" : "tensor-core result");
    }
  }
  return MFG_OK;
}

}  // extern "C"
