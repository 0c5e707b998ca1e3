// Synthetic inputs for the launch-shape autotuner (mfg_plan_autotune): a batch with the plan's
// sizes whose entries are uniform in (-1, 1), drawn from a counter hash (the SplitMix64
// finaliser of seed, matrix and element index), so every candidate shape sees the same bytes.
// Cholesky plans get a diagonal of n + 1: with off-diagonal entries below 1 in magnitude the
// matrix is strictly diagonally dominant with a positive diagonal, hence positive definite.
#include <cuda_runtime.h>

#include "mf_device.cuh"
#include "mf_kernels.h"

namespace mfg {

__device__ __forceinline__ double tune_uniform(unsigned long long seed, long long mat, long long e) {
  unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(mat + 1) +
                         0xBF58476D1CE4E5B9ull * (unsigned long long)(e + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * 0x1.0p-52 - 1.0;  // (z >> 11) / 2^53 * 2 - 1
}

// One warp per matrix (grid-stride over the batch).
__global__ void tune_fill_kernel(BatchArgs p, int spd, unsigned long long seed) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long mat = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
       mat < p.count; mat += warps) {
    const int n = p.n[mat];
    const long long lda = p.lda[mat];
    double* a = p.a + p.a_off[mat];
    for (long long e = lane; e < (long long)n * n; e += 32) {
      const int j = (int)(e / n);
      const int i = (int)(e - (long long)j * n);
      a[(long long)j * lda + i] = (spd && i == j) ? (double)n + 1.0 : tune_uniform(seed, mat, e);
    }
    if (p.nrhs > 0) {
      double* b = p.b + p.b_off[mat];
      for (long long e = lane; e < (long long)n * p.nrhs; e += 32)
        b[e] = tune_uniform(seed ^ 0x5555555555555555ull, mat, e);
    }
  }
}

cudaError_t launch_tune_fill(const BatchArgs& args, int spd, cudaStream_t s) {
  if (args.count <= 0) return cudaSuccess;
  long long blocks = ((long long)args.count + 7) / 8;
  if (blocks > 4096) blocks = 4096;
  tune_fill_kernel<<<(unsigned)blocks, 256, 0, s>>>(args, spd, 0x243F6A8885A308D3ull);
  return cudaGetLastError();
}

// QR plans: A (m-by-n, leading dimension lda) and the right-hand sides (m per column) uniform in
// (-1, 1), one warp per matrix.
__global__ void tune_fill_qr_kernel(QrBatchArgs<double> p, unsigned long long seed) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long mat = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
       mat < p.count; mat += warps) {
    const int m = p.m[mat], n = p.n[mat];
    const long long lda = p.lda[mat];
    double* a = p.a + p.a_off[mat];
    for (long long e = lane; e < (long long)m * n; e += 32) {
      const int j = (int)(e / m);
      const int i = (int)(e - (long long)j * m);
      a[(long long)j * lda + i] = tune_uniform(seed, mat, e);
    }
    if (p.nrhs > 0) {
      double* b = p.b + p.b_off[mat];
      for (long long e = lane; e < (long long)m * p.nrhs; e += 32)
        b[e] = tune_uniform(seed ^ 0x5555555555555555ull, mat, e);
    }
  }
}

cudaError_t launch_tune_fill_qr(const QrBatchArgs<double>& args, cudaStream_t s) {
  if (args.count <= 0) return cudaSuccess;
  long long blocks = ((long long)args.count + 7) / 8;
  if (blocks > 4096) blocks = 4096;
  tune_fill_qr_kernel<<<(unsigned)blocks, 256, 0, s>>>(args, 0x13198A2E03707344ull);
  return cudaGetLastError();
}

}  // namespace mfg
