/* Seeded synthetic inputs for the benchmark and the tests (host code, not part of the C ABI).
 *
 * Counter-based generator: element i of stream `stream` under `seed` is
 * SplitMix64(seed + (stream << 40) + i), so any slice can be generated independently and in
 * parallel and every run sees the same bytes.  SplitMix64 is the published mixer of Steele, Lea
 * and Flood ("Fast splittable pseudorandom number generators", OOPSLA 2014).  Normal deviates use
 * the Box–Muller transform on pairs of uniforms.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

/* Uniform in [0, 1) with 53 random bits. */
static inline double u01(uint64_t seed, uint64_t stream, uint64_t i) {
  return (double)(splitmix64(seed + (stream << 40) + i) >> 11) * (1.0 / 9007199254740992.0);
}

static inline double normal_at(uint64_t seed, uint64_t stream, uint64_t i) {
  /* Box–Muller on the uniform pair (2k, 2k+1); even i takes the cosine branch. */
  const uint64_t k = i >> 1;
  const double u1 = 1.0 - u01(seed, stream, 2 * k);      /* (0, 1] */
  const double u2 = u01(seed, stream, 2 * k + 1);
  const double r = sqrt(-2.0 * log(u1));
  const double t = 6.283185307179586 * u2;
  return (i & 1) ? r * sin(t) : r * cos(t);
}

typedef struct {
  double* out;
  int64_t begin, end;
  uint64_t seed, stream, offset;
  double lo, hi;
  int kind; /* 0 normal, 1 uniform */
} job_t;

static void* run_job(void* p) {
  job_t* j = (job_t*)p;
  for (int64_t i = j->begin; i < j->end; i++) {
    const uint64_t idx = j->offset + (uint64_t)i;
    j->out[i] = j->kind == 0 ? normal_at(j->seed, j->stream, idx)
                             : j->lo + (j->hi - j->lo) * u01(j->seed, j->stream, idx);
  }
  return NULL;
}

static void fill(double* out, int64_t count, uint64_t seed, uint64_t stream, uint64_t offset,
                 double lo, double hi, int kind, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  if (count < 65536) nthreads = 1;
  pthread_t th[256];
  job_t jobs[256];
  const int64_t chunk = (count + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; t++) {
    jobs[t].out = out;
    jobs[t].begin = t * chunk < count ? t * chunk : count;
    jobs[t].end = (t + 1) * chunk < count ? (t + 1) * chunk : count;
    jobs[t].seed = seed;
    jobs[t].stream = stream;
    jobs[t].offset = offset;
    jobs[t].lo = lo;
    jobs[t].hi = hi;
    jobs[t].kind = kind;
  }
  if (nthreads == 1) {
    run_job(&jobs[0]);
    return;
  }
  for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, run_job, &jobs[t]);
  for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
}

void mfs_normal(double* out, int64_t count, uint64_t seed, uint64_t stream, uint64_t offset,
                int nthreads) {
  fill(out, count, seed, stream, offset, 0.0, 1.0, 0, nthreads);
}

void mfs_uniform(double* out, int64_t count, uint64_t seed, uint64_t stream, uint64_t offset,
                 double lo, double hi, int nthreads) {
  fill(out, count, seed, stream, offset, lo, hi, 1, nthreads);
}
