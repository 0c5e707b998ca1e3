// MatFlat CPU oracle — TEST INFRASTRUCTURE ONLY.
//
// A plain C++ restatement of the arithmetic of MatFlat 0.8.2 (sinshu/matflat, C#) for the
// factorization hot path: Internals.Dot/Norm/MulAdd/DivInplace/SwapRows, Factorization.Lu,
// Factorization.Cholesky, Factorization.Qr (+ QrOrthogonalFactor, QrUpperTriangularFactor),
// Blas.SolveTriangular, Blas.MulMatMat, Blas.MulMatVec and Factorization.LuInverse, for the
// float, double and Complex overloads.  Every routine cites the reference file:line it follows.
//
// It exists to check the CUDA library (tests, the smoke check) and to time the reference
// algorithm on the host cores (the CPU baseline leg of bench.py).  The product library never
// links it, calls it or falls back to it.
//
// Arithmetic contract.  MatFlat evaluates every product and sum separately rounded (RyuJIT does
// not contract a*b+c into an FMA), so this file MUST be compiled with -ffp-contract=off and no
// fast-math; the build recipe next to it does so.  The summation trees below reproduce the C#
// evaluation order exactly: `sum += x0*y0 + x1*y1` evaluates the right-hand pair first.
//
// Parity pin.  The reference is C# and no .NET runtime exists on either machine, so the
// reference itself cannot be executed.  The restatement is pinned against the reference test
// suite's own oracle (OpenBLAS LAPACK/BLAS via scipy, at the tolerances and shapes of
// MatFlatTest/*.cs) and against its literal fixtures; see tests/test_oracle_pin.py.

#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>
#include <atomic>
#include <algorithm>

namespace {

// ---------------------------------------------------------------------------------------------
// .NET System.Numerics.Complex arithmetic, restated (textbook formulas, no FMA):
//   (a+bi)(c+di) = (ac - bd) + (bc + ad)i ;  division by Smith's algorithm (Smith, CACM 1962),
//   which is what System.Numerics.Complex.op_Division uses.
struct cplx {
  double re, im;
};
static inline cplx cadd(cplx x, cplx y) { return {x.re + y.re, x.im + y.im}; }
static inline cplx csub(cplx x, cplx y) { return {x.re - y.re, x.im - y.im}; }
static inline cplx cmul(cplx x, cplx y) {
  return {x.re * y.re - x.im * y.im, x.im * y.re + x.re * y.im};
}
static inline cplx cdiv(cplx x, cplx y) {
  double a = x.re, b = x.im, c = y.re, d = y.im;
  if (std::fabs(d) < std::fabs(c)) {
    double doc = d / c;
    return {(a + b * doc) / (c + d * doc), (b - a * doc) / (c + d * doc)};
  } else {
    double cod = c / d;
    return {(b + a * cod) / (d + c * cod), (-a + b * cod) / (d + c * cod)};
  }
}
static inline cplx cconj(cplx x) { return {x.re, -x.im}; }
// Internals.MulConj (Internals.cs:22-29): conj(x) * y
static inline cplx cmulconj(cplx x, cplx y) {
  double a = x.re, b = -x.im, c = y.re, d = y.im;
  return {a * c - b * d, a * d + b * c};
}
// Internals.MulConjConj (Internals.cs:32-39): conj(x) * conj(y)
static inline cplx cmulconjconj(cplx x, cplx y) {
  double a = x.re, b = -x.im, c = y.re, d = -y.im;
  return {a * c - b * d, a * d + b * c};
}
// Internals.FastMagnitude (Internals.cs:16-19)
static inline double cfastmag(cplx x) { return std::fabs(x.re) + std::fabs(x.im); }

// ---------------------------------------------------------------------------------------------
// Internals.Dot, strided double (Internals.cs:265-292); the contiguous twin (:178-205) is the
// same tree with unit strides.
static double dot_d(int n, const double* x, long incx, const double* y, long incy) {
  double sum;
  if (n & 1) {
    sum = x[0] * y[0];
    x += incx;
    y += incy;
    n--;
  } else {
    sum = 0.0;
  }
  while (n > 0) {
    sum += x[0] * y[0] + x[incx] * y[incy];
    x += 2 * incx;
    y += 2 * incy;
    n -= 2;
  }
  return sum;
}

// Internals.Dot, strided float widened to double (Internals.cs:236-263; contiguous :149-176).
static double dot_s(int n, const float* x, long incx, const float* y, long incy) {
  double sum;
  if (n & 1) {
    sum = (double)x[0] * (double)y[0];
    x += incx;
    y += incy;
    n--;
  } else {
    sum = 0.0;
  }
  while (n > 0) {
    sum += (double)x[0] * (double)y[0] + (double)x[incx] * (double)y[incy];
    x += 2 * incx;
    y += 2 * incy;
    n -= 2;
  }
  return sum;
}

// Internals.Dot, Complex (Internals.cs:294-321; contiguous :207-234).
static cplx dot_z(int n, const cplx* x, long incx, const cplx* y, long incy) {
  cplx sum;
  if (n & 1) {
    sum = cmul(x[0], y[0]);
    x += incx;
    y += incy;
    n--;
  } else {
    sum = {0.0, 0.0};
  }
  while (n > 0) {
    sum = cadd(sum, cadd(cmul(x[0], y[0]), cmul(x[incx], y[incy])));
    x += 2 * incx;
    y += 2 * incy;
    n -= 2;
  }
  return sum;
}

// Internals.DotConj, Complex (Internals.cs:352-379; contiguous :323-350): sum conj(x)*y.
static cplx dotconj_z(int n, const cplx* x, long incx, const cplx* y, long incy) {
  cplx sum;
  if (n & 1) {
    sum = cmulconj(x[0], y[0]);
    x += incx;
    y += incy;
    n--;
  } else {
    sum = {0.0, 0.0};
  }
  while (n > 0) {
    sum = cadd(sum, cadd(cmulconj(x[0], y[0]), cmulconj(x[incx], y[incy])));
    x += 2 * incx;
    y += 2 * incy;
    n -= 2;
  }
  return sum;
}

// Internals.Norm (Internals.cs:435-460 double, :381-406 float, :489-514 Complex).
static double norm_d(int n, const double* x) {
  double sum;
  if (n & 1) {
    sum = x[0] * x[0];
    x++;
    n--;
  } else {
    sum = 0.0;
  }
  while (n > 0) {
    sum += x[0] * x[0] + x[1] * x[1];
    x += 2;
    n -= 2;
  }
  return std::sqrt(sum);
}
static double norm_s(int n, const float* x) {
  double sum;
  if (n & 1) {
    sum = (double)x[0] * (double)x[0];
    x++;
    n--;
  } else {
    sum = 0.0;
  }
  while (n > 0) {
    sum += (double)x[0] * (double)x[0] + (double)x[1] * (double)x[1];
    x += 2;
    n -= 2;
  }
  return std::sqrt(sum);
}
static double norm_z(int n, const cplx* x) {
  double sum;
  if (n & 1) {
    sum = x[0].re * x[0].re + x[0].im * x[0].im;
    x++;
    n--;
  } else {
    sum = 0.0;
  }
  while (n > 0) {
    sum += x[0].re * x[0].re + x[0].im * x[0].im + x[1].re * x[1].re + x[1].im * x[1].im;
    x += 2;
    n -= 2;
  }
  return std::sqrt(sum);
}

// Internals.MulAdd (Internals.cs:49-73): dst += x*y element by element (the pairing of the
// loop does not change any value: every element is updated once).
template <typename T>
static void muladd(int n, const T* x, T y, T* dst) {
  for (int i = 0; i < n; i++) dst[i] += x[i] * y;
}
static void muladd_z(int n, const cplx* x, cplx y, cplx* dst) {
  for (int i = 0; i < n; i++) dst[i] = cadd(dst[i], cmul(x[i], y));
}
// Internals.MulConjAdd (Internals.cs:75-99): dst += conj(x) * y[i]
static void mulconjadd_z(int n, cplx x, const cplx* y, cplx* dst) {
  for (int i = 0; i < n; i++) dst[i] = cadd(dst[i], cmulconj(x, y[i]));
}

// Internals.DivInplace (Internals.cs:125-147): true division, element by element.
template <typename T>
static void divinplace(int n, T* x, T y) {
  for (int i = 0; i < n; i++) x[i] /= y;
}
static void divinplace_z(int n, cplx* x, cplx y) {
  for (int i = 0; i < n; i++) x[i] = cdiv(x[i], y);
}

// Internals.SwapRows (Internals.cs:567-576).
template <typename T>
static void swaprows(int n, T* x, T* y, long inc) {
  for (int c = 0; c < n; c++) {
    T t = x[c * inc];
    x[c * inc] = y[c * inc];
    y[c * inc] = t;
  }
}

// Blas.MulSub (Blas.SolveTriangular.cs:397-421): dst -= x*y, element by element.
template <typename T>
static void mulsub(int n, const T* x, long incx, T y, T* dst, long incdst) {
  for (int i = 0; i < n; i++) dst[i * incdst] -= x[i * incx] * y;
}
static void mulsub_z(int n, const cplx* x, long incx, cplx y, cplx* dst, long incdst) {
  for (int i = 0; i < n; i++) dst[i * incdst] = csub(dst[i * incdst], cmul(x[i * incx], y));
}
// Blas.MulSubConj (Blas.SolveTriangular.cs:423-447): dst -= conj(x) * y
static void mulsubconj_z(int n, const cplx* x, long incx, cplx y, cplx* dst, long incdst) {
  for (int i = 0; i < n; i++)
    dst[i * incdst] = csub(dst[i * incdst], cmulconj(x[i * incx], y));
}

}  // namespace

extern "C" {

// =============================================================================================
// LU with partial pivoting: Factorization.LuCore (Factorization.Lu.cs:296-350 double,
// :240-294 float, :352-406 Complex).  Returns the pivot sign.  `work` holds m elements.
int orc_dlu(int m, int n, double* a, int lda, int* piv) {
  std::vector<double> workv(m);
  double* work = workv.data();
  for (int i = 0; i < m; i++) piv[i] = i;
  int sign = 1;
  double* colj = a;
  for (int j = 0; j < n; j++) {
    std::memcpy(work, colj, sizeof(double) * m);
    for (int i = 0; i < m; i++) {
      double s = dot_d(std::min(i, j), a + i, lda, work, 1);
      colj[i] = work[i] -= s;
    }
    int p = j;
    for (int i = j + 1; i < m; i++)
      if (std::fabs(work[i]) > std::fabs(work[p])) p = i;
    if (p != j) {
      swaprows(n, a + p, a + j, lda);
      std::swap(piv[p], piv[j]);
      sign = -sign;
    }
    if (j < m) {
      double diag = colj[j];
      if (diag != 0.0) divinplace(m - j - 1, colj + j + 1, diag);
    }
    colj += lda;
  }
  return sign;
}

int orc_slu(int m, int n, float* a, int lda, int* piv) {
  std::vector<float> workv(m);
  float* work = workv.data();
  for (int i = 0; i < m; i++) piv[i] = i;
  int sign = 1;
  float* colj = a;
  for (int j = 0; j < n; j++) {
    std::memcpy(work, colj, sizeof(float) * m);
    for (int i = 0; i < m; i++) {
      float s = (float)dot_s(std::min(i, j), a + i, lda, work, 1);
      colj[i] = work[i] -= s;
    }
    int p = j;
    for (int i = j + 1; i < m; i++)
      if (std::fabs(work[i]) > std::fabs(work[p])) p = i;
    if (p != j) {
      swaprows(n, a + p, a + j, lda);
      std::swap(piv[p], piv[j]);
      sign = -sign;
    }
    if (j < m) {
      float diag = colj[j];
      if (diag != 0.0f) divinplace(m - j - 1, colj + j + 1, diag);
    }
    colj += lda;
  }
  return sign;
}

int orc_zlu(int m, int n, double* a_, int lda, int* piv) {
  cplx* a = reinterpret_cast<cplx*>(a_);
  std::vector<cplx> workv(m);
  cplx* work = workv.data();
  for (int i = 0; i < m; i++) piv[i] = i;
  int sign = 1;
  cplx* colj = a;
  for (int j = 0; j < n; j++) {
    std::memcpy(work, colj, sizeof(cplx) * m);
    for (int i = 0; i < m; i++) {
      cplx s = dot_z(std::min(i, j), a + i, lda, work, 1);
      work[i] = csub(work[i], s);
      colj[i] = work[i];
    }
    int p = j;
    for (int i = j + 1; i < m; i++)
      if (cfastmag(work[i]) > cfastmag(work[p])) p = i;
    if (p != j) {
      swaprows(n, a + p, a + j, lda);
      std::swap(piv[p], piv[j]);
      sign = -sign;
    }
    if (j < m) {
      cplx diag = colj[j];
      if (!(diag.re == 0.0 && diag.im == 0.0)) divinplace_z(m - j - 1, colj + j + 1, diag);
    }
    colj += lda;
  }
  return sign;
}

// =============================================================================================
// Cholesky A = L*L^H: Factorization.Cholesky (Factorization.Cholesky.cs:114-168 double,
// :33-87 float, :195-249 Complex).  Reads the upper triangle, writes L to the lower triangle,
// zeroes the strict upper triangle.  Returns 0, or j+1 for the first column whose pivot is not
// positive (MatFlat throws MatrixFactorizationException there; the array is left as it was at
// that point, without the final clearing pass).
int orc_dcholesky(int n, double* a, int lda) {
  double* colj = a;
  for (int j = 0; j < n; j++) {
    double s = 0.0;
    double* colk = a;
    for (int k = 0; k < j; k++) {
      double t = (colj[k] - dot_d(k, a + j, lda, a + k, lda)) / colk[k];
      colk[j] = t;
      s += t * t;
      colk += lda;
    }
    s = colj[j] - s;
    if (s > 0) {
      colj[j] = std::sqrt(s);
    } else {
      return j + 1;
    }
    colj += lda;
  }
  colj = a + lda;
  for (int j = 1; j < n; j++) {
    std::memset(colj, 0, sizeof(double) * j);
    colj += lda;
  }
  return 0;
}

int orc_scholesky(int n, float* a, int lda) {
  float* colj = a;
  for (int j = 0; j < n; j++) {
    double s = 0.0;
    float* colk = a;
    for (int k = 0; k < j; k++) {
      double t = ((double)colj[k] - dot_s(k, a + j, lda, a + k, lda)) / (double)colk[k];
      colk[j] = (float)t;
      s += t * t;
      colk += lda;
    }
    s = (double)colj[j] - s;
    if (s > 0) {
      colj[j] = (float)std::sqrt(s);
    } else {
      return j + 1;
    }
    colj += lda;
  }
  colj = a + lda;
  for (int j = 1; j < n; j++) {
    std::memset(colj, 0, sizeof(float) * j);
    colj += lda;
  }
  return 0;
}

int orc_zcholesky(int n, double* a_, int lda) {
  cplx* a = reinterpret_cast<cplx*>(a_);
  cplx* colj = a;
  for (int j = 0; j < n; j++) {
    double s = 0.0;
    cplx* colk = a;
    for (int k = 0; k < j; k++) {
      cplx t = cdiv(csub(colj[k], dotconj_z(k, a + j, lda, a + k, lda)), colk[k]);
      colk[j] = {t.re, -t.im};
      s += t.re * t.re + t.im * t.im;
      colk += lda;
    }
    s = colj[j].re - s;
    if (s > 0) {
      colj[j] = {std::sqrt(s), 0.0};
    } else {
      return j + 1;
    }
    colj += lda;
  }
  colj = a + lda;
  for (int j = 1; j < n; j++) {
    std::memset(colj, 0, sizeof(cplx) * j);
    colj += lda;
  }
  return 0;
}

// =============================================================================================
// Householder QR in the Mapack format: Factorization.Qr (Factorization.Qr.cs:115-172 double,
// :32-89 float, :198-255 Complex).  No reflector sign choice; rdiag[k] = -norm.
void orc_dqr(int m, int n, double* a, int lda, double* rdiag) {
  double* colk = a;
  for (int k = 0; k < n; k++) {
    double norm = norm_d(m - k, colk + k);
    if (norm != 0.0) {
      divinplace(m - k, colk + k, norm);
      colk[k] += 1.0;
      for (int j = k + 1; j < n; j++) {
        double* colj = a + (long)lda * j;
        double s = -dot_d(m - k, colk + k, 1, colj + k, 1) / colk[k];
        muladd(m - k, colk + k, s, colj + k);
      }
    }
    rdiag[k] = -norm;
    colk += lda;
  }
}

void orc_sqr(int m, int n, float* a, int lda, float* rdiag) {
  float* colk = a;
  for (int k = 0; k < n; k++) {
    float norm = (float)norm_s(m - k, colk + k);
    if (norm != 0.0f) {
      divinplace(m - k, colk + k, norm);
      colk[k] += 1.0f;
      for (int j = k + 1; j < n; j++) {
        float* colj = a + (long)lda * j;
        float s = -(float)(dot_s(m - k, colk + k, 1, colj + k, 1) / (double)colk[k]);
        muladd(m - k, colk + k, s, colj + k);
      }
    }
    rdiag[k] = -norm;
    colk += lda;
  }
}

void orc_zqr(int m, int n, double* a_, int lda, double* rdiag) {
  cplx* a = reinterpret_cast<cplx*>(a_);
  cplx* colk = a;
  for (int k = 0; k < n; k++) {
    double norm = norm_z(m - k, colk + k);
    if (norm != 0.0) {
      // DivInplace<Complex>(…, norm): Complex / Complex(norm, 0).
      divinplace_z(m - k, colk + k, cplx{norm, 0.0});
      colk[k] = cadd(colk[k], cplx{1.0, 0.0});
      for (int j = k + 1; j < n; j++) {
        cplx* colj = a + (long)lda * j;
        cplx d = dotconj_z(m - k, colk + k, 1, colj + k, 1);
        cplx s = cdiv(cplx{-d.re, -d.im}, colk[k]);
        muladd_z(m - k, colk + k, s, colj + k);
      }
    }
    rdiag[k] = -norm;
    colk += lda;
  }
}

// QrOrthogonalFactor (Factorization.Qr.cs:357-413 double, :278-334 float, :436-492 Complex).
void orc_dqr_q(int m, int n, const double* a, int lda, double* q, int ldq) {
  for (int k = n - 1; k >= 0; k--) {
    double* qColk = q + (long)ldq * k;
    const double* aColk = a + (long)lda * k;
    std::memset(qColk, 0, sizeof(double) * m);
    qColk[k] = 1.0;
    for (int j = k; j < n; j++) {
      double* qColj = q + (long)ldq * j;
      if (aColk[k] != 0) {
        double s = -dot_d(m - k, aColk + k, 1, qColj + k, 1) / aColk[k];
        muladd(m - k, aColk + k, s, qColj + k);
      }
    }
  }
}

void orc_sqr_q(int m, int n, const float* a, int lda, float* q, int ldq) {
  for (int k = n - 1; k >= 0; k--) {
    float* qColk = q + (long)ldq * k;
    const float* aColk = a + (long)lda * k;
    std::memset(qColk, 0, sizeof(float) * m);
    qColk[k] = 1.0f;
    for (int j = k; j < n; j++) {
      float* qColj = q + (long)ldq * j;
      if (aColk[k] != 0) {
        float s = -(float)(dot_s(m - k, aColk + k, 1, qColj + k, 1) / (double)aColk[k]);
        muladd(m - k, aColk + k, s, qColj + k);
      }
    }
  }
}

void orc_zqr_q(int m, int n, const double* a_, int lda, double* q_, int ldq) {
  const cplx* a = reinterpret_cast<const cplx*>(a_);
  cplx* q = reinterpret_cast<cplx*>(q_);
  for (int k = n - 1; k >= 0; k--) {
    cplx* qColk = q + (long)ldq * k;
    const cplx* aColk = a + (long)lda * k;
    std::memset(qColk, 0, sizeof(cplx) * m);
    qColk[k] = {1.0, 0.0};
    for (int j = k; j < n; j++) {
      cplx* qColj = q + (long)ldq * j;
      if (!(aColk[k].re == 0.0 && aColk[k].im == 0.0)) {
        // Factorization.Qr.cs:487-488: s = -DotConj(qColj, aColk) / aColk[k];
        // MulConjAdd(s, aColk, qColj): q += conj(s) * a.
        cplx d = dotconj_z(m - k, qColj + k, 1, aColk + k, 1);
        cplx s = cdiv(cplx{-d.re, -d.im}, aColk[k]);
        mulconjadd_z(m - k, s, aColk + k, qColj + k);
      }
    }
  }
}

// QrUpperTriangularFactor (Factorization.Qr.cs:597-650 double, :518-571 float, :677-730 Complex).
void orc_dqr_r(int m, int n, const double* a, int lda, double* r, int ldr, const double* rdiag) {
  (void)m;
  for (int i = 0; i < n; i++) {
    std::memcpy(r + (long)ldr * i, a + (long)lda * i, sizeof(double) * i);
    r[(long)ldr * i + i] = rdiag[i];
    std::memset(r + (long)ldr * i + i + 1, 0, sizeof(double) * (n - i - 1));
  }
}
void orc_sqr_r(int m, int n, const float* a, int lda, float* r, int ldr, const float* rdiag) {
  (void)m;
  for (int i = 0; i < n; i++) {
    std::memcpy(r + (long)ldr * i, a + (long)lda * i, sizeof(float) * i);
    r[(long)ldr * i + i] = rdiag[i];
    std::memset(r + (long)ldr * i + i + 1, 0, sizeof(float) * (n - i - 1));
  }
}
void orc_zqr_r(int m, int n, const double* a_, int lda, double* r_, int ldr, const double* rdiag) {
  (void)m;
  const cplx* a = reinterpret_cast<const cplx*>(a_);
  cplx* r = reinterpret_cast<cplx*>(r_);
  for (int i = 0; i < n; i++) {
    std::memcpy(r + (long)ldr * i, a + (long)lda * i, sizeof(cplx) * i);
    r[(long)ldr * i + i] = {rdiag[i], 0.0};
    std::memset(r + (long)ldr * i + i + 1, 0, sizeof(cplx) * (n - i - 1));
  }
}

// =============================================================================================
// Triangular solve, non-unit diagonal: Blas.SolveTriangular (Blas.SolveTriangular.cs:162-242
// double, :44-124 float, :280-395 Complex).  uplo: 121 Upper, 122 Lower.  trans: 111 NoTrans,
// 112 Trans, 113 ConjTrans, 114 ConjNoTrans.  Returns 0, or -1 for an invalid enum.
enum { UPPER = 121, LOWER = 122, NOTRANS = 111, TRANS = 112, CONJTRANS = 113, CONJNOTRANS = 114 };

int orc_dtrsv(int uplo, int trans, int n, const double* a, int lda, double* x, int incx) {
  if (uplo == UPPER) {
    if (trans == NOTRANS) {
      for (int i = n - 1; i >= 0; i--) {
        long p = (long)incx * i;
        const double* aColi = a + (long)lda * i;
        x[p] /= aColi[i];
        mulsub(i, aColi, 1, x[p], x, incx);
      }
    } else if (trans == TRANS) {
      for (int j = 0; j < n; j++) {
        long p = (long)incx * j;
        x[p] = (x[p] - dot_d(j, a + (long)lda * j, 1, x, incx)) / a[(long)lda * j + j];
      }
    } else {
      return -1;
    }
  } else if (uplo == LOWER) {
    if (trans == NOTRANS) {
      for (int i = 0; i < n; i++) {
        long p = (long)incx * i;
        x[p] = (x[p] - dot_d(i, a + i, lda, x, incx)) / a[(long)lda * i + i];
      }
    } else if (trans == TRANS) {
      for (int j = n - 1; j >= 0; j--) {
        long p = (long)incx * j;
        x[p] /= a[(long)j * lda + j];
        mulsub(j, a + j, lda, x[p], x, incx);
      }
    } else {
      return -1;
    }
  } else {
    return -1;
  }
  return 0;
}

int orc_strsv(int uplo, int trans, int n, const float* a, int lda, float* x, int incx) {
  if (uplo == UPPER) {
    if (trans == NOTRANS) {
      for (int i = n - 1; i >= 0; i--) {
        long p = (long)incx * i;
        const float* aColi = a + (long)lda * i;
        x[p] /= aColi[i];
        mulsub(i, aColi, 1, x[p], x, incx);
      }
    } else if (trans == TRANS) {
      for (int j = 0; j < n; j++) {
        long p = (long)incx * j;
        x[p] = (float)(((double)x[p] - dot_s(j, a + (long)lda * j, 1, x, incx)) /
                       (double)a[(long)lda * j + j]);
      }
    } else {
      return -1;
    }
  } else if (uplo == LOWER) {
    if (trans == NOTRANS) {
      for (int i = 0; i < n; i++) {
        long p = (long)incx * i;
        x[p] = (float)(((double)x[p] - dot_s(i, a + i, lda, x, incx)) / (double)a[(long)lda * i + i]);
      }
    } else if (trans == TRANS) {
      for (int j = n - 1; j >= 0; j--) {
        long p = (long)incx * j;
        x[p] /= a[(long)j * lda + j];
        mulsub(j, a + j, lda, x[p], x, incx);
      }
    } else {
      return -1;
    }
  } else {
    return -1;
  }
  return 0;
}

int orc_ztrsv(int uplo, int trans, int n, const double* a_, int lda, double* x_, int incx) {
  const cplx* a = reinterpret_cast<const cplx*>(a_);
  cplx* x = reinterpret_cast<cplx*>(x_);
  if (uplo == UPPER) {
    if (trans == NOTRANS) {
      for (int i = n - 1; i >= 0; i--) {
        long p = (long)incx * i;
        const cplx* aColi = a + (long)lda * i;
        x[p] = cdiv(x[p], aColi[i]);
        mulsub_z(i, aColi, 1, x[p], x, incx);
      }
    } else if (trans == TRANS) {
      for (int j = 0; j < n; j++) {
        long p = (long)incx * j;
        x[p] = cdiv(csub(x[p], dot_z(j, a + (long)lda * j, 1, x, incx)), a[(long)lda * j + j]);
      }
    } else if (trans == CONJNOTRANS) {
      for (int i = n - 1; i >= 0; i--) {
        long p = (long)incx * i;
        const cplx* aColi = a + (long)lda * i;
        x[p] = cdiv(x[p], cconj(aColi[i]));
        mulsubconj_z(i, aColi, 1, x[p], x, incx);
      }
    } else if (trans == CONJTRANS) {
      for (int j = 0; j < n; j++) {
        long p = (long)incx * j;
        x[p] = cdiv(csub(x[p], dotconj_z(j, a + (long)lda * j, 1, x, incx)),
                    cconj(a[(long)lda * j + j]));
      }
    } else {
      return -1;
    }
  } else if (uplo == LOWER) {
    if (trans == NOTRANS) {
      for (int i = 0; i < n; i++) {
        long p = (long)incx * i;
        x[p] = cdiv(csub(x[p], dot_z(i, a + i, lda, x, incx)), a[(long)lda * i + i]);
      }
    } else if (trans == TRANS) {
      for (int j = n - 1; j >= 0; j--) {
        long p = (long)incx * j;
        x[p] = cdiv(x[p], a[(long)j * lda + j]);
        mulsub_z(j, a + j, lda, x[p], x, incx);
      }
    } else if (trans == CONJNOTRANS) {
      for (int i = 0; i < n; i++) {
        long p = (long)incx * i;
        x[p] = cdiv(csub(x[p], dotconj_z(i, a + i, lda, x, incx)), cconj(a[(long)lda * i + i]));
      }
    } else if (trans == CONJTRANS) {
      for (int j = n - 1; j >= 0; j--) {
        long p = (long)incx * j;
        x[p] = cdiv(x[p], cconj(a[(long)j * lda + j]));
        mulsubconj_z(j, a + j, lda, x[p], x, incx);
      }
    } else {
      return -1;
    }
  } else {
    return -1;
  }
  return 0;
}

// =============================================================================================
// C = op(A) * op(B), no alpha/beta: Blas.MulMatMat (Blas.MulMatMat.cs:226-368 double,
// :45-187 float).  Each element is one Internals.Dot of length k.
int orc_dgemm(int transa, int transb, int m, int n, int k, const double* a, int lda,
              const double* b, int ldb, double* c, int ldc) {
  if ((transa != NOTRANS && transa != TRANS) || (transb != NOTRANS && transb != TRANS)) return -1;
  for (int j = 0; j < n; j++) {
    for (int i = 0; i < m; i++) {
      const double* x;
      long incx;
      const double* y;
      long incy;
      if (transa == NOTRANS) {
        x = a + i;
        incx = lda;
      } else {
        x = a + (long)lda * i;
        incx = 1;
      }
      if (transb == NOTRANS) {
        y = b + (long)ldb * j;
        incy = 1;
      } else {
        y = b + j;
        incy = ldb;
      }
      c[(long)ldc * j + i] = dot_d(k, x, incx, y, incy);
    }
  }
  return 0;
}

int orc_sgemm(int transa, int transb, int m, int n, int k, const float* a, int lda,
              const float* b, int ldb, float* c, int ldc) {
  if ((transa != NOTRANS && transa != TRANS) || (transb != NOTRANS && transb != TRANS)) return -1;
  for (int j = 0; j < n; j++) {
    for (int i = 0; i < m; i++) {
      const float* x;
      long incx;
      const float* y;
      long incy;
      if (transa == NOTRANS) {
        x = a + i;
        incx = lda;
      } else {
        x = a + (long)lda * i;
        incx = 1;
      }
      if (transb == NOTRANS) {
        y = b + (long)ldb * j;
        incy = 1;
      } else {
        y = b + j;
        incy = ldb;
      }
      c[(long)ldc * j + i] = (float)dot_s(k, x, incx, y, incy);
    }
  }
  return 0;
}

// Complex MulMatMat (Blas.MulMatMat.cs:407-575) with its unpaired sequential dots
// Dot_NN/CN/NC/CC (:598-648).
int orc_zgemm(int transa, int transb, int m, int n, int k, const double* a_, int lda,
              const double* b_, int ldb, double* c_, int ldc) {
  const cplx* a = reinterpret_cast<const cplx*>(a_);
  const cplx* b = reinterpret_cast<const cplx*>(b_);
  cplx* c = reinterpret_cast<cplx*>(c_);
  auto valid = [](int t) { return t == NOTRANS || t == TRANS || t == CONJTRANS || t == CONJNOTRANS; };
  if (!valid(transa) || !valid(transb)) return -1;
  bool ca = (transa == CONJNOTRANS || transa == CONJTRANS);
  bool cb = (transb == CONJNOTRANS || transb == CONJTRANS);
  bool ta = (transa == TRANS || transa == CONJTRANS);
  bool tb = (transb == TRANS || transb == CONJTRANS);
  for (int j = 0; j < n; j++) {
    for (int i = 0; i < m; i++) {
      const cplx* x = ta ? a + (long)lda * i : a + i;
      long incx = ta ? 1 : lda;
      const cplx* y = tb ? b + j : b + (long)ldb * j;
      long incy = tb ? ldb : 1;
      cplx sum = {0.0, 0.0};
      for (int t = 0; t < k; t++) {
        cplx xv = x[t * incx], yv = y[t * incy];
        cplx p;
        if (ca && cb) p = cmulconjconj(xv, yv);
        else if (ca) p = cmulconj(xv, yv);
        else if (cb) p = cmulconj(yv, xv);
        else p = cmul(xv, yv);
        sum = cadd(sum, p);
      }
      c[(long)ldc * j + i] = sum;
    }
  }
  return 0;
}

// y = op(A) x: Blas.MulMatVec (Blas.MulMatVec.cs:138-236), used to form Q^T b for the
// least-squares composition Qr -> QrOrthogonalFactor -> MulMatVec(Trans) -> SolveTriangular.
int orc_dgemv(int trans, int m, int n, const double* a, int lda, const double* x, int incx,
              double* y, int incy) {
  if (trans == NOTRANS) {
    for (int i = 0; i < m; i++) y[(long)incy * i] = dot_d(n, a + i, lda, x, incx);
  } else if (trans == TRANS) {
    for (int i = 0; i < n; i++) y[(long)incy * i] = dot_d(m, a + (long)lda * i, 1, x, incx);
  } else {
    return -1;
  }
  return 0;
}
int orc_sgemv(int trans, int m, int n, const float* a, int lda, const float* x, int incx,
              float* y, int incy) {
  if (trans == NOTRANS) {
    for (int i = 0; i < m; i++) y[(long)incy * i] = (float)dot_s(n, a + i, lda, x, incx);
  } else if (trans == TRANS) {
    for (int i = 0; i < n; i++) y[(long)incy * i] = (float)dot_s(m, a + (long)lda * i, 1, x, incx);
  } else {
    return -1;
  }
  return 0;
}

// Blas.Dot / Blas.L2Norm / Blas.Outer, double (Blas.VectorOperations.cs:143-174, :50-60,
// :292-334): Internals.Dot's tree; L2Norm = Math.Sqrt of the same tree over x*x
// (Internals.Norm, Internals.cs:435-460); Outer a(i,j) = y_j * x_i.
double orc_ddot(int n, const double* x, int incx, const double* y, int incy) {
  return dot_d(n, x, incx, y, incy);
}
double orc_dnrm2(int n, const double* x, int incx) { return std::sqrt(dot_d(n, x, incx, x, incx)); }
void orc_dger(int m, int n, const double* x, int incx, const double* y, int incy, double* a,
              int lda) {
  for (int j = 0; j < n; j++) {
    const double t = y[(long)incy * j];
    for (int i = 0; i < m; i++) a[(long)lda * j + i] = t * x[(long)incx * i];
  }
}

// The float and Complex overloads (Blas.MulMatVec.cs:38-136, :238-336; Blas.VectorOperations.cs
// :23-48, :77-108, :110-141, :176-246, :248-290, :336-420).  Float dots and norms are the double
// tree over widened operands, cast to float; Complex MulMatVec uses Dot for NoTrans / Trans and
// DotConj for ConjNoTrans / ConjTrans; the Complex norm is a double.
int orc_zgemv(int trans, int m, int n, const double* a_, int lda, const double* x_, int incx,
              double* y_, int incy) {
  const cplx* a = (const cplx*)a_;
  const cplx* x = (const cplx*)x_;
  cplx* y = (cplx*)y_;
  if (trans == NOTRANS) {
    for (int i = 0; i < m; i++) y[(long)incy * i] = dot_z(n, a + i, lda, x, incx);
  } else if (trans == TRANS) {
    for (int i = 0; i < n; i++) y[(long)incy * i] = dot_z(m, a + (long)lda * i, 1, x, incx);
  } else if (trans == CONJNOTRANS) {
    for (int i = 0; i < m; i++) y[(long)incy * i] = dotconj_z(n, a + i, lda, x, incx);
  } else if (trans == CONJTRANS) {
    for (int i = 0; i < n; i++) y[(long)incy * i] = dotconj_z(m, a + (long)lda * i, 1, x, incx);
  } else {
    return -1;
  }
  return 0;
}
float orc_sdot(int n, const float* x, int incx, const float* y, int incy) {
  return (float)dot_s(n, x, incx, y, incy);
}
void orc_zdot(int n, const double* x, int incx, const double* y, int incy, int conj,
              double* out) {
  const cplx r = conj ? dotconj_z(n, (const cplx*)x, incx, (const cplx*)y, incy)
                      : dot_z(n, (const cplx*)x, incx, (const cplx*)y, incy);
  out[0] = r.re;
  out[1] = r.im;
}
float orc_snrm2(int n, const float* x, int incx) {
  return (float)std::sqrt(dot_s(n, x, incx, x, incx));
}
double orc_dznrm2(int n, const double* x_, int incx) {
  const cplx* x = (const cplx*)x_;
  double sum = 0.0;
  if (n & 1) {
    sum = x[0].re * x[0].re + x[0].im * x[0].im;
    x += incx;
    n--;
  }
  while (n > 0) {
    sum += x[0].re * x[0].re + x[0].im * x[0].im + x[incx].re * x[incx].re +
           x[incx].im * x[incx].im;
    x += 2 * (long)incx;
    n -= 2;
  }
  return std::sqrt(sum);
}
void orc_sger(int m, int n, const float* x, int incx, const float* y, int incy, float* a,
              int lda) {
  for (int j = 0; j < n; j++) {
    const float t = y[(long)incy * j];
    for (int i = 0; i < m; i++) a[(long)lda * j + i] = t * x[(long)incx * i];
  }
}
void orc_zger(int m, int n, const double* x_, int incx, const double* y_, int incy, double* a_,
              int lda, int conj) {
  const cplx* x = (const cplx*)x_;
  const cplx* y = (const cplx*)y_;
  cplx* a = (cplx*)a_;
  for (int j = 0; j < n; j++) {
    cplx t = y[(long)incy * j];
    if (conj) t.im = -t.im;
    for (int i = 0; i < m; i++) a[(long)lda * j + i] = cmul(t, x[(long)incx * i]);
  }
}

// =============================================================================================
// Factorization.LuInverse (Factorization.LuInverse.cs:123-199): A^-1 from the LU factors.
// Returns 0, or 1 when a diagonal entry of U is zero (MatFlat throws there, before writing).
int orc_dlu_inverse(int n, double* a, int lda, const int* piv) {
  for (int j = 0; j < n; j++)
    if (a[(long)lda * j + j] == 0.0) return 1;
  std::vector<double> workv((size_t)n * n + n);
  double* work = workv.data();
  double* diag = work + (size_t)n * n;
  for (int j = 0; j < n; j++) {
    double* aColj = a + (long)lda * j;
    std::memcpy(work + (size_t)n * j, aColj, sizeof(double) * n);
    diag[j] = aColj[j];
    std::memset(aColj, 0, sizeof(double) * n);
  }
  for (int j = 0; j < n; j++) a[(long)lda * piv[j] + j] = 1.0;
  for (int j = 0; j < n; j++) work[(size_t)n * j + j] = 1.0;
  for (int j = 0; j < n; j++) orc_dtrsv(LOWER, NOTRANS, n, work, n, a + (long)lda * j, 1);
  for (int j = 0; j < n; j++) work[(size_t)n * j + j] = diag[j];
  for (int j = 0; j < n; j++) orc_dtrsv(UPPER, NOTRANS, n, work, n, a + (long)lda * j, 1);
  return 0;
}

// The float and Complex overloads (Factorization.LuInverse.cs:27-103, :219-295): the same steps
// with float SolveTriangular and with Complex SolveTriangular / Complex.One (the zero test is
// re == 0 && im == 0 for Complex).
int orc_slu_inverse(int n, float* a, int lda, const int* piv) {
  for (int j = 0; j < n; j++)
    if (a[(long)lda * j + j] == 0.0f) return 1;
  std::vector<float> workv((size_t)n * n + n);
  float* work = workv.data();
  float* diag = work + (size_t)n * n;
  for (int j = 0; j < n; j++) {
    float* aColj = a + (long)lda * j;
    std::memcpy(work + (size_t)n * j, aColj, sizeof(float) * n);
    diag[j] = aColj[j];
    std::memset(aColj, 0, sizeof(float) * n);
  }
  for (int j = 0; j < n; j++) a[(long)lda * piv[j] + j] = 1.0f;
  for (int j = 0; j < n; j++) work[(size_t)n * j + j] = 1.0f;
  for (int j = 0; j < n; j++) orc_strsv(LOWER, NOTRANS, n, work, n, a + (long)lda * j, 1);
  for (int j = 0; j < n; j++) work[(size_t)n * j + j] = diag[j];
  for (int j = 0; j < n; j++) orc_strsv(UPPER, NOTRANS, n, work, n, a + (long)lda * j, 1);
  return 0;
}
int orc_zlu_inverse(int n, double* a, int lda, const int* piv) {
  for (int j = 0; j < n; j++) {
    const double* d = a + 2 * ((long)lda * j + j);
    if (d[0] == 0.0 && d[1] == 0.0) return 1;
  }
  std::vector<double> workv((size_t)2 * ((size_t)n * n + n));
  double* work = workv.data();
  double* diag = work + (size_t)2 * n * n;
  for (int j = 0; j < n; j++) {
    double* aColj = a + 2 * (long)lda * j;
    std::memcpy(work + (size_t)2 * n * j, aColj, sizeof(double) * 2 * n);
    diag[2 * j] = aColj[2 * j];
    diag[2 * j + 1] = aColj[2 * j + 1];
    std::memset(aColj, 0, sizeof(double) * 2 * n);
  }
  for (int j = 0; j < n; j++) {
    a[2 * ((long)lda * piv[j] + j)] = 1.0;
    a[2 * ((long)lda * piv[j] + j) + 1] = 0.0;
  }
  for (int j = 0; j < n; j++) {
    work[2 * ((size_t)n * j + j)] = 1.0;
    work[2 * ((size_t)n * j + j) + 1] = 0.0;
  }
  for (int j = 0; j < n; j++) orc_ztrsv(LOWER, NOTRANS, n, work, n, a + 2 * (long)lda * j, 1);
  for (int j = 0; j < n; j++) {
    work[2 * ((size_t)n * j + j)] = diag[2 * j];
    work[2 * ((size_t)n * j + j) + 1] = diag[2 * j + 1];
  }
  for (int j = 0; j < n; j++) orc_ztrsv(UPPER, NOTRANS, n, work, n, a + 2 * (long)lda * j, 1);
  return 0;
}

// =============================================================================================
// Composite per-matrix workloads of the batched paths.  Each composes the routines above in
// the order MatFlat's own idioms give.

// Solve A x = b from the LU factors of one square matrix, for nrhs right-hand sides stored
// column after column with leading dimension ldb.  P*b first (b'[i] = b[piv[i]]), then the
// unit-lower solve in MatFlat's LuInverse idiom (trsv Lower/NoTrans against L with its diagonal
// set to 1.0, Factorization.LuInverse.cs:174-182 — dividing by 1.0 is exact, so this equals a
// solve that skips the division), then trsv Upper/NoTrans against U (:184-192).
void orc_dlu_solve(int n, const double* lu, int lda, const int* piv, int nrhs, double* b, int ldb) {
  std::vector<double> l((size_t)n * n);
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) l[(size_t)j * n + i] = lu[(long)lda * j + i];
  for (int j = 0; j < n; j++) l[(size_t)j * n + j] = 1.0;
  std::vector<double> tmp(n);
  for (int r = 0; r < nrhs; r++) {
    double* x = b + (long)ldb * r;
    for (int i = 0; i < n; i++) tmp[i] = x[piv[i]];
    std::memcpy(x, tmp.data(), sizeof(double) * n);
    orc_dtrsv(LOWER, NOTRANS, n, l.data(), n, x, 1);
    orc_dtrsv(UPPER, NOTRANS, n, lu, lda, x, 1);
  }
}

// The same solve for the float and Complex overloads (MatFlat's float / Complex SolveTriangular;
// Complex arrays are interleaved (re, im) doubles).
void orc_slu_solve(int n, const float* lu, int lda, const int* piv, int nrhs, float* b, int ldb) {
  std::vector<float> l((size_t)n * n);
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) l[(size_t)j * n + i] = lu[(long)lda * j + i];
  for (int j = 0; j < n; j++) l[(size_t)j * n + j] = 1.0f;
  std::vector<float> tmp(n);
  for (int r = 0; r < nrhs; r++) {
    float* x = b + (long)ldb * r;
    for (int i = 0; i < n; i++) tmp[i] = x[piv[i]];
    std::memcpy(x, tmp.data(), sizeof(float) * n);
    orc_strsv(LOWER, NOTRANS, n, l.data(), n, x, 1);
    orc_strsv(UPPER, NOTRANS, n, lu, lda, x, 1);
  }
}
void orc_zlu_solve(int n, const double* lu, int lda, const int* piv, int nrhs, double* b,
                   int ldb) {
  std::vector<double> l((size_t)2 * n * n);
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) {
      l[2 * ((size_t)j * n + i)] = lu[2 * ((long)lda * j + i)];
      l[2 * ((size_t)j * n + i) + 1] = lu[2 * ((long)lda * j + i) + 1];
    }
  for (int j = 0; j < n; j++) {
    l[2 * ((size_t)j * n + j)] = 1.0;
    l[2 * ((size_t)j * n + j) + 1] = 0.0;
  }
  std::vector<double> tmp((size_t)2 * n);
  for (int r = 0; r < nrhs; r++) {
    double* x = b + (long)2 * ldb * r;
    for (int i = 0; i < n; i++) {
      tmp[2 * i] = x[2 * piv[i]];
      tmp[2 * i + 1] = x[2 * piv[i] + 1];
    }
    std::memcpy(x, tmp.data(), sizeof(double) * 2 * n);
    orc_ztrsv(LOWER, NOTRANS, n, l.data(), n, x, 1);
    orc_ztrsv(UPPER, NOTRANS, n, lu, lda, x, 1);
  }
}

// Least squares min ||A x - b|| for one tall matrix (m >= n), composed from MatFlat's own
// routines since MatFlat has no QR solve: Qr, QrOrthogonalFactor, MulMatVec(Trans) for Q^T b,
// QrUpperTriangularFactor, SolveTriangular(Upper, NoTrans).  a is overwritten by the QR factors;
// x receives n entries.
void orc_dqr_ls(int m, int n, double* a, int lda, const double* b, double* x) {
  std::vector<double> rdiag(n), q((size_t)m * n), r((size_t)n * n);
  orc_dqr(m, n, a, lda, rdiag.data());
  orc_dqr_q(m, n, a, lda, q.data(), m);
  orc_dgemv(TRANS, m, n, q.data(), m, b, 1, x, 1);
  orc_dqr_r(m, n, a, lda, r.data(), n, rdiag.data());
  orc_dtrsv(UPPER, NOTRANS, n, r.data(), n, x, 1);
}
// Complex: x = R^-1 (Q^H b) with Q^H b from MulMatMat(ConjTrans, NoTrans) (Blas.MulMatMat.cs:
// 407-575) and R x = y by SolveTriangular(Upper, NoTrans) Complex.
void orc_zqr_ls(int m, int n, double* a, int lda, const double* b, double* x) {
  std::vector<double> rdiag(n), q((size_t)2 * m * n), r((size_t)2 * n * n);
  orc_zqr(m, n, a, lda, rdiag.data());
  orc_zqr_q(m, n, a, lda, q.data(), m);
  orc_zgemm(CONJTRANS, NOTRANS, n, 1, m, q.data(), m, b, m, x, n);
  orc_zqr_r(m, n, a, lda, r.data(), n, rdiag.data());
  orc_ztrsv(UPPER, NOTRANS, n, r.data(), n, x, 1);
}
void orc_sqr_ls(int m, int n, float* a, int lda, const float* b, float* x) {
  std::vector<float> rdiag(n), q((size_t)m * n), r((size_t)n * n);
  orc_sqr(m, n, a, lda, rdiag.data());
  orc_sqr_q(m, n, a, lda, q.data(), m);
  orc_sgemv(TRANS, m, n, q.data(), m, b, 1, x, 1);
  orc_sqr_r(m, n, a, lda, r.data(), n, rdiag.data());
  orc_strsv(UPPER, NOTRANS, n, r.data(), n, x, 1);
}

// Differentiable Cholesky / log-determinant / solve, composed from MatFlat's routines:
// L = Cholesky(K); z = L^-1 y (SolveTriangular Lower/NoTrans); quad = Internals.Dot(z, z);
// log det K = 2 * sum_i log L_ii; alpha = L^-T z (SolveTriangular Lower/Trans);
// W = L^-1 column by column (SolveTriangular Lower/NoTrans applied to e_c);
// K^-1 = W^T W (Blas.MulMatMat(Trans, NoTrans), Blas.MulMatMat.cs:226-368, which is exactly
// symmetric: C[i,j] and C[j,i] are the same dot); grad = K^-1 - alpha alpha^T, upper triangle
// computed and mirrored to a full symmetric matrix (leading dimension lda).
// On exit k holds L, y holds alpha.  Returns Cholesky's code (0 = success).
int orc_dchol_grad(int n, double* k, int lda, double* y, double* loss, double* g) {
  int info = orc_dcholesky(n, k, lda);
  if (info != 0) {
    *loss = std::nan("");
    return info;
  }
  orc_dtrsv(LOWER, NOTRANS, n, k, lda, y, 1);
  const double quad = dot_d(n, y, 1, y, 1);
  double logsum = 0.0;
  for (int i = 0; i < n; i++) logsum = logsum + std::log(k[(long)i * lda + i]);
  orc_dtrsv(LOWER, TRANS, n, k, lda, y, 1);
  *loss = quad + 2.0 * logsum;
  std::vector<double> w((size_t)n * n), c((size_t)n * n);
  for (int j = 0; j < n; j++) {
    double* wj = w.data() + (size_t)n * j;
    for (int i = 0; i < n; i++) wj[i] = (i == j) ? 1.0 : 0.0;
    orc_dtrsv(LOWER, NOTRANS, n, k, lda, wj, 1);
  }
  orc_dgemm(TRANS, NOTRANS, n, n, n, w.data(), n, w.data(), n, c.data(), n);
  for (int j = 0; j < n; j++)
    for (int i = 0; i <= j; i++) g[(long)j * lda + i] = c[(size_t)n * j + i] - y[i] * y[j];
  for (int j = 0; j < n; j++)
    for (int r = j + 1; r < n; r++) g[(long)j * lda + r] = g[(long)r * lda + j];
  return 0;
}

// Front half of the generalized eigenproblem, double (Factorization.GevdCore, Factorization.Gevd.cs:
// 330-365): Cholesky(B) in place (:335-343), C filled symmetrically from A's upper triangle
// (:346-357), every row of C solved with SolveTriangular(Lower, NoTrans) at stride n (:358-361),
// then every column (:362-365): C = L^-1 A L^-T, leading dimension n.  Returns 0, or Cholesky's
// k+1 (MatFlat throws "The right-hand side matrix is not positive definite." there).
int orc_dgevd_front(int n, const double* a, int lda, double* b, int ldb, double* c) {
  const int info = orc_dcholesky(n, b, ldb);
  if (info != 0) return info;
  for (int j = 0; j < n; j++) {
    const double* aColj = a + (long)lda * j;
    for (int i = 0; i < j; i++) {
      c[(long)n * j + i] = aColj[i];
      c[(long)n * i + j] = aColj[i];
    }
    c[(long)n * j + j] = aColj[j];
  }
  for (int i = 0; i < n; i++) orc_dtrsv(LOWER, NOTRANS, n, b, ldb, c + i, n);
  for (int i = 0; i < n; i++) orc_dtrsv(LOWER, NOTRANS, n, b, ldb, c + (long)n * i, 1);
  return 0;
}

// Float overload (Factorization.Gevd.cs:282-318): the same steps with float storage, through the
// float Cholesky and SolveTriangular (double dots, float results).
int orc_sgevd_front(int n, const float* a, int lda, float* b, int ldb, float* c) {
  const int info = orc_scholesky(n, b, ldb);
  if (info != 0) return info;
  for (int j = 0; j < n; j++) {
    const float* aColj = a + (long)lda * j;
    for (int i = 0; i < j; i++) {
      c[(long)n * j + i] = aColj[i];
      c[(long)n * i + j] = aColj[i];
    }
    c[(long)n * j + j] = aColj[j];
  }
  for (int i = 0; i < n; i++) orc_strsv(LOWER, NOTRANS, n, b, ldb, c + i, n);
  for (int i = 0; i < n; i++) orc_strsv(LOWER, NOTRANS, n, b, ldb, c + (long)n * i, 1);
  return 0;
}

// Complex overload (Factorization.Gevd.cs:378-422): B = L L^H; C(i,j) = A(i,j) above the diagonal,
// conj(A(j,i)) below it, A(j,j) on it (:393-406); each row of C is conjugated, solved at stride n
// and conjugated back (:407-418); then every column is solved (:419-422).  Interleaved doubles.
int orc_zgevd_front(int n, const double* a_, int lda, double* b_, int ldb, double* c_) {
  const int info = orc_zcholesky(n, b_, ldb);
  if (info != 0) return info;
  const cplx* a = reinterpret_cast<const cplx*>(a_);
  cplx* c = reinterpret_cast<cplx*>(c_);
  for (int j = 0; j < n; j++) {
    const cplx* aColj = a + (long)lda * j;
    for (int i = 0; i < j; i++) {
      c[(long)n * j + i] = aColj[i];
      c[(long)n * i + j] = cconj(aColj[i]);
    }
    c[(long)n * j + j] = aColj[j];
  }
  for (int i = 0; i < n; i++) {
    for (int k = 0; k < n; k++) c[(long)n * k + i] = cconj(c[(long)n * k + i]);
    orc_ztrsv(LOWER, NOTRANS, n, b_, ldb, reinterpret_cast<double*>(c + i), n);
    for (int k = 0; k < n; k++) c[(long)n * k + i] = cconj(c[(long)n * k + i]);
  }
  for (int i = 0; i < n; i++)
    orc_ztrsv(LOWER, NOTRANS, n, b_, ldb, reinterpret_cast<double*>(c + (long)n * i), 1);
  return 0;
}

// ---------------------------------------------------------------------------------------------
// Batched drivers over std::thread.  Matrices are packed: matrix i starts at a + a_off[i]
// (elements), has order n[i] and leading dimension n[i]; vectors start at b + b_off[i].
// Work is split by an atomic counter over the batch (dynamic chunks), which balances uneven n.

}  // extern "C"

template <typename F>
static void parallel_for(long count, int nthreads, F f) {
  if (nthreads <= 1) {
    for (long i = 0; i < count; i++) f(i);
    return;
  }
  std::atomic<long> next(0);
  const long chunk = 16;
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; t++) {
    th.emplace_back([&]() {
      for (;;) {
        long s = next.fetch_add(chunk);
        if (s >= count) break;
        long e = std::min(count, s + chunk);
        for (long i = s; i < e; i++) f(i);
      }
    });
  }
  for (auto& x : th) x.join();
}

extern "C" {

// Config "Cholesky then SolveTriangular": per matrix, Cholesky; then L y = b (Lower/NoTrans)
// and L^T x = y (Lower/Trans).  info[i] = Cholesky return code; b is left untouched on failure.
void orc_dchol_solve_batched(long count, const int* n, const int64_t* a_off, double* a,
                             const int64_t* b_off, double* b, int* info, int nthreads) {
  parallel_for(count, nthreads, [&](long i) {
    int ni = n[i];
    double* ai = a + a_off[i];
    int r = orc_dcholesky(ni, ai, ni);
    info[i] = r;
    if (r == 0) {
      orc_dtrsv(LOWER, NOTRANS, ni, ai, ni, b + b_off[i], 1);
      orc_dtrsv(LOWER, TRANS, ni, ai, ni, b + b_off[i], 1);
    }
  });
}

// Float and Complex overloads: Cholesky, then L y = b and L^T x = y (float) or L^H x = y
// (Complex: Lower/ConjTrans, A = L L^H) for nrhs columns (ldb = n[i]; offsets in elements).
void orc_schol_solve_batched(long count, const int* n, const int64_t* a_off, float* a,
                             const int64_t* b_off, float* b, int nrhs, int* info, int nthreads) {
  parallel_for(count, nthreads, [&](long i) {
    const int ni = n[i];
    float* ai = a + a_off[i];
    const int r = orc_scholesky(ni, ai, ni);
    info[i] = r;
    if (r == 0)
      for (int c = 0; c < nrhs; c++) {
        float* x = b + b_off[i] + (long)ni * c;
        orc_strsv(LOWER, NOTRANS, ni, ai, ni, x, 1);
        orc_strsv(LOWER, TRANS, ni, ai, ni, x, 1);
      }
  });
}
void orc_zchol_solve_batched(long count, const int* n, const int64_t* a_off, double* a,
                             const int64_t* b_off, double* b, int nrhs, int* info, int nthreads) {
  parallel_for(count, nthreads, [&](long i) {
    const int ni = n[i];
    double* ai = a + 2 * a_off[i];
    const int r = orc_zcholesky(ni, ai, ni);
    info[i] = r;
    if (r == 0)
      for (int c = 0; c < nrhs; c++) {
        double* x = b + 2 * (b_off[i] + (long)ni * c);
        orc_ztrsv(LOWER, NOTRANS, ni, ai, ni, x, 1);
        orc_ztrsv(LOWER, CONJTRANS, ni, ai, ni, x, 1);
      }
  });
}

// Config "LU + forward/back solve": per matrix, Lu then the solve above for nrhs columns
// (ldb = n[i]).  sign[i] receives Lu's return value.
void orc_dlu_solve_batched(long count, const int* n, const int64_t* a_off, double* a,
                           const int64_t* piv_off, int* piv, const int64_t* b_off, double* b,
                           int nrhs, int* sign, int nthreads) {
  parallel_for(count, nthreads, [&](long i) {
    int ni = n[i];
    double* ai = a + a_off[i];
    int* pi = piv + piv_off[i];
    sign[i] = orc_dlu(ni, ni, ai, ni, pi);
    if (nrhs > 0) orc_dlu_solve(ni, ai, ni, pi, nrhs, b + b_off[i], ni);
  });
}

// Batched Factorization.LuInverse over LU factors (lda = n): info[i] = 0, or j+1 for the first
// zero diagonal entry of U (LuInverse.cs:145-152 throws there; the matrix is left unchanged).
void orc_dlu_inverse_batched(long count, const int* n, const int64_t* a_off, double* a,
                             const int64_t* piv_off, const int* piv, int* info, int nthreads) {
  parallel_for(count, nthreads, [&](long i) {
    const int ni = n[i];
    double* ai = a + a_off[i];
    int bad = 0;
    for (int j = 0; j < ni && !bad; j++)
      if (ai[(long)ni * j + j] == 0.0) bad = j + 1;
    info[i] = bad;
    if (!bad) orc_dlu_inverse(ni, ai, ni, piv + piv_off[i]);
  });
}

// The float and Complex overloads of the batched LuInverse (offsets in elements).
void orc_slu_inverse_batched(long count, const int* n, const int64_t* a_off, float* a,
                             const int64_t* piv_off, const int* piv, int* info, int nthreads) {
  parallel_for(count, nthreads, [&](long i) {
    const int ni = n[i];
    float* ai = a + a_off[i];
    int bad = 0;
    for (int j = 0; j < ni && !bad; j++)
      if (ai[(long)ni * j + j] == 0.0f) bad = j + 1;
    info[i] = bad;
    if (!bad) orc_slu_inverse(ni, ai, ni, piv + piv_off[i]);
  });
}
void orc_zlu_inverse_batched(long count, const int* n, const int64_t* a_off, double* a,
                             const int64_t* piv_off, const int* piv, int* info, int nthreads) {
  parallel_for(count, nthreads, [&](long i) {
    const int ni = n[i];
    double* ai = a + 2 * a_off[i];
    int bad = 0;
    for (int j = 0; j < ni && !bad; j++) {
      const double* d = ai + 2 * ((long)ni * j + j);
      if (d[0] == 0.0 && d[1] == 0.0) bad = j + 1;
    }
    info[i] = bad;
    if (!bad) orc_zlu_inverse(ni, ai, ni, piv + piv_off[i]);
  });
}

// Batched GEVD front half (lda = ldb = n): pair i is A at a + a_off[i], B at b + b_off[i], and C
// is written at c + a_off[i].
void orc_dgevd_front_batched(long count, const int* n, const int64_t* a_off, const double* a,
                             const int64_t* b_off, double* b, double* c, int* info, int nthreads) {
  parallel_for(count, nthreads, [&](long i) {
    info[i] = orc_dgevd_front(n[i], a + a_off[i], n[i], b + b_off[i], n[i], c + a_off[i]);
  });
}
void orc_sgevd_front_batched(long count, const int* n, const int64_t* a_off, const float* a,
                             const int64_t* b_off, float* b, float* c, int* info, int nthreads) {
  parallel_for(count, nthreads, [&](long i) {
    info[i] = orc_sgevd_front(n[i], a + a_off[i], n[i], b + b_off[i], n[i], c + a_off[i]);
  });
}
// Complex: offsets in Complex elements, arrays as interleaved doubles.
void orc_zgevd_front_batched(long count, const int* n, const int64_t* a_off, const double* a,
                             const int64_t* b_off, double* b, double* c, int* info, int nthreads) {
  parallel_for(count, nthreads, [&](long i) {
    info[i] = orc_zgevd_front(n[i], a + 2 * a_off[i], n[i], b + 2 * b_off[i], n[i],
                              c + 2 * a_off[i]);
  });
}

// Float and Complex overloads of the batched LU + solve (offsets in elements of the type).
void orc_slu_solve_batched(long count, const int* n, const int64_t* a_off, float* a,
                           const int64_t* piv_off, int* piv, const int64_t* b_off, float* b,
                           int nrhs, int* sign, int nthreads) {
  parallel_for(count, nthreads, [&](long i) {
    const int ni = n[i];
    sign[i] = orc_slu(ni, ni, a + a_off[i], ni, piv + piv_off[i]);
    if (nrhs > 0) orc_slu_solve(ni, a + a_off[i], ni, piv + piv_off[i], nrhs, b + b_off[i], ni);
  });
}
void orc_zlu_solve_batched(long count, const int* n, const int64_t* a_off, double* a,
                           const int64_t* piv_off, int* piv, const int64_t* b_off, double* b,
                           int nrhs, int* sign, int nthreads) {
  parallel_for(count, nthreads, [&](long i) {
    const int ni = n[i];
    double* ai = a + 2 * a_off[i];
    sign[i] = orc_zlu(ni, ni, ai, ni, piv + piv_off[i]);
    if (nrhs > 0) orc_zlu_solve(ni, ai, ni, piv + piv_off[i], nrhs, b + 2 * b_off[i], ni);
  });
}

// Config "differentiable Cholesky": per matrix orc_dchol_grad (lda = n); g has the layout of a.
void orc_dchol_grad_batched(long count, const int* n, const int64_t* a_off, double* a,
                            const int64_t* b_off, double* y, double* loss, double* g, int* info,
                            int nthreads) {
  parallel_for(count, nthreads, [&](long i) {
    info[i] = orc_dchol_grad(n[i], a + a_off[i], n[i], y + b_off[i], loss + i, g + a_off[i]);
  });
}

// Config "QR + least squares": a_off/m/n per matrix (lda = m), b has m entries, x has n.
void orc_dqr_ls_batched(long count, const int* m, const int* n, const int64_t* a_off, double* a,
                        const int64_t* b_off, const double* b, const int64_t* x_off, double* x,
                        int nthreads) {
  parallel_for(count, nthreads, [&](long i) {
    orc_dqr_ls(m[i], n[i], a + a_off[i], m[i], b + b_off[i], x + x_off[i]);
  });
}
void orc_sqr_ls_batched(long count, const int* m, const int* n, const int64_t* a_off, float* a,
                        const int64_t* b_off, const float* b, const int64_t* x_off, float* x,
                        int nthreads) {
  parallel_for(count, nthreads, [&](long i) {
    orc_sqr_ls(m[i], n[i], a + a_off[i], m[i], b + b_off[i], x + x_off[i]);
  });
}

}  // extern "C"
