"""matflat_gb300 — GB300-native implementation of MatFlat's factorization hot path.

The compute path is the CUDA library `libmatflat_gpu.so` (C ABI in include/matflat_gpu.h).  This
package is the host-side mirror of MatFlat's C# surface over that ABI, for Python callers, the
tests and the benchmark:

  * `Factorization` and `Blas` keep MatFlat's static-method names and argument meaning
    (MatFlat/Factorization*.cs, MatFlat/Blas*.cs).  Where C# takes `double*`, these take a 1-D
    numpy array holding the column-major data with its leading dimension, and work in place.
  * MatFlat's exceptions are mirrored: ArgumentException, ArgumentNullException,
    MatrixFactorizationException (with MatFlat's messages).
  * `LuBatch` / `LuInverseBatch` / `CholeskyBatch` are the batched overloads (device-resident
    batches).

There is no CPU fallback: if the CUDA library is missing or no GPU is present, every call raises.
"""
from ._api import (  # noqa: F401
    ArgumentException,
    ArgumentNullException,
    Blas,
    CholeskyBatch,
    Factorization,
    GevdFrontBatch,
    LuBatch,
    LuInverseBatch,
    MatFlatException,
    MatrixFactorizationException,
    MixedSolveBatch,
    QrBatch,
    StridedBlas,
    Transpose,
    Uplo,
    context,
    library,
    library_path,
    selftest_dmul,
    selftest_ddiv,
)

__version__ = "0.1.0"
