"""CPU-side checks of the C ABI: the library builds for sm_103a, loads, and exports exactly the
entry points include/*.h declares (no GPU is touched)."""
import ctypes
import glob
import os
import re

from tests.conftest import ROOT


def declared_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        syms |= set(re.findall(r"MFG_API\s+[\w\s\*]+?\b(mfg_\w+)\s*\(", text))
    return syms


def test_header_declares_entry_points():
    syms = declared_symbols()
    for must in ("mfg_create", "mfg_dgetrf", "mfg_dpotrf", "mfg_dgeqrf", "mfg_dtrsv", "mfg_dgemm",
                 "mfg_dgetrf_batched", "mfg_dpotrf_batched", "mfg_dgeqrf_batched"):
        assert must in syms


def test_library_exports_every_declared_symbol():
    from matflat_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [s for s in sorted(declared_symbols()) if not hasattr(lib, s)]
    assert not missing, missing


def test_library_exports_nothing_undeclared():
    from matflat_gb300 import build
    path = build.build()
    out = os.popen("nm -D --defined-only %s" % path).read()
    exported = set(re.findall(r" T (mfg_\w+)", out))
    assert exported == declared_symbols()


def test_create_without_device_fails_loudly():
    """With no visible GPU the library refuses to create a context (no CPU fallback)."""
    import subprocess
    import sys
    code = ("import os,ctypes; os.environ['CUDA_VISIBLE_DEVICES']=''; "
            "lib=ctypes.CDLL(%r); h=ctypes.c_void_p(); "
            "print(lib.mfg_create(ctypes.byref(h)))" % os.path.join(
                ROOT, "matflat_gb300", "_lib", "libmatflat_gpu.so"))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                         timeout=120)
    assert out.stdout.strip() == "-1001", out.stdout + out.stderr


def test_python_facade_raises_without_device():
    import subprocess
    import sys
    code = ("import os; os.environ['CUDA_VISIBLE_DEVICES']=''; import sys; sys.path.insert(0, %r);"
            "import numpy as np, matflat_gb300 as mf\n"
            "try:\n mf.Factorization.Lu(2,2,np.zeros(4),2,np.zeros(2,np.int32)); print('ran')\n"
            "except RuntimeError as e: print('raised')" % ROOT)
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                         timeout=120)
    assert out.stdout.strip() == "raised", out.stdout + out.stderr


def test_every_status_code_is_returned_somewhere():
    """Each MFG_ERR_* status the header declares is produced by some code path of the library
    (named in code, not only in comments): the ABI promises no status that can never occur."""
    header = open(os.path.join(ROOT, "include", "matflat_gpu.h")).read()
    codes = set(re.findall(r"\b(MFG_ERR_\w+)\s*=", header))
    assert codes, "no status codes found"
    src = ""
    for f in glob.glob(os.path.join(ROOT, "matflat_gb300", "csrc", "*.cu")):
        text = re.sub(r"/\*.*?\*/", "", open(f).read(), flags=re.S)
        src += re.sub(r"//[^\n]*", "", text)
    unused = [c for c in sorted(codes) if not re.search(r"\b%s\b" % c, src)]
    assert not unused, unused


def test_library_package_is_torch_free_and_loads_no_workload_helper():
    """The product package imports neither torch nor the benchmark's input generator."""
    for f in glob.glob(os.path.join(ROOT, "matflat_gb300", "*.py")):
        text = open(f).read()
        assert not re.search(r"^\s*(import torch|from torch)", text, re.M), f
        assert not re.search(r"^\s*(import workloads|from workloads)", text, re.M), f
        assert "libworkloads_synth" not in text, f
