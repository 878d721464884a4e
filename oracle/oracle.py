"""ctypes loader for the CPU oracle (oracle/ggks_oracle.c).

TEST INFRASTRUCTURE ONLY: the tests, the smoke check and the CPU-baseline leg
of bench.py use this module as the checker.  The product library never imports
it.

Every function takes and returns numpy arrays.  ``k`` follows the reference's
wrapper convention (bucketMultiselect.cu:842-846): k-th LARGEST, 1-based, so
``out[i] == ascending[n - k[i]]`` (multiselectTimingFunctions.cu:46).
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libggks_oracle.so")
SRC_PATH = os.path.join(_HERE, "ggks_oracle.c")
SRC_CPP = os.path.join(_HERE, "ggks_oracle_stdsort.cpp")
HDR_PATH = os.path.join(_HERE, "ggks_oracle.h")

_lib = None

_SUFFIX = {np.dtype(np.float32): "f32", np.dtype(np.float64): "f64",
           np.dtype(np.uint32): "u32"}


def build(force=False):
    """Compile the oracle (gcc for the C restatement, g++ for the std::sort
    baseline) into oracle/libggks_oracle.so."""
    srcs = (SRC_PATH, SRC_CPP, HDR_PATH)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(p) for p in srcs)):
        return LIB_PATH
    tmp = LIB_PATH + f".{os.getpid()}"
    o_c, o_cpp = tmp + ".c.o", tmp + ".cpp.o"
    subprocess.run(["gcc", "-O3", "-std=c11", "-fPIC", "-pthread", "-c", SRC_PATH, "-o", o_c],
                   check=True)
    subprocess.run(["g++", "-O3", "-std=c++17", "-fPIC", "-c", SRC_CPP, "-o", o_cpp], check=True)
    subprocess.run(["g++", "-shared", "-pthread", o_c, o_cpp, "-o", tmp, "-lm"], check=True)
    os.replace(tmp, LIB_PATH)  # atomic: concurrent builders never see a partial file
    for f in (o_c, o_cpp):
        os.remove(f)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        for sfx in ("f32", "f64", "u32"):
            f = getattr(L, "ggks_oracle_multiselect_" + sfx)
            f.argtypes = [P, ctypes.c_uint64, P, ctypes.c_uint32, P, ctypes.c_int]
            f.restype = ctypes.c_int
            f = getattr(L, "ggks_oracle_topk_" + sfx)
            f.argtypes = [P, ctypes.c_uint64, ctypes.c_uint32, P, ctypes.c_int]
            f.restype = ctypes.c_int
            f = getattr(L, "ggks_oracle_bucket_multiselect_" + sfx)
            f.argtypes = [P, ctypes.c_uint32, P, ctypes.c_uint32, P, ctypes.c_uint64]
            f.restype = ctypes.c_int
            f = getattr(L, "ggks_oracle_multiselect_stdsort_" + sfx)
            f.argtypes = [P, ctypes.c_uint64, P, ctypes.c_uint32, P]
            f.restype = ctypes.c_int
        for sfx in ("u32", "u64"):
            f = getattr(L, "ggks_oracle_sort_keys_" + sfx)
            f.argtypes = [P, ctypes.c_uint64, ctypes.c_int]
            f.restype = ctypes.c_int
        _lib = L
    return _lib


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def _check(rc, what):
    if rc != 0:
        raise ValueError(f"{what}: oracle status {rc}")


def multiselect(vec, k, threads=1):
    """Sort-and-choose multiselect (multiselectTimingFunctions.cu:51-95)."""
    vec = np.ascontiguousarray(vec)
    k = np.ascontiguousarray(k, dtype=np.uint32)
    out = np.empty(len(k), dtype=vec.dtype)
    sfx = _SUFFIX[vec.dtype]
    rc = getattr(lib(), "ggks_oracle_multiselect_" + sfx)(
        _ptr(vec), vec.size, _ptr(k), k.size, _ptr(out), int(threads))
    _check(rc, "multiselect")
    return out


def multiselect_stdsort(vec, k):
    """Sort-and-choose multiselect with one thread's std::sort (the CPU
    baseline of the benchmark)."""
    vec = np.ascontiguousarray(vec)
    k = np.ascontiguousarray(k, dtype=np.uint32)
    out = np.empty(len(k), dtype=vec.dtype)
    sfx = _SUFFIX[vec.dtype]
    rc = getattr(lib(), "ggks_oracle_multiselect_stdsort_" + sfx)(
        _ptr(vec), vec.size, _ptr(k), k.size, _ptr(out))
    _check(rc, "multiselect_stdsort")
    return out


def topk(vec, K, threads=1):
    """Sort-and-choose top-k (multiselectTimingFunctions.cu:156-177)."""
    vec = np.ascontiguousarray(vec)
    out = np.empty(int(K), dtype=vec.dtype)
    sfx = _SUFFIX[vec.dtype]
    rc = getattr(lib(), "ggks_oracle_topk_" + sfx)(
        _ptr(vec), vec.size, int(K), _ptr(out), int(threads))
    _check(rc, "topk")
    return out


def bucket_multiselect(vec, k, seed=1):
    """The reference's bucket algorithm run on the CPU
    (bucketMultiselect.cu:521-871)."""
    vec = np.ascontiguousarray(vec)
    k = np.ascontiguousarray(k, dtype=np.uint32)
    out = np.empty(len(k), dtype=vec.dtype)
    sfx = _SUFFIX[vec.dtype]
    rc = getattr(lib(), "ggks_oracle_bucket_multiselect_" + sfx)(
        _ptr(vec), vec.size, _ptr(k), k.size, _ptr(out), int(seed))
    _check(rc, "bucket_multiselect")
    return out


def sort_keys(keys, threads=1):
    keys = np.array(keys, copy=True)
    sfx = "u32" if keys.dtype == np.uint32 else "u64"
    rc = getattr(lib(), "ggks_oracle_sort_keys_" + sfx)(_ptr(keys), keys.size, int(threads))
    _check(rc, "sort_keys")
    return keys
