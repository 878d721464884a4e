"""The reference's bucket multiselect on the GPU -- test and measurement
infrastructure (the GPU tests and the bench's reference-GPU leg use it as a
checker and a comparison; the product never imports it).

Two parts, both built into oracle/_ref/ (git-ignored; built files there travel
to the GPU machine with the tree):
  ref_kernels.cubin   the reference's own kernels (bucketMultiselect.cu,
                      multiselectTimingFunctions.cu) compiled for sm_103a from
                      its sources in place (GGKS_REFERENCE, default
                      /root/reference) -- built only where those sources are;
  libggks_ref_gpu.so  ref_gpu/ref_gpu_host.cu: the reference's host code
                      (phaseOne, generatePivots, bucketMultiselectWrapper and
                      the timing adapters) restated, loading the cubin and
                      launching its kernels in the reference's order -- built
                      wherever nvcc is, once the cubin exists.

k's follow the reference's wrapper convention: k-th LARGEST, 1-based.
Vectors handed to the device entry must be readable one element past n (the
reference's sampling can read x[n]; ref_gpu_host.cu says why), which
``padded_device_copy`` provides.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC_DIR = os.path.join(HERE, "ref_gpu")
OUT_DIR = os.path.join(HERE, "_ref")
CUBIN = os.path.join(OUT_DIR, "ref_kernels.cubin")
LIB = os.path.join(OUT_DIR, "libggks_ref_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
REF_SOURCES = ("bucketMultiselect.cu", "multiselectTimingFunctions.cu")

_SUFFIX = {np.dtype(np.float32): "f32", np.dtype(np.float64): "f64",
           np.dtype(np.uint32): "u32"}
_lib = None
_lock = threading.Lock()


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _reference_root():
    return os.environ.get("GGKS_REFERENCE", "/root/reference")


def _stale(out, deps):
    return not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(d) for d in deps)


def build_cubin(force=False):
    """Compiles the reference's kernels where its sources are; returns the
    cubin's path, or None without the sources (an existing cubin is kept)."""
    ref = _reference_root()
    srcs = [os.path.join(ref, s) for s in REF_SOURCES]
    if not all(os.path.isfile(s) for s in srcs):
        return CUBIN if os.path.exists(CUBIN) else None
    tu = os.path.join(SRC_DIR, "ref_kernels.cu")
    deps = srcs + [tu, os.path.join(SRC_DIR, "ref_gpu_shim.h"), __file__]
    if force or _stale(CUBIN, deps):
        os.makedirs(OUT_DIR, exist_ok=True)
        tmp = CUBIN + f".{os.getpid()}"
        cmd = [_nvcc(), "-cubin", *ARCH, "-O3", "-std=c++17", "-w", "-I", SRC_DIR,
               f'-DGGKS_REF_BUCKET_MULTISELECT="{srcs[0]}"',
               f'-DGGKS_REF_TIMING_FUNCTIONS="{srcs[1]}"', tu, "-o", tmp]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compiling the reference's kernels failed:\n" + r.stderr[-4000:])
        os.replace(tmp, CUBIN)
    return CUBIN


def build_host(force=False):
    """Compiles the restated host driver (needs nvcc, not the reference)."""
    src = os.path.join(SRC_DIR, "ref_gpu_host.cu")
    if force or _stale(LIB, [src, __file__]):
        os.makedirs(OUT_DIR, exist_ok=True)
        tmp = LIB + f".{os.getpid()}"
        cmd = [_nvcc(), *ARCH, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", src,
               "-o", tmp, "-lcuda"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compiling the reference's host driver failed:\n" + r.stderr[-4000:])
        os.replace(tmp, LIB)
    return LIB


def build(force=False):
    """Builds what can be built here: the cubin where the reference's sources
    are, the host driver wherever the cubin is.  Returns why the reference's
    GPU path is unavailable, or None when both parts exist."""
    if build_cubin(force) is None:
        return "the reference's kernels were never compiled (no cubin, no reference sources)"
    build_host(force)
    return None


def unavailable():
    """None when the reference's GPU path can run here, else why not."""
    if not os.path.exists(CUBIN):
        return "no cubin of the reference's kernels (oracle/_ref/ref_kernels.cubin)"
    if not os.path.exists(LIB):
        return "host driver not built (oracle/_ref/libggks_ref_gpu.so)"
    return None


def lib():
    global _lib
    with _lock:
        if _lib is None:
            why = unavailable()
            if why:
                raise RuntimeError(why)
            L = ctypes.CDLL(LIB)
            P, I, U = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint
            L.ggks_refgpu_load.argtypes = [ctypes.c_char_p]
            L.ggks_refgpu_load.restype = I
            L.ggks_refgpu_device_shape.argtypes = [P, P]
            L.ggks_refgpu_device_shape.restype = I
            for s in ("f32", "f64", "u32"):
                f = getattr(L, "ggks_refgpu_bucket_multiselect_" + s)
                f.argtypes = [P, I, P, I, P, I, I, P]
                f.restype = I
                for name, args in (("time_bucket_multiselect_", [P, U, P, U, P]),
                                   ("time_bucket_topk_", [P, U, U, P]),
                                   ("time_sort_choose_multiselect_", [P, U, P, U, P]),
                                   ("time_sort_choose_topk_", [P, U, U, P])):
                    f = getattr(L, "ggks_refgpu_" + name + s)
                    f.argtypes = args
                    f.restype = ctypes.c_float
            rc = L.ggks_refgpu_load(CUBIN.encode())
            if rc != 0:
                raise RuntimeError(f"loading the reference's kernels failed ({rc})")
            _lib = L
    return _lib


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def device_shape():
    """(SM count, max threads per block): the launch shape the reference's
    timing adapters pass (multiselectTimingFunctions.cu:113)."""
    sms, mt = ctypes.c_int(), ctypes.c_int()
    if lib().ggks_refgpu_device_shape(ctypes.byref(sms), ctypes.byref(mt)) != 0:
        raise RuntimeError("cudaGetDeviceProperties failed")
    return sms.value, mt.value


def padded_device_copy(x):
    """A torch device tensor of n + 1 elements: x, then x[0] (the element the
    reference's sampling may read past the end)."""
    import torch
    x = np.ascontiguousarray(x)
    carrier = x.view(np.int32) if x.dtype == np.uint32 else x
    t = torch.empty(x.size + 1, dtype=torch.from_numpy(carrier[:1]).dtype, device="cuda")
    t[:x.size].copy_(torch.from_numpy(carrier))
    t[x.size:].copy_(torch.from_numpy(carrier[:1]))
    return t


def bucket_multiselect_device(d_ptr, n, k, dtype):
    """bucketMultiselectWrapper on a resident vector (d_ptr from
    padded_device_copy); returns (outputs, wrapper milliseconds)."""
    dtype = np.dtype(dtype)
    k = np.ascontiguousarray(k, dtype=np.uint32)
    out = np.empty(k.size, dtype=dtype)
    ms = ctypes.c_float()
    sms, mt = device_shape()
    f = getattr(lib(), "ggks_refgpu_bucket_multiselect_" + _SUFFIX[dtype])
    rc = f(ctypes.c_void_p(d_ptr), int(n), _ptr(k), int(k.size), _ptr(out), sms, mt,
           ctypes.byref(ms))
    if rc != 1:
        raise RuntimeError("the reference's bucketMultiselectWrapper failed")
    return out, ms.value


def _timed(name, x, arg, nout):
    x = np.ascontiguousarray(x)
    out = np.empty(nout, dtype=x.dtype)
    f = getattr(lib(), "ggks_refgpu_" + name + _SUFFIX[x.dtype])
    if isinstance(arg, np.ndarray):
        ms = f(_ptr(x), x.size, _ptr(arg), arg.size, _ptr(out))
    else:
        ms = f(_ptr(x), x.size, int(arg), _ptr(out))
    if ms < 0:
        raise RuntimeError(f"the reference's {name.rstrip('_')} failed")
    return out, float(ms)


def time_bucket_multiselect(x, k):
    """timeBucketMultiselect (multiselectTimingFunctions.cu:100-122) on a host
    vector: (outputs in k order, milliseconds of the wrapper)."""
    k = np.ascontiguousarray(k, dtype=np.uint32)
    return _timed("time_bucket_multiselect_", x, k, k.size)


def time_bucket_topk(x, K):
    """timeBucketTopkselect (:205-231): the K largest, descending."""
    return _timed("time_bucket_topk_", x, K, K)


def time_sort_choose_multiselect(x, k):
    """timeSortAndChooseMultiselect (:51-95): Thrust sort on the device."""
    k = np.ascontiguousarray(k, dtype=np.uint32)
    return _timed("time_sort_choose_multiselect_", x, k, k.size)


def time_sort_choose_topk(x, K):
    """timeSortAndChooseTopkselect (:156-177)."""
    return _timed("time_sort_choose_topk_", x, K, K)
