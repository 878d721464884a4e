"""Python binding (ctypes) of libggks_gb300.so, the GB300 GGKS bucket
multiselect / top-k library, plus Python mirrors of the reference's host-side
interface for this path:

* ``bucketMultiselectWrapper``   -- BucketMultiselect::bucketMultiselectWrapper
  (bucketMultiselect.cu:837-871): device vector, k list (k-th largest),
  outputs in k order; blocks/threads accepted and ignored.
* ``timeBucketMultiselect`` / ``timeBucketTopkselect`` -- the timing adapters
  of multiselectTimingFunctions.cu:100-122 and :205-231, returning a
  ``Results`` (time in ms, values) like ``results_t<T>`` (:11-14).

The CUDA library must be built (``ggks_build.build()``); importing this module
without it raises -- there is no CPU fallback.
"""
import ctypes
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libggks_gb300.so")

OK, INVALID_ARG, OOM, CUDA_ERROR, TIMEOUT, INTERNAL, NO_DEVICE, UNSUPPORTED = range(8)
FLAG_OUT_DEVICE = 1
FLAG_AUTOTUNE = 2
FLAG_TOPK_PIPELINE = 4
FLAG_NO_SMALL = 8
NUM_PASSES = 6
PASS_NAMES = ("sample", "hist", "scan", "plan", "compact", "finish")
NUM_BATCH_PHASES = 5
BATCH_PHASE_NAMES = ("table", "hist", "plan", "compact", "finish")

_SFX = {np.dtype(np.float32): "f32", np.dtype(np.float64): "f64", np.dtype(np.uint32): "u32"}


class GgksError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        super().__init__(f"{what}: ggks status {status} ({status_string(status)})")


class Opts(ctypes.Structure):
    _fields_ = [("ctx", ctypes.c_void_p), ("stream", ctypes.c_void_p),
                ("flags", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class Stats(ctypes.Structure):
    _fields_ = [("calls", ctypes.c_uint64), ("launches", ctypes.c_uint64),
                ("pass_launches", ctypes.c_uint64 * NUM_PASSES),
                ("pass_ms", ctypes.c_double * NUM_PASSES),
                ("bytes_in", ctypes.c_uint64), ("survivors", ctypes.c_uint64),
                ("retries", ctypes.c_uint64), ("recursions", ctypes.c_uint64),
                ("host_ingested", ctypes.c_uint64), ("host_staged", ctypes.c_uint64),
                ("batch_calls", ctypes.c_uint64), ("batch_problems", ctypes.c_uint64),
                ("batch_phase_ms", ctypes.c_double * NUM_BATCH_PHASES),
                ("batch_grid", ctypes.c_uint64), ("spec_calls", ctypes.c_uint64),
                ("spec_ctas", ctypes.c_uint64), ("topk_threshold_calls", ctypes.c_uint64),
                ("topk_misses", ctypes.c_uint64), ("batch_spec_tiles", ctypes.c_uint64),
                ("small_calls", ctypes.c_uint64), ("small_misses", ctypes.c_uint64)]

    def as_dict(self):
        return {"calls": self.calls, "launches": self.launches,
                "pass_launches": dict(zip(PASS_NAMES, list(self.pass_launches))),
                "pass_ms": dict(zip(PASS_NAMES, list(self.pass_ms))),
                "bytes_in": self.bytes_in, "survivors": self.survivors,
                "retries": self.retries, "recursions": self.recursions,
                "host_ingested": self.host_ingested, "host_staged": self.host_staged,
                "batch_calls": self.batch_calls, "batch_problems": self.batch_problems,
                "batch_phase_ms": dict(zip(BATCH_PHASE_NAMES, list(self.batch_phase_ms))),
                "batch_grid": self.batch_grid, "spec_calls": self.spec_calls,
                "spec_ctas": self.spec_ctas, "topk_threshold_calls": self.topk_threshold_calls,
                "topk_misses": self.topk_misses, "batch_spec_tiles": self.batch_spec_tiles,
                "small_calls": self.small_calls, "small_misses": self.small_misses}


DTYPE_CODES = {np.dtype(np.float32): 0, np.dtype(np.float64): 1, np.dtype(np.uint32): 2}
REQ_TOPK = 1
REQ_HOST_VECTOR = 2


class ServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("max_batch", ctypes.c_uint32),
                ("hbm_cap_bytes", ctypes.c_uint64), ("hbm_reserve_bytes", ctypes.c_uint64),
                ("lanes", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class Request(ctypes.Structure):
    _fields_ = [("dtype", ctypes.c_int32), ("flags", ctypes.c_uint32), ("vec", ctypes.c_void_p),
                ("n", ctypes.c_uint64), ("k", ctypes.c_void_p), ("num_k", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class ServerStats(ctypes.Structure):
    _fields_ = [(f, ctypes.c_uint64) for f in (
        "submitted", "completed", "batches", "batched_requests", "max_batch_seen", "launches",
        "uploads", "upload_bytes", "peak_bytes", "in_flight_bytes", "concurrent_launches",
        "hbm_waits", "admit_budget_bytes", "single_calls", "recursions")] + [
        ("batch_phase_ms", ctypes.c_double * NUM_BATCH_PHASES), ("kernel_ms", ctypes.c_double),
        ("group_ms", ctypes.c_double), ("device_busy_ms", ctypes.c_double),
        ("device_span_ms", ctypes.c_double)]

    def as_dict(self):
        d = {f: int(getattr(self, f)) for f, t in self._fields_ if t is ctypes.c_uint64}
        d["batch_phase_ms"] = dict(zip(BATCH_PHASE_NAMES, list(self.batch_phase_ms)))
        d["kernel_ms"] = float(self.kernel_ms)
        d["group_ms"] = float(self.group_ms)
        d["device_busy_ms"] = float(self.device_busy_ms)
        d["device_span_ms"] = float(self.device_span_ms)
        return d


# every symbol declared in include/ggks.h
EXPORTS = [
    "ggks_multiselect_f32", "ggks_multiselect_f64", "ggks_multiselect_u32",
    "ggks_multiselect_host_f32", "ggks_multiselect_host_f64", "ggks_multiselect_host_u32",
    "ggks_topk_f32", "ggks_topk_f64", "ggks_topk_u32",
    "ggks_topk_host_f32", "ggks_topk_host_f64", "ggks_topk_host_u32",
    "ggks_context_create", "ggks_context_destroy", "ggks_context_get_stats",
    "ggks_context_reset_stats", "ggks_context_set_profiling", "ggks_status_string",
    "ggks_version", "ggks_multiselect_noalloc_f32",
    "ggks_multiselect_batch_f32", "ggks_multiselect_batch_f64", "ggks_multiselect_batch_u32",
    "ggks_topk_batch_f32", "ggks_topk_batch_f64", "ggks_topk_batch_u32",
    "ggks_batch_last_tuning", "ggks_batch_set_tuning",
    "ggks_server_create", "ggks_server_destroy", "ggks_server_submit", "ggks_server_wait",
    "ggks_server_get_stats", "ggks_server_set_tuning",
    "ggks_select_f32", "ggks_select_f64", "ggks_select_u32",
]

_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with ggks_build.build()")
    L = ctypes.CDLL(LIB_PATH)
    P, U64, U32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32
    for sfx in ("f32", "f64", "u32"):
        for nm in ("ggks_multiselect_", "ggks_multiselect_host_"):
            f = getattr(L, nm + sfx)
            f.argtypes = [P, U64, P, U32, P, ctypes.POINTER(Opts)]
            f.restype = ctypes.c_int
        for nm in ("ggks_topk_", "ggks_topk_host_", "ggks_select_"):
            f = getattr(L, nm + sfx)
            f.argtypes = [P, U64, U32, P, ctypes.POINTER(Opts)]
            f.restype = ctypes.c_int
    for sfx in ("f32", "f64", "u32"):
        f = getattr(L, "ggks_multiselect_batch_" + sfx)
        f.argtypes = [P, P, U32, P, P, P, ctypes.POINTER(Opts)]
        f.restype = ctypes.c_int
        f = getattr(L, "ggks_topk_batch_" + sfx)
        f.argtypes = [P, P, U32, P, P, ctypes.POINTER(Opts)]
        f.restype = ctypes.c_int
    L.ggks_batch_last_tuning.argtypes = [P, ctypes.POINTER(ctypes.c_uint32),
                                         ctypes.POINTER(ctypes.c_uint32)]
    L.ggks_batch_last_tuning.restype = ctypes.c_int
    L.ggks_batch_set_tuning.argtypes = [P, U32, U32]
    L.ggks_batch_set_tuning.restype = ctypes.c_int
    L.ggks_server_create.argtypes = [ctypes.POINTER(ServerConfig), ctypes.POINTER(ctypes.c_void_p)]
    L.ggks_server_destroy.argtypes = [P]
    L.ggks_server_submit.argtypes = [P, ctypes.POINTER(Request), P, ctypes.POINTER(U64)]
    L.ggks_server_wait.argtypes = [P, U64, ctypes.POINTER(ctypes.c_double)]
    L.ggks_server_get_stats.argtypes = [P, ctypes.POINTER(ServerStats)]
    L.ggks_server_set_tuning.argtypes = [P, U32, U32]
    for nm in ("create", "destroy", "submit", "wait", "get_stats", "set_tuning"):
        getattr(L, "ggks_server_" + nm).restype = ctypes.c_int
    L.ggks_multiselect_noalloc_f32.argtypes = [P, U64, P, U32, P, P]
    L.ggks_multiselect_noalloc_f32.restype = ctypes.c_int
    L.ggks_context_create.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    L.ggks_context_destroy.argtypes = [P]
    L.ggks_context_get_stats.argtypes = [P, ctypes.POINTER(Stats)]
    L.ggks_context_reset_stats.argtypes = [P]
    L.ggks_context_set_profiling.argtypes = [P, ctypes.c_int]
    L.ggks_status_string.argtypes = [ctypes.c_int]
    L.ggks_status_string.restype = ctypes.c_char_p
    for f in (L.ggks_context_create, L.ggks_context_destroy, L.ggks_context_get_stats,
              L.ggks_context_reset_stats, L.ggks_context_set_profiling, L.ggks_version):
        f.restype = ctypes.c_int
    _lib = L
    return L


def status_string(st):
    try:
        return lib().ggks_status_string(int(st)).decode()
    except ImportError:
        return "?"


def _check(st, what):
    if st != OK:
        raise GgksError(st, what)


class Context:
    """An owned ggks_context (device, stream, workspace)."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        _check(lib().ggks_context_create(int(device), ctypes.byref(h)), "context_create")
        self.handle = h

    def close(self):
        if self.handle:
            hv = self.handle.value if isinstance(self.handle, ctypes.c_void_p) else self.handle
            for key in [k for k in _opts_refs if k[0] == hv]:
                del _opts_refs[key]
            lib().ggks_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stats(self):
        return get_stats(self)

    def reset_stats(self):
        reset_stats(self)

    def set_profiling(self, on=True, passes=None):
        set_profiling(self, on, passes)


def _h(ctx):
    return ctx.handle if isinstance(ctx, Context) else ctx


def _opts(ctx=None, stream=None, flags=0):
    o = Opts()
    o.ctx = _h(ctx)
    o.stream = stream
    o.flags = flags
    return o


_opts_refs = {}


def _opts_ref(ctx, stream, flags):
    """A reference to an Opts for (context, stream, flags), built once: a call
    of the pointer entry points then costs no structure construction."""
    h = _h(ctx)
    key = (h.value if isinstance(h, ctypes.c_void_p) else h, stream, flags)
    r = _opts_refs.get(key)
    if r is None:
        o = _opts(ctx, stream, flags)
        r = _opts_refs[key] = (o, ctypes.byref(o))  # the Opts lives as long as its reference
    return r[1]


def _addr(a):
    """Data address of a numpy array (cheaper than a.ctypes.data)."""
    return a.__array_interface__["data"][0]


def get_stats(ctx=None):
    s = Stats()
    _check(lib().ggks_context_get_stats(_h(ctx), ctypes.byref(s)), "get_stats")
    return s.as_dict()


def reset_stats(ctx=None):
    _check(lib().ggks_context_reset_stats(_h(ctx)), "reset_stats")


def set_profiling(ctx=None, on=True, passes=None):
    """Time the passes with CUDA events: all of them, or only those named in
    passes (names of PASS_NAMES)."""
    if not on:
        v = 0
    elif passes is None:
        v = 1
    else:
        mask = 0
        for p in passes:
            mask |= 1 << PASS_NAMES.index(p)
        v = ctypes.c_int32(0x80000000 | mask).value
    _check(lib().ggks_context_set_profiling(_h(ctx), v), "set_profiling")


# ---------------------------------------------------------------------------
# raw entry points (pointers)
# ---------------------------------------------------------------------------


def multiselect_ptr(d_ptr, n, dtype, k, ctx=None, stream=None, out=None, out_device_ptr=None,
                    small=True):
    """Multiselect of a device vector at d_ptr (n elements of dtype).
    Returns a host array of len(k) values, or writes to out_device_ptr.
    small=False runs the pipeline where the one-launch small-vector path
    (at most 2^20 elements and 1024 k's) would apply (same results)."""
    dtype = np.dtype(dtype)
    k = np.ascontiguousarray(k, dtype=np.uint32)
    flags = 0 if small else FLAG_NO_SMALL
    if out_device_ptr is not None:
        flags |= FLAG_OUT_DEVICE
        optr = out_device_ptr
    else:
        if out is None:
            out = np.empty(k.size, dtype=dtype)
        optr = _addr(out)
    st = getattr(lib(), "ggks_multiselect_" + _SFX[dtype])(
        d_ptr, int(n), _addr(k), k.size, optr, _opts_ref(ctx, stream, flags))
    _check(st, "multiselect")
    return out


def topk_ptr(d_ptr, n, dtype, K, ctx=None, stream=None, out=None, out_device_ptr=None,
             pipeline=False, small=True):
    """The K largest of the device vector at d_ptr, descending.  pipeline=True
    forces the histogram / compaction pipeline; small=False keeps the threshold
    path or the pipeline where the one-launch small-vector path (at most 2^18
    elements, K <= 1024) would apply (same results)."""
    dtype = np.dtype(dtype)
    flags = (FLAG_TOPK_PIPELINE if pipeline else 0) | (0 if small else FLAG_NO_SMALL)
    if out_device_ptr is not None:
        flags |= FLAG_OUT_DEVICE
        optr = out_device_ptr
    else:
        if out is None:
            out = np.empty(int(K), dtype=dtype)
        optr = _addr(out)
    st = getattr(lib(), "ggks_topk_" + _SFX[dtype])(
        d_ptr, int(n), int(K), optr, _opts_ref(ctx, stream, flags))
    _check(st, "topk")
    return out


def select_ptr(d_ptr, n, dtype, k, ctx=None, stream=None):
    """The k-th largest (1-based) of the device vector at d_ptr."""
    dtype = np.dtype(dtype)
    out = np.empty(1, dtype=dtype)
    o = _opts(ctx, stream)
    st = getattr(lib(), "ggks_select_" + _SFX[dtype])(ctypes.c_void_p(d_ptr), int(n), int(k),
                                                       out.ctypes.data, ctypes.byref(o))
    _check(st, "select")
    return out[0]


def multiselect_noalloc_f32(d_ptr, n, d_k_ptr, num_k, d_out_ptr, stream=None):
    """ggks_multiselect_noalloc_f32: every pointer is device memory; returns
    the ggks status (no exception), like the C call."""
    return lib().ggks_multiselect_noalloc_f32(ctypes.c_void_p(d_ptr), int(n),
                                              ctypes.c_void_p(d_k_ptr), int(num_k),
                                              ctypes.c_void_p(d_out_ptr), stream)


def multiselect_host(h_vec, k, ctx=None, stream=None, out=None):
    """Multiselect of a host vector (copied to the device inside the call)."""
    h_vec = np.ascontiguousarray(h_vec)
    k = np.ascontiguousarray(k, dtype=np.uint32)
    if out is None:
        out = np.empty(k.size, dtype=h_vec.dtype)
    o = _opts(ctx, stream)
    st = getattr(lib(), "ggks_multiselect_host_" + _SFX[h_vec.dtype])(
        h_vec.ctypes.data, h_vec.size, k.ctypes.data, k.size, out.ctypes.data, ctypes.byref(o))
    _check(st, "multiselect_host")
    return out


def topk_host(h_vec, K, ctx=None, stream=None, out=None, pipeline=False):
    """The K largest of a host vector (copied to the device inside the call),
    descending.  pipeline=True forces the histogram / compaction pipeline."""
    h_vec = np.ascontiguousarray(h_vec)
    if out is None:
        out = np.empty(int(K), dtype=h_vec.dtype)
    o = _opts(ctx, stream, FLAG_TOPK_PIPELINE if pipeline else 0)
    st = getattr(lib(), "ggks_topk_host_" + _SFX[h_vec.dtype])(
        h_vec.ctypes.data, h_vec.size, int(K), out.ctypes.data, ctypes.byref(o))
    _check(st, "topk_host")
    return out


def _batch_arrays(ptrs, ns):
    ptrs = np.ascontiguousarray(np.asarray(ptrs, dtype=np.uint64))
    ns = np.ascontiguousarray(np.asarray(ns, dtype=np.uint64))
    assert ptrs.size == ns.size
    return ptrs, ns


def multiselect_batch_ptr(ptrs, ns, dtype, k_lists, ctx=None, stream=None, autotune=False,
                          out_device_ptr=None):
    """Batched multiselect: problem p is the device vector at ptrs[p] with
    ns[p] elements of dtype and the k list k_lists[p] (k-th largest).  One
    persistent launch selects every problem.  Returns a list of host arrays
    (one per problem), or None when writing to out_device_ptr (outputs
    concatenated in problem order)."""
    dtype = np.dtype(dtype)
    ptrs, ns = _batch_arrays(ptrs, ns)
    sizes = np.array([len(k) for k in k_lists], dtype=np.int64)
    off = np.zeros(len(k_lists) + 1, dtype=np.uint32)
    np.cumsum(sizes, out=off[1:])
    ks = (np.concatenate([np.asarray(k, dtype=np.uint32) for k in k_lists])
          if len(k_lists) else np.zeros(0, np.uint32))
    ks = np.ascontiguousarray(ks, dtype=np.uint32)
    flags = FLAG_AUTOTUNE if autotune else 0
    if out_device_ptr is not None:
        flags |= FLAG_OUT_DEVICE
        optr, out = out_device_ptr, None
    else:
        out = np.empty(int(off[-1]), dtype=dtype)
        optr = out.ctypes.data
    o = _opts(ctx, stream, flags)
    st = getattr(lib(), "ggks_multiselect_batch_" + _SFX[dtype])(
        ptrs.ctypes.data, ns.ctypes.data, ptrs.size, off.ctypes.data,
        ks.ctypes.data if ks.size else None, ctypes.c_void_p(optr), ctypes.byref(o))
    _check(st, "multiselect_batch")
    if out is None:
        return None
    return [out[off[p]:off[p + 1]] for p in range(ptrs.size)]


def topk_batch_ptr(ptrs, ns, dtype, Ks, ctx=None, stream=None, autotune=False):
    """Batched top-k: the Ks[p] largest of each device vector, descending."""
    dtype = np.dtype(dtype)
    ptrs, ns = _batch_arrays(ptrs, ns)
    Ks = np.ascontiguousarray(np.asarray(Ks, dtype=np.uint32))
    off = np.zeros(Ks.size + 1, dtype=np.int64)
    np.cumsum(Ks, out=off[1:])
    out = np.empty(int(off[-1]), dtype=dtype)
    o = _opts(ctx, stream, FLAG_AUTOTUNE if autotune else 0)
    st = getattr(lib(), "ggks_topk_batch_" + _SFX[dtype])(
        ptrs.ctypes.data, ns.ctypes.data, ptrs.size, Ks.ctypes.data, out.ctypes.data,
        ctypes.byref(o))
    _check(st, "topk_batch")
    return [out[off[p]:off[p + 1]] for p in range(ptrs.size)]


class PreparedBatch:
    """A batched multiselect (k_lists) or top-k (Ks) whose argument arrays are
    built once, the way a C or C++ caller keeps them: each call runs one
    ggks_multiselect_batch_* / ggks_topk_batch_* and returns the concatenated
    outputs (problem order); split() cuts them per problem."""

    def __init__(self, ptrs, ns, dtype, k_lists=None, Ks=None, ctx=None, stream=None,
                 autotune=False):
        self.dtype = np.dtype(dtype)
        self.ptrs, self.ns = _batch_arrays(ptrs, ns)
        if Ks is not None:
            self.Ks = np.ascontiguousarray(np.asarray(Ks, dtype=np.uint32))
            sizes = self.Ks.astype(np.int64)
            self.fn = getattr(lib(), "ggks_topk_batch_" + _SFX[self.dtype])
        else:
            self.Ks = None
            sizes = np.array([len(k) for k in k_lists], dtype=np.int64)
            self.fn = getattr(lib(), "ggks_multiselect_batch_" + _SFX[self.dtype])
            self.ks = np.ascontiguousarray(
                np.concatenate([np.asarray(k, dtype=np.uint32) for k in k_lists])
                if len(k_lists) else np.zeros(0, np.uint32), dtype=np.uint32)
        self.off = np.zeros(self.ptrs.size + 1, dtype=np.uint32)
        np.cumsum(sizes, out=self.off[1:])
        self.out = np.empty(int(self.off[-1]), dtype=self.dtype)
        self.opts = _opts(ctx, stream, FLAG_AUTOTUNE if autotune else 0)
        self.num_outputs = int(self.off[-1])

    def __call__(self):
        if self.Ks is not None:
            st = self.fn(self.ptrs.ctypes.data, self.ns.ctypes.data, self.ptrs.size,
                         self.Ks.ctypes.data, self.out.ctypes.data, ctypes.byref(self.opts))
        else:
            st = self.fn(self.ptrs.ctypes.data, self.ns.ctypes.data, self.ptrs.size,
                         self.off.ctypes.data, self.ks.ctypes.data if self.ks.size else None,
                         self.out.ctypes.data, ctypes.byref(self.opts))
        _check(st, "batch")
        return self.out

    def split(self, out=None):
        out = self.out if out is None else out
        return [out[self.off[p]:self.off[p + 1]] for p in range(self.ptrs.size)]


class Server:
    """A ggks_server: requests submitted from any thread are admitted under an
    HBM cap and coalesced into batched launches (continuous batching)."""

    def __init__(self, device=0, hbm_cap_bytes=64 << 30, max_batch=0, hbm_reserve_bytes=0,
                 lanes=0):
        cfg = ServerConfig(int(device), int(max_batch), int(hbm_cap_bytes),
                           int(hbm_reserve_bytes), int(lanes), 0)
        h = ctypes.c_void_p()
        _check(lib().ggks_server_create(ctypes.byref(cfg), ctypes.byref(h)), "server_create")
        self.handle = h
        self._keep = {}

    def submit(self, ptr, n, dtype, k=None, K=None, host=False, out=None):
        """Submit one request (k list, or K for top-k) on the vector at ptr
        (device memory, or host memory with host=True).  Returns a ticket."""
        dtype = np.dtype(dtype)
        flags = REQ_HOST_VECTOR if host else 0
        if K is not None:
            flags |= REQ_TOPK
            karr, num = None, int(K)
        else:
            karr = np.ascontiguousarray(k, dtype=np.uint32)
            num = karr.size
        if out is None:
            out = np.empty(num, dtype=dtype)
        r = Request(DTYPE_CODES[dtype], flags, ctypes.c_void_p(ptr), int(n),
                    karr.ctypes.data if karr is not None else None, num, 0)
        t = ctypes.c_uint64()
        _check(lib().ggks_server_submit(self.handle, ctypes.byref(r), out.ctypes.data,
                                        ctypes.byref(t)), "server_submit")
        self._keep[t.value] = out
        return t.value

    def wait(self, ticket):
        """Block until the request is done: (values, latency in ms)."""
        lat = ctypes.c_double()
        st = lib().ggks_server_wait(self.handle, int(ticket), ctypes.byref(lat))
        out = self._keep.pop(ticket, None)
        _check(st, "server_wait")
        return out, lat.value

    def stats(self):
        s = ServerStats()
        _check(lib().ggks_server_get_stats(self.handle, ctypes.byref(s)), "server_stats")
        return s.as_dict()

    def set_tuning(self, div, tile):
        _check(lib().ggks_server_set_tuning(self.handle, int(div), int(tile)), "server_tuning")

    def close(self):
        if self.handle:
            lib().ggks_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_set_tuning(ctx=None, div=0, tile=0):
    """Pin the batched path's bucket divisor and tile size on a context
    (div = 0: back to the autotuner / default)."""
    _check(lib().ggks_batch_set_tuning(_h(ctx), int(div), int(tile)), "batch_set_tuning")


def batch_last_tuning(ctx=None):
    """(div, tile) used by the context's last batched call."""
    d, t = ctypes.c_uint32(), ctypes.c_uint32()
    _check(lib().ggks_batch_last_tuning(_h(ctx), ctypes.byref(d), ctypes.byref(t)),
           "batch_last_tuning")
    return d.value, t.value


# ---------------------------------------------------------------------------
# torch-tensor conveniences (device memory is plumbing; torch is optional)
# ---------------------------------------------------------------------------
_TORCH_NP = {"torch.float32": np.float32, "torch.float64": np.float64, "torch.uint32": np.uint32,
             "torch.int32": np.uint32}


def _tensor_dtype(t):
    return np.dtype(_TORCH_NP[str(t.dtype)])


def multiselect(t, k, ctx=None, stream=None):
    """Multiselect of a contiguous CUDA tensor (float32 / float64 / uint32;
    an int32 tensor is read as uint32 bits)."""
    assert t.is_cuda and t.is_contiguous()
    return multiselect_ptr(t.data_ptr(), t.numel(), _tensor_dtype(t), k, ctx=ctx, stream=stream)


def topk(t, K, ctx=None, stream=None):
    assert t.is_cuda and t.is_contiguous()
    return topk_ptr(t.data_ptr(), t.numel(), _tensor_dtype(t), K, ctx=ctx, stream=stream)


# ---------------------------------------------------------------------------
# mirrors of the reference's host interface
# ---------------------------------------------------------------------------


def bucketMultiselectWrapper(d_vector, length, kVals, numKs, outputs, blocks=0, threads=0,
                             dtype=None):
    """BucketMultiselect::bucketMultiselectWrapper (bucketMultiselect.cu:837-871).
    d_vector: a CUDA tensor or a device pointer (then dtype is required);
    kVals: host k's (k-th largest); outputs: a host numpy array of numKs values,
    filled in k order.  blocks/threads are accepted and ignored.  Returns 1
    like the reference; errors raise GgksError instead of being silent."""
    if hasattr(d_vector, "data_ptr"):
        ptr, dtype = d_vector.data_ptr(), _tensor_dtype(d_vector)
    else:
        ptr = int(d_vector)
    k = np.ascontiguousarray(np.asarray(kVals)[:numKs], dtype=np.uint32)
    multiselect_ptr(ptr, length, dtype, k, out=outputs)
    return 1


def bucketSelectWrapper(d_vector, length, K, blocks=0, threads=0, dtype=None):
    """BucketSelect::bucketSelectWrapper (bucketSelect.cu:453-471): the K-th
    largest element of the device vector (a CUDA tensor, or a pointer with
    dtype); blocks / threads are accepted and ignored."""
    if hasattr(d_vector, "data_ptr"):
        ptr, dtype = d_vector.data_ptr(), _tensor_dtype(d_vector)
    else:
        ptr = int(d_vector)
    return select_ptr(ptr, length, dtype, K)


def randomizedBucketSelectWrapper(d_vector, length, K, blocks=0, threads=0, dtype=None):
    """RandomizedBucketSelect::randomizedBucketSelectWrapper
    (randomizedBucketSelect.cu:861-881): same contract, same exact path."""
    return bucketSelectWrapper(d_vector, length, K, blocks, threads, dtype)


class Results:
    """results_t<T> (multiselectTimingFunctions.cu:11-14): time (ms), vals."""

    def __init__(self, time_ms, vals):
        self.time = time_ms
        self.vals = vals


def timeBucketMultiselect(h_vec, kVals, kCount=None, ctx=None):
    """timeBucketMultiselect (multiselectTimingFunctions.cu:100-122): the
    vector is copied to the device before the timer starts; the wrapper call is
    timed."""
    import torch
    kVals = np.asarray(kVals, dtype=np.uint32)[: (kCount or len(kVals))]
    d = torch.from_numpy(np.ascontiguousarray(h_vec)).cuda()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    vals = multiselect_ptr(d.data_ptr(), d.numel(), h_vec.dtype, kVals, ctx=ctx)
    t1 = time.perf_counter()
    del d
    return Results((t1 - t0) * 1e3, vals)


def timeBucketTopkselect(h_vec, kCount, ctx=None):
    """timeBucketTopkselect (multiselectTimingFunctions.cu:205-231): the K
    largest, descending."""
    import torch
    d = torch.from_numpy(np.ascontiguousarray(h_vec)).cuda()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    vals = topk_ptr(d.data_ptr(), d.numel(), h_vec.dtype, kCount, ctx=ctx)
    t1 = time.perf_counter()
    del d
    return Results((t1 - t0) * 1e3, vals)
