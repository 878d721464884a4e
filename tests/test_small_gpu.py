"""The one-launch small-vector path (csrc/ggks_small.cuh) on the GPU: a device
vector of at most 2^20 elements with at most 1024 k's (a top-k of at most
1024 from at most 2^18) is selected by one thread-block cluster in one kernel.  Every result is
compared bit for bit with the oracle (sort-and-choose,
multiselectTimingFunctions.cu:51-95 / :156-177) and with the pipeline on the
same input; the statistics show which path answered, and inputs the cluster
leaves to the pipeline (a bucket whose needed bins do not fit) must still be
exact."""
import numpy as np
import pytest

from gpu_util import DeviceArray, assert_same

pytestmark = pytest.mark.gpu

MAX_N = 1 << 20
MAX_TOPK_N = 1 << 18
MAX_REQ = 1024


@pytest.fixture(scope="module")
def g():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ggks
    ggks.lib()
    return ggks


@pytest.fixture(scope="module")
def orc():
    import oracle
    oracle.build()
    return oracle


def _call(g, fn, *args, **kw):
    ctx = g.Context(0)
    try:
        got = fn(*args, ctx=ctx, **kw)
        return got, ctx.stats()
    finally:
        ctx.close()


CASES = [("f32", "uniform", 1 << 20), ("f32", "normal", MAX_N - 3), ("f32", "cauchy", 777_777),
         ("f32", "half_normal", 1 << 16), ("f32", "noisy", 123_457), ("f32", "killer", 1 << 20),
         ("f64", "uniform_pm1e6", 1 << 20), ("f64", "normal", 300_007), ("f64", "cauchy", MAX_N),
         ("u32", "uniform", MAX_N), ("u32", "sorted", 1 << 19), ("u32", "uniform16", 1 << 20)]


@pytest.mark.parametrize("dtype,dist,n", CASES, ids=[f"{a}-{b}-{c}" for a, b, c in CASES])
def test_small_path_vs_oracle_and_pipeline(g, orc, dtype, dist, n):
    import ggks_problems as gp
    x = gp.generate(dtype, dist, n, seed=n % 89)
    ks = np.concatenate([gp.k_pgrid(n, 101), gp.k_uniform_random(n, 600, 2),
                         gp.k_cluster(n, 99, 3), gp.k_normal(n, 50, 4)])
    assert ks.size <= MAX_REQ
    d = DeviceArray(x)
    want = orc.multiselect(x, ks, threads=8)
    got, st = _call(g, g.multiselect_ptr, d.ptr, n, x.dtype, ks)
    assert_same(got, want, f"small {dtype}/{dist}/{n}")
    assert st["small_calls"] + st["small_misses"] == 1
    if dist not in ("killer", "uniform16"):
        assert st["small_calls"] == 1 and st["launches"] == 1, st
    got_p, st_p = _call(g, g.multiselect_ptr, d.ptr, n, x.dtype, ks, small=False)
    assert_same(got_p, got, "pipeline")
    assert st_p["small_calls"] == 0 and st_p["small_misses"] == 0


@pytest.mark.parametrize("dtype,dist,n,K", [("f32", "uniform", MAX_TOPK_N, 32),
                                            ("f32", "normal", 200_001, 1024),
                                            ("u32", "uniform16", MAX_TOPK_N, 500),
                                            ("f64", "normal", 100_003, 1),
                                            ("u32", "sorted", 1 << 17, 777)])
def test_small_path_topk(g, orc, dtype, dist, n, K):
    import ggks_problems as gp
    x = gp.generate(dtype, dist, n, seed=K)
    d = DeviceArray(x)
    want = orc.topk(x, K, threads=8)
    got, st = _call(g, g.topk_ptr, d.ptr, n, x.dtype, K)
    assert_same(got, want, f"small top-k {dtype}/{dist}/{n}/{K}")
    assert st["small_calls"] + st["small_misses"] == 1
    got_p, _ = _call(g, g.topk_ptr, d.ptr, n, x.dtype, K, pipeline=True)
    assert_same(got_p, want, "pipeline top-k")


def test_small_path_limits(g, orc):
    """2^20 elements with 1024 k's take the small path; one more element or
    one more k takes the pipeline; a reversed copy of the vector and every
    rank of a tiny one stay exact."""
    import ggks_problems as gp
    x = gp.uniform_f32(MAX_N + 1, 31)
    ks = gp.k_uniform_random(MAX_N, MAX_REQ, 7)
    d = DeviceArray(x)
    got, st = _call(g, g.multiselect_ptr, d.ptr, MAX_N, x.dtype, ks)
    assert_same(got, orc.multiselect(x[:MAX_N], ks, 8), "2^20, 1024 k's")
    assert st["small_calls"] == 1
    got, st = _call(g, g.multiselect_ptr, d.ptr, MAX_N + 1, x.dtype, ks)
    assert_same(got, orc.multiselect(x, ks, 8), "2^20 + 1")
    assert st["small_calls"] == 0 and st["small_misses"] == 0
    ks2 = np.append(ks, np.uint32(5))
    got, st = _call(g, g.multiselect_ptr, d.ptr, MAX_N, x.dtype, ks2)
    assert_same(got, orc.multiselect(x[:MAX_N], ks2, 8), "1025 k's")
    assert st["small_calls"] == 0
    r = x[:MAX_N][::-1].copy()
    dr = DeviceArray(r)
    got, st = _call(g, g.multiselect_ptr, dr.ptr, MAX_N, r.dtype, ks)
    assert_same(got, orc.multiselect(r, ks, 8), "reversed")
    for n in (1, 2, 7, 100, 1000):
        y = gp.normal_f32(n, n)
        dy = DeviceArray(y)
        kk = np.arange(1, n + 1, dtype=np.uint32)
        got, st = _call(g, g.multiselect_ptr, dy.ptr, n, y.dtype, kk)
        assert_same(got, orc.multiselect(y, kk), f"every rank of n={n}")
        assert st["small_calls"] == 1


@pytest.mark.parametrize("dtype,extra,nk", [(np.float64, 3000, 300), (np.float64, 20000, 30),
                                            (np.float32, 3000, 300), (np.float32, 40000, 300)])
def test_small_path_medium_and_large_segments(g, orc, dtype, extra, nk):
    """A tight cluster puts thousands of keys into one bucket: the CTA sorts a
    segment of up to 64 KB of keys whole (a bitonic network in shared
    memory) and hands a larger one to finish_slot.  float64: distinct keys
    2^-45 apart near 0.5 -- 20000 of them narrow the bucket's bins too little
    for finish_slot, which leaves the call to the pipeline; float32: copies
    of 0.5 (finish_slot answers a bin of one key from its key).  The k's fall
    on and around the cluster, and at both ends."""
    r = np.random.default_rng(extra)
    n = 1 << 20
    x = r.random(n).astype(dtype)
    pos = r.choice(n, extra, replace=False)
    if dtype == np.float64:
        x[pos] = 0.5 + np.arange(extra) * 2.0 ** -45
    else:
        x[pos] = np.float32(0.5)
    below = int(np.count_nonzero(x < 0.5))  # ranks [below, below + extra) hold the cluster
    ks = np.unique(np.concatenate([
        n - below - np.arange(0, extra, max(1, extra // nk)),  # inside the cluster
        [n - below + 1, n - below - extra, 1, n, n // 3]])).astype(np.uint32)
    ks = ks[(ks >= 1) & (ks <= n)]
    d = DeviceArray(x)
    got, st = _call(g, g.multiselect_ptr, d.ptr, n, x.dtype, ks)
    assert_same(got, orc.multiselect(x, ks, 8), f"cluster {dtype.__name__} {extra}")
    assert st["small_calls"] + st["small_misses"] == 1
    if extra <= 3000 or dtype == np.float32:
        assert st["small_calls"] == 1
    got, st = _call(g, g.topk_ptr, d.ptr, n, x.dtype, 1000)
    assert_same(got, orc.topk(x, 1000, 8), "top-1000")


def test_small_path_leaves_oversized_buckets_to_the_pipeline(g, orc):
    """Half the vector within 2^22 keys of 1.0: the cluster's bucket has
    needed bins that do not fit the finisher, so the kernel sets its miss
    flag and the pipeline (with its recursive level) answers."""
    import ggks_problems as gp
    r = np.random.default_rng(0)
    n = MAX_N
    base = r.random(n) * 2.0
    m = n // 2
    base[:m] = 1.0 + r.integers(0, 1 << 20, m) * 2.0 ** -50
    r.shuffle(base)
    d = DeviceArray(base)
    ks = np.concatenate([gp.k_pgrid(n, 101), gp.k_distinct(n, 300, 1)])
    got, st = _call(g, g.multiselect_ptr, d.ptr, n, np.float64, ks)
    assert_same(got, orc.multiselect(base, ks, 8), "oversized bucket")
    assert st["small_misses"] == 1 and st["small_calls"] == 0
    assert st["recursions"] > 0


def test_small_path_repeated_and_mixed_calls(g, orc):
    """Calls of the small path, the threshold top-k and the pipeline on one
    context, on one stream of the caller, back to back."""
    import torch

    import ggks_problems as gp
    ctx = g.Context(0)
    s = torch.cuda.Stream()
    for it in range(6):
        n = (1 << 20) - 17 * it
        x = gp.generate("f32", "normal", n, seed=it)
        d = DeviceArray(x)
        ks = gp.k_distinct(n, 257, it)
        assert_same(g.multiselect_ptr(d.ptr, n, x.dtype, ks, ctx=ctx, stream=s.cuda_stream),
                    orc.multiselect(x, ks, 8), f"small {it}")
        assert_same(g.topk_ptr(d.ptr, n, x.dtype, 2000, ctx=ctx, stream=s.cuda_stream),
                    orc.topk(x, 2000, 8), f"threshold {it}")
        big = gp.k_distinct(n, 1500, it)
        assert_same(g.multiselect_ptr(d.ptr, n, x.dtype, big, ctx=ctx),
                    orc.multiselect(x, big, 8), f"pipeline {it}")
    st = ctx.stats()
    assert st["small_calls"] == 6 and st["topk_threshold_calls"] == 6
    ctx.close()


def test_small_path_device_output_and_host_vectors(g, orc):
    import torch

    import ggks_problems as gp
    x = gp.uniform_f32(1 << 20, 5)
    ks = gp.k_pgrid(x.size, 101)
    d = DeviceArray(x)
    out = torch.empty(ks.size, dtype=torch.float32, device="cuda")
    g.multiselect_ptr(d.ptr, x.size, x.dtype, ks, out_device_ptr=out.data_ptr())
    torch.cuda.synchronize()
    assert_same(out.cpu().numpy(), orc.multiselect(x, ks), "device output")
    for dtype in ("f32", "f64", "u32"):
        y = gp.generate(dtype, "uniform" if dtype != "f64" else "uniform_pm1e6", 300_001, 9)
        kk = gp.k_distinct(y.size, 333, 3)
        assert_same(g.multiselect_host(y, kk), orc.multiselect(y, kk), f"host {dtype}")
        assert_same(g.topk_host(y, 111), orc.topk(y, 111), f"host top-k {dtype}")
