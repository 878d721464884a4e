"""GPU parity tests: the CUDA path through the C ABI against the golden
fixtures and against the oracle (sort-and-choose, multiselectTimingFunctions.cu
:51-95 / :156-177) on seeded inputs.  Every comparison is bit-exact."""
import os

import numpy as np
import pytest

from conftest import golden_files, load_golden
from gpu_util import DeviceArray, assert_same

pytestmark = pytest.mark.gpu

GOLDEN = golden_files()


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


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_golden_multiselect(g, path):
    f = load_golden(path)
    d = DeviceArray(f["vec"])
    got = g.multiselect_ptr(d.ptr, d.n, d.dtype, f["k"])
    assert_same(got, f["expected"], os.path.basename(path))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_golden_topk(g, path):
    f = load_golden(path)
    d = DeviceArray(f["vec"])
    got = g.topk_ptr(d.ptr, d.n, d.dtype, int(f["topk_K"]))
    assert_same(got, f["topk_expected"], os.path.basename(path))


CASES = [
    ("f32", "uniform", 1 << 20), ("f32", "normal", 1 << 20), ("f32", "half_normal", 999_983),
    ("f32", "cauchy", 1 << 21), ("f32", "killer", 1 << 20), ("f32", "noisy", 1 << 19),
    ("f32", "ones_twos", 1 << 20), ("f32", "all_ones", 300_001), ("f32", "uint_valued", 1 << 21),
    ("f32", "huge_uniform", 65_537), ("f32", "normal100", 4_000_037),
    ("f64", "uniform_pm1e6", 1 << 20), ("f64", "normal", 777_777), ("f64", "killer", 1 << 19),
    ("f64", "cauchy", 1 << 20), ("f64", "uint_valued", 1 << 20),
    ("u32", "uniform", 1 << 21), ("u32", "sorted", 1 << 20), ("u32", "zero_to_four", 1_000_003),
    ("u32", "uniform16", 1 << 21),
]


# small: the one-launch small-vector path where it applies (at most 2^21
# elements and 1024 k's), else the pipeline on the same inputs
PATHS = [True, False]
PATH_IDS = ["small", "pipeline"]


@pytest.mark.parametrize("small", PATHS, ids=PATH_IDS)
@pytest.mark.parametrize("dtype,dist,n", CASES, ids=[f"{a}-{b}-{c}" for a, b, c in CASES])
def test_multiselect_vs_oracle(g, orc, dtype, dist, n, small):
    import ggks_problems as gp
    x = gp.generate(dtype, dist, n, seed=n % 97)
    ks = np.concatenate([gp.k_pgrid(n, 101), gp.k_uniform_random(n, 400, 3),
                         gp.k_cluster(n, 45, 4), gp.k_sectioned(n, 64, 5), gp.k_normal(n, 50, 6)])
    d = DeviceArray(x)
    got = g.multiselect_ptr(d.ptr, n, x.dtype, ks, small=small)
    want = orc.multiselect(x, ks, threads=8)
    assert_same(got, want, f"{dtype}/{dist}/{n}")


@pytest.mark.parametrize("small", PATHS, ids=PATH_IDS)
@pytest.mark.parametrize("n", [1, 2, 3, 5, 31, 32, 33, 1023, 1024, 1025, 65535, 65536, 65537, 131073])
def test_small_and_ragged_sizes(g, orc, n, small):
    import ggks_problems as gp
    for dtype, dist in (("f32", "normal"), ("f64", "uniform"), ("u32", "uniform16")):
        x = gp.generate(dtype, dist, n, seed=n)
        # every k (in three calls of at most 1024 for the small path's limit)
        ks = np.arange(1, n + 1, dtype=np.uint32) if n <= 2048 else gp.k_pgrid(n, 101)
        d = DeviceArray(x)
        want = orc.multiselect(x, ks)
        for lo in range(0, ks.size, 1024):
            assert_same(g.multiselect_ptr(d.ptr, n, x.dtype, ks[lo:lo + 1024], small=small),
                        want[lo:lo + 1024], f"{dtype} n={n}")
        K = min(n, 700)
        assert_same(g.topk_ptr(d.ptr, n, x.dtype, K, small=small), orc.topk(x, K),
                    f"topk {dtype} n={n}")


@pytest.mark.parametrize("small", PATHS, ids=PATH_IDS)
@pytest.mark.parametrize("offset", [1, 2, 3])
def test_unaligned_views(g, orc, offset, small):
    """Vectors that start off a 16-byte boundary take the scalar head path."""
    import ggks_problems as gp
    for dtype, dist in (("f32", "uniform"), ("u32", "uniform"), ("f64", "normal")):
        n = 300_007
        x = gp.generate(dtype, dist, n, seed=offset)
        d = DeviceArray(x, pad_front=offset)
        ks = gp.k_pgrid(n, 101)
        assert_same(g.multiselect_ptr(d.ptr, n, x.dtype, ks, small=small),
                    orc.multiselect(x, ks), f"{dtype} offset {offset}")


TOPK = [("f32", "uniform", 1 << 22, 32), ("f32", "uniform", 1 << 22, 1024),
        ("f32", "uniform", 1 << 22, 65536), ("u32", "uniform16", 1 << 22, 32),
        ("u32", "uniform16", 1 << 22, 65536), ("f32", "cauchy", 1 << 21, 5000),
        ("f64", "normal", 1 << 21, 4096), ("f32", "ones_twos", 1 << 20, 3000),
        ("u32", "sorted", 1 << 22, 65536), ("f32", "killer", 1 << 20, 777)]


@pytest.mark.parametrize("dtype,dist,n,K", TOPK, ids=[f"{a}-{b}-{c}-{d}" for a, b, c, d in TOPK])
def test_topk_vs_oracle(g, orc, dtype, dist, n, K):
    import ggks_problems as gp
    x = gp.generate(dtype, dist, n, seed=K)
    d = DeviceArray(x)
    got = g.topk_ptr(d.ptr, n, x.dtype, K)
    want = orc.topk(x, K, threads=8)
    assert_same(got, want, f"topk {dtype}/{dist}/{n}/{K}")
    # the K largest as a multiset, in descending order
    assert np.all(got[:-1] >= got[1:]) or x.dtype != np.float32


def test_presorted_and_reversed_topk(g, orc):
    import ggks_problems as gp
    x = np.sort(gp.uniform_f32(1 << 22, 9))
    for arr in (x, x[::-1].copy()):
        d = DeviceArray(arr)
        for K in (32, 1024, 65536):
            assert_same(g.topk_ptr(d.ptr, arr.size, arr.dtype, K), orc.topk(arr, K, threads=8),
                        f"presorted K={K}")
        ks = gp.k_distinct(arr.size, 1001, 1)
        assert_same(g.multiselect_ptr(d.ptr, arr.size, arr.dtype, ks), orc.multiselect(arr, ks, 8),
                    "presorted multiselect")


def test_duplicate_and_unsorted_ks(g, orc):
    import ggks_problems as gp
    n = 1 << 20
    x = gp.normal_f32(n, 2)
    ks = np.array([5, 1, n, 5, 77, n, 1, 123456, 5] * 11, dtype=np.uint32)
    d = DeviceArray(x)
    assert_same(g.multiselect_ptr(d.ptr, n, x.dtype, ks), orc.multiselect(x, ks), "dup ks")
    ks = np.arange(1, 70_001, dtype=np.uint32)[::-1].copy()  # many k's, one region
    assert_same(g.multiselect_ptr(d.ptr, n, x.dtype, ks), orc.multiselect(x, ks), "dense ks")


def test_repeated_calls_one_context(g, orc):
    """Device state (per-slice sample counts at the workspace head, grid-barrier
    counters, tickets) re-arms between calls of different shapes, with the
    pipeline and the one-launch small-vector path taking turns."""
    import ggks_problems as gp
    ctx = g.Context(0)
    small_expected = 0
    for it, (dtype, dist, n) in enumerate([("f32", "uniform", 1 << 21), ("u32", "uniform", 5000),
                                           ("f64", "normal", 1 << 20), ("f32", "uniform", 1 << 21),
                                           ("f32", "cauchy", 123_457)] * 2):
        x = gp.generate(dtype, dist, n, seed=7)
        ks = gp.k_pgrid(n, 101)
        d = DeviceArray(x)
        small = it % 2 == 1
        small_expected += small and n <= (1 << 20)
        got = g.multiselect_ptr(d.ptr, n, x.dtype, ks, ctx=ctx, small=small)
        assert_same(got, orc.multiselect(x, ks), f"call {it}")
    st = ctx.stats()
    assert st["calls"] == 10
    assert st["small_calls"] == small_expected
    assert st["launches"] >= 7 * (10 - small_expected) + small_expected
    ctx.close()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_single_key_buckets_tracked(g, orc, dtype):
    """Integer-valued floats in [0, 256): every value's bucket spans many keys
    but holds one.  The histogram pass tracks each bucket's key, so every
    requested bucket is answered from its key and nothing is compacted.  A
    second key 5 ulps from one value (inside the same bucket) must be seen as
    a second key, and that bucket compacted and selected as usual."""
    import ggks_problems as gp
    n = 1 << 22 if dtype == np.float32 else 1 << 21
    r = np.random.default_rng(17)
    x = r.integers(0, 256, n).astype(dtype)
    ks = gp.k_distinct(n, 1001, 5)
    d = DeviceArray(x)
    ctx = g.Context(0)
    assert_same(g.multiselect_ptr(d.ptr, n, x.dtype, ks, ctx=ctx, small=False),
                orc.multiselect(x, ks, 8), "integer valued")
    assert ctx.stats()["survivors"] == 0
    y = x.copy()
    pick = np.nonzero(y == 200)[0][::3]
    y[pick] = np.nextafter(np.nextafter(np.nextafter(np.nextafter(np.nextafter(
        y[pick], dtype(300)), dtype(300)), dtype(300)), dtype(300)), dtype(300))
    d = DeviceArray(y)
    ctx.reset_stats()
    assert_same(g.multiselect_ptr(d.ptr, n, y.dtype, ks, ctx=ctx, small=False),
                orc.multiselect(y, ks, 8), "integer valued, one bucket with two keys")
    # the small-vector path on the same inputs
    assert_same(g.multiselect_ptr(d.ptr, n, y.dtype, ks, ctx=ctx), orc.multiselect(y, ks, 8),
                "integer valued, one bucket with two keys (small path)")
    ctx.close()


def test_fresh_context_while_default_stream_busy(g, orc):
    """A context's workspace is cleared when it is allocated.  The clearing
    must be ordered on the context's own (non-blocking) stream: issued to the
    legacy default stream while other work keeps that stream busy, it would
    run whenever that work ends -- in the middle of whichever call is then in
    flight.  The default stream is held by a bounded spin while calls on a
    fresh context run back to back past its end; every result must be exact."""
    import torch

    import ggks_problems as gp
    n = 1 << 24
    x = gp.uniform_f32(n, 8)
    ks = gp.k_distinct(n, 1001, 3)
    want = orc.multiselect(x, ks, 8)
    d = DeviceArray(x)
    torch.cuda.synchronize()
    ctx = g.Context(0)
    torch.cuda._sleep(40_000_000)  # ~20 ms on the default stream
    for i in range(120):
        assert_same(g.multiselect_ptr(d.ptr, n, x.dtype, ks, ctx=ctx), want, f"call {i}")
    torch.cuda.synchronize()
    ctx.close()


def test_host_vector_entry_points(g, orc):
    import ggks_problems as gp
    for dtype, dist in (("f32", "normal"), ("f64", "uniform"), ("u32", "uniform")):
        x = gp.generate(dtype, dist, 1 << 20, seed=4)
        ks = gp.k_distinct(x.size, 257, 2)
        assert_same(g.multiselect_host(x, ks), orc.multiselect(x, ks), f"host {dtype}")
        assert_same(g.topk_host(x, 999), orc.topk(x, 999), f"host topk {dtype}")


def test_device_output_flag(g, orc):
    import torch

    import ggks_problems as gp
    x = gp.uniform_f32(1 << 20, 5)
    ks = gp.k_pgrid(x.size, 101)
    d = DeviceArray(x)
    out = torch.empty(ks.size, dtype=torch.float32, device="cuda")
    g.multiselect_ptr(d.ptr, x.size, x.dtype, ks, out_device_ptr=out.data_ptr())
    torch.cuda.synchronize()
    assert_same(out.cpu().numpy(), orc.multiselect(x, ks), "device output")


def test_oversized_segments_recurse(g, orc):
    """A cluster of nearly equal values that the sampled splitter table cannot
    cut finely enough: its bucket exceeds shared memory, is listed, and is
    selected again on its keys (recursive level)."""
    import ggks_problems as gp
    r = np.random.default_rng(0)
    n = 1 << 21
    base = r.random(n) * 2.0
    m = n // 2
    base[:m] = 1.0 + r.integers(0, 1 << 20, m) * 2.0 ** -50  # within 2^22 keys of 1.0
    r.shuffle(base)
    ctx = g.Context(0)
    d = DeviceArray(base)
    ks = np.concatenate([gp.k_pgrid(n, 101), gp.k_distinct(n, 300, 1)])
    got = g.multiselect_ptr(d.ptr, n, np.float64, ks, ctx=ctx, small=False)
    assert_same(got, orc.multiselect(base, ks, 8), "recursive f64 cluster")
    assert ctx.stats()["recursions"] > 0
    got = g.topk_ptr(d.ptr, n, np.float64, 20000, ctx=ctx)
    assert_same(got, orc.topk(base, 20000, 8), "recursive f64 top-k")
    # f32: 16 neighbouring floats share half of the mass
    x = gp.uniform_f32(1 << 22, 3) * 2
    idx = r.choice(x.size, x.size // 2, replace=False)
    x[idx] = (np.float32(1.0).view(np.uint32) + r.integers(0, 16, idx.size).astype(np.uint32)).view(
        np.float32)
    d = DeviceArray(x)
    ks = gp.k_pgrid(x.size, 101)
    assert_same(g.multiselect_ptr(d.ptr, x.size, x.dtype, ks, ctx=ctx), orc.multiselect(x, ks, 8),
                "f32 cluster")
    ctx.close()


def test_survivor_overflow_regrows(g, orc):
    """When the active buckets hold more elements than the survivor buffer, the
    buffer is regrown and compaction + finish re-run."""
    import ggks_problems as gp
    r = np.random.default_rng(1)
    n = 1 << 23
    x = r.random(n) * 2.0
    m = (n * 3) // 4
    x[:m] = 1.0 + r.integers(0, 1 << 16, m) * 2.0 ** -52
    r.shuffle(x)
    ctx = g.Context(0)
    d = DeviceArray(x)
    ks = gp.k_pgrid(n, 101)
    assert_same(g.multiselect_ptr(d.ptr, n, np.float64, ks, ctx=ctx), orc.multiselect(x, ks, 8),
                "overflow")
    st = ctx.stats()
    assert st["retries"] > 0
    ctx.close()


def test_reference_harness_mirror(g, orc):
    """compareMultiselectAlgorithms (compareMultiselect.hpp:46-224): every
    distribution, sort-and-choose vs bucketMultiselectWrapper, error count 0."""
    import ggks_problems as gp
    errors = 0
    for dtype, gens in gp.GENERATORS.items():
        for dist in gens:
            n = 1 << 18
            h_vec = gp.generate(dtype, dist, n, seed=11)
            kVals = gp.k_uniform(n, 101)
            oracle_vals = orc.multiselect(h_vec, kVals)  # algorithm 0
            d = DeviceArray(h_vec)
            outputs = np.empty(kVals.size, dtype=h_vec.dtype)
            ret = g.bucketMultiselectWrapper(d.ptr, n, kVals, kVals.size, outputs, 152, 1024,
                                             dtype=h_vec.dtype)
            assert ret == 1
            errors += int(np.count_nonzero(outputs.view(np.uint8).reshape(kVals.size, -1)
                                           != oracle_vals.view(np.uint8).reshape(kVals.size, -1)))
    assert errors == 0


def test_reference_bucket_algorithm_agrees(g, orc):
    """The reference's own bucket algorithm (restated on the CPU) and the GPU
    path give the same answers."""
    import ggks_problems as gp
    for dtype, dist in (("f32", "normal"), ("f64", "uniform"), ("u32", "uniform"),
                        ("f32", "cauchy")):
        n = 200_003
        x = gp.generate(dtype, dist, n, 21)
        ks = gp.k_uniform(n, 101)
        d = DeviceArray(x)
        assert_same(g.multiselect_ptr(d.ptr, n, x.dtype, ks), orc.bucket_multiselect(x, ks, 9),
                    f"{dtype}/{dist}")


@pytest.mark.parametrize("offset", [0, 1, 3])
def test_pinned_host_vector_ingest(g, orc, offset):
    """A pinned host vector is read over the CPU-GPU link by the histogram
    pass, which also writes the device copy; views off a 16-byte boundary
    keep their alignment in the copy."""
    import torch

    import ggks_problems as gp
    for dtype, dist, tdt in (("f32", "normal", torch.float32), ("f64", "cauchy", torch.float64),
                             ("u32", "uniform", torch.int32)):
        n = (1 << 20) + 7
        x = gp.generate(dtype, dist, n, seed=offset + 1)
        pin = torch.empty(n + offset, dtype=tdt, pin_memory=True)
        view = pin.numpy().view(x.dtype)[offset:]
        view[:] = x
        ks = gp.k_distinct(n, 333, offset)
        assert_same(g.multiselect_host(view, ks), orc.multiselect(x, ks), f"pinned {dtype}")
        assert_same(g.topk_host(view, 2048), orc.topk(x, 2048), f"pinned topk {dtype}")


@pytest.mark.parametrize("dtype", ["f32", "u32", "f64"])
def test_narrow_span_with_far_outliers(g, orc, dtype):
    """Almost every element is one of two neighbouring keys, so the sampled
    span is tiny; a few far outliers lie beyond every slice and take the
    splitter table's top entry (a right shift by the whole key width)."""
    n = 1 << 22
    r = np.random.default_rng(11)
    if dtype == "f32":
        a = np.float32(1.0)
        x = np.where(r.random(n) < 0.5, a, np.nextafter(a, np.float32(2))).astype(np.float32)
        x[r.integers(0, n, 5)] = np.float32(1e6)
        x[r.integers(0, n, 5)] = np.float32(-1e6)
    elif dtype == "u32":
        x = np.where(r.random(n) < 0.5, 1000, 1001).astype(np.uint32)
        x[r.integers(0, n, 5)] = np.uint32(0xFFFFFF00)
        x[r.integers(0, n, 5)] = np.uint32(3)
    else:
        x = np.where(r.random(n) < 0.5, 1.0, np.nextafter(1.0, 2.0))
        x[r.integers(0, n, 5)] = 1e300
        x[r.integers(0, n, 5)] = -1e300
    d = DeviceArray(x)
    ks = np.concatenate([np.arange(1, 12), np.arange(n - 11, n + 1), [n // 2, n // 2 + 1]])
    ks = ks.astype(np.uint32)
    assert_same(g.multiselect_ptr(d.ptr, n, x.dtype, ks), orc.multiselect(x, ks), dtype)
    assert_same(g.topk_ptr(d.ptr, n, x.dtype, 20), orc.topk(x, 20), f"topk {dtype}")


@pytest.mark.parametrize("dtype,dist", [("f32", "normal"), ("f32", "ones_twos"), ("f64", "cauchy"),
                                        ("u32", "uniform16"), ("u32", "sorted")])
def test_single_k_select(g, orc, dtype, dist):
    """bucketSelectWrapper / randomizedBucketSelectWrapper (bucketSelect.cu:453-471,
    randomizedBucketSelect.cu:861-881): the K-th largest, one value."""
    import ggks_problems as gp
    for n in (1, 7, 1000, 1 << 20):
        x = gp.generate(dtype, dist, n, seed=n)
        d = DeviceArray(x)
        for K in sorted({1, n, (n + 1) // 2, max(1, n // 3)}):
            want = orc.multiselect(x, [K])
            got = np.array([g.bucketSelectWrapper(d.ptr, n, K, 152, 1024, dtype=x.dtype)],
                           dtype=x.dtype)
            assert_same(got, want, f"bucketSelect {dtype}/{dist} n={n} K={K}")
            got = np.array([g.randomizedBucketSelectWrapper(d.ptr, n, K, dtype=x.dtype)],
                           dtype=x.dtype)
            assert_same(got, want, f"randomizedBucketSelect {dtype}/{dist} n={n} K={K}")


def test_many_slots_and_many_requests_per_slot(g, orc):
    """Request counters per slot: thousands of requests in a few slots (top-k,
    shared-memory counters) and more slots than shared memory holds (the
    global counters)."""
    import ggks_problems as gp
    n = 1 << 22
    x = gp.generate("f32", "normal", n, seed=31)
    d = DeviceArray(x)
    ks = gp.k_distinct(n, 20_000, 4)  # > 6144 slots
    assert_same(g.multiselect_ptr(d.ptr, n, x.dtype, ks), orc.multiselect(x, ks, 8), "20k ks")
    assert_same(g.topk_ptr(d.ptr, n, x.dtype, 100_000), orc.topk(x, 100_000, 8), "top 100k")
