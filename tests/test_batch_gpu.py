"""GPU parity tests of the batched multiselect / top-k (one persistent launch
over many vectors): every output is compared bit for bit with the oracle
(sort-and-choose, multiselectTimingFunctions.cu:51-95 / :156-177) and with the
single-vector entry points on the same vectors."""
import numpy as np
import pytest

from gpu_util import DeviceArray, assert_same

pytestmark = pytest.mark.gpu


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


def _check_batch(g, orc, vecs, klists, dtype, what, ctx=None, autotune=False, offsets=None):
    offsets = offsets or [0] * len(vecs)
    devs = [DeviceArray(v, pad_front=o) for v, o in zip(vecs, offsets)]
    got = g.multiselect_batch_ptr([d.ptr for d in devs], [v.size for v in vecs], dtype, klists,
                                  ctx=ctx, autotune=autotune)
    for p, (v, ks) in enumerate(zip(vecs, klists)):
        if len(ks) == 0:
            assert got[p].size == 0
            continue
        assert_same(got[p], orc.multiselect(v, ks), f"{what} problem {p} (n={v.size})")
    return devs, got


def test_batch_mixed_sizes_and_distributions(g, orc):
    import ggks_problems as gp
    sizes = [1, 2, 3, 5, 17, 31, 32, 33, 255, 1000, 1023, 1024, 1025, 4095, 4096, 8191, 8192,
             8193, 65535, 65537, 100_003, 1 << 20, (1 << 20) + 3, 3_000_017]
    vecs, klists = [], []
    r = np.random.default_rng(11)
    for i, n in enumerate(sizes):
        dist = gp.BATCH_DISTS[i % len(gp.BATCH_DISTS)]
        vecs.append(gp.generate("f32", dist, n, seed=i))
        nk = int(r.integers(1, 65))
        ks = r.integers(1, n + 1, nk).astype(np.uint32)
        if i % 3 == 0:
            ks = np.concatenate([ks, [1, n, ks[0]]]).astype(np.uint32)  # extremes, duplicate
        klists.append(ks)
    devs, got = _check_batch(g, orc, vecs, klists, np.float32, "mixed")
    # same outputs as the single-vector entry point
    for p, (d, ks) in enumerate(zip(devs, klists)):
        assert_same(got[p], g.multiselect_ptr(d.ptr, d.n, np.float32, ks), f"vs plain {p}")


@pytest.mark.parametrize("dtype,dists", [
    ("f64", ("uniform", "normal", "cauchy", "uint_valued", "killer", "uniform_pm1e6")),
    ("u32", ("uniform", "sorted", "zero_to_four", "uniform16")),
    ("f32", ("half_normal", "huge_uniform", "all_ones", "ones_twos", "noisy", "killer",
             "normal100")),
])
def test_batch_element_types_and_adversarial_inputs(g, orc, dtype, dists):
    import ggks_problems as gp
    r = np.random.default_rng(5)
    vecs, klists = [], []
    for i in range(3 * len(dists)):
        dist = dists[i % len(dists)]
        n = int(2 ** r.uniform(8, 21))
        vecs.append(gp.generate(dtype, dist, n, seed=100 + i))
        klists.append(np.concatenate([gp.k_pgrid(n, min(n, 33)),
                                      r.integers(1, n + 1, 20)]).astype(np.uint32))
    _check_batch(g, orc, vecs, klists, gp.DTYPES[dtype], f"{dtype} batch")


def test_batch_workload_sample(g, orc):
    """A slice of the batched workload's generator: log-uniform lengths,
    four distributions, 1-64 k's each."""
    import ggks_problems as gp
    probs = gp.batch_problems(96, seed=3, lo_log2=10, hi_log2=20)
    vecs = [gp.batch_vector(p) for p in probs]
    _check_batch(g, orc, vecs, [p["k"] for p in probs], np.float32, "workload")


def test_batch_unaligned_vectors(g, orc):
    """Vectors that start off a 16-byte boundary: scalar head, vector body,
    scalar tail inside every tile."""
    import ggks_problems as gp
    for dtype in ("f32", "u32", "f64"):
        sizes = [70_001, 5, 1 << 18, 4099, 300_007, 12]
        vecs = [gp.generate(dtype, "uniform", n, seed=i) for i, n in enumerate(sizes)]
        klists = [gp.k_pgrid(n, min(n, 41)) for n in sizes]
        _check_batch(g, orc, vecs, klists, gp.DTYPES[dtype], f"unaligned {dtype}",
                     offsets=[1 + i % 3 for i in range(len(sizes))])


def test_topk_batch(g, orc):
    import ggks_problems as gp
    specs = [("uniform", 1 << 20, 32), ("uint_valued", 1 << 19, 4096), ("normal", 5000, 5000),
             ("cauchy", 3, 2), ("uniform", 1 << 22, 1024), ("normal", 77_777, 0),
             ("uniform", 1, 1)]
    vecs = [gp.generate("f32", d, n, seed=n) for d, n, _ in specs]
    Ks = [K for _, _, K in specs]
    devs = [DeviceArray(v) for v in vecs]
    got = g.topk_batch_ptr([d.ptr for d in devs], [v.size for v in vecs], np.float32, Ks)
    for p, (v, K) in enumerate(zip(vecs, Ks)):
        assert got[p].size == K
        if K:
            assert_same(got[p], orc.topk(v, K), f"topk problem {p}")
    # u32 with heavy duplicates, and a presorted vector
    x = gp.generate("u32", "uniform16", 1 << 21, seed=1)
    s = np.sort(gp.generate("u32", "uniform", 1 << 20, seed=2))
    dx, ds = DeviceArray(x), DeviceArray(s)
    got = g.topk_batch_ptr([dx.ptr, ds.ptr], [x.size, s.size], np.uint32, [65536, 1024])
    assert_same(got[0], orc.topk(x, 65536), "topk u32 uniform16")
    assert_same(got[1], orc.topk(s, 1024), "topk u32 presorted")


def test_batch_skips_problems_without_outputs(g, orc):
    import ggks_problems as gp
    a = gp.generate("f32", "normal", 10_000, seed=1)
    b = gp.generate("f32", "uniform", 20_000, seed=2)
    da, db = DeviceArray(a), DeviceArray(b)
    ka = np.array([1, 5000, 10_000], dtype=np.uint32)
    got = g.multiselect_batch_ptr([0, da.ptr, 0, db.ptr, 0], [0, a.size, 0, b.size, 0],
                                  np.float32, [[], ka, [], [7], []])
    assert [x.size for x in got] == [0, 3, 0, 1, 0]
    assert_same(got[1], orc.multiselect(a, ka), "a")
    assert_same(got[3], orc.multiselect(b, [7]), "b")


def test_batch_autotune_keeps_results(g, orc):
    import ggks_problems as gp
    probs = gp.batch_problems(40, seed=8, lo_log2=10, hi_log2=19)
    vecs = [gp.batch_vector(p) for p in probs]
    ks = [p["k"] for p in probs]
    ctx = g.Context(0)
    _check_batch(g, orc, vecs, ks, np.float32, "autotune", ctx=ctx, autotune=True)
    div, tile = g.batch_last_tuning(ctx)
    assert div in (256, 1024, 4096) and tile in (1 << 16, 1 << 18, 1 << 20)
    # the choice is cached for this shape: the next call runs once
    before = ctx.stats()["launches"]
    _check_batch(g, orc, vecs, ks, np.float32, "tuned", ctx=ctx, autotune=True)
    assert ctx.stats()["launches"] - before == 1
    assert g.batch_last_tuning(ctx) == (div, tile)
    ctx.close()


def test_batch_survivor_overflow_and_single_key_bins(g, orc):
    """Half the vector is four neighbouring floats just above 1.0, which share
    one bucket: that bucket exceeds the first survivor estimate (the batch runs
    again with a larger buffer), and the finisher answers its ranks from bins
    one key wide."""
    r = np.random.default_rng(2)
    n = 1 << 22
    x = (r.random(n) * 1e6).astype(np.float32)
    one = np.float32(1.0).view(np.uint32)
    x[: n // 2] = (one + r.integers(0, 4, n // 2).astype(np.uint32)).view(np.float32)
    r.shuffle(x)
    y = r.random(5000).astype(np.float32)
    ctx = g.Context(0)
    ks = np.array([1, n // 4, n // 2, n // 2 + 1, 3 * n // 4, n], dtype=np.uint32)
    _check_batch(g, orc, [y, x, y], [[1, 2500], ks, [5000]], np.float32, "overflow", ctx=ctx)
    assert ctx.stats()["retries"] >= 1
    ctx.close()


def test_batch_deferred_segments_recurse(g, orc):
    """float64: 30% of the vector is two neighbouring keys (1.0 and the next
    double), the rest a narrow normal around them plus a few huge values, so
    the buckets around 1.0 are about 2^40 keys wide: the finisher's bin holding
    the two keys holds some 600 000 of them (even over the segment's actual
    key range) and exceeds its shared memory.  The slot is selected again on
    its keys (recursive level)."""
    r = np.random.default_rng(3)
    n = 1 << 21
    x = 1.0 + r.standard_normal(n) * 1e-3
    m = (3 * n) // 10
    x[:m] = np.where(r.random(m) < 0.5, 1.0, np.nextafter(1.0, 2.0))
    x[-16:] = np.array([1e300, -1e300] * 8)
    r.shuffle(x)
    ctx = g.Context(0)
    ks = np.concatenate([gp_pgrid(n, 41), [n // 2, n // 2 + 1]]).astype(np.uint32)
    _check_batch(g, orc, [x[:1000].copy(), x], [[1, 1000], ks], np.float64, "deferred", ctx=ctx)
    assert ctx.stats()["recursions"] >= 1
    ctx.close()


def gp_pgrid(n, count):
    import ggks_problems as gp
    return gp.k_pgrid(n, count)


def test_batch_many_small_problems(g, orc):
    r = np.random.default_rng(4)
    vecs, klists = [], []
    for i in range(3000):
        n = int(r.integers(1, 400))
        vecs.append(r.standard_normal(n).astype(np.float32))
        klists.append(r.integers(1, n + 1, int(r.integers(1, 9))).astype(np.uint32))
    _check_batch(g, orc, vecs, klists, np.float32, "small")


def test_batch_device_output_and_repeated_calls(g, orc):
    import torch

    import ggks_problems as gp
    ctx = g.Context(0)
    for it in range(3):
        probs = gp.batch_problems(20, seed=50 + it, lo_log2=10, hi_log2=18)
        vecs = [gp.batch_vector(p) for p in probs]
        ks = [p["k"] for p in probs]
        devs = [DeviceArray(v) for v in vecs]
        total = sum(len(k) for k in ks)
        out = torch.empty(total, dtype=torch.float32, device="cuda")
        g.multiselect_batch_ptr([d.ptr for d in devs], [v.size for v in vecs], np.float32, ks,
                                ctx=ctx, out_device_ptr=out.data_ptr())
        torch.cuda.synchronize()
        want = np.concatenate([orc.multiselect(v, k) for v, k in zip(vecs, ks)])
        assert_same(out.cpu().numpy(), want, f"device output, call {it}")
    assert ctx.stats()["batch_calls"] == 3
    ctx.close()


def test_batch_pinned_tunings_agree(g, orc):
    """Every bucket divisor / tile size gives the same, exact results."""
    import ggks_problems as gp
    probs = gp.batch_problems(24, seed=21, lo_log2=10, hi_log2=20)
    vecs = [gp.batch_vector(p) for p in probs]
    ks = [p["k"] for p in probs]
    ctx = g.Context(0)
    for div, tile in ((16, 4096), (256, 1 << 16), (1024, 1 << 18), (4096, 1 << 20), (1 << 20, 1 << 22)):
        g.batch_set_tuning(ctx, div, tile)
        _check_batch(g, orc, vecs, ks, np.float32, f"div {div} tile {tile}", ctx=ctx)
        assert g.batch_last_tuning(ctx) == (div, tile)
    g.batch_set_tuning(ctx, 0, 0)
    ctx.close()


def test_batch_single_key_buckets(g, orc):
    """Buckets holding one repeated key are answered without survivors only
    when every tile saw that same key: tiles of 1.0 followed by tiles of the
    next float up (one key per tile, two keys per bucket), the two keys
    interleaved inside tiles, integer-valued floats, and the largest key."""
    r = np.random.default_rng(9)
    n = 1 << 22
    one = np.float32(1.0)
    up = np.nextafter(one, np.float32(2.0))
    halves = np.concatenate([np.full(n // 2, one), np.full(n // 2, up)]).astype(np.float32)
    halves[0], halves[-1] = -1e6, 1e6
    mixed = np.where(r.random(n) < 0.5, one, up).astype(np.float32)
    mixed[0], mixed[-1] = -1e6, 1e6
    ints = np.floor(r.random(n) * 256).astype(np.float32)
    nan_top = ints.copy()
    nan_top[r.integers(0, n, 1000)] = np.uint32(0xFFFFFFFF).view(np.float32)  # largest key
    vecs = [halves, mixed, ints, nan_top]
    ks = [np.concatenate([gp_pgrid(n, 64), [n // 2 - 1, n // 2, n // 2 + 1, n // 2 + 2]]).astype(
        np.uint32) for _ in vecs]
    ctx = g.Context(0)
    for div, tile in ((1024, 1 << 20), (256, 1 << 18), (4096, 1 << 16)):
        g.batch_set_tuning(ctx, div, tile)
        _check_batch(g, orc, vecs, ks, np.float32, f"single-key div {div} tile {tile}", ctx=ctx)
    ctx.close()


def test_batch_many_slots_and_large_topk(g, orc):
    """Per-problem request counters: a problem with more slots than the plan
    phase's shared memory holds, and top-k problems with thousands of
    requests in a few slots."""
    import ggks_problems as gp
    n = 1 << 22
    a = gp.generate("f32", "uniform", n, seed=41)
    b = gp.generate("f32", "normal", 300_000, seed=42)
    ka = gp.k_distinct(n, 6000, 5)
    kb = np.arange(1, 4097, dtype=np.uint32)  # the 4096 largest, as a k list
    ctx = g.Context(0)
    g.batch_set_tuning(ctx, 256, 1 << 20)
    _check_batch(g, orc, [a, b], [ka, kb], np.float32, "many slots", ctx=ctx)
    ctx.close()


@pytest.mark.parametrize("spread", [300, 6000])
def test_batch_mid_size_segments(g, orc, spread):
    """Vectors of 2^23-2^24 elements put 1000-4000 keys in a bucket (8192
    buckets a problem at most): a slot with at most four requests is answered
    by one warp's radix select, one with five or more by a whole CTA.  The
    k's: spread ranks (one request a slot), groups of three and of five
    adjacent ranks, and ranks on a dense cluster (3000 copies of one value:
    its bin does not fit the warp's buffer, so a CTA finishes the slot after
    the warps); heavy duplicates, whose bins are one key wide.  300 spread
    k's a problem leave the batch's mid-size slots to CTAs, 6000 give the
    warps enough of them."""
    import ggks_problems as gp
    r = np.random.default_rng(23)

    def ks_for(n, seed):
        rr = np.random.default_rng(seed)
        sp = gp.k_distinct(n, spread, seed)
        base = rr.integers(10, n - 10, 40)
        threes = (base[:20, None] + np.arange(3)).ravel()
        fives = (base[20:, None] + np.arange(5)).ravel()
        return np.concatenate([sp, threes, fives, [1, n]]).astype(np.uint32)

    n = 1 << 23
    a = gp.generate("f32", "normal", n, seed=1)
    c = r.random(n).astype(np.float32)
    c[r.choice(n, 3000, replace=False)] = np.float32(0.5)
    below = int(np.count_nonzero(c < 0.5))
    # two requests on the cluster (a warp tries, its CTA finishes), and the
    # same vector with nine requests on and around it (a CTA's slot)
    kc2 = np.concatenate([ks_for(n, 3), [n - below, n - below - 1500]])
    kc9 = np.concatenate([n - below - np.array([0, 1, 1500, 2999]),
                          n - below - 3000 + np.arange(-2, 1), n - below + np.arange(1, 3)])
    _check_batch(g, orc, [a, c, c], [ks_for(n, 2), kc2.astype(np.uint32), kc9.astype(np.uint32)],
                 np.float32, "mid f32")
    u = gp.generate("u32", "uniform", 1 << 24, seed=4)
    # 256 copies of each value of [0, 2^16): buckets of a few values, whose
    # bins are one key wide (answered from the bin, however many copies)
    v = gp.generate("u32", "uniform16", 1 << 24, seed=10)
    _check_batch(g, orc, [u, v], [ks_for(u.size, 5), ks_for(v.size, 11)], np.uint32, "mid u32")
    w = gp.generate("f32", "uint_valued", 1 << 23, seed=12)
    _check_batch(g, orc, [w], [ks_for(w.size, 13)], np.float32, "mid integer-valued f32")
    d = gp.generate("f64", "cauchy", n, seed=6)
    e = gp.generate("f64", "normal", 3 << 21, seed=7)
    _check_batch(g, orc, [d, e], [ks_for(n, 8), ks_for(e.size, 9)], np.float64, "mid f64")
