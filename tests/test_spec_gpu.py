"""Speculative compaction on the GPU: when the requested ranks cluster (top-k,
one k, k's near both ends), the histogram pass also keeps the elements of the
buckets the sample predicts, and compaction reads those in place of the
vector.  (Top-k calls here force the pipeline: small K otherwise take the
threshold path, tests/test_topk_threshold_gpu.py.)  Every result is compared bit for bit with the oracle (sort-and-choose,
multiselectTimingFunctions.cu:51-95 / :156-177), including the cases where the
prediction misses or a CTA's candidates overflow and compaction falls back to
the vector."""
import numpy as np
import pytest

from gpu_util import DeviceArray, assert_same

pytestmark = pytest.mark.gpu

SAMPLES = 65536
SEED = 0x5EED


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


def sampled_positions(n):
    """Positions the sampling pass reads for a vector of n > 65536 elements:
    pairs of neighbours, sample i at murmur3's 32-bit finaliser of
    (i / 2) * 0x9E3779B9 + seed scaled to [0, n - 1), plus i mod 2."""
    i = np.arange(SAMPLES, dtype=np.uint64)
    a = ((i >> np.uint64(1)) * 0x9E3779B9 + SEED) & 0xFFFFFFFF
    a ^= a >> 16
    a = (a * 0x85EBCA6B) & 0xFFFFFFFF
    a ^= a >> 13
    a = (a * 0xC2B2AE35) & 0xFFFFFFFF
    a ^= a >> 16
    return ((a * np.uint64(n - 1)) >> np.uint64(32)) + (i & np.uint64(1))


def run(g, fn, *args, **kw):
    ctx = g.Context(0)
    try:
        got = fn(*args, ctx=ctx, **kw)
        return got, ctx.stats()
    finally:
        ctx.close()


TOPK = [("f32", "uniform", 1 << 22, 1024), ("f32", "normal", 1 << 22, 65536),
        ("f32", "cauchy", 3_000_017, 777), ("f64", "normal", 1 << 21, 4096),
        ("u32", "uniform", 1 << 22, 32), ("u32", "uniform16", 1 << 21, 5000),
        ("f32", "half_normal", 1 << 20, 1)]


@pytest.mark.parametrize("dtype,dist,n,K", TOPK, ids=[f"{a}-{b}-{c}-{d}" for a, b, c, d in TOPK])
def test_topk_reads_candidates(g, orc, dtype, dist, n, K):
    import ggks_problems as gp
    x = gp.generate(dtype, dist, n, seed=K + 1)
    d = DeviceArray(x)
    got, st = run(g, g.topk_ptr, d.ptr, n, x.dtype, K, pipeline=True)
    assert_same(got, orc.topk(x, K, threads=8), f"topk {dtype}/{dist}/{n}/{K}")
    assert st["spec_calls"] == 1
    if dist != "uniform16":  # 2^16 values: the top buckets may hold one key each
        assert st["spec_ctas"] > 0


def test_clustered_ks_two_windows(g, orc):
    """k's at both ends: two windows, each open towards its end of the order."""
    import ggks_problems as gp
    n = 1 << 22
    x = gp.normal_f32(n, 12)
    ks = np.concatenate([np.arange(1, 11), np.arange(n - 9, n + 1)]).astype(np.uint32)
    d = DeviceArray(x)
    got, st = run(g, g.multiselect_ptr, d.ptr, n, x.dtype, ks)
    assert_same(got, orc.multiselect(x, ks, 8), "both ends")
    assert st["spec_calls"] == 1 and st["spec_ctas"] > 0
    # one k in the middle, and a few neighbours of it
    for ks in ([n // 2], [n // 3, n // 3 + 1, n // 3 + 5000]):
        ks = np.array(ks, dtype=np.uint32)
        got, st = run(g, g.multiselect_ptr, d.ptr, n, x.dtype, ks)
        assert_same(got, orc.multiselect(x, ks), f"middle {ks.tolist()}")
        assert st["spec_calls"] == 1 and st["spec_ctas"] > 0


def test_spread_ks_do_not_speculate(g, orc):
    import ggks_problems as gp
    n = 1 << 21
    x = gp.uniform_f32(n, 13)
    ks = gp.k_pgrid(n, 101)
    d = DeviceArray(x)
    got, st = run(g, g.multiselect_ptr, d.ptr, n, x.dtype, ks)
    assert_same(got, orc.multiselect(x, ks, 8), "p-grid")
    assert st["spec_calls"] == 0 and st["spec_ctas"] == 0


def test_prediction_miss_falls_back(g, orc):
    """A vector whose sampled positions misrepresent it: 90 % of the elements
    lie in [2, 3) but half of the sampled ones lie in [0, 1).  The median
    sits far above the sample's median, so the predicted buckets miss the
    median's bucket: compaction must read the vector (no CTA reads
    candidates) and the result must still be exact."""
    r = np.random.default_rng(21)
    n = 1 << 22
    x = np.where(r.random(n) < 0.9, 2.0 + r.random(n), r.random(n)).astype(np.float32)
    pos = sampled_positions(n).astype(np.int64)
    half = np.arange(SAMPLES) % 2 == 0
    x[pos[half]] = r.random(int(half.sum())).astype(np.float32)
    x[pos[~half]] = (2.0 + r.random(int((~half).sum()))).astype(np.float32)
    ks = np.array([n // 2], dtype=np.uint32)
    d = DeviceArray(x)
    got, st = run(g, g.multiselect_ptr, d.ptr, n, x.dtype, ks)
    assert_same(got, orc.multiselect(x, ks), "miss")
    assert st["spec_calls"] == 1 and st["spec_ctas"] == 0


def test_presorted_candidates_fill_few_ctas(g, orc):
    """Ascending input: the top elements sit in the last tiles, so a few CTAs
    hold every candidate.  Their warps take as many pool chunks as they need,
    and every CTA reads its candidate lists (most of them empty)."""
    import ggks_problems as gp
    n = 1 << 22
    x = np.sort(gp.uniform_f32(n, 14))
    d = DeviceArray(x)
    for K in (1024, 65536):
        got, st = run(g, g.topk_ptr, d.ptr, n, x.dtype, K, pipeline=True)
        assert_same(got, orc.topk(x, K, 8), f"sorted K={K}")
        assert st["spec_calls"] == 1
        assert st["spec_ctas"] == min(n // 65536, 152)


def test_speculation_with_survivor_overflow(g, orc):
    """Three quarters of the vector in one narrow cluster above the rest, at
    positions the sample never reads: the table predicts few candidates and
    keeps them, but the top bucket (keys above the sampled span) holds the
    whole cluster, so its survivors exceed the survivor buffer.  The buffer is
    regrown and the re-run compaction reads the vector (the candidates were in
    the old buffer).  The cluster's elements are all candidates: the pool runs
    out long before, so no CTA could have read candidates anyway."""
    r = np.random.default_rng(3)
    n = 1 << 23
    x = 3.0 + r.integers(0, 1 << 16, n) * 2.0 ** -50
    pos = np.unique(sampled_positions(n).astype(np.int64))
    spread = np.setdiff1d(r.choice(n, n // 4, replace=False), pos)
    x[spread] = r.random(spread.size) * 2.0
    x[pos] = r.random(pos.size) * 2.0
    d = DeviceArray(x)
    got, st = run(g, g.topk_ptr, d.ptr, n, np.float64, 100, pipeline=True)
    assert_same(got, orc.topk(x, 100, 8), "cluster top-k")
    assert st["spec_calls"] == 1 and st["spec_ctas"] == 0
    assert st["retries"] > 0


def test_host_vector_topk_speculates(g, orc):
    """The pinned-host entry: the first pass reads the host vector, writes the
    device copy and keeps the candidates."""
    import ggks_problems as gp
    x = gp.normal_f32(1 << 22, 15)
    assert_same(g.topk_host(x, 2048, pipeline=True), orc.topk(x, 2048, 8), "host topk")
    ks = np.array([7, 1 << 21], dtype=np.uint32)
    assert_same(g.multiselect_host(x, ks), orc.multiselect(x, ks), "host two k's")
