"""GPU tests of speculative compaction in the batched kernel: problems whose
requested ranks cluster (top-k, k's close together) keep the keys inside a
window taken from their sample while counting, and the compaction phase reads
those candidates in place of the tile.  Every output is compared bit for bit
with the oracle (sort-and-choose, multiselectTimingFunctions.cu:51-95 /
:156-177); the statistics show whether tiles read candidates, and the
fallbacks (a tile whose list overflows, a sample that misplaces the window)
are forced."""
import numpy as np
import pytest

from gpu_util import DeviceArray, assert_same

pytestmark = pytest.mark.gpu

MAX_S = 8192  # samples per problem in the batched kernel


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


def batch_sampled_positions(n, itemsize):
    """Elements the batched table phase samples from a problem of n > 8192
    elements: chunks of 32 bytes' worth of consecutive elements, chunk c at
    murmur3's 32-bit finaliser of c * 0x9E3779B9 + 0x5EED scaled to the
    n / chunk chunk positions."""
    ch = 32 // itemsize
    c = np.arange(MAX_S // ch, dtype=np.uint64)
    a = (c * np.uint64(0x9E3779B9) + np.uint64(0x5EED)) & np.uint64(0xFFFFFFFF)
    a ^= a >> np.uint64(16)
    a = (a * np.uint64(0x85EBCA6B)) & np.uint64(0xFFFFFFFF)
    a ^= a >> np.uint64(13)
    a = (a * np.uint64(0xC2B2AE35)) & np.uint64(0xFFFFFFFF)
    a ^= a >> np.uint64(16)
    pos = ((a * np.uint64(n // ch)) >> np.uint64(32)) * np.uint64(ch)
    return (pos[:, None] + np.arange(ch, dtype=np.uint64)[None, :]).ravel()


def run_topk(g, vecs, Ks, dtype):
    ctx = g.Context()
    devs = [DeviceArray(v) for v in vecs]
    got = g.topk_batch_ptr([d.ptr for d in devs], [v.size for v in vecs], dtype, Ks, ctx=ctx)
    st = ctx.stats()
    ctx.close()
    return got, st


@pytest.mark.parametrize("dtype,dists", [
    ("f32", ("uniform", "normal", "cauchy", "uniform")),
    ("u32", ("uniform", "uniform", "sorted", "uniform")),
    ("f64", ("uniform_pm1e6", "normal", "cauchy", "normal")),
])
def test_topk_batch_reads_candidates(g, orc, dtype, dists):
    import ggks_problems as gp
    sizes = [1 << 17, 300_001, 1 << 21, (1 << 22) + 5]
    Ks = [16, 100, 1024, 4096]
    vecs = [gp.generate(dtype, d, n, seed=7 + i) for i, (d, n) in enumerate(zip(dists, sizes))]
    npdt = vecs[0].dtype
    got, st = run_topk(g, vecs, Ks, npdt)
    for p, (v, K) in enumerate(zip(vecs, Ks)):
        assert_same(got[p], orc.topk(v, K, threads=8), f"{dtype} {dists[p]} n={v.size} K={K}")
    assert st["batch_spec_tiles"] > 0


def test_clustered_ks_batch_speculate(g, orc):
    """Multiselects whose k's lie close together (both ends, the middle) read
    candidates too; spread k lists do not speculate."""
    import ggks_problems as gp
    n = 1 << 21
    vecs = [gp.generate("f32", d, n, seed=30 + i)
            for i, d in enumerate(("uniform", "normal", "cauchy", "uint_valued"))]
    klists = [np.arange(1, 65, dtype=np.uint32),                   # the 64 largest
              np.arange(n - 40, n + 1, dtype=np.uint32),           # the 41 smallest
              (n // 2 + np.arange(-300, 300, 7)).astype(np.uint32),  # around the median
              gp.k_distinct(n, 50, 3)]                             # spread: no window
    ctx = g.Context()
    devs = [DeviceArray(v) for v in vecs]
    got = g.multiselect_batch_ptr([d.ptr for d in devs], [n] * 4, np.float32, klists, ctx=ctx)
    st = ctx.stats()
    ctx.close()
    for p, (v, ks) in enumerate(zip(vecs, klists)):
        assert_same(got[p], orc.multiselect(v, ks, 8), f"clustered problem {p}")
    assert st["batch_spec_tiles"] > 0


def test_presorted_tiles_overflow_and_read_their_elements(g, orc):
    """Ascending input puts a top-k's candidates in the last tiles, whose areas
    overflow: those tiles read their elements, the others their (empty)
    lists.  Descending input puts them in the first tiles."""
    import ggks_problems as gp
    up = np.sort(gp.generate("f32", "uniform", 1 << 22, seed=5))
    down = up[::-1].copy()
    got, st = run_topk(g, [up, down], [2048, 2048], np.float32)
    assert_same(got[0], orc.topk(up, 2048), "ascending")
    assert_same(got[1], orc.topk(down, 2048), "descending")
    assert st["batch_spec_tiles"] > 0


@pytest.mark.parametrize("where", ["sample_high", "sample_low"])
def test_misleading_sample_falls_back(g, orc, where):
    """The sampled chunks hold the vector's largest values (the window's lower
    threshold lands above the K-th largest: the plan sees a slot outside the
    window and the whole problem reads its elements) or its smallest (the
    threshold lands far too low: every tile's list overflows).  Results stay
    exact either way."""
    import ggks_problems as gp
    n = 1 << 21
    x = gp.generate("f32", "uniform", n, seed=9)
    pos = batch_sampled_positions(n, 4)
    if where == "sample_high":
        x[pos] = np.float32(2.0) + x[pos]
    else:
        x[pos] = x[pos] - np.float32(2.0)
    other = gp.generate("f32", "normal", 1 << 20, seed=10)
    got, st = run_topk(g, [x, other], [1024, 300], np.float32)
    assert_same(got[0], orc.topk(x, 1024), f"misleading sample ({where})")
    assert_same(got[1], orc.topk(other, 300), "neighbour problem")


def test_speculating_batch_matches_plain_calls(g, orc):
    """A served-like mix of top-k and multiselect problems of every size gives
    the single-vector entry point's answers."""
    import ggks_problems as gp
    r = np.random.default_rng(4)
    vecs, klists = [], []
    for i in range(24):
        n = int(2 ** r.uniform(12, 22))
        vecs.append(gp.generate("f32", gp.BATCH_DISTS[i % 4], n, seed=100 + i))
        if i % 3 == 0:
            K = int(min(n, r.integers(16, 4097)))
            klists.append(np.arange(1, K + 1, dtype=np.uint32))
        else:
            klists.append(r.integers(1, n + 1, int(r.integers(8, 200))).astype(np.uint32))
    devs = [DeviceArray(v) for v in vecs]
    got = g.multiselect_batch_ptr([d.ptr for d in devs], [v.size for v in vecs], np.float32,
                                  klists)
    for p, (d, v, ks) in enumerate(zip(devs, vecs, klists)):
        want = orc.multiselect(v, ks, 8)
        assert_same(got[p], want, f"mix problem {p}")
        assert_same(g.multiselect_ptr(d.ptr, d.n, np.float32, ks), want, f"plain {p}")
