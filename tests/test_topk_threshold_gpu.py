"""Top-k by a sampled threshold (csrc/ggks_topk.cuh) on the GPU: for K <= 4096
of a vector larger than the sample, one streaming pass keeps the elements at
or above a threshold taken from the sample and one CTA selects the K largest
of them.  Every result is compared bit for bit with the oracle (sort-and-
choose, multiselectTimingFunctions.cu:156-177) and with the pipeline on the
same input, including inputs built so that the threshold's candidates fall
short and the call falls back to the pipeline."""
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
    """Positions the sampling pass reads for a vector of n > 65536 elements
    (pairs of neighbours at murmur3-hashed positions)."""
    i = np.arange(SAMPLES, dtype=np.uint64)
    a = ((i >> np.uint64(1)) * 0x9E3779B9 + SEED) & 0xFFFFFFFF
    a ^= a >> 16
    a = (a * 0x85EBCA6B) & 0xFFFFFFFF
    a ^= a >> 13
    a = (a * 0xC2B2AE35) & 0xFFFFFFFF
    a ^= a >> 16
    return ((a * np.uint64(n - 1)) >> np.uint64(32)) + (i & np.uint64(1))


def _topk(g, x, K, **kw):
    """The threshold path where it applies (small=False: not the one-launch
    small-vector path, which takes small vectors first)."""
    kw.setdefault("small", False)
    ctx = g.Context(0)
    try:
        d = DeviceArray(x)
        got = g.topk_ptr(d.ptr, x.size, x.dtype, K, ctx=ctx, **kw)
        return got, ctx.stats()
    finally:
        ctx.close()


CASES = [("f32", "uniform", 1 << 22, 1), ("f32", "uniform", 1 << 22, 32),
         ("f32", "normal", 1 << 22, 1024), ("f32", "cauchy", 3_000_017, 4096),
         ("f32", "half_normal", 65_537 + 1024, 1024), ("f32", "killer", 1 << 20, 777),
         ("f32", "uint_valued", 1 << 21, 4096), ("f32", "ones_twos", 1 << 20, 100),
         ("f32", "all_ones", 1 << 20, 33), ("f64", "normal", 1 << 21, 4096),
         ("f64", "uniform_pm1e6", 1 << 20, 1), ("f64", "uint_valued", 1 << 20, 2048),
         ("u32", "uniform", 1 << 22, 32), ("u32", "uniform16", 1 << 22, 4096),
         ("u32", "sorted", 1 << 21, 1000), ("u32", "zero_to_four", 1 << 20, 4096)]


@pytest.mark.parametrize("dtype,dist,n,K", CASES, ids=[f"{a}-{b}-{c}-{d}" for a, b, c, d in CASES])
def test_threshold_topk_vs_oracle(g, orc, dtype, dist, n, K):
    import ggks_problems as gp
    x = gp.generate(dtype, dist, n, seed=K + 7)
    got, st = _topk(g, x, K)
    want = orc.topk(x, K, 8)
    assert_same(got, want, f"threshold top-k {dtype}/{dist}/{n}/{K}")
    assert st["topk_threshold_calls"] + st["topk_misses"] == 1
    if dist != "killer":
        # (the bucket killer's head of 2^-126 .. 2^126 stretches the sampled
        # span so far that the threshold's fine slice holds most of the
        # vector, and the pick's gather does not fit: a miss, by design)
        assert st["topk_misses"] == 0, "a plain input fell back to the pipeline"
    # the pipeline gives the same answer
    got_p, st_p = _topk(g, x, K, pipeline=True)
    assert_same(got_p, want, "pipeline")
    assert st_p["topk_threshold_calls"] == 0


@pytest.mark.parametrize("K", [32, 1024, 4096])
def test_threshold_topk_sorted_and_reversed(g, orc, K):
    """Ascending input: every candidate sits in the last tiles, so a few warps
    hold them all; descending: in the first."""
    import ggks_problems as gp
    x = np.sort(gp.uniform_f32(1 << 22, 3))
    for arr in (x, x[::-1].copy()):
        got, st = _topk(g, arr, K)
        assert_same(got, orc.topk(arr, K, 8), f"sorted K={K}")
        assert st["topk_threshold_calls"] == 1


def test_threshold_topk_falls_back_when_the_sample_misses(g, orc):
    """Every position the sample reads holds one of the largest values (the
    rest lies below them): the sample puts the threshold among its own few
    largest keys, the filter keeps only those -- fewer than K -- and the call
    runs the pipeline."""
    r = np.random.default_rng(5)
    n = 1 << 22
    x = r.random(n).astype(np.float32)
    pos = np.unique(sampled_positions(n).astype(np.int64))
    x[pos] = 2.0 + r.random(pos.size).astype(np.float32)
    for K in (32, 4096):
        got, st = _topk(g, x, K)
        assert_same(got, orc.topk(x, K, 8), f"miss K={K}")
        assert st["topk_misses"] == 1 and st["topk_threshold_calls"] == 0


def test_threshold_topk_too_many_equal_candidates_fall_back(g, orc):
    """Half the vector is two neighbouring floats at the top: the bin of the
    K-th largest holds far more keys than the pick CTA gathers (two distinct
    keys, so not a one-key bin), and the call runs the pipeline."""
    r = np.random.default_rng(6)
    n = 1 << 21
    x = r.random(n).astype(np.float32)
    half = r.choice(n, n // 2, replace=False)
    x[half] = np.where(r.random(half.size) < 0.5, np.float32(3.0),
                       np.nextafter(np.float32(3.0), np.float32(4.0)))
    # a far key above them keeps the bins wide
    x[r.integers(0, n)] = np.float32(1e30)
    got, st = _topk(g, x, 4096)
    assert_same(got, orc.topk(x, 4096, 8), "equal candidates")
    assert st["topk_threshold_calls"] + st["topk_misses"] == 1


def test_threshold_topk_host_vectors(g, orc):
    """Host entry points: a pinned vector is read in place by the sample and
    filter passes, which write the device copy; a pageable one is staged."""
    import torch

    import ggks_problems as gp
    x = gp.normal_f32((1 << 22) + 3, 21)
    pin = torch.empty(x.size, dtype=torch.float32, pin_memory=True)
    pin.numpy()[:] = x
    for K in (1, 100, 4096):
        assert_same(g.topk_host(pin.numpy(), K), orc.topk(x, K, 8), f"pinned K={K}")
        assert_same(g.topk_host(x, K), orc.topk(x, K, 8), f"pageable K={K}")


def test_threshold_topk_repeated_calls_one_context(g, orc):
    """The slice counts at the workspace head and the sample ticket re-arm
    between threshold calls, pipeline calls and multiselects on one context."""
    import ggks_problems as gp
    ctx = g.Context(0)
    for it, (dist, n, K) in enumerate([("normal", 1 << 21, 64), ("uniform", 1 << 20, 4096),
                                       ("cauchy", 1 << 22, 1), ("normal", 1 << 21, 65536)] * 2):
        x = gp.generate("f32", dist, n, seed=it)
        d = DeviceArray(x)
        assert_same(g.topk_ptr(d.ptr, n, x.dtype, K, ctx=ctx, small=False), orc.topk(x, K, 8),
                    f"call {it}")
        ks = gp.k_pgrid(n, 101)
        assert_same(g.multiselect_ptr(d.ptr, n, x.dtype, ks, ctx=ctx, small=False),
                    orc.multiselect(x, ks, 8), f"multiselect {it}")
    st = ctx.stats()
    assert st["topk_threshold_calls"] == 6
    ctx.close()


def test_threshold_topk_far_outlier_sorts_together(g, orc):
    """One key far above the rest stretches the pick's bins until nearly every
    candidate shares the bottom bin: the gathered keys are sorted together
    (bitonic) rather than bin by bin, and the answer is the same."""
    import ggks_problems as gp
    x = gp.uniform_f32(1 << 22, 17)
    x[12345] = np.float32(1e30)
    for K in (1, 32, 100):
        got, st = _topk(g, x, K)
        assert_same(got, orc.topk(x, K, 8), f"far outlier K={K}")
        assert st["topk_threshold_calls"] == 1
