"""The multiselect that allocates nothing (ggks_multiselect_noalloc_f32).

Callers that may not allocate when they select -- an engine whose device
memory all belongs to its own allocator, which budgets every byte, or a
latency-bound loop where an allocation would stall on the driver -- use this
entry point: its scratch is a fixed device array inside the library, and
input, k list and output are the caller's device buffers.  These tests call it
through the C ABI, twice in a row on different inputs, and compare each result
bit for bit with the regular entry point (ggks_multiselect_f32) and with the
oracle (sort-and-choose).  This file is collected last so that a run stopping
at the first failure has already run every other test; every test here also
passes alone in a fresh process.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_N = 1 << 21
MAX_K = 2048
GUARD = 64  # sentinel entries after d_out


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


def _device(arr):
    import torch
    carrier = arr.view(np.int32) if arr.dtype == np.uint32 else arr
    return torch.from_numpy(np.ascontiguousarray(carrier)).cuda()


def _out(num_k):
    """Device output of num_k floats followed by GUARD sentinel floats."""
    import torch
    t = torch.full((num_k + GUARD,), float("nan"), dtype=torch.float32, device="cuda")
    t[num_k:] = -12345.0
    return t


def _call(g, x, ks, stream=None):
    """One no-allocation call on device copies of x and ks; returns (status,
    outputs, guard intact)."""
    import torch
    d_x, d_k = _device(x), _device(ks.astype(np.uint32))
    d_out = _out(ks.size)
    torch.cuda.synchronize()
    st = g.multiselect_noalloc_f32(d_x.data_ptr(), x.size, d_k.data_ptr(), ks.size,
                                   d_out.data_ptr(), stream)
    res = d_out.cpu().numpy()
    return st, res[:ks.size], bool(np.all(res[ks.size:] == np.float32(-12345.0)))


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_noalloc_matches_regular_entry_point_on_two_calls(g, orc):
    import ggks_problems as gp
    cases = (("normal", 1 << 21, 1), ("cauchy", 1_500_007, 2))
    for dist, n, seed in cases:
        x = gp.generate("f32", dist, n, seed)
        ks = np.concatenate([gp.k_pgrid(n, 101), gp.k_distinct(n, 900, seed)]).astype(np.uint32)
        st, got, guard = _call(g, x, ks)
        assert st == g.OK, g.status_string(st)
        assert guard
        want = g.multiselect_ptr(_device(x).data_ptr(), n, np.float32, ks)
        # bit-exact, the tolerance of every parity test in this suite
        assert np.array_equal(_bits(got), _bits(want)), dist
        assert np.array_equal(_bits(got), _bits(orc.multiselect(x, ks, 8))), dist


@pytest.mark.parametrize("n", [1, 2, 1000, 65535, 65536, 65537])
def test_noalloc_small_sizes(g, orc, n):
    """Small vectors sample every element (S = n) on a single histogram CTA."""
    import ggks_problems as gp
    x = gp.generate("f32", "normal", n, n)
    ks = np.arange(1, n + 1, dtype=np.uint32) if n <= MAX_K else gp.k_distinct(n, 777, 3)
    for rep in range(2):
        st, got, guard = _call(g, x, ks)
        assert st == g.OK, g.status_string(st)
        assert guard
        assert np.array_equal(_bits(got), _bits(orc.multiselect(x, ks))), (n, rep)


def test_noalloc_most_ks_and_largest_n(g, orc):
    """num_k at its limit (2048: more requests than one plan thread each)
    and n at its limit, twice in a row."""
    import ggks_problems as gp
    for seed, dist in ((5, "uniform"), (6, "half_normal")):
        x = gp.generate("f32", dist, MAX_N, seed)
        ks = gp.k_distinct(MAX_N, MAX_K, seed)
        st, got, guard = _call(g, x, ks)
        assert st == g.OK, g.status_string(st)
        assert guard
        assert np.array_equal(_bits(got), _bits(orc.multiselect(x, ks, 8))), dist


def test_noalloc_on_a_caller_stream(g, orc):
    """The call runs on the caller's (non-default) stream and returns with the
    results in d_out."""
    import torch

    import ggks_problems as gp
    s = torch.cuda.Stream()
    x = gp.generate("f32", "uniform", 300_001, 9)
    ks = gp.k_pgrid(x.size, 101)
    for rep in range(2):
        with torch.cuda.stream(s):
            st, got, guard = _call(g, x, ks, stream=s.cuda_stream)
        assert st == g.OK, g.status_string(st)
        assert guard
        assert np.array_equal(_bits(got), _bits(orc.multiselect(x, ks))), rep


def test_noalloc_unsupported_heavy_cluster_stays_in_bounds(g, orc):
    """Half of the vector is 2048 neighbouring floats (512 copies each), the
    rest spread over the whole float range: the cluster's few buckets hold far
    more keys than a finishing CTA can sort, which needs a recursive level
    with a workspace of its own.  The call reports GGKS_UNSUPPORTED and writes
    nothing past d_out; a later call on a plain input is exact again."""
    import ggks_problems as gp
    r = np.random.default_rng(3)
    n = MAX_N
    x = np.empty(n, dtype=np.float32)
    half = n // 2
    x[:half] = (np.float32(1.0).view(np.uint32) + (np.arange(half) % 2048).astype(np.uint32)).view(
        np.float32)
    x[half:] = (r.uniform(-1e38, 1e38, n - half)).astype(np.float32)
    r.shuffle(x)
    ks = gp.k_distinct(n, MAX_K, 2)
    st, got, guard = _call(g, x, ks)
    assert guard, "wrote past d_out"
    assert st == g.UNSUPPORTED, g.status_string(st)
    # the regular entry point selects it (recursively)
    want = orc.multiselect(x, ks, 8)
    assert np.array_equal(_bits(g.multiselect_ptr(_device(x).data_ptr(), n, np.float32, ks)),
                          _bits(want))
    y = gp.generate("f32", "normal", 100_000, 4)
    ky = gp.k_pgrid(y.size, 101)
    st, got, guard = _call(g, y, ky)
    assert st == g.OK and guard
    assert np.array_equal(_bits(got), _bits(orc.multiselect(y, ky)))


def test_noalloc_allocates_nothing(g):
    """After a first call on the device, further calls leave the device's free
    memory unchanged (no allocation anywhere: neither in the library nor by a
    library routine it calls)."""
    import torch

    import ggks_problems as gp
    x = gp.generate("f32", "normal", 1 << 20, 12)
    ks = gp.k_distinct(x.size, 1001, 1).astype(np.uint32)
    d_x, d_k = _device(x), _device(ks)
    d_out = _out(ks.size)
    s = torch.cuda.Stream()
    assert g.multiselect_noalloc_f32(d_x.data_ptr(), x.size, d_k.data_ptr(), ks.size,
                                     d_out.data_ptr(), s.cuda_stream) == g.OK
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(20):
        assert g.multiselect_noalloc_f32(d_x.data_ptr(), x.size, d_k.data_ptr(), ks.size,
                                         d_out.data_ptr(), s.cuda_stream) == g.OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_sizes_beyond_its_limits(g):
    import torch
    x = torch.zeros(16, dtype=torch.float32, device="cuda")
    k = torch.ones(4, dtype=torch.int32, device="cuda")
    out = torch.empty(4, dtype=torch.float32, device="cuda")
    assert g.multiselect_noalloc_f32(x.data_ptr(), MAX_N + 1, k.data_ptr(), 4,
                                     out.data_ptr()) == g.INVALID_ARG
    assert g.multiselect_noalloc_f32(x.data_ptr(), 16, k.data_ptr(), MAX_K + 1,
                                     out.data_ptr()) == g.INVALID_ARG
    assert g.multiselect_noalloc_f32(x.data_ptr(), 0, k.data_ptr(), 4,
                                     out.data_ptr()) == g.INVALID_ARG
    bad = torch.tensor([1, 2, 0, 3], dtype=torch.int32, device="cuda")  # k = 0
    assert g.multiselect_noalloc_f32(x.data_ptr(), 16, bad.data_ptr(), 4,
                                     out.data_ptr()) == g.INVALID_ARG
    bad = torch.tensor([1, 2, 17, 3], dtype=torch.int32, device="cuda")  # k > n
    assert g.multiselect_noalloc_f32(x.data_ptr(), 16, bad.data_ptr(), 4,
                                     out.data_ptr()) == g.INVALID_ARG
