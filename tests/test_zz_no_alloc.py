"""The multiselect that allocates nothing (ggks_multiselect_noalloc_f32).

Callers that cannot allocate at the point of the call -- a CUDA graph being
captured, an engine whose memory another allocator owns, a latency-critical
path -- use this entry point: its scratch is a fixed device array inside the
library, and input, k list and output are the caller's device buffers.  These
tests call it through the C ABI twice in a row on different inputs and compare
each result bit for bit with the regular entry point, ggks_multiselect_f32.
This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ggks
    ggks.lib()
    return ggks


def _device(arr):
    import torch
    carrier = arr.view(np.int32) if arr.dtype == np.uint32 else arr
    return torch.from_numpy(np.ascontiguousarray(carrier)).cuda()


def test_noalloc_matches_regular_entry_point_on_two_calls(g):
    import torch

    import ggks_problems as gp
    cases = (("normal", 1 << 21, 1), ("cauchy", 1_500_007, 2))
    for dist, n, seed in cases:
        x = gp.generate("f32", dist, n, seed)
        ks = np.concatenate([gp.k_pgrid(n, 101), gp.k_distinct(n, 900, seed)]).astype(np.uint32)
        d_x, d_k = _device(x), _device(ks)
        d_out = torch.empty(ks.size, dtype=torch.float32, device="cuda")
        st = g.multiselect_noalloc_f32(d_x.data_ptr(), n, d_k.data_ptr(), ks.size,
                                       d_out.data_ptr())
        assert st == g.OK, g.status_string(st)
        got = d_out.cpu().numpy()
        want = g.multiselect_ptr(d_x.data_ptr(), n, np.float32, ks)
        # bit-exact, the tolerance of every parity test in this suite
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), dist


def test_noalloc_rejects_sizes_beyond_its_limits(g):
    import torch
    x = torch.zeros(16, dtype=torch.float32, device="cuda")
    k = torch.ones(4, dtype=torch.int32, device="cuda")
    out = torch.empty(4, dtype=torch.float32, device="cuda")
    max_n = 1 << 21
    assert g.multiselect_noalloc_f32(x.data_ptr(), max_n + 1, k.data_ptr(), 4,
                                     out.data_ptr()) == g.INVALID_ARG
    assert g.multiselect_noalloc_f32(x.data_ptr(), 16, k.data_ptr(), 2049,
                                     out.data_ptr()) == g.INVALID_ARG
    bad = torch.tensor([1, 2, 0, 3], dtype=torch.int32, device="cuda")  # k = 0
    assert g.multiselect_noalloc_f32(x.data_ptr(), 16, bad.data_ptr(), 4,
                                     out.data_ptr()) == g.INVALID_ARG
