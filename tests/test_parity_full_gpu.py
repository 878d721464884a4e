"""Parity at the configurations' own sizes: every input of the large
configuration (2^28 float32 normal / Cauchy / half-normal, 2^28 uint32, 2^27
float64; 1001 distinct k's), every top-k input (2^26 float32 uniform, uint32
over [0, 2^16), ascending float32; K = 32 / 1024 / 65536) and the plain
configuration exactly (2^20 float32 uniform, seed 0, k = floor(p (n - 1)) + 1
for 101 p's), against sort-and-choose (multiselectTimingFunctions.cu:51-95,
:156-177) run on every host core.

The reference checks every timed run against sort-and-choose at the size it
timed (compareMultiselect.hpp:164-185, compareTopkselect.hpp:165-185); these
are the same inputs the benchmark times.  Behaviour that only appears at
these sizes -- tiles of 8 vectors per thread, the survivor buffer's regrowth,
1024 copies of every uint32 value over [0, 2^16) -- is covered here.
Every comparison is bit-exact."""
import os

import numpy as np
import pytest

import ggks_problems as gp
from gpu_util import assert_same

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


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


def _device(x):
    import torch
    carrier = x.view(np.int32) if x.dtype == np.uint32 else x
    return torch.from_numpy(carrier).cuda()


def test_plain_configuration_exact(g, orc):
    x, k = gp.config_p()
    assert x.size == 1 << 20 and k.size == 101 and k[0] == 1 and k[-1] == x.size
    d = _device(x)
    want = orc.multiselect(x, k, THREADS)
    for _ in range(2):  # a fresh context's first call and a warm one
        assert_same(g.multiselect_ptr(d.data_ptr(), x.size, x.dtype, k), want, "P")
    # top-k of the same input (the k list k = 1..K of timeBucketTopkselect)
    assert_same(g.topk_ptr(d.data_ptr(), x.size, x.dtype, 101), orc.topk(x, 101, THREADS),
                "P top-101")


@pytest.mark.parametrize("name", [c[0] for c in gp.L_INPUTS])
def test_large_configuration(g, orc, name):
    import torch
    x, k = gp.config_l(name)
    assert k.size == gp.L_NUM_K and np.unique(k).size == k.size
    d = _device(x)
    ctx = g.Context(0)
    got = g.multiselect_ptr(d.data_ptr(), x.size, x.dtype, k, ctx=ctx)
    want = orc.multiselect(x, k, THREADS)
    assert_same(got, want, f"L {name}")
    # the same call again on the warm context (grown survivor buffer)
    assert_same(g.multiselect_ptr(d.data_ptr(), x.size, x.dtype, k, ctx=ctx), want,
                f"L {name} again")
    ctx.close()
    del d
    torch.cuda.empty_cache()


@pytest.mark.parametrize("name", list(gp.T_INPUTS))
def test_topk_configuration(g, orc, name):
    import torch

    x = gp.config_t(name)
    d = _device(x)
    ctx = g.Context(0)
    want = orc.topk(x, max(gp.T_KS), THREADS)  # descending: every K is a prefix
    for K in gp.T_KS:
        got = g.topk_ptr(d.data_ptr(), x.size, x.dtype, K, ctx=ctx)
        assert_same(got, want[:K], f"T {name} K={K}")
    # the multiset of the K largest: no element of the rest exceeds the K-th
    kth = want[max(gp.T_KS) - 1]
    assert np.count_nonzero(x > kth) < max(gp.T_KS)
    if name != "u32_uniform16":
        # buckets whose every rank is requested are finished in rounds, not
        # by a recursive level
        assert ctx.stats()["recursions"] == 0
    ctx.close()
    del d
    torch.cuda.empty_cache()
