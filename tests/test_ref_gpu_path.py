"""The reference's own GPU kernels against this path, on the GPU.

oracle/ref_gpu.py runs the reference's bucket multiselect with its own
kernels (bucketMultiselect.cu:129-325, compiled for sm_103a from its sources)
under a restatement of its host code (phaseOne, :521-833).  Here its answers
must equal, bit for bit, this path's and sort-and-choose's on:
  * the committed fixtures of the reference run on the host CPU
    (tests/golden/ref_*.npz): the reference's kernels on the GPU reproduce
    them, which ties the host build that made them to the real device code;
  * the plain configuration exactly (2^20, seed 0, 101 k's on the p grid),
    also through the reference's GPU sort-and-choose (its own oracle,
    multiselectTimingFunctions.cu:51-95);
  * every input of the large configuration at its full size (1001 k's);
  * the top-k configuration's inputs at 2^26, K = 32 / 1024 / 65536 (k =
    1..K, timeBucketTopkselect, :205-231).
The inputs hold no NaN and no -0.0, where the reference's native `<` is not
a total order, and no k list made only of 1 and n (the reference then reads
outside its arrays).  Skipped where the reference's kernels were never
compiled (the cubin is built only beside the reference's sources)."""
import os
import sys

import numpy as np
import pytest

import ggks_problems as gp
from conftest import GOLDEN_DIR, ref_files
from gpu_util import DeviceArray, assert_same

sys.path.insert(0, GOLDEN_DIR)
import ref_inputs as ri  # noqa: E402

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
def rg():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ref_gpu
    why = ref_gpu.unavailable()
    if why:
        pytest.skip("reference GPU path unavailable: " + why)
    ref_gpu.lib()
    return ref_gpu


@pytest.fixture(scope="module")
def orc():
    import oracle
    oracle.build()
    return oracle


REF = ref_files()


@pytest.mark.parametrize("path", REF, ids=[os.path.basename(p)[4:-4] for p in REF])
def test_reference_gpu_reproduces_host_fixtures(rg, path):
    f, vec = ri.load_case(path)
    name = os.path.basename(path)
    if str(f["kind"]) == "topk":
        got, ms = rg.time_bucket_topk(vec, int(f["k"][0]))
    else:
        got, ms = rg.time_bucket_multiselect(vec, f["k"])
    assert ms >= 0
    assert_same(got, f["expected"], name + " (reference kernels on the GPU)")


def test_plain_configuration(g, rg, orc):
    x, k = gp.config_p()
    want = orc.multiselect(x, k, THREADS)
    got, _ = rg.time_bucket_multiselect(x, k)
    assert_same(got, want, "P: reference bucket multiselect on the GPU")
    got, _ = rg.time_sort_choose_multiselect(x, k)
    assert_same(got, want, "P: reference sort-and-choose on the GPU")
    d = DeviceArray(x)
    assert_same(g.multiselect_ptr(d.ptr, d.n, d.dtype, k), want, "P: this path")
    # the device-vector entry, as the bench times it
    p = rg.padded_device_copy(x)
    got, ms = rg.bucket_multiselect_device(p.data_ptr(), x.size, k, x.dtype)
    assert ms > 0
    assert_same(got, want, "P: reference wrapper on a resident vector")


@pytest.mark.parametrize("name", [c[0] for c in gp.L_INPUTS])
def test_large_configuration(g, rg, orc, name):
    import torch
    x, k = gp.config_l(name)
    want = orc.multiselect(x, k, THREADS)
    p = rg.padded_device_copy(x)
    got_ref, _ = rg.bucket_multiselect_device(p.data_ptr(), x.size, k, x.dtype)
    got = g.multiselect_ptr(p.data_ptr(), x.size, x.dtype, k)
    del p
    torch.cuda.empty_cache()
    assert_same(got_ref, want, f"L {name}: reference kernels")
    assert_same(got, got_ref, f"L {name}: this path vs the reference's kernels")


@pytest.mark.parametrize("name", list(gp.T_INPUTS))
def test_topk_configuration(g, rg, orc, name):
    x = gp.config_t(name)
    want = orc.topk(x, max(gp.T_KS), THREADS)
    d = DeviceArray(x)
    for K in gp.T_KS:
        got_ref, _ = rg.time_bucket_topk(x, K)
        assert_same(got_ref, want[:K], f"T {name} K={K}: reference kernels")
        assert_same(g.topk_ptr(d.ptr, d.n, d.dtype, K), got_ref,
                    f"T {name} K={K}: this path vs the reference's kernels")
