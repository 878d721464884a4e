"""GPU parity against outputs of the reference itself.

tests/golden/ref_*.npz hold the reference's own answers
(bucketMultiselectWrapper through timeBucketMultiselect / timeBucketTopkselect,
multiselectTimingFunctions.cu:100-122, :205-231) for the plain configuration
exactly, the large configuration's shapes at 2^22, the top-k configuration's
inputs at 2^22 and duplicate-heavy, sorted, tiny and edge-k cases.  The CUDA
path must return the same bits through every entry: device vectors, host
vectors, the top-k pipeline and threshold paths, the single-k select and the
reference-named mirrors."""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN_DIR, ref_files
from gpu_util import DeviceArray, assert_same

sys.path.insert(0, GOLDEN_DIR)
import ref_inputs as ri  # noqa: E402

pytestmark = pytest.mark.gpu

REF = ref_files()
IDS = [os.path.basename(p)[4:-4] for p in REF]


@pytest.fixture(scope="module")
def g():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ggks
    ggks.lib()
    return ggks


@pytest.mark.parametrize("path", REF, ids=IDS)
def test_device_vector_matches_reference(g, path):
    f, vec = ri.load_case(path)
    d = DeviceArray(vec)
    name = os.path.basename(path)
    if str(f["kind"]) == "topk":
        K = int(f["k"][0])
        assert_same(g.topk_ptr(d.ptr, d.n, d.dtype, K), f["expected"], name)
        assert_same(g.topk_ptr(d.ptr, d.n, d.dtype, K, pipeline=True), f["expected"],
                    name + " (pipeline)")
    else:
        assert_same(g.multiselect_ptr(d.ptr, d.n, d.dtype, f["k"]), f["expected"], name)


@pytest.mark.parametrize("path", REF, ids=IDS)
def test_host_vector_matches_reference(g, path):
    f, vec = ri.load_case(path)
    name = os.path.basename(path)
    if str(f["kind"]) == "topk":
        assert_same(g.topk_host(vec, int(f["k"][0])), f["expected"], name)
    else:
        assert_same(g.multiselect_host(vec, f["k"]), f["expected"], name)


MULTI = [p for p in REF if str(np.load(p)["kind"]) == "multiselect"]


@pytest.mark.parametrize("path", MULTI, ids=[os.path.basename(p)[4:-4] for p in MULTI])
def test_single_k_select_matches_reference(g, path):
    f, vec = ri.load_case(path)
    d = DeviceArray(vec)
    for i in (0, len(f["k"]) // 2, len(f["k"]) - 1):
        got = np.array([g.select_ptr(d.ptr, d.n, d.dtype, int(f["k"][i]))], dtype=vec.dtype)
        assert_same(got, f["expected"][i:i + 1], f"{os.path.basename(path)} k[{i}]")


def test_reference_named_mirrors(g):
    """The mirrors of the reference's harness entries, on the plain
    configuration and one top-k input."""
    f, vec = ri.load_case(os.path.join(GOLDEN_DIR, "ref_p_f32_uniform_2p20_pgrid.npz"))
    r = g.timeBucketMultiselect(vec, f["k"])
    assert_same(r.vals, f["expected"], "timeBucketMultiselect")
    import torch
    out = np.empty(f["k"].size, dtype=np.float32)
    d = torch.from_numpy(vec).cuda()
    assert g.bucketMultiselectWrapper(d, d.numel(), f["k"], f["k"].size, out, 152, 1024) == 1
    assert_same(out, f["expected"], "bucketMultiselectWrapper")
    f, vec = ri.load_case(os.path.join(GOLDEN_DIR, "ref_t_f32_uniform_2p22_K1024.npz"))
    r = g.timeBucketTopkselect(vec, 1024)
    assert_same(r.vals, f["expected"], "timeBucketTopkselect")
