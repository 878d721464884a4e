"""CPU tests: the oracle pinned by outputs of the reference itself.

tests/golden/ref_*.npz hold what the reference's own code returned
(bucketMultiselectWrapper through timeBucketMultiselect / timeBucketTopkselect,
multiselectTimingFunctions.cu:100-122, :205-231, checked there against the
reference's sort-and-choose, :51-95, :156-177) on inputs regenerated here from
their recipes.  Both oracle restatements -- sort-and-choose and the
reference's bucket algorithm -- must reproduce every output bit for bit.
Where the reference sources are present, the host build of the reference is
also re-run on the small cases, so a fixture that went stale is caught."""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN_DIR, bits, ref_files

sys.path.insert(0, GOLDEN_DIR)
import ref_inputs as ri  # noqa: E402

REF = ref_files()
IDS = [os.path.basename(p)[4:-4] for p in REF]


def test_reference_fixtures_present():
    names = [os.path.basename(p) for p in REF]
    assert len(names) >= 25
    assert any(n.startswith("ref_p_") for n in names)
    assert sum(n.startswith("ref_l_") for n in names) >= 5
    assert sum(n.startswith("ref_t_") for n in names) >= 5


@pytest.mark.parametrize("path", REF, ids=IDS)
def test_inputs_regenerate_bit_identically(path):
    ri.load_case(path)  # raises on a digest mismatch


@pytest.mark.parametrize("path", REF, ids=IDS)
def test_sort_and_choose_matches_reference(oracle_mod, path):
    g, vec = ri.load_case(path)
    if str(g["kind"]) == "topk":
        out = oracle_mod.topk(vec, int(g["k"][0]), threads=4)
    else:
        out = oracle_mod.multiselect(vec, g["k"], threads=4)
    assert np.array_equal(bits(out), bits(g["expected"]))


@pytest.mark.parametrize("path", REF, ids=IDS)
def test_restated_bucket_algorithm_matches_reference(oracle_mod, path):
    g, vec = ri.load_case(path)
    if str(g["kind"]) == "topk":
        k = np.arange(1, int(g["k"][0]) + 1, dtype=np.uint32)
    else:
        k = g["k"]
    out = oracle_mod.bucket_multiselect(vec, k, seed=3)
    assert np.array_equal(bits(out), bits(g["expected"]))


def test_numpy_float32_draws_restated():
    """The plain configuration's input recipe restates numpy's float32 draws."""
    import ggks_problems as gp
    for n in (1, 2, 7, 4096):
        assert np.array_equal(bits(ri.numpy_random_f32(n, 0)), bits(gp.uniform_f32(n, 0)))


@pytest.fixture(scope="module")
def reference_lib():
    import build_ref
    try:
        path = build_ref.build()
    except RuntimeError as e:  # a toolchain problem, not a parity result
        pytest.skip(f"host build of the reference failed: {e}")
    if path is None:
        pytest.skip("reference sources not present")
    sys.path.insert(0, GOLDEN_DIR)
    import make_ref_golden
    return make_ref_golden.Reference(path)


SMALL = [p for p in REF if int(np.load(p)["n"]) <= (1 << 18)]


@pytest.mark.parametrize("path", SMALL, ids=[os.path.basename(p)[4:-4] for p in SMALL])
def test_reference_rerun_matches_fixture(reference_lib, path):
    g, vec = ri.load_case(path)
    if str(g["kind"]) == "topk":
        out = reference_lib.topk("bucket", vec, int(g["k"][0]))
    else:
        out = reference_lib.multiselect("bucket", vec, np.ascontiguousarray(g["k"]))
    assert np.array_equal(bits(out), bits(g["expected"]))
