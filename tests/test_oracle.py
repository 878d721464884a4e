"""CPU tests of the oracle: pinned against the golden fixtures (closed-form
known answers and numpy cross-checks), and the reference's bucket algorithm
(restated on the CPU) against sort-and-choose."""
import os

import numpy as np
import pytest

from conftest import bits, golden_files, load_golden

GOLDEN = golden_files()


def test_fixtures_present():
    names = [os.path.basename(p) for p in GOLDEN]
    assert sum(n.startswith("kat_") for n in names) >= 10
    assert sum(n.startswith("xcheck_") for n in names) >= 10


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_sort_and_choose_matches_golden(oracle_mod, path):
    g = load_golden(path)
    out = oracle_mod.multiselect(g["vec"], g["k"])
    assert np.array_equal(bits(out), bits(g["expected"]))
    out4 = oracle_mod.multiselect(g["vec"], g["k"], threads=4)
    assert np.array_equal(bits(out4), bits(g["expected"]))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_topk_matches_golden(oracle_mod, path):
    g = load_golden(path)
    out = oracle_mod.topk(g["vec"], int(g["topk_K"]), threads=3)
    assert np.array_equal(bits(out), bits(g["topk_expected"]))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_reference_bucket_algorithm_matches_golden(oracle_mod, path):
    g = load_golden(path)
    if "specials" in path:
        pytest.skip("the reference's projection arithmetic is undefined on NaN/inf")
    out = oracle_mod.bucket_multiselect(g["vec"], g["k"], seed=5)
    assert np.array_equal(bits(out), bits(g["expected"]))


def test_invalid_k_rejected(oracle_mod):
    v = np.arange(10, dtype=np.uint32)
    for bad in ([0], [11]):
        with pytest.raises(ValueError):
            oracle_mod.multiselect(v, np.array(bad, dtype=np.uint32))
    with pytest.raises(ValueError):
        oracle_mod.topk(v, 11)


@pytest.mark.parametrize("dtype", [np.uint32, np.uint64])
def test_parallel_radix_sort(oracle_mod, dtype):
    r = np.random.default_rng(0)
    x = r.integers(0, np.iinfo(dtype).max, 200003, dtype=dtype)
    x[::7] = x[3]
    for t in (1, 2, 7):
        assert np.array_equal(oracle_mod.sort_keys(x, threads=t), np.sort(x))
