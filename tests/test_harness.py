"""The comparison harness mirror (compareMultiselect.hpp:46-224) and its CSV
report (read back as readMultiselectOutputfile.cpp:91-140 does).  The CPU test
compares the oracle with a deliberately wrong algorithm; the GPU test runs the
reference's pairing, sort-and-choose against bucket multiselect, over every
reference distribution and k distribution."""
import pytest


def _sort_and_choose(orc):
    import time

    import ggks

    def fn(h_vec, k_vals):
        t0 = time.perf_counter()
        vals = orc.multiselect(h_vec, k_vals)
        return ggks.Results((time.perf_counter() - t0) * 1e3, vals)
    return fn


def test_report_format_and_error_count(oracle_mod, tmp_path):
    import ggks
    import ggks_harness as gh

    def wrong(h_vec, k_vals):
        vals = oracle_mod.multiselect(h_vec, k_vals).copy()
        vals[::7] += 1.0  # every 7th output wrong
        return ggks.Results(1.5, vals)

    csv = tmp_path / "report.csv"
    algs = [("Sort and Choose Multiselect", _sort_and_choose(oracle_mod)),
            ("Bucket Multiselect", wrong)]
    flags = gh.compare_multiselect(algs, 5000, 30, "f32", 1, 0, 2, str(csv), seed=3)
    assert all(f > 0 for f in flags)
    recs = gh.read_multiselect_report(str(csv))
    assert len(recs) == 2
    for r, f in zip(recs, flags):
        assert r["size"] == 5000 and r["k"] == 30
        assert r["arrayDistribution"] == "NORMAL FLOATS"
        assert r["kDistribution"] == "Uniform Random Ks"
        assert r["names"] == ["Sort and Choose Multiselect", "Bucket Multiselect"]
        assert r["errorFlag"] == f
        assert r["ratios"][0] == 1.0
    text = csv.read_text()
    assert "ERROR ON TEST 0 of 2 tests!!!!!" in text and "wrong k = " in text


@pytest.mark.gpu
def test_reference_pairing_over_every_distribution(oracle_mod, tmp_path):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ggks
    import ggks_harness as gh
    import ggks_problems as gp
    csv = tmp_path / "report.csv"
    algs = [("Sort and Choose Multiselect", _sort_and_choose(oracle_mod)),
            ("Bucket Multiselect", ggks.timeBucketMultiselect)]
    total = 0
    for dtype, dists in gp.REFERENCE_DISTRIBUTIONS.items():
        for g in range(len(dists)):
            for kg in range(len(gp.REFERENCE_K_DISTRIBUTIONS)):
                total += 1
                flags = gh.compare_multiselect(algs, 1 << 16, 101, dtype, g, kg, 1, str(csv),
                                               seed=g * 10 + kg)
                assert flags == [0], (dtype, dists[g], kg)
    recs = gh.read_multiselect_report(str(csv))
    assert len(recs) == total
    assert all(r["errorFlag"] == 0 for r in recs)
