"""Mirror of the reference's comparison harness for this path and of its CSV
report, so that reports written here feed the reference's summarizers.

* ``compare_multiselect`` follows compareMultiselectAlgorithms
  (compareMultiselect.hpp:46-224): per test it generates a vector and a k list
  with the named distributions, runs every timing function in a shuffled order
  on a fresh copy, takes algorithm 0's results as the correct ones, counts the
  outputs of the other algorithms that differ, and appends one line to the CSV
  report:

      size,numKs,<vector distribution>,<k distribution>,<name>,<time ms>,...,<error count>

  with an error paragraph before the count for every wrong output (as at
  compareMultiselect.hpp:168-177).
* ``read_multiselect_report`` parses those lines like readLine in
  readMultiselectOutputfile.cpp:91-140 (size, k count, distributions, name /
  time pairs, time ratios to algorithm 0, error flag).

Timing functions are ``fn(h_vec, kVals) -> Results`` (``ggks.Results``: time
in ms and values in k order), e.g. ``ggks.timeBucketMultiselect``; the caller
chooses algorithm 0, the reference's sort-and-choose in its harness.
"""
import numpy as np

import ggks_problems as gp


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint8).reshape(a.size, -1)


def compare_multiselect(timing_functions, size, num_ks, dtype, generate_type, k_generate_type,
                        num_tests, csv_path, seed=0):
    """Run num_tests tests of `size` elements and num_ks k's; timing_functions
    is a list of (name, fn).  Returns the per-test error counts."""
    dist, dist_name = gp.REFERENCE_DISTRIBUTIONS[dtype][generate_type]
    k_name, k_gen = gp.REFERENCE_K_DISTRIBUTIONS[k_generate_type]
    rng = np.random.default_rng(seed)
    flags = []
    with open(csv_path, "a") as f:
        for i in range(num_tests):
            test_seed = int(rng.integers(0, 2**31))
            h_vec = gp.generate(dtype, dist, size, test_seed)
            k_vals = np.clip(np.asarray(k_gen(size, num_ks, test_seed), dtype=np.int64), 1,
                             size).astype(np.uint32)
            f.write(f"{size},{num_ks},{dist_name},{k_name},")
            results = [None] * len(timing_functions)
            for j in rng.permutation(len(timing_functions)):
                results[j] = timing_functions[j][1](h_vec.copy(), k_vals)
            for j, (name, _) in enumerate(timing_functions):
                f.write(f"{name},{results[j].time},")
            flag = 0
            ref = _bits(results[0].vals)
            for m in range(1, len(timing_functions)):
                got = _bits(results[m].vals)
                for j in np.nonzero((got != ref).any(axis=1))[0]:
                    flag += 1
                    f.write(f"\nERROR ON TEST {i} of {num_tests} tests!!!!!\n")
                    f.write(f"vector size = {size}\nvector seed = {test_seed}\n")
                    f.write(f"numKs = {num_ks}\n")
                    f.write(f"wrong k = {k_vals[j]} kIndex = {j} wrong result = "
                            f"{results[m].vals[j]} correct result = {results[0].vals[j]}\n")
            f.write(f"{flag}\n")
            flags.append(flag)
    return flags


def read_multiselect_report(csv_path, num_algorithms=2):
    """Result lines of a report: dicts with size, k, arrayDistribution,
    kDistribution, names, times, ratios (time / algorithm 0's time) and
    errorFlag.  Error paragraphs are skipped; the count that follows one
    becomes its test's errorFlag."""
    out = []
    with open(csv_path) as f:
        for line in f:
            parts = line.rstrip("\n").split(",")
            if len(parts) == 1 and parts[0].isdigit() and out and out[-1]["errorFlag"] is None:
                out[-1]["errorFlag"] = int(parts[0])
                continue
            if len(parts) < 5 + 2 * num_algorithms or not parts[0].isdigit():
                continue
            rec = {"size": int(parts[0]), "k": int(parts[1]), "arrayDistribution": parts[2],
                   "kDistribution": parts[3], "names": [], "times": []}
            p = 4
            for _ in range(num_algorithms):
                rec["names"].append(parts[p])
                rec["times"].append(float(parts[p + 1]))
                p += 2
            rec["ratios"] = [t / rec["times"][0] if rec["times"][0] else float("inf")
                             for t in rec["times"]]
            rec["errorFlag"] = int(parts[p]) if p < len(parts) and parts[p] else None
            out.append(rec)
    return out
