"""Generate tests/golden/ref_*.npz: outputs of the reference itself.

Run (in a tree that has the reference sources; see oracle/build_ref.py):
    python tests/golden/make_ref_golden.py

The reference's own bucket multiselect path (bucketMultiselect.cu:521-871
through timeBucketMultiselect / timeBucketTopkselect,
multiselectTimingFunctions.cu:100-122, :205-231) and its own oracle
(timeSortAndChooseMultiselect / -Topkselect, :51-95, :156-177) are compiled
for the host CPU by oracle/build_ref.py and run here on each case's input.
The two must agree (the script stops otherwise); their common answer is the
fixture's expected output.  Each file holds:
  kind       "multiselect" or "topk"
  recipe, n, seed, sha256   the input (tests/golden/ref_inputs.py) and its digest
  k          k-th largest, 1-based (multiselect), or K (top-k)
  expected   the reference's outputs: out[i] = the k[i]-th largest (multiselect),
             the K largest in descending order (top-k)
Inputs avoid NaN and signed zeros, where the reference's native `<` order is
not total.  k lists avoid the reference's known faults: none is made only of
k = 1 and k = n (bucketMultiselect.cu:714-730 then reads uninitialised data),
and every list is short enough for copyValuesInChunk's one pass over
blocks x 1024 threads (:321-324) on the emulated 152-SM device.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import ref_inputs as ri  # noqa: E402
import build_ref  # noqa: E402

SUFFIX = {np.dtype(np.float32): "f32", np.dtype(np.float64): "f64", np.dtype(np.uint32): "u32"}


def k_distinct(n, count, seed):
    r = np.random.PCG64(seed).random_raw(4 * count)
    ks = []
    seen = set()
    for w in r:
        v = int(w % np.uint64(n)) + 1
        if v not in seen:
            seen.add(v)
            ks.append(v)
            if len(ks) == min(count, n):
                break
    return np.array(ks, dtype=np.uint32)


def k_pgrid(n, count=101):
    p = np.arange(count, dtype=np.float64) / (count - 1)
    return (np.floor(p * (n - 1)) + 1).astype(np.uint32)


def k_cluster(n, count, seed):
    c = int(np.random.PCG64(seed).random_raw(1)[0] % np.uint64(n - 2 * count)) + count
    return (c + np.arange(-count // 2, count - count // 2)).astype(np.uint32)


def k_edges(n, seed):
    """k = 1 and k = n among others, duplicates and an unsorted order."""
    mid = k_distinct(n, 40, seed)
    k = np.concatenate([[1, n, 2, n - 1], mid, [1, n, int(mid[0])]]).astype(np.uint32)
    r = np.random.Generator(np.random.PCG64(seed + 1))
    r.shuffle(k)
    return k


# (name, recipe, n, seed, k-list builder or ("topk", K))
CASES = [
    # the plain configuration exactly: 2^20 float32 uniform [0,1) seed 0, 101 k's on the p grid
    ("p_f32_uniform_2p20_pgrid", "numpy_random_f32", 1 << 20, 0, lambda n: k_pgrid(n, 101)),
    # the large configuration's shapes at 2^22 (2^21 for float64), 1001 distinct k's
    ("l_f32_bell_2p22_1001k", "bell_f32", 1 << 22, 1, lambda n: k_distinct(n, 1001, 101)),
    ("l_f32_heavy_tail_2p22_1001k", "heavy_tail_f32", 1 << 22, 2, lambda n: k_distinct(n, 1001, 102)),
    ("l_f32_half_bell_2p22_1001k", "half_bell_f32", 1 << 22, 3, lambda n: k_distinct(n, 1001, 103)),
    ("l_u32_uniform_2p22_1001k", "uniform_u32", 1 << 22, 4, lambda n: k_distinct(n, 1001, 104)),
    ("l_f64_pm1e6_2p21_1001k", "pm1e6_f64", 1 << 21, 5, lambda n: k_distinct(n, 1001, 105)),
    # duplicates, order, edges and small sizes
    ("f32_int_valued_2p20_1001k", "int_valued_f32", 1 << 20, 6, lambda n: k_distinct(n, 1001, 106)),
    ("u32_u16_valued_2p20_501k", "u16_valued_u32", 1 << 20, 7, lambda n: k_distinct(n, 501, 107)),
    ("u32_few_valued_2p18_64k", "few_valued_u32", 1 << 18, 8, lambda n: k_distinct(n, 64, 108)),
    ("f32_ones_twos_2p18_1001k", "ones_twos_f32", 1 << 18, 9, lambda n: k_distinct(n, 1001, 109)),
    ("f32_all_equal_10000_33k", "all_equal_f32", 10000, 0, lambda n: k_distinct(n, 33, 110)),
    ("f32_sorted_2p20_101k", "sorted_f32", 1 << 20, 11, lambda n: k_pgrid(n, 101)),
    ("u32_sorted_65537_257k", "sorted_u32", 65537, 12, lambda n: k_distinct(n, 257, 112)),
    ("f32_uniform_1000_edges", "uniform_f32", 1000, 13, lambda n: k_edges(n, 113)),
    ("f32_bell_4097_every_k", "bell_f32", 4097, 14, lambda n: np.arange(1, n + 1, dtype=np.uint32)),
    ("f64_bell_65537_cluster", "bell_f64", 65537, 15, lambda n: k_cluster(n, 257, 115)),
    ("f32_heavy_tail_2p20_edges", "heavy_tail_f32", 1 << 20, 16, lambda n: k_edges(n, 116)),
    ("u32_uniform_300001_cluster", "uniform_u32", 300001, 17, lambda n: k_cluster(n, 1024, 117)),
    # top-k: the top-k configuration's inputs at 2^22
    ("t_f32_uniform_2p22_K32", "uniform_f32", 1 << 22, 20, ("topk", 32)),
    ("t_f32_uniform_2p22_K1024", "uniform_f32", 1 << 22, 20, ("topk", 1024)),
    ("t_f32_uniform_2p22_K65536", "uniform_f32", 1 << 22, 20, ("topk", 65536)),
    ("t_u32_u16_valued_2p22_K32", "u16_valued_u32", 1 << 22, 21, ("topk", 32)),
    ("t_u32_u16_valued_2p22_K1024", "u16_valued_u32", 1 << 22, 21, ("topk", 1024)),
    ("t_f32_sorted_2p22_K32", "sorted_f32", 1 << 22, 22, ("topk", 32)),
    ("t_f32_sorted_2p22_K4096", "sorted_f32", 1 << 22, 22, ("topk", 4096)),
    ("t_f64_bell_2p20_K1024", "bell_f64", 1 << 20, 23, ("topk", 1024)),
    ("t_f32_bell_100000_K777", "bell_f32", 100000, 24, ("topk", 777)),
]


class Reference:
    def __init__(self, path):
        self.L = ctypes.CDLL(str(path))
        P = ctypes.c_void_p
        for sfx in SUFFIX.values():
            for name in ("bucket_multiselect", "sort_choose_multiselect"):
                f = getattr(self.L, f"ggks_ref_{name}_{sfx}")
                f.argtypes = [P, ctypes.c_uint, P, ctypes.c_uint, P]
                f.restype = ctypes.c_float
            for name in ("bucket_topk", "sort_choose_topk"):
                f = getattr(self.L, f"ggks_ref_{name}_{sfx}")
                f.argtypes = [P, ctypes.c_uint, ctypes.c_uint, P]
                f.restype = ctypes.c_float

    def multiselect(self, which, vec, k):
        out = np.empty(k.size, dtype=vec.dtype)
        f = getattr(self.L, f"ggks_ref_{which}_multiselect_{SUFFIX[vec.dtype]}")
        if f(vec.ctypes.data, vec.size, k.ctypes.data, k.size, out.ctypes.data) < 0:
            raise RuntimeError("reference call failed")
        return out

    def topk(self, which, vec, K):
        out = np.empty(K, dtype=vec.dtype)
        f = getattr(self.L, f"ggks_ref_{which}_topk_{SUFFIX[vec.dtype]}")
        if f(vec.ctypes.data, vec.size, K, out.ctypes.data) < 0:
            raise RuntimeError("reference call failed")
        return out


def bits(a):
    return a.view(np.uint64 if a.dtype.itemsize == 8 else np.uint32)


def main():
    os.environ.setdefault("GGKS_EMU_SMS", "152")
    lib = build_ref.build()
    if lib is None:
        sys.exit("the reference sources are not present: nothing generated")
    ref = Reference(lib)
    for name, recipe, n, seed, kspec in CASES:
        vec = ri.make(recipe, n, seed)
        if isinstance(kspec, tuple):
            K = kspec[1]
            a = ref.topk("bucket", vec, K)
            b = ref.topk("sort_choose", vec, K)
            k = np.array([K], dtype=np.uint32)
            kind = "topk"
        else:
            k = np.ascontiguousarray(kspec(n), dtype=np.uint32)
            a = ref.multiselect("bucket", vec, k)
            b = ref.multiselect("sort_choose", vec, k)
            kind = "multiselect"
        if not np.array_equal(bits(a), bits(b)):
            bad = int(np.count_nonzero(bits(a) != bits(b)))
            sys.exit(f"{name}: the reference's bucket path and its sort-and-choose "
                     f"disagree on {bad} outputs")
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), kind=kind, recipe=recipe,
                            n=np.int64(n), seed=np.int64(seed), sha256=ri.digest(vec),
                            k=k, expected=a)
        print(f"ref_{name}.npz: {kind}, n={n}, {k.size if kind == 'multiselect' else K} "
              f"{'k' if kind == 'multiselect' else 'K'}; bucket path == sort-and-choose")


if __name__ == "__main__":
    main()
