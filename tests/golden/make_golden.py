"""Generate the golden fixtures in tests/golden/*.npz.

Run:  python tests/golden/make_golden.py

Two kinds of fixture:

* ``kat_*`` -- known-answer vectors whose expected outputs are written down in
  closed form, with no sort involved, from the reference's deterministic
  generators: generateUniformZeroToFourUints (generateProblems.cu:46-51),
  generateOnesTwosFloats (:154-177), generateAllOnesFloats (:180-197), the
  power-of-two head of generateBucketKillerFloats / Doubles (:363-365,
  :419-421), a sorted uint vector (:34-44, identity in place of the curand
  draw), and k lists from generateKUniform (:506-513) and generateKSectioned
  (:559-576).  A hand-ordered set of IEEE special values (signed zeros,
  subnormals, infinities, NaNs) pins the key order policy.
* ``xcheck_*`` -- seeded random inputs whose expected outputs come from
  numpy's sort of the order-preserving keys, an implementation independent of
  the oracle and of the CUDA path.

Each file holds: vec, k (k-th largest, 1-based), expected (out[i] =
ascending[n - k[i]]), topk_K and topk_expected (the K largest, descending).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "ggks-multiselect_gb300"))
import ggks_problems as gp  # noqa: E402


def keys_of(vec):
    if vec.dtype == np.float32:
        b = vec.view(np.uint32)
        return np.where(b & np.uint32(0x80000000), ~b, b | np.uint32(0x80000000))
    if vec.dtype == np.float64:
        b = vec.view(np.uint64)
        return np.where(b & np.uint64(1 << 63), ~b, b | np.uint64(1 << 63))
    return vec.copy()


def numpy_expected(vec, k, K):
    order = np.argsort(keys_of(vec), kind="stable")
    asc = vec[order]
    n = vec.size
    exp = asc[n - k.astype(np.int64)]
    topk = asc[::-1][:K].copy()
    return exp, topk


def save(name, vec, k, expected, K, topk_expected, source):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, vec=vec, k=k.astype(np.uint32), expected=expected,
                        topk_K=np.uint32(K), topk_expected=topk_expected,
                        source=np.array(source))
    return path


def kat_zero_to_four(n):
    vec = gp.zero_to_four_u32(n)
    counts = [n // 4 + (1 if v < n % 4 else 0) for v in range(4)]

    def kth_largest(k):
        acc = 0
        for v in (3, 2, 1, 0):
            acc += counts[v]
            if k <= acc:
                return v
        raise AssertionError

    ks = np.concatenate([gp.k_uniform(n, min(n, 101)),
                         (n // 3 + np.arange(min(n, 50))).astype(np.uint32)])
    ks = np.clip(ks, 1, n).astype(np.uint32)
    exp = np.array([kth_largest(int(k)) for k in ks], dtype=np.uint32)
    K = min(n, 1024)
    topk = np.array([kth_largest(k) for k in range(1, K + 1)], dtype=np.uint32)
    save(f"kat_zero_to_four_u32_n{n}", vec, ks, exp, K, topk,
         "generateUniformZeroToFourUints (generateProblems.cu:46-51) x "
         "generateKUniform (:506-513) + a sectioned k run; closed form")


def kat_ones_twos(n):
    vec = gp.ones_twos_f32(n, 7)
    n2 = (n * 50) // 100
    ks = gp.k_uniform(n, min(n, 101))
    exp = np.where(ks <= n2, np.float32(2.0), np.float32(1.0)).astype(np.float32)
    K = min(n, 2048)
    kk = np.arange(1, K + 1)
    topk = np.where(kk <= n2, np.float32(2.0), np.float32(1.0)).astype(np.float32)
    save(f"kat_ones_twos_f32_n{n}", vec, ks, exp, K, topk,
         "generateOnesTwosFloats (generateProblems.cu:154-177) x generateKUniform; "
         "closed form")


def kat_all_ones(n):
    vec = gp.all_ones_f32(n)
    ks = gp.k_uniform(n, 64)
    exp = np.ones(ks.size, dtype=np.float32)
    K = min(n, 100)
    save(f"kat_all_ones_f32_n{n}", vec, ks, exp, K, np.ones(K, dtype=np.float32),
         "generateAllOnesFloats (generateProblems.cu:180-197); closed form")


def kat_killer_head_f32(reverse):
    e = np.arange(-126, 127)
    vec = np.exp2(e.astype(np.float64)).astype(np.float32)
    if reverse:
        vec = vec[::-1].copy()
    n = vec.size
    ks = np.arange(1, n + 1, dtype=np.uint32)
    exp = np.exp2((126 - (ks.astype(np.int64) - 1)).astype(np.float64)).astype(np.float32)
    K = n
    save(f"kat_killer_head_f32_{'rev' if reverse else 'asc'}", vec, ks, exp, K, exp.copy(),
         "power-of-two head of generateBucketKillerFloats (generateProblems.cu:363-365); "
         "closed form")


def kat_killer_head_f64():
    e = np.arange(-1022, 1023)
    vec = np.exp2(e.astype(np.float64))
    gp._rng(3).shuffle(vec)
    n = vec.size
    ks = np.arange(1, n + 1, dtype=np.uint32)
    exp = np.exp2((1022 - (ks.astype(np.int64) - 1)).astype(np.float64))
    K = 300
    save("kat_killer_head_f64_shuffled", vec, ks, exp, K, exp[:K].copy(),
         "power-of-two head of generateBucketKillerDoubles (generateProblems.cu:419-421), "
         "shuffled; closed form")


def kat_sorted_identity(n):
    vec = np.arange(n, dtype=np.uint32)
    ks = np.concatenate([gp.k_uniform(n, 101), np.array([1, 2, n - 1, n], dtype=np.uint32)])
    exp = (n - ks.astype(np.int64)).astype(np.uint32)
    K = 777
    topk = (n - 1 - np.arange(K)).astype(np.uint32)
    save(f"kat_sorted_identity_u32_n{n}", vec, ks, exp, K, topk,
         "sorted uints (generateProblems.cu:34-44) with the identity in place of the "
         "curand draw; closed form")


def kat_specials(dtype):
    """IEEE special values listed in ascending key order."""
    if dtype == np.float32:
        bits = np.array([
            0xFFC00001,  # negative NaN, large payload: lowest key
            0xFFC00000,  # negative quiet NaN
            0xFF800000,  # -inf
            0xFF7FFFFF,  # -max
            0xBF800000,  # -1
            0x80800000,  # -min normal
            0x80000001,  # -min subnormal
            0x80000000,  # -0
            0x00000000,  # +0
            0x00000001,  # +min subnormal
            0x00800000,  # +min normal
            0x3F800000,  # 1
            0x7F7FFFFF,  # +max
            0x7F800000,  # +inf
            0x7FC00000,  # +quiet NaN
            0x7FC00001,  # +NaN, larger payload: highest key
        ], dtype=np.uint32)
        asc = bits.view(np.float32)
    else:
        bits = np.array([
            0xFFF8000000000001, 0xFFF8000000000000, 0xFFF0000000000000,
            0xFFEFFFFFFFFFFFFF, 0xBFF0000000000000, 0x8010000000000000,
            0x8000000000000001, 0x8000000000000000, 0x0000000000000000,
            0x0000000000000001, 0x0010000000000000, 0x3FF0000000000000,
            0x7FEFFFFFFFFFFFFF, 0x7FF0000000000000, 0x7FF8000000000000,
            0x7FF8000000000001,
        ], dtype=np.uint64)
        asc = bits.view(np.float64)
    # three copies of every value, shuffled
    vec = np.concatenate([asc, asc, asc])
    perm = gp._rng(11).permutation(vec.size)
    vec = vec[perm].copy()
    n = vec.size
    asc_full = np.repeat(asc, 3)
    ks = np.arange(1, n + 1, dtype=np.uint32)
    exp = asc_full[n - ks.astype(np.int64)].copy()
    K = n
    topk = asc_full[::-1].copy()
    tag = "f32" if dtype == np.float32 else "f64"
    save(f"kat_specials_{tag}", vec, ks, exp, K, topk,
         "IEEE specials in key order (keyConversion.cu:9-23): NaN(-) < -inf < ... < -0 < "
         "+0 < ... < +inf < NaN(+); closed form")


def xcheck(dtype, dist, n, seed):
    vec = gp.generate(dtype, dist, n, seed)
    if n <= 300:
        ks = np.arange(1, n + 1, dtype=np.uint32)
    else:
        ks = np.concatenate([gp.k_pgrid(n, 101), gp.k_cluster(n, 27, seed + 1)])
    K = min(n, 512)
    exp, topk = numpy_expected(vec, ks, K)
    save(f"xcheck_{dtype}_{dist}_n{n}_s{seed}", vec, ks, exp, K, topk,
         f"seeded {dist} ({dtype}), expected from numpy's sort of the keys")


def main():
    for n in (1, 3, 1000, 4096, 65537):
        kat_zero_to_four(n)
    for n in (2, 1001, 65536):
        kat_ones_twos(n)
    kat_all_ones(5000)
    kat_killer_head_f32(False)
    kat_killer_head_f32(True)
    kat_killer_head_f64()
    kat_sorted_identity(4099)
    kat_specials(np.float32)
    kat_specials(np.float64)
    cases = [
        ("f32", "uniform", 1, 0), ("f32", "uniform", 2, 1), ("f32", "uniform", 17, 2),
        ("f32", "uniform", 4096, 0), ("f32", "normal", 10007, 1),
        ("f32", "half_normal", 3001, 3), ("f32", "cauchy", 20000, 2),
        ("f32", "killer", 8192, 4), ("f32", "noisy", 5000, 5),
        ("f32", "uint_valued", 30000, 6), ("f32", "normal100", 999, 7),
        ("f64", "uniform_pm1e6", 12345, 8), ("f64", "normal", 4000, 9),
        ("f64", "killer", 6000, 10), ("f64", "uint_valued", 9000, 11),
        ("u32", "uniform", 16384, 12), ("u32", "uniform16", 20000, 13),
        ("u32", "sorted", 7777, 14),
    ]
    for c in cases:
        xcheck(*c)
    names = sorted(f for f in os.listdir(HERE) if f.endswith(".npz"))
    print(f"{len(names)} fixtures written to {HERE}")


if __name__ == "__main__":
    main()
