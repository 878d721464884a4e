"""Seeded host-side problem generators for GGKS multiselect / top-k.

These restate the distribution recipes of the reference's generators
(generateProblems.cu) with numpy's PCG64 in place of curand, so every input is
reproducible from (distribution, n, seed) on any machine.  The k-list
generators follow generateProblems.cu:489-584.

k convention everywhere: k-th LARGEST, 1-based (bucketMultiselect.cu:842-846).
"""
import numpy as np

# ---------------------------------------------------------------------------
# value distributions
# ---------------------------------------------------------------------------


def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def uniform_f32(n, seed):
    """generateUniformFloats (generateProblems.cu:62-68): uniform [0,1)."""
    return _rng(seed).random(n, dtype=np.float32)


def normal_f32(n, seed, sigma=1.0):
    """generateNormalFloats (:70-76) and generateNormalFloats100 (:301-307)."""
    x = _rng(seed).standard_normal(n, dtype=np.float32)
    if sigma != 1.0:
        x *= np.float32(sigma)
    return x


def half_normal_f32(n, seed):
    """generateHalfNormalFloats (:322-341): |N(0,1)|."""
    return np.abs(normal_f32(n, seed))


def cauchy_f32(n, seed):
    """generateCauchyFloats (:212-247): tan(pi (u - 1/2)) with u == 1 -> 0.9999
    and u == 0 -> 0.0001 (:218-221)."""
    u = uniform_f32(n, seed)
    u[u == np.float32(1.0)] = np.float32(0.9999)
    u[u == np.float32(0.0)] = np.float32(0.0001)
    return np.tan(np.float32(np.pi) * (u - np.float32(0.5))).astype(np.float32)


def huge_uniform_f32(n, seed):
    """generateHugeUniformFloats (:287-298): uniform [0,1) times 1e6."""
    return uniform_f32(n, seed) * np.float32(1000000)


def all_ones_f32(n, seed=0):
    """generateAllOnesFloats (:180-197)."""
    return np.ones(n, dtype=np.float32)


def ones_twos_f32(n, seed):
    """generateOnesTwosFloats (:154-177): (n*50)/100 twos, the rest ones,
    shuffled."""
    n2 = (n * 50) // 100
    x = np.ones(n, dtype=np.float32)
    x[:n2] = 2.0
    _rng(seed).shuffle(x)
    return x


def noisy_f32(n, seed):
    """generateNoisyVector (:249-277): N(0, 0.01) plus 1.0 on 20% of the
    entries."""
    r = _rng(seed)
    x = (r.standard_normal(n, dtype=np.float32) * np.float32(0.01)).astype(np.float32)
    ones = np.zeros(n, dtype=np.float32)
    ones[: (n * 20) // 100] = 1.0
    r.shuffle(ones)
    return (x + ones).astype(np.float32)


def killer_f32(n, seed):
    """generateBucketKillerFloats (:353-367): uniform bits masked with
    0x80EFFFFF, sorted, with 2^i (i = -126..126) written over the head."""
    b = _rng(seed).random(n, dtype=np.float32).view(np.uint32) & np.uint32(0x80EFFFFF)
    x = np.sort(b).view(np.float32).copy()
    m = min(n, 253)
    x[:m] = np.exp2(np.arange(-126, -126 + m, dtype=np.float64)).astype(np.float32)
    return x


def uint_valued_f32(n, seed):
    """Integer-valued floats in [0,256) (heavy duplicates)."""
    return _rng(seed).integers(0, 256, n, dtype=np.int32).astype(np.float32)


def uniform_f64(n, seed, lo=0.0, hi=1.0):
    """generateUniformDoubles (:385-391); lo/hi rescale it (the large f64
    workload is uniform [-1e6, 1e6))."""
    x = _rng(seed).random(n, dtype=np.float64)
    if lo != 0.0 or hi != 1.0:
        x = lo + (hi - lo) * x
    return x


def normal_f64(n, seed):
    """generateNormalDoubles (:393-399)."""
    return _rng(seed).standard_normal(n, dtype=np.float64)


def cauchy_f64(n, seed):
    u = _rng(seed).random(n, dtype=np.float64)
    u[u == 0.0] = 0.0001
    return np.tan(np.pi * (u - 0.5))


def killer_f64(n, seed):
    """generateBucketKillerDoubles (:409-423): masked with 0x800FFFFFFFFFFFFF,
    sorted, 2^i (i = -1022..1022) over the head."""
    b = _rng(seed).random(n, dtype=np.float64).view(np.uint64) & np.uint64(0x800FFFFFFFFFFFFF)
    x = np.sort(b).view(np.float64).copy()
    m = min(n, 2045)
    x[:m] = np.exp2(np.arange(-1022, -1022 + m, dtype=np.float64))
    return x


def uint_valued_f64(n, seed):
    return _rng(seed).integers(0, 256, n, dtype=np.int32).astype(np.float64)


def uniform_u32(n, seed, hi=1 << 32):
    """generateUniformUnsignedIntegers (:25-31); hi < 2^32 gives the
    heavy-duplicate top-k input (uniform over [0, 2^16))."""
    return _rng(seed).integers(0, hi, n, dtype=np.uint64).astype(np.uint32)


def sorted_u32(n, seed):
    """generateSortedArrayUints (:34-44)."""
    return np.sort(uniform_u32(n, seed))


def zero_to_four_u32(n, seed=0):
    """generateUniformZeroToFourUints (:46-51): i % 4."""
    return (np.arange(n, dtype=np.uint64) % 4).astype(np.uint32)


GENERATORS = {
    "f32": {
        "uniform": uniform_f32, "normal": normal_f32, "half_normal": half_normal_f32,
        "cauchy": cauchy_f32, "huge_uniform": huge_uniform_f32, "all_ones": all_ones_f32,
        "ones_twos": ones_twos_f32, "noisy": noisy_f32, "killer": killer_f32,
        "normal100": lambda n, s: normal_f32(n, s, 100.0), "uint_valued": uint_valued_f32,
    },
    "f64": {
        "uniform": uniform_f64, "normal": normal_f64, "killer": killer_f64,
        "cauchy": cauchy_f64, "uint_valued": uint_valued_f64,
        "uniform_pm1e6": lambda n, s: uniform_f64(n, s, -1e6, 1e6),
    },
    "u32": {
        "uniform": uniform_u32, "sorted": sorted_u32, "zero_to_four": zero_to_four_u32,
        "uniform16": lambda n, s: uniform_u32(n, s, 1 << 16),
    },
}

DTYPES = {"f32": np.float32, "f64": np.float64, "u32": np.uint32}


def generate(dtype, dist, n, seed):
    return np.ascontiguousarray(GENERATORS[dtype][dist](int(n), int(seed)))


# ---------------------------------------------------------------------------
# k lists (k-th largest, 1-based)
# ---------------------------------------------------------------------------


def k_pgrid(n, count=101):
    """k = floor(p (n-1)) + 1 for p = 0, 1/(count-1), ..., 1."""
    p = np.arange(count, dtype=np.float64) / (count - 1)
    return (np.floor(p * (n - 1)) + 1).astype(np.uint32)


def k_uniform(n, count):
    """generateKUniform (generateProblems.cu:506-513), float32 arithmetic as
    written there."""
    k = np.empty(count, dtype=np.uint32)
    i = np.arange(count, dtype=np.float32)
    k[:] = ((i / np.float32(count)) * np.float32(n)).astype(np.uint32)
    k[0] = 1
    k[count - 1] = n
    return k


def k_uniform_random(n, count, seed):
    """generateKUniformRandom (:489-504) with the k = 0 case mapped to 1."""
    u = _rng(seed).random(count, dtype=np.float64)
    return np.clip((u * n).astype(np.uint64) + 1, 1, n).astype(np.uint32)


def k_distinct(n, count, seed):
    """count distinct k's uniform over [1, n]."""
    count = min(count, n)
    r = _rng(seed)
    ks = set()
    while len(ks) < count:
        ks.update((r.integers(1, n + 1, count - len(ks))).tolist())
    out = np.array(sorted(ks), dtype=np.uint32)
    r.shuffle(out)
    return out


def k_normal(n, count, seed):
    """generateKNormal (:515-530): (|N| + 7) n / 14."""
    z = np.abs(_rng(seed).standard_normal(count))
    return np.clip(((z + 7) * (n / 14.0)).astype(np.uint64), 1, n).astype(np.uint32)


def k_cluster(n, count, seed):
    """generateKCluster (:533-557): clusters of 9 consecutive k's."""
    k = np.ones(count, dtype=np.uint32)
    u = _rng(seed).random(max(count // 9, 1))
    fi = 0
    for i in range(4, count, 9):
        c = int(u[fi] * (n - 10) + 5)
        fi += 1
        k[i] = c
        for j in range(1, 5):
            k[i - j] = c - j
            if i + j < count:
                k[i + j] = c + j
    return np.clip(k, 1, n).astype(np.uint32)


def k_sectioned(n, count, seed):
    """generateKSectioned (:559-576): count consecutive k's from a random
    start."""
    u = _rng(seed).random()
    start = max(1, int(u * (n - count)))
    return (start + np.arange(count, dtype=np.uint64)).clip(1, n).astype(np.uint32)


# ---------------------------------------------------------------------------
# the single-vector configurations, as seeded inputs (the benchmark times them;
# the full-size parity tests check the same inputs)
# ---------------------------------------------------------------------------
# plain: 2^20 float32 uniform [0, 1), seed 0, 101 k's on the p grid
P_LOG2N = 20
# large: 1001 distinct k's uniform in [1, n] (seed 100 + the input's seed)
L_NUM_K = 1001
L_INPUTS = (  # (name, dtype, distribution, log2 n, seed)
    ("f32_normal", "f32", "normal", 28, 1),
    ("f32_cauchy", "f32", "cauchy", 28, 2),
    ("f32_half_normal", "f32", "half_normal", 28, 3),
    ("u32_uniform", "u32", "uniform", 28, 4),
    ("f64_uniform_pm1e6", "f64", "uniform_pm1e6", 27, 5),
)
# top-k: 2^26 elements, K in T_KS; the ascending input is the sorted float32 one
T_LOG2N = 26
T_KS = (32, 1024, 65536)
T_INPUTS = ("f32_uniform", "u32_uniform16", "f32_sorted")


def config_p():
    """The plain configuration: (vector, k list)."""
    n = 1 << P_LOG2N
    return uniform_f32(n, 0), k_pgrid(n, 101)


def config_l(name, log2n=None):
    """One input of the large configuration: (vector, k list); log2n
    overrides the size (smaller runs of the same recipe)."""
    for nm, dt, dist, lg, seed in L_INPUTS:
        if nm == name:
            n = 1 << (lg if log2n is None else log2n)
            return generate(dt, dist, n, seed), k_distinct(n, L_NUM_K, 100 + seed)
    raise KeyError(name)


def config_t(name, log2n=T_LOG2N):
    """One input of the top-k configuration."""
    n = 1 << log2n
    if name == "f32_uniform":
        return uniform_f32(n, 0)
    if name == "u32_uniform16":
        return uniform_u32(n, 1, 1 << 16)
    if name == "f32_sorted":
        return np.sort(uniform_f32(n, 0))
    raise KeyError(name)


# ---------------------------------------------------------------------------
# batched workload: many independent vectors of uneven lengths
# ---------------------------------------------------------------------------
BATCH_DISTS = ("uniform", "normal", "cauchy", "uint_valued")


def batch_problems(count, seed, lo_log2=10.0, hi_log2=22.0, k_lo=1, k_hi=64):
    """The problem list of a batched multiselect: lengths log-uniform in
    [2^lo_log2, 2^hi_log2], each vector's distribution drawn uniformly from
    BATCH_DISTS (float32: uniform [0,1), normal(0,1), standard Cauchy,
    integer-valued floats in [0,256)), each with k_lo..k_hi k's drawn
    uniformly from [1, length].  Returns a list of dicts with keys dist, n,
    seed (the vector's data seed) and k (uint32 array)."""
    r = _rng(seed)
    lens = np.floor(2.0 ** r.uniform(lo_log2, hi_log2, count)).astype(np.int64)
    lens = np.clip(lens, 1, None)
    dists = r.integers(0, len(BATCH_DISTS), count)
    nks = r.integers(k_lo, k_hi + 1, count)
    out = []
    for i in range(count):
        n = int(lens[i])
        ks = r.integers(1, n + 1, int(nks[i]), dtype=np.int64).astype(np.uint32)
        out.append({"dist": BATCH_DISTS[int(dists[i])], "n": n, "seed": int(seed) * 100003 + i,
                    "k": ks})
    return out


def batch_vector(prob):
    """The float32 data of one batch problem (numpy, seeded)."""
    return generate("f32", prob["dist"], prob["n"], prob["seed"])


def batch_vectors_device(probs, seed, device):
    """float32 vectors of batch_problems() generated on a CUDA device with one
    seeded torch generator, in problem order (uniform [0,1) = rand, normal =
    randn, Cauchy = tan(pi (u - 1/2)), integer-valued = floor(256 u))."""
    import math

    import torch
    gen = torch.Generator(device=device)
    gen.manual_seed(int(seed))
    out = []
    for p in probs:
        n, d = p["n"], p["dist"]
        if d == "normal":
            v = torch.randn(n, device=device, generator=gen)
        else:
            u = torch.rand(n, device=device, generator=gen)
            if d == "uniform":
                v = u
            elif d == "cauchy":
                v = torch.tan(math.pi * (u - 0.5))
            else:
                v = torch.floor(u * 256.0)
        out.append(v.contiguous())
    return out


# ---------------------------------------------------------------------------
# served workload: a stream of mixed requests
# ---------------------------------------------------------------------------


def serving_pool(counts, seed, device, lo_log2=12.0, hi_log2=26.0):
    """Resident vectors of the served workload, generated on a CUDA device:
    counts = {"f32": a, "u32": b, "f64": c} vectors with lengths log-uniform in
    [2^lo_log2, 2^hi_log2]; float vectors draw from uniform / normal / Cauchy /
    integer-valued [0,256), uint32 vectors from uniform [0,2^32) / [0,2^16).
    Returns {dtype: [tensor, ...]} (uint32 data in int32 tensors)."""
    import math

    import torch
    r = _rng(seed)
    gen = torch.Generator(device=device)
    gen.manual_seed(int(seed))
    pool = {}
    for dt in ("f32", "u32", "f64"):
        pool[dt] = []
        for _ in range(counts.get(dt, 0)):
            n = int(2.0 ** r.uniform(lo_log2, hi_log2))
            if dt == "u32":
                hi = (1 << 32) if r.random() < 0.5 else (1 << 16)
                v = torch.randint(0, hi, (n,), device=device, generator=gen, dtype=torch.int64)
                v = (v - (v >= (1 << 31)).to(torch.int64) * (1 << 32)).to(torch.int32)  # bits
            else:
                fdt = torch.float32 if dt == "f32" else torch.float64
                d = BATCH_DISTS[int(r.integers(0, len(BATCH_DISTS)))]
                if d == "normal":
                    v = torch.randn(n, device=device, generator=gen, dtype=fdt)
                else:
                    u = torch.rand(n, device=device, generator=gen, dtype=fdt)
                    v = u if d == "uniform" else (torch.tan(math.pi * (u - 0.5)) if d == "cauchy"
                                                  else torch.floor(u * 256.0))
            pool[dt].append(v.contiguous())
    return pool


def serving_trace(pool_sizes, rate, count, seed):
    """A Poisson request stream: arrival times (s) at `rate` requests/s; each
    request picks float32 / uint32 / float64 in ratio 6:3:1, a vector of that
    type from the pool, and is a multiselect with 8-1024 k's (70%) or a top-k
    with K in [16, 4096] (30%, K <= n).  pool_sizes = {dtype: [n, ...]}."""
    r = _rng(seed)
    t = np.cumsum(r.exponential(1.0 / rate, count))
    t -= t[0]
    out = []
    for i in range(count):
        dt = ("f32",) * 6 + ("u32",) * 3 + ("f64",)
        dt = dt[int(r.integers(0, 10))]
        vi = int(r.integers(0, len(pool_sizes[dt])))
        n = pool_sizes[dt][vi]
        if r.random() < 0.7:
            ks = r.integers(1, n + 1, int(r.integers(8, 1025))).astype(np.uint32)
            out.append({"t": float(t[i]), "dtype": dt, "vec": vi, "k": ks, "K": None})
        else:
            out.append({"t": float(t[i]), "dtype": dt, "vec": vi, "k": None,
                        "K": int(min(n, r.integers(16, 4097)))})
    return out


# ---------------------------------------------------------------------------
# the reference's names, in its order (generateProblems.cu:53-55, :369-376,
# :425-428, :581-584): the comparison harness writes them into its CSV report
# ---------------------------------------------------------------------------
REFERENCE_DISTRIBUTIONS = {
    "f32": [("uniform", "UNIFORM FLOATS"), ("normal", "NORMAL FLOATS"),
            ("killer", "KILLER FLOATS"), ("half_normal", "HALF NORMAL FLOATS"),
            ("normal100", "NORMAL FLOATS 100"), ("huge_uniform", "HUGE UNIFORM FLOATS"),
            ("noisy", "NOISY FLOATS"), ("all_ones", "ALL ONES FLOATS"),
            ("ones_twos", "ONES TWOS FLOAT"), ("cauchy", "CAUCHY FLOAT")],
    "f64": [("uniform", "UNIFORM DOUBLES"), ("normal", "NORMAL DOUBLES"),
            ("killer", "KILLER DOUBLES")],
    "u32": [("uniform", "UNIFORM UNSIGNED INTEGERS"), ("sorted", "SORTED UINTS"),
            ("zero_to_four", "UNIFORM 0-4")],
}

REFERENCE_K_DISTRIBUTIONS = [
    ("Uniform Random Ks", lambda n, c, s: k_uniform_random(n, c, s)),
    ("Uniform Ks", lambda n, c, s: k_uniform(n, c)),
    ("Normal Random Ks", lambda n, c, s: k_normal(n, c, s)),
    ("Cluster Ks", lambda n, c, s: k_cluster(n, c, s)),
    ("Sectioned Ks", lambda n, c, s: k_sectioned(n, c, s)),
]
