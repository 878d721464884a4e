"""Input recipes of the reference-output fixtures (tests/golden/ref_*.npz).

Every recipe is built from raw PCG64 words (np.random.PCG64(seed).random_raw,
an integer stream fixed by the algorithm) and IEEE operations that round
exactly (+, -, *, /, abs, float64 -> float32 casts), so the same (recipe, n,
seed) gives the same bits on any machine and any numpy: the fixtures store
the recipe and a SHA-256 of the input, never the input.

The distributions stand in for the benchmark's shapes: a bell curve (sum of
four uniforms, scaled to unit variance) for normal(0,1), its absolute value for
the half-normal, a ratio of two uniforms for Cauchy's heavy tails.
"""
import hashlib

import numpy as np

_TWO_M24 = 1.0 / (1 << 24)
_TWO_M53 = 1.0 / (1 << 53)


def _raw(n, seed):
    return np.random.PCG64(int(seed)).random_raw(int(n))


def _u53(n, seed):
    """Uniform [0, 1) doubles with 53 random bits."""
    return (_raw(n, seed) >> np.uint64(11)).astype(np.float64) * _TWO_M53


def numpy_random_f32(n, seed):
    """np.random.Generator(PCG64(seed)).random(n, dtype=float32), restated from
    the raw words: numpy draws 32-bit words low half first, then high half,
    and maps w to (w >> 8) * 2^-24."""
    raw = _raw((n + 1) // 2, seed)
    w = np.empty(2 * raw.size, dtype=np.uint32)
    w[0::2] = (raw & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    w[1::2] = (raw >> np.uint64(32)).astype(np.uint32)
    return ((w[:n] >> np.uint32(8)).astype(np.float32) * np.float32(_TWO_M24)).astype(np.float32)


def uniform_f32(n, seed):
    return ((_raw(n, seed) >> np.uint64(40)).astype(np.float64) * _TWO_M24).astype(np.float32)


def bell_f32(n, seed):
    s = _u53(n, seed) + _u53(n, seed + 1000) + _u53(n, seed + 2000) + _u53(n, seed + 3000)
    return ((s - 2.0) * 1.7320508075688772).astype(np.float32)


def half_bell_f32(n, seed):
    return np.abs(bell_f32(n, seed))


def heavy_tail_f32(n, seed):
    a = _u53(n, seed) * 2.0 - 1.0
    b = _u53(n, seed + 1000) * 2.0 - 1.0 + _TWO_M53
    return (a / b).astype(np.float32)


def int_valued_f32(n, seed):
    return (_raw(n, seed) >> np.uint64(56)).astype(np.float32)


def sorted_f32(n, seed):
    return np.sort(uniform_f32(n, seed))


def ones_twos_f32(n, seed):
    return ((_raw(n, seed) >> np.uint64(63)) + np.uint64(1)).astype(np.float32)


def all_equal_f32(n, seed):
    return np.full(n, 0.75, dtype=np.float32)


def uniform_u32(n, seed):
    return (_raw(n, seed) & np.uint64(0xFFFFFFFF)).astype(np.uint32)


def u16_valued_u32(n, seed):
    return (_raw(n, seed) >> np.uint64(48)).astype(np.uint32)


def few_valued_u32(n, seed):
    return (_raw(n, seed) >> np.uint64(60)).astype(np.uint32)


def sorted_u32(n, seed):
    return np.sort(uniform_u32(n, seed))


def pm1e6_f64(n, seed):
    return _u53(n, seed) * 2e6 - 1e6


def bell_f64(n, seed):
    s = _u53(n, seed) + _u53(n, seed + 1000) + _u53(n, seed + 2000) + _u53(n, seed + 3000)
    return (s - 2.0) * 1.7320508075688772


RECIPES = {
    "numpy_random_f32": numpy_random_f32,
    "uniform_f32": uniform_f32,
    "bell_f32": bell_f32,
    "half_bell_f32": half_bell_f32,
    "heavy_tail_f32": heavy_tail_f32,
    "int_valued_f32": int_valued_f32,
    "sorted_f32": sorted_f32,
    "ones_twos_f32": ones_twos_f32,
    "all_equal_f32": all_equal_f32,
    "uniform_u32": uniform_u32,
    "u16_valued_u32": u16_valued_u32,
    "few_valued_u32": few_valued_u32,
    "sorted_u32": sorted_u32,
    "pm1e6_f64": pm1e6_f64,
    "bell_f64": bell_f64,
}


def make(recipe, n, seed):
    return np.ascontiguousarray(RECIPES[str(recipe)](int(n), int(seed)))


def digest(vec):
    return hashlib.sha256(np.ascontiguousarray(vec).tobytes()).hexdigest()


def load_case(path):
    """(fixture dict, regenerated input); raises if the input's digest does not
    match the one the fixture was made from."""
    g = dict(np.load(path, allow_pickle=False))
    vec = make(str(g["recipe"]), int(g["n"]), int(g["seed"]))
    if digest(vec) != str(g["sha256"]):
        raise AssertionError(f"{path}: regenerated input differs from the fixture's")
    return g, vec
