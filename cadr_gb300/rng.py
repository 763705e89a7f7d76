"""Counter-based random numbers for the seeded synthetic scenes.

Every value is a pure function of (seed, stream name, attempt, index), so a
scene is reproduced bit for bit on any machine, in any order, from any
subset of indices.  The floating-point helpers use only IEEE basic
operations (+, -, *, /, sqrt, frexp, ldexp), never the platform's libm,
so x86 and Arm builds of numpy give identical bits.

Generator: SplitMix64 (Steele, Lea, Flood, "Fast splittable pseudorandom
number generators", OOPSLA 2014) applied to a keyed counter.
"""
from __future__ import annotations

import numpy as np

_U64 = np.uint64
_GOLDEN = _U64(0x9E3779B97F4A7C15)


def splitmix64(x: np.ndarray) -> np.ndarray:
    """SplitMix64 finaliser of a uint64 array (wrapping arithmetic)."""
    x = np.asarray(x, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = x + _GOLDEN
        z = (z ^ (z >> _U64(30))) * _U64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> _U64(27))) * _U64(0x94D049BB133111EB)
    return z ^ (z >> _U64(31))


def _fnv1a(name: str) -> int:
    h = 0xCBF29CE484222325
    for b in name.encode():
        h ^= b
        h = (h * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
    return h


class Stream:
    """A named random stream of one seed."""

    def __init__(self, seed: int, name: str):
        k = splitmix64(np.array([(seed * 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF], np.uint64))
        k = splitmix64(k ^ np.array([_fnv1a(name)], np.uint64))
        self.key = k[0]

    def u64(self, idx: np.ndarray, attempt: int = 0) -> np.ndarray:
        idx = np.asarray(idx, dtype=np.uint64)
        a = splitmix64(np.array([attempt], np.uint64) ^ np.array([self.key], np.uint64))[0]
        return splitmix64(splitmix64(idx ^ a) + a)

    def uniform(self, idx: np.ndarray, attempt: int = 0) -> np.ndarray:
        """Uniform float64 in [0, 1) with 53 random bits."""
        return (self.u64(idx, attempt) >> _U64(11)).astype(np.float64) * (2.0 ** -53)

    def uniform_range(self, idx, lo, hi, attempt: int = 0) -> np.ndarray:
        return lo + (hi - lo) * self.uniform(idx, attempt)

    def integers(self, idx, lo: int, hi_inclusive: int, attempt: int = 0) -> np.ndarray:
        """Uniform integers in [lo, hi_inclusive] (multiply-shift, no modulo bias
        beyond 2^-32 for the ranges used here)."""
        span = np.uint64(hi_inclusive - lo + 1)
        u = self.u64(idx, attempt) >> _U64(32)
        return (lo + ((u * span) >> _U64(32))).astype(np.int64)


# ---------------------------------------------------------------------------
# Elementary functions from basic operations only.

_LN2 = 0.6931471805599453094
_SQRT_HALF = 0.70710678118654752440


def det_log(x: np.ndarray) -> np.ndarray:
    """Natural logarithm for x > 0: x = m * 2^e with m in [sqrt(1/2), sqrt(2)),
    log m = 2 atanh(t), t = (m-1)/(m+1), by its odd power series."""
    x = np.asarray(x, dtype=np.float64)
    m, e = np.frexp(x)  # m in [0.5, 1)
    small = m < _SQRT_HALF
    m = np.where(small, m * 2.0, m)
    e = np.where(small, e - 1, e).astype(np.float64)
    t = (m - 1.0) / (m + 1.0)
    t2 = t * t
    acc = np.zeros_like(t)
    for k in range(27, 0, -2):  # sum_{k odd} t^k / k, Horner in t^2
        acc = acc * t2 + 1.0 / k
    return 2.0 * t * acc + e * _LN2


def det_exp(x: np.ndarray) -> np.ndarray:
    """Exponential: x = k ln2 + r, |r| <= ln2/2, exp r by its Taylor series."""
    x = np.asarray(x, dtype=np.float64)
    k = np.round(x / _LN2)
    r = x - k * _LN2
    acc = np.ones_like(r)
    for n in range(22, 0, -1):  # Horner of sum r^n / n!
        acc = 1.0 + acc * r / n
    return np.ldexp(acc, k.astype(np.int64))


def det_pow(base: np.ndarray, p: float) -> np.ndarray:
    return det_exp(p * det_log(base))


# ---------------------------------------------------------------------------
# Rejection samplers (vectorised over indices, attempt by attempt).

def unit_quaternions(stream: Stream, n: int) -> np.ndarray:
    """Uniformly distributed unit quaternions (uniform random rotations):
    points drawn uniformly in the 4-cube, kept inside the unit 4-ball and
    normalised.  Returns float64 [n, 4] = (w, x, y, z)."""
    out = np.empty((n, 4), np.float64)
    pending = np.arange(n, dtype=np.uint64)
    attempt = 0
    while pending.size:
        q = np.stack([stream.uniform(pending * _U64(4) + _U64(c), attempt) * 2.0 - 1.0
                      for c in range(4)], axis=1)
        s = ((q[:, 0] * q[:, 0] + q[:, 1] * q[:, 1]) + q[:, 2] * q[:, 2]) + q[:, 3] * q[:, 3]
        ok = (s <= 1.0) & (s > 1e-6)
        out[pending[ok].astype(np.int64)] = q[ok] / np.sqrt(s[ok])[:, None]
        pending = pending[~ok]
        attempt += 1
        if attempt > 200:
            raise RuntimeError("rejection sampler did not converge")
    return out


def normals(stream: Stream, n: int) -> np.ndarray:
    """Standard normal deviates by Marsaglia's polar method."""
    out = np.empty(n, np.float64)
    pending = np.arange(n, dtype=np.uint64)
    attempt = 0
    while pending.size:
        u = stream.uniform(pending * _U64(2), attempt) * 2.0 - 1.0
        v = stream.uniform(pending * _U64(2) + _U64(1), attempt) * 2.0 - 1.0
        s = u * u + v * v
        ok = (s < 1.0) & (s > 0.0)
        so = s[ok]
        out[pending[ok].astype(np.int64)] = u[ok] * np.sqrt(-2.0 * det_log(so) / so)
        pending = pending[~ok]
        attempt += 1
        if attempt > 200:
            raise RuntimeError("rejection sampler did not converge")
    return out


def lognormal(stream: Stream, n: int, mu: float, sigma: float) -> np.ndarray:
    return det_exp(mu + sigma * normals(stream, n))


def zipf_choice(stream: Stream, n: int, k: int, s: float) -> np.ndarray:
    """Draws n indices in [0, k) with P(i) proportional to (i+1)^-s."""
    w = det_exp(-s * det_log(np.arange(1, k + 1, dtype=np.float64)))
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    u = stream.uniform(np.arange(n, dtype=np.uint64))
    return np.minimum(np.searchsorted(cdf, u, side="right"), k - 1).astype(np.int64)
