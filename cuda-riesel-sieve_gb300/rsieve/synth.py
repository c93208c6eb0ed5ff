"""Seeded synthetic sieve jobs with the shapes of the benchmark workloads.

The generator is a counter-based splitmix64 stream evaluated with numpy, so a
(seed, shape) pair gives the same job on every machine and numpy version.

Workloads (all Riesel k*b^n-1, uint64 arithmetic):
  plain_small    b=745, 22 distinct odd k in [3, 1e6], n in [180000, 250000],
                 each n kept with probability 0.05; p in [1e9, 1.02e9)
  plain_steady   the same job over p in [1e13, 1e13 + 1e11)
  wide_2_50      b=2, 1000 distinct odd k in [3, 1e7], n in [1e6, 3e6] at 2%;
                 p in [2^50, 2^50 + 5e10)
  batch_job(i)   base uniform in [2, 1024] (no perfect powers), k-count
                 log-uniform in [1, 1000], odd k in [3, 1e7], n-start uniform in
                 [1e5, 1e6], width log-uniform in [1e4, 2e6], density in [1%, 10%],
                 a 1e9-wide p window starting uniform in [1e12, 2^60]
"""
from __future__ import annotations

import math

import numpy as np

M64 = (1 << 64) - 1
_GOLD = np.uint64(0x9E3779B97F4A7C15)


def _mix(z: np.ndarray) -> np.ndarray:
    z = z.astype(np.uint64, copy=True)
    with np.errstate(over="ignore"):
        z += _GOLD
        z ^= z >> np.uint64(30)
        z *= np.uint64(0xBF58476D1CE4E5B9)
        z ^= z >> np.uint64(27)
        z *= np.uint64(0x94D049BB133111EB)
        z ^= z >> np.uint64(31)
    return z


def _key(seed: int, tag: str) -> int:
    h = seed & M64
    for ch in tag.encode():
        h = int(_mix(np.array([h ^ ch], dtype=np.uint64))[0])
    return h


def stream(seed: int, tag: str, start: int, count: int) -> np.ndarray:
    """count uint64 values of stream (seed, tag) from index start."""
    k = np.uint64(_key(seed, tag))
    idx = np.arange(start, start + count, dtype=np.uint64)
    with np.errstate(over="ignore"):
        return _mix(idx * np.uint64(0xD1B54A32D192ED03) + k)


def uniform(seed: int, tag: str, count: int) -> np.ndarray:
    """count doubles in [0, 1)."""
    return (stream(seed, tag, 0, count) >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))


def _distinct_odd_ks(seed: int, tag: str, nk: int, lo: int, hi: int) -> np.ndarray:
    ks: list[int] = []
    seen = set()
    start = 0
    while len(ks) < nk:
        vals = stream(seed, tag, start, 4 * nk + 16)
        start += len(vals)
        for v in vals:
            k = lo + int(v) % (hi - lo + 1)
            k |= 1
            if k > hi:
                k -= 2
            if k < lo or k in seen:
                continue
            seen.add(k)
            ks.append(k)
            if len(ks) == nk:
                break
    return np.array(ks, dtype=np.uint32)


def make_job(seed: int, base: int, nk: int, kmin: int, kmax: int, nmin: int, nmax: int, density: float):
    """(base, sign, ks, nlists): n kept independently with the given probability."""
    ks = _distinct_odd_ks(seed, "k", nk, kmin, kmax)
    width = nmax - nmin + 1
    thr = np.uint64(min(M64, int(density * 2.0**64)))
    nlists = []
    for i in range(nk):
        u = stream(seed, f"n{i}", 0, width)
        keep = np.nonzero(u < thr)[0].astype(np.uint32) + np.uint32(nmin)
        if keep.size == 0:
            keep = np.array([nmin], dtype=np.uint32)
        nlists.append(keep)
    return base, -1, ks, nlists


def plain_job(seed: int = 1):
    """b=745, 22 odd k in [3, 1e6], n in [180000, 250000] at 5%."""
    return make_job(seed, 745, 22, 3, 10**6, 180000, 250000, 0.05)


PLAIN_SMALL_RANGE = (10**9, 102 * 10**7 - 1)
PLAIN_STEADY_RANGE = (10**13, 10**13 + 10**11 - 1)


def wide_job(seed: int = 1):
    """b=2, 1000 odd k in [3, 1e7], n in [1e6, 3e6] at 2%."""
    return make_job(seed, 2, 1000, 3, 10**7, 10**6, 3 * 10**6, 0.02)


WIDE_RANGE = (1 << 50, (1 << 50) + 5 * 10**10 - 1)


def _is_perfect_power(b: int) -> bool:
    for e in range(2, 11):
        r = round(b ** (1.0 / e))
        for c in (r - 1, r, r + 1):
            if c > 1 and c**e == b:
                return True
    return False


def batch_job(seed: int, i: int):
    """Job i of the mixed batch: ((base, sign, ks, nlists), (p0, p1))."""
    u = uniform(seed, f"batch{i}", 8)
    bases = [b for b in range(2, 1025) if not _is_perfect_power(b)]
    base = bases[int(u[0] * len(bases))]
    nk = int(round(math.exp(u[1] * math.log(1000.0))))
    nk = max(1, min(1000, nk))
    nstart = 10**5 + int(u[2] * (10**6 - 10**5))
    width = int(round(math.exp(math.log(1e4) + u[3] * (math.log(2e6) - math.log(1e4)))))
    density = 0.01 + u[4] * 0.09
    p0 = int(1e12 + u[5] * ((1 << 60) - 1e12))
    job = make_job(seed * 1000 + i, base, nk, 3, 10**7, nstart, nstart + width - 1, density)
    return job, (p0, p0 + 10**9 - 1)


def to_abcd(base: int, sign: int, ks, nlists) -> str:
    """srsieve ABCD text: a header with the first n, then n deltas."""
    out = []
    s = "-1" if sign < 0 else "+1"
    for k, ns in zip(ks, nlists):
        ns = np.asarray(ns, dtype=np.int64)
        out.append(f"ABCD {int(k)}*{base}^$a{s} [{int(ns[0])}]")
        if len(ns) > 1:
            out.append("\n".join(map(str, np.diff(ns).tolist())))
    return "\n".join(out) + "\n"
