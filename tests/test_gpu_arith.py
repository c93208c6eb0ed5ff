"""Device arithmetic against exact integer arithmetic (run on the GB300 machine).

Every modular product the kernels are built from (rs_arith.cuh, generalising
the reference's montmul and modul64, kernel_v0.24.6.cu:150-270) is evaluated on
the GPU through rs_gpu_modmul_check and compared with Python's exact integers,
at random points and at the edges of each product's domain: p just above 2^33
(the short product's lower bound), c*p just below 2^63 (its upper bound), p near
2^62 and just below 2^63, x = 0, p-1 and 2^64-1 where the domain allows them.
"""
import random

import pytest

pytestmark = pytest.mark.gpu

M64 = 1 << 64


def _primes(oracle_mod):
    ps = [3, 5, 7, 11, 2**31 - 1, 4294967311]
    ps += oracle_mod.primes(2**33, 2**33 + 400).tolist()[:3]
    ps += oracle_mod.primes(2**40 - 2000, 2**40).tolist()[-2:]
    ps += oracle_mod.primes(10**13, 10**13 + 2000).tolist()[:2]
    ps += oracle_mod.primes(2**50, 2**50 + 3000).tolist()[:2]
    ps += oracle_mod.primes(2**62 - 3000, 2**62).tolist()[-2:]
    ps += oracle_mod.primes(2**63 - 3000, 2**63 - 1).tolist()[-3:]
    return [int(p) for p in ps]


def _run(rs, op, rows):
    a, b, c, p = zip(*rows)
    return [int(x) for x in rs.modmul_check(op, a, b, c, p)]


def _check(rs, op, rows, want):
    got = _run(rs, op, rows)
    bad = [(r, g, w) for r, g, w in zip(rows, got, want) if g != w]
    assert not bad, f"{op}: {len(bad)} of {len(rows)} wrong, first {bad[:3]}"


def test_montgomery_products(rs, oracle_mod):
    rng = random.Random(1)
    rows = []
    for p in _primes(oracle_mod):
        for a in (0, 1, p - 1, M64 - 1, rng.randrange(M64), rng.randrange(p)):
            for b in (0, 1, p - 1, rng.randrange(p)):
                rows.append((a, b, 0, p))
    want = [a * b * pow(M64, -1, p) % p for a, b, _, p in rows]
    _check(rs, "montmul", rows, want)
    _check(rs, "montmul_ptx", rows, want)


def test_from_mont_and_shoup_const(rs, oracle_mod):
    rng = random.Random(2)
    rows_f, rows_s, want_s = [], [], []
    for p in _primes(oracle_mod):
        for x in (0, 1, p - 1, rng.randrange(p), rng.randrange(p)):
            rows_f.append((x, 0, 0, p))
            rows_s.append(((x << 64) % p, 0, 0, p))  # the Montgomery form of w = x
            want_s.append((x << 64) // p)
    _check(rs, "from_mont", rows_f, [x * pow(M64, -1, p) % p for x, _, _, p in rows_f])
    _check(rs, "shoup_const", rows_s, want_s)


def test_shoup_products(rs, oracle_mod):
    rng = random.Random(3)
    rows, rows32 = [], []
    for p in _primes(oracle_mod):
        for w in (0, 1, p - 1, rng.randrange(p)):
            wq = (w << 64) // p
            for x in (0, 1, p - 1, M64 - 1, rng.randrange(M64)):
                rows.append((x, w, wq, p))
            for x in (0, 1, 2**32 - 1, rng.randrange(2**32)):
                rows32.append((x, w, wq, p))
    _check(rs, "shoup", rows, [x * w % p for x, w, _, p in rows])
    _check(rs, "shoup32", rows32, [x * w % p for x, w, _, p in rows32])


def test_shoup_by_32bit_constant(rs, oracle_mod):
    """shoup_mul_w32: w*2^32 < p, so that floor(w*2^64/p) fits 32 bits."""
    rng = random.Random(4)
    rows = []
    for p in _primes(oracle_mod):
        wmax = (p - 1) >> 32
        if wmax < 1:
            continue
        for w in {w for w in (1, 2, wmax, rng.randrange(1, wmax + 1)) if w <= wmax}:
            wq = (w << 64) // p
            assert wq < 2**32
            for x in (0, 1, p - 1, M64 - 1, rng.randrange(M64)):
                rows.append((x, w, wq, p))
    assert len(rows) > 50
    _check(rs, "shoup_w32", rows, [x * w % p for x, w, _, p in rows])


def test_short_product(rs, oracle_mod):
    """mul_small: x < p, p > 2^33, c*p < 2^63 (both bounds reached)."""
    rng = random.Random(5)
    rows = []
    for p in _primes(oracle_mod):
        if p <= 2**33:
            continue
        cmax = min((2**63 - 1) // p, 2**32 - 1)
        rc = M64 // p
        assert rc < 2**32
        for c in {1, 2, cmax, max(1, cmax - 1), rng.randrange(1, cmax + 1), 555025 if 555025 <= cmax else 1}:
            for x in (0, 1, p - 1, p - 2, rng.randrange(p), rng.randrange(p)):
                rows.append((x, c, rc, p))
    _check(rs, "mul_small", rows, [x * c % p for x, c, _, p in rows])


def test_montgomery_constants_and_powers(rs, oracle_mod):
    rng = random.Random(6)
    ps = _primes(oracle_mod)
    rows = [(0, 0, 0, p) for p in ps]
    _check(rs, "pinv", rows, [(-pow(p, -1, M64)) % M64 for p in ps])
    _check(rs, "one", rows, [M64 % p for p in ps])
    _check(rs, "r2", rows, [(M64 * M64) % p for p in ps])
    rows = []
    for p in ps:
        for a in (0, 1, 2, p - 1, rng.randrange(p)):
            for e in (0, 1, 2, 18, 1152, 89999, p - 2, M64 - 1):
                rows.append((a, e, 0, p))
    _check(rs, "pow", rows, [pow(a, e, p) for a, e, _, p in rows])


def test_product_rates(rs):
    """The measured product rates are positive, and the inline-PTX Montgomery
    chain and the C form are within a factor of two of each other."""
    r = rs.bench_products()
    assert all(v > 0 for v in r.values()), r
    assert 0.5 < r["montmul_ptx"] / r["montmul"] < 2.0, r
