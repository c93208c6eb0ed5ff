"""The CPU oracle, pinned against the reference's own known answers and
against brute force on small cases (no GPU)."""
import hashlib
import os

import numpy as np
import pytest

from conftest import GOLDEN


def test_fixture_digest(kat):
    with open(os.path.join(GOLDEN, "sr_745.abcd"), "rb") as f:
        assert hashlib.sha256(f.read()).hexdigest() == kat["sr_745_sha256"]


def test_structural_kat(oracle_mod, sr745_text, kat):
    """kernel_v0.24.6.cu:1086-1255 on sr_745.abcd: Q=18, 198 rows, x-range 3743."""
    job = oracle_mod.Job.from_abcd(sr745_text)
    s = kat["structure"]
    pl = job.ref_plan(0, s["hash_elems"])
    assert (pl.Q, pl.rows, pl.x_range, pl.tmin, pl.tmax) == (s["Q"], s["rows"], s["x_range"], s["tmin"], s["tmax"])
    assert [list(t) for t in zip(pl.row_k, pl.row_r)] == s["row_order"]
    # -Q 18 forced gives the same plan on this file
    assert job.ref_plan(18, 512).Q == 18


def test_reference_q_fallback_on_dense_data(oracle_mod, rs):
    """On dense synthetic data the reference keeps Q=1 even with -Q 18
    (minWork starts at the Q=1 cost, kernel_v0.24.6.cu:1089-1141)."""
    import rsieve.synth as S

    b, s, ks, nl = S.plain_job(1)
    job = oracle_mod.Job.from_abcd(S.to_abcd(b, s, ks, nl))
    assert job.ref_plan(0, 512).Q == 1
    assert job.ref_plan(18, 512).Q == 1


def test_datless_kat(oracle_mod, sr745_text, kat):
    d = kat["datless"]
    assert oracle_mod.verify(d["p"], d["k"], d["b"], d["n"], -1)
    job = oracle_mod.Job.from_abcd(sr745_text)
    f, npr = job.sieve(d["p"] - 1000, d["p"] + 1000, datless=True)
    assert (d["p"], d["k"], d["n"]) in [tuple(map(int, x)) for x in f]
    f2, _ = job.sieve(d["p"] - 1000, d["p"] + 1000, datless=False)
    assert all(int(x["p"]) != d["p"] or int(x["n"]) != d["n"] for x in f2)


def test_negative_kat(oracle_mod, sr745_text, kat):
    """sr_745.abcd was sieved to 5e12: no factor below that."""
    job = oracle_mod.Job.from_abcd(sr745_text)
    f, npr = job.sieve(10**9, 10**9 + 2 * 10**6, datless=False)
    assert npr > 90000
    assert len(f) == 0
    lim = kat["negative"]["sieved_to"]
    f, npr = job.sieve(lim - 10**6, lim, datless=False)
    assert len(f) == 0


def _brute(base, sign, ks, nlists, p0, p1, datless=False):
    """Pure-Python check of every (p, k, n) -- tiny cases only."""
    from sympy import isprime

    out = []
    nmin = min(min(x) for x in nlists)
    nmax = max(max(x) for x in nlists)
    for p in range(max(3, p0), p1 + 1):
        if p % 2 == 0 or not isprime(p):
            continue
        for k, ns in zip(ks, nlists):
            cand = range(nmin, nmax + 1) if datless else ns
            for n in cand:
                if (k * pow(base, n, p) - (1 if sign < 0 else -1)) % p == 0:
                    out.append((p, k, n))
    return sorted(set(out))


@pytest.mark.parametrize("sign", [-1, 1])
@pytest.mark.parametrize("datless", [False, True])
def test_oracle_vs_brute_force(oracle_mod, sign, datless):
    rng = np.random.default_rng(5)
    base = 3
    ks = [7, 12, 25, 81]
    nlists = [sorted(set(rng.integers(20, 140, size=25).tolist())) for _ in ks]
    job = oracle_mod.Job.from_arrays(base, sign, ks, [np.array(x) for x in nlists])
    f, _ = job.sieve(3, 3000, datless=datless)
    got = sorted((int(a), int(b), int(c)) for a, b, c in f)
    assert got == _brute(base, sign, ks, nlists, 3, 3000, datless)


def test_oracle_small_p_and_divisors(oracle_mod):
    """p dividing b or k, p smaller than k, tiny multiplicative orders."""
    base = 10
    ks = [3, 5, 11, 21]
    nlists = [list(range(1, 40)) for _ in ks]
    job = oracle_mod.Job.from_arrays(base, -1, ks, [np.array(x) for x in nlists])
    f, _ = job.sieve(3, 400)
    got = sorted((int(a), int(b), int(c)) for a, b, c in f)
    assert got == _brute(base, -1, ks, nlists, 3, 400)


def test_oracle_primes(oracle_mod):
    from sympy import primerange

    for lo, hi in [(3, 10000), (10**9, 10**9 + 20000), (10**12 + 5, 10**12 + 9999)]:
        got = oracle_mod.primes(lo, hi).tolist()
        assert got == [p for p in primerange(max(lo, 3), hi + 1) if p > 2]


def test_oracle_jacobi(oracle_mod):
    from sympy import jacobi_symbol

    rng = np.random.default_rng(3)
    for _ in range(500):
        n = int(rng.integers(1, 10**12)) * 2 + 1
        a = int(rng.integers(0, 2**40))
        assert oracle_mod.jacobi(a, n) == jacobi_symbol(a, n)


def test_oracle_abcd_errors(oracle_mod):
    with pytest.raises(ValueError):
        oracle_mod.Job.from_abcd("12\n")
    with pytest.raises(ValueError):
        oracle_mod.Job.from_abcd("ABCD 3*2^$a-1 [10]\n-5\n")
    with pytest.raises(ValueError):
        oracle_mod.Job.from_abcd("ABCD 3*2^$a-1 [10]\nABCD 5*3^$a-1 [10]\n")


# --- reference projection: what one run of the reference executable writes ---

def _trip(f):
    return {(int(x["p"]), int(x["k"]), int(x["n"])) for x in f}


def test_projection_reproduces_datless_kat(oracle_mod, sr745_text, kat):
    """On the reference's own file and default range with -Q 18 -m 8 -v, the
    projection writes exactly the debug prime's factor of kernel_v0.24.6.cu:244;
    with verification on it writes nothing (n = 242670 is not a candidate)."""
    d = kat["datless"]
    lo = kat["default_range"]["low"]
    hi = lo + kat["default_range"]["width_per_scale"]
    job = oracle_mod.Job.from_abcd(sr745_text)
    f, ncand = job.sieve_ref(lo, hi, Qin=18, hash_m=8, verify=False)
    assert _trip(f) == {(d["p"], d["k"], d["n"])}
    f, _ = job.sieve_ref(lo, hi, Qin=18, hash_m=8, verify=True)
    assert len(f) == 0
    # below smallP_max^2 (s = 256) the reference's probable primes are the primes
    _, npr = job.sieve(lo, hi, datless=True)
    assert ncand == npr


def test_projection_is_subset_of_complete_set(oracle_mod):
    """On dense synthetic data the reference falls back to Q=1 and writes at
    most one factor per prime: its output is a strict subset of the complete
    set (verified and datless), as stated in the contract differences."""
    import rsieve.synth as S

    b, s, ks, nl = S.plain_job(1)
    job = oracle_mod.Job.from_arrays(b, s, ks, [np.asarray(x) for x in nl])
    p0, p1 = 10**9, 10**9 + 2 * 10**6
    for verify in (True, False):
        ref, ncand = job.sieve_ref(p0, p1, Qin=18, hash_m=8, verify=verify)
        full, npr = job.sieve(p0, p1, datless=not verify)
        assert ncand == npr
        r, c = _trip(ref), _trip(full)
        assert r <= c and len(r) < len(c)
        assert len({p for p, _, _ in r}) == len(r)  # one report per prime
        assert len(r) >= 5


def test_projection_sends_composites_above_small_prime_bound(oracle_mod):
    """With -s 1 the reference's probable-prime source keeps composites above
    (the 4096th odd prime)^2 ~ 1.5e9; every line it writes still divides."""
    import rsieve.synth as S

    b, s, ks, nl = S.plain_job(1)
    job = oracle_mod.Job.from_arrays(b, s, ks, [np.asarray(x) for x in nl])
    p0, p1 = 5 * 10**9, 5 * 10**9 + 2 * 10**6
    ref, ncand = job.sieve_ref(p0, p1, Qin=0, hash_m=8, small_prime_scale=1, verify=False)
    npr = len(oracle_mod.primes(p0, p1))
    assert ncand > npr
    for p, k, n in _trip(ref):
        assert oracle_mod.verify(p, k, b, n, -1)
