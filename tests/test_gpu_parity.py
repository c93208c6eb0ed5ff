"""Parity of the CUDA path with the CPU oracle (run on the GB300 machine).

Bit-exact factor sets: the GPU reports every (p,k,n) the oracle reports and
nothing else, on seeded synthetic jobs, on the reference's own sr_745.abcd,
and on edge cases (Sierpinski, even k, base 2, p dividing b or k, tiny p,
x range starting at 0, forced Q/m, datless).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _set(f):
    """(p, k, n) triples of a factor array (rsieve's or the oracle's)."""
    return [(int(x["p"]), int(x["k"]), int(x["n"])) for x in f]


_WIDE = []


def _wide_job():
    """The wide job (40M candidates, slow to generate), made once per session."""
    import rsieve.synth as S

    if not _WIDE:
        _WIDE.append(S.wide_job(1))
    return _WIDE[0]


def _both(rs, oracle_mod, base, sign, ks, nlists, p0, p1, datless=False, **opts):
    """GPU and oracle factor sets of one job on [p0, p1]; st["info"] is the GPU job's plan."""
    job = rs.Job(base=base, sign=sign, ks=ks, nlists=nlists, datless=int(datless), **opts)
    g, st = job.sieve(p0, p1)
    st["info"] = dict(job.info)
    oj = oracle_mod.Job.from_arrays(base, sign, ks, [np.asarray(x) for x in nlists])
    o, npr = oj.sieve(p0, p1, datless=datless)
    job.close()
    assert st["primes"] == npr
    assert sum(st["primes_by_step"].values()) == st["primes"]
    return _set(g), _set(o), st


def test_arith_montmul_and_jacobi(rs, oracle_mod):
    rng = np.random.default_rng(11)
    ps = oracle_mod.primes(10**13, 10**13 + 3000).tolist()
    ps += oracle_mod.primes(2**62 - 200000, 2**62).tolist()
    ps += oracle_mod.primes(2**63 - 20000, 2**63 - 1).tolist()
    ps += [3, 5, 7, 2**31 - 1, 4294967311]
    a, b, p = [], [], []
    for P in ps:
        for _ in range(4):
            a.append(int(rng.integers(0, P)) if P > 2 else 1)
            b.append(int(rng.integers(0, P)))
            p.append(P)
        a += [P - 1, 0, 1 % P, (1 << 32) % P]
        b += [P - 1, P - 1, P - 1, (1 << 32) % P]
        p += [P, P, P, P]
    mm, jj = rs.arith_check(a, b, p)
    for i in range(len(a)):
        assert int(mm[i]) == a[i] * b[i] % p[i], (a[i], b[i], p[i])
        k = a[i] & 0xFFFFFFFF
        assert int(jj[i]) == oracle_mod.jacobi(k, p[i]), (k, p[i])


@pytest.mark.parametrize("lo,hi", [
    (3, 200000), (10**9, 10**9 + 3 * 10**6), (10**13 - 10**6, 10**13 + 10**6),
    (2**50, 2**50 + 10**6), (2**62 - 10**6, 2**62 + 10**6), (2**63 - 10**6, 2**63 - 1),
    (101, 101), (100, 103), (2**32 - 50, 2**32 + 50),
])
def test_gpu_primes_match_oracle(rs, oracle_mod, lo, hi):
    g = rs.gpu_primes(lo, hi)
    o = oracle_mod.primes(lo, hi)
    assert np.array_equal(g, o)


def test_plain_small_full(rs, oracle_mod):
    """The small plain workload in full: b=745, 22 k, p in [1e9, 1.02e9)."""
    import rsieve.synth as S

    b, s, ks, nl = S.plain_job(1)
    p0, p1 = S.PLAIN_SMALL_RANGE
    g, o, st = _both(rs, oracle_mod, b, s, ks, nl, p0, p1)
    assert len(o) > 0
    assert g == o


def test_plain_steady_subwindow(rs, oracle_mod):
    """The 1e8-wide sub-window [1e13, 1e13+1e8) of the steady-state workload,
    complete and datless.  Factors are rare this high (the oracle finds 0 and 1),
    so the non-empty parity of this exact kernel path is test_benchmark_path_near_2_33."""
    import rsieve.synth as S

    b, s, ks, nl = S.plain_job(1)
    for datless in (False, True):
        g, o, st = _both(rs, oracle_mod, b, s, ks, nl, 10**13, 10**13 + 10**8 - 1, datless=datless)
        assert g == o
        assert st["primes"] > 3 * 10**6
        assert st["primes_by_step"]["short"] == st["primes"] and st["paired_primes"] > st["primes"] // 4


# The benchmark job's plan: Q = 2, one warp per prime, integer rows kept in the
# records (row form 1).  Just above 2^33 its baby steps take the short product
# by b^Q (the form the benchmark window at 1e13 runs) and factors are still
# plentiful: the oracle reports 8 / 78 (Riesel, complete / datless) on a 1e7
# window and 8 Sierpinski factors on a 3e7 window.
_NEAR_2_33 = 2**33 + 1


@pytest.mark.parametrize("sign,datless,width", [(-1, False, 10**7), (-1, True, 10**7), (1, False, 3 * 10**7),
                                                (1, True, 10**7)])
def test_benchmark_path_near_2_33(rs, oracle_mod, sign, datless, width):
    """The benchmark's own kernel path on a window where the oracle reports
    factors: warp-per-prime BSGS with short baby products, integer rows and,
    for primes with (b/p) = 1, the row-pair giant path; the counters of
    rs_stats show that path ran."""
    import rsieve.synth as S

    b, _, ks, nl = S.plain_job(1)
    g, o, st = _both(rs, oracle_mod, b, sign, ks, nl, _NEAR_2_33, _NEAR_2_33 + width - 1, datless=datless)
    info = st["info"]
    assert (info["Q"], info["warps_per_prime"], info["row_form"]) == (2, 1, 3)
    assert len(o) >= 5
    assert g == o
    assert st["primes_by_step"]["short"] == st["primes"]
    assert st["primes"] // 4 < st["paired_primes"] < st["primes"]


@pytest.mark.parametrize("baby_step", ["shoup", "short"])
def test_benchmark_job_forced_baby_step(rs, oracle_mod, baby_step):
    """The same window with the baby-step product forced: Shoup's full product
    (no row pairs, which ride on the short product) and the short one."""
    import rsieve.synth as S

    b, s, ks, nl = S.plain_job(1)
    form = {"shoup": rs.BABY_SHOUP, "short": rs.BABY_SHORT}[baby_step]
    g, o, st = _both(rs, oracle_mod, b, s, ks, nl, _NEAR_2_33, _NEAR_2_33 + 10**7 - 1, datless=True,
                     baby_step=form)
    assert len(o) >= 5 and g == o
    assert st["primes_by_step"][baby_step] == st["primes"]
    assert (st["paired_primes"] > 0) == (baby_step == "short")


@pytest.mark.parametrize("opts", [{}, {"Q": 18}, {"Q": 2}, {"Q": 18, "hash_m": 5}, {"Q": 6, "hash_m": 9}])
def test_sr745_vs_oracle(rs, oracle_mod, sr745_text, opts):
    """The reference's own test file (datless, so hits exist at small p)."""
    job = rs.Job(sr745_text, datless=1, **opts)
    g, st = job.sieve(10**6, 10**6 + 4 * 10**6)
    oj = oracle_mod.Job.from_abcd(sr745_text)
    o, npr = oj.sieve(10**6, 10**6 + 4 * 10**6, datless=True)
    job.close()
    assert st["primes"] == npr
    assert _set(g) == _set(o)
    assert len(o) > 100


def test_sr745_negative_kat(rs, sr745_text, kat):
    """Sieved to 5e12 (sr_745.abcd:1): no candidate has a factor below it."""
    lim = kat["negative"]["sieved_to"]
    job = rs.Job(sr745_text)
    g, st = job.sieve(lim - 2 * 10**8, lim)
    assert len(g) == 0 and st["primes"] > 6 * 10**6
    g, st = job.sieve(10**9, 10**9 + 10**8)
    assert len(g) == 0


def test_sr745_datless_kat(rs, sr745_text, kat):
    """102297149781479 | 18300*745^242670-1 (kernel_v0.24.6.cu:244); n is not a candidate."""
    d = kat["datless"]
    lo = kat["default_range"]["low"]
    for Q in (0, 18):
        job = rs.Job(sr745_text, datless=1, Q=Q)
        g, st = job.sieve(lo, lo + kat["default_range"]["width_per_scale"])
        assert (d["p"], d["k"], d["n"]) in _set(g)
        job.close()
    job = rs.Job(sr745_text)
    g, st = job.sieve(d["p"] - 10**5, d["p"] + 10**5)
    assert (d["p"], d["k"], d["n"]) not in _set(g)


@pytest.mark.parametrize("case", [
    # base, sign, ks, n range, density, p0, p1, opts
    (2, -1, [3, 5, 7, 9, 15, 27], (1000, 3000), 0.3, 10**7, 10**7 + 10**6, {}),
    (2, 1, [3, 5, 7, 9, 15, 27], (1000, 3000), 0.3, 10**7, 10**7 + 10**6, {}),
    (10, -1, [4, 12, 48, 96, 1024], (50, 900), 0.5, 3, 300000, {}),
    (3, -1, [2, 4, 8, 16], (1, 40), 1.0, 3, 100000, {"Q": 6}),
    (745, -1, [18300, 1160], (5, 20), 1.0, 3, 50000, {"Q": 18}),
    (6, 1, [1, 35, 77], (100, 20000), 0.1, 10**9, 10**9 + 10**6, {"Q": 3}),
    (1024, -1, [3, 7, 11], (5000, 60000), 0.05, 10**12, 10**12 + 10**6, {}),
])
def test_edge_cases(rs, oracle_mod, case):
    base, sign, ks, (nlo, nhi), dens, p0, p1, opts = case
    rng = np.random.default_rng(abs(hash((base, sign, nlo))) % 2**32)
    nlists = []
    for _ in ks:
        ns = np.arange(nlo, nhi + 1)
        keep = ns[rng.random(ns.size) < dens]
        if keep.size == 0:
            keep = ns[:1]
        nlists.append(keep.astype(np.uint32))
    for datless in (False, True):
        g, o, st = _both(rs, oracle_mod, base, sign, ks, nlists, p0, p1, datless=datless, **opts)
        assert g == o, (case, datless, len(g), len(o))


def test_range_additivity_and_boundaries(rs, oracle_mod):
    """[a,c] == [a,b] + [b+1,c]; primes exactly at p0 and p1 are included."""
    import rsieve.synth as S

    b, s, ks, nl = S.plain_job(2)
    job = rs.Job(base=b, sign=s, ks=ks, nlists=nl, datless=1)
    a, c = 10**9, 10**9 + 4 * 10**6
    full, _ = job.sieve(a, c)
    mid = a + 1234567
    left, _ = job.sieve(a, mid)
    right, _ = job.sieve(mid + 1, c)
    assert _set(full) == _set(left) + _set(right)
    ps = sorted({x[0] for x in _set(full)})
    assert ps, "datless window should have hits"
    p = ps[len(ps) // 2]
    at, _ = job.sieve(p, p)
    assert {x[0] for x in _set(at)} == {p}
    job.close()


def test_every_factor_verifies_at_scale(rs, oracle_mod):
    """A 1e10-wide slice of the steady-state workload: every factor passes an
    independent modexp check (size-independent property)."""
    import rsieve.synth as S

    b, s, ks, nl = S.plain_job(1)
    job = rs.Job(base=b, sign=s, ks=ks, nlists=nl)
    g, st = job.sieve(10**13, 10**13 + 10**10)
    cand = {(int(k), int(n)) for k, ns in zip(ks, nl) for n in ns}
    for p, k, n in _set(g):
        assert oracle_mod.verify(p, k, b, n, s)
        assert (k, n) in cand
    assert st["primes"] > 3 * 10**8
    job.close()


def test_wide_config_window(rs, oracle_mod):
    """The wide workload (b=2, 1000 k in [3, 1e7], n in [1e6, 3e6] at 2%) on a
    2e6-wide window at 2^50, complete and datless."""
    import rsieve.synth as S

    b, s, ks, nl = _wide_job()
    p0 = S.WIDE_RANGE[0]
    for datless in (False, True):
        g, o, st = _both(rs, oracle_mod, b, s, ks, nl, p0, p0 + 2 * 10**6, datless=datless)
        assert g == o
    assert st["primes"] > 50000


@pytest.mark.parametrize("baby_step,datless", [("auto", False), ("auto", True), ("high", True), ("shoup", True)])
def test_wide_job_near_2_35(rs, oracle_mod, baby_step, datless):
    """The wide job's own path (16 warps per prime, row ids only) on a window
    where the oracle reports factors (7 complete, 487 datless on 2e5 at 2^35),
    with each baby-step product the CTA kernel has: the short product (auto),
    Shoup's product by the 32-bit constant b^Q (valid: 2 * 2^32 < p) and
    Shoup's full product."""
    import rsieve.synth as S

    b, s, ks, nl = _wide_job()
    form = {"auto": rs.BABY_AUTO, "high": rs.BABY_HIGH, "shoup": rs.BABY_SHOUP}[baby_step]
    p0 = 2**35 + 1
    g, o, st = _both(rs, oracle_mod, b, s, ks, nl, p0, p0 + 2 * 10**5 - 1, datless=datless, baby_step=form)
    assert st["info"]["warps_per_prime"] == 16
    assert len(o) >= 5 and g == o
    want = {"auto": "short", "high": "high", "shoup": "shoup"}[baby_step]
    assert st["primes_by_step"][want] == st["primes"]


@pytest.mark.parametrize("mode", ["auto", "always", "never"])
def test_character_table_modes(rs, oracle_mod, mode):
    """The quadratic characters from bit tables built when they pay (auto: here,
    on a 2e5-wide window, only tables of k' below ~6,000), all at creation
    (always) or none (never), on the wide b=2 job (1000 k up to 1e7) at 2^35,
    both complete and datless: the same factor sets as the oracle."""
    b, s, ks, nl = _wide_job()
    m = {"auto": rs.TABLES_AUTO, "always": rs.TABLES_ALWAYS, "never": rs.TABLES_NEVER}[mode]
    p0 = 2**35 + 1
    for datless in (False, True):
        g, o, st = _both(rs, oracle_mod, b, s, ks, nl, p0, p0 + 2 * 10**5 - 1, datless=datless, char_tables=m)
        assert len(o) >= 5 and g == o


def test_character_tables_built_as_primes_accumulate(rs, oracle_mod):
    """One job (auto tables) over consecutive windows of growing width: each
    call builds the tables its primes pay for, and every window's factors
    equal the oracle's; sieving the first window again gives the same set."""
    import rsieve.synth as S

    (b, s, ks, nl), _ = S.batch_job(7, 20)  # a CTA-layout job of many k
    oj = oracle_mod.Job.from_arrays(b, s, ks, [np.asarray(x) for x in nl])
    p0 = 2**33 + 1
    wins = [(p0, p0 + 2 * 10**5 - 1), (p0 + 2 * 10**5, p0 + 10**6 - 1), (p0 + 10**6, p0 + 6 * 10**6 - 1)]
    with rs.Job(base=b, sign=s, ks=ks, nlists=nl, datless=1) as job:
        first = None
        for a, z in wins:
            g, st = job.sieve(a, z)
            o, npr = oj.sieve(a, z, datless=True)
            assert st["primes"] == npr and _set(g) == _set(o)
            first = first or _set(g)
        assert _set(job.sieve(*wins[0])[0]) == first


@pytest.mark.parametrize("i", [0, 1, 2, 3])
def test_batch_shaped_jobs(rs, oracle_mod, i):
    """Jobs drawn from the mixed-batch distribution (random base, k count,
    n range, density, p window up to 2^60), on a narrow window each."""
    import rsieve.synth as S

    (b, s, ks, nl), (p0, p1) = S.batch_job(7, i)
    g, o, st = _both(rs, oracle_mod, b, s, ks, nl, 10**6, 10**6 + 3 * 10**5, datless=True)
    assert g == o and len(o) > 0
    g, o, st = _both(rs, oracle_mod, b, s, ks, nl, p0, p0 + 3 * 10**5, datless=True)
    assert g == o and st["primes"] > 1000


@pytest.mark.parametrize("i,form,wpp", [(20, 1, 16), (5, 0, 16), (8, 2, 16), (4, 3, 1), (19, 3, 1), (48, 1, 1),
                                        (62, 2, 1)])
def test_row_forms(rs, oracle_mod, i, form, wpp):
    """Each form of the giant-step start values on each kernel: per-prime
    residues (form 0), the integers k*b^r kept in the records (form 1),
    k*b^r read by row id (form 2) and an active-row mask (form 3), with a warp
    (wpp 1) or a CTA (16) per prime, on mixed-batch jobs at small p (with
    factors), just above 2^33 and in their own window near 2^60."""
    import rsieve.synth as S

    (b, s, ks, nl), (p0, _) = S.batch_job(7, i)
    info = rs.plan_abcd(S.to_abcd(b, s, ks, nl), datless=1)
    assert (info["row_form"], info["warps_per_prime"]) == (form, wpp)
    g, o, st = _both(rs, oracle_mod, b, s, ks, nl, 10**6, 10**6 + 2 * 10**5, datless=True)
    assert g == o and len(o) > 0
    # just above 2^33, where the faster baby-step products start to apply
    # (jobs with few k need a wider window for factors)
    width = 2 * 10**6 if len(ks) < 50 else 2 * 10**5
    g, o, st = _both(rs, oracle_mod, b, s, ks, nl, _NEAR_2_33, _NEAR_2_33 + width - 1, datless=True)
    assert g == o and len(o) >= 3
    g, o, st = _both(rs, oracle_mod, b, s, ks, nl, p0, p0 + 2 * 10**5, datless=True)
    assert g == o and st["primes"] > 1000


def test_autotune_keeps_results(rs):
    """Measured autotuning picks one of the cost model's cheapest layouts and
    leaves the factor set unchanged."""
    import rsieve.synth as S

    b, s, ks, nl = S.plain_job(1)
    lo, hi = 10**9, 102 * 10**7 - 1  # the small workload, which has factors
    with rs.Job(base=b, sign=s, ks=ks, nlists=nl) as j:
        want, _ = j.sieve(lo, hi)
    with rs.Job(base=b, sign=s, ks=ks, nlists=nl) as j:
        before = dict(j.info)
        info = j.autotune(10**13, 10**13 + 3 * 10**8, candidates=3)
        got, _ = j.sieve(lo, hi)
    assert _set(got) == _set(want) and len(want) > 0
    assert info["Q"] >= 1 and info["baby_steps"] * info["giant_steps"] >= info["x_range"]
    assert info["num_candidates"] == before["num_candidates"]


@pytest.mark.parametrize("hash_m,sign", [(11, -1), (12, 1)])
def test_cta_layout_more_giant_steps(rs, oracle_mod, hash_m, sign):
    """The CTA-per-prime kernel with 8 and 4 giant steps per lane (baby steps
    capped by -m), both signs, against the oracle near 2^50."""
    import rsieve.synth as S

    b, _, ks, nl = _wide_job()
    p0 = S.WIDE_RANGE[0]
    job = rs.Job(base=b, sign=sign, ks=ks, nlists=nl, hash_m=hash_m)
    assert job.info["warps_per_prime"] == 16 and job.info["giant_steps"] >= 128
    job.close()
    g, o, st = _both(rs, oracle_mod, b, sign, ks, nl, p0, p0 + 5 * 10**5, hash_m=hash_m)
    assert g == o
    assert st["primes"] > 10000
    # a window with factors, just above 2^35
    q0 = 2**35 + 1
    for datless in (False, True):
        g, o, st = _both(rs, oracle_mod, b, sign, ks, nl, q0, q0 + 2 * 10**5 - 1, datless=datless, hash_m=hash_m)
        assert g == o
    assert len(o) >= 5


def test_sierpinski_row_pairs_near_1e13(rs, oracle_mod):
    """k*b^n+1 on the dense benchmark-shaped job at 1e13, where the baby steps
    use the short product and primes with (b/p) = 1 take the row-pair path."""
    import rsieve.synth as S

    b, _, ks, nl = S.plain_job(3)
    for datless in (False, True):
        g, o, st = _both(rs, oracle_mod, b, 1, ks, nl, 10**13, 10**13 + 2 * 10**7, datless=datless)
        assert g == o
    assert st["primes"] > 600000


def _mixed_file():
    """Three (base, sign) groups in one ABCD text, interleaved, some k shared
    between groups: b=745 Riesel (the plain job), b=2 Riesel, b=745 Sierpinski."""
    import rsieve.synth as S

    b0, _, ks0, nl0 = S.plain_job(1)
    _, _, ks1, nl1 = S.make_job(11, 2, 12, 3, 10**6, 180000, 250000, 0.05)
    groups = [(745, -1, ks0, nl0), (2, -1, ks1, nl1), (745, 1, ks0[:6], nl0[:6])]
    lines = []
    for i in range(max(len(g[2]) for g in groups)):
        for b, c, ks, nl in groups:
            if i < len(ks):
                lines.append(S.to_abcd(b, c, ks[i:i + 1], nl[i:i + 1]))
    return "".join(lines), groups


@pytest.mark.parametrize("datless", [False, True])
def test_per_sequence_bases(rs, oracle_mod, datless):
    """A file whose headers carry different bases and signs (the reference uses
    the first header's base for every k, kernel_v0.24.6.cu:1009-1016): every
    sequence is sieved with its own base and sign, each factor names them, and
    the set equals the oracle's per group, on a window with factors."""
    text, groups = _mixed_file()
    p0, p1 = _NEAR_2_33, _NEAR_2_33 + 10**7 - 1
    with rs.Job(text, datless=int(datless)) as job:
        assert job.info["parts"] == 3
        assert job.info["num_k"] == sum(len(g[2]) for g in groups)
        g, st = job.sieve(p0, p1)
    got = [(int(x["p"]), int(x["k"]), int(x["n"]), int(x["b"]), int(x["c"])) for x in g]
    want = []
    npr = 0
    for b, c, ks, nl in groups:
        oj = oracle_mod.Job.from_arrays(b, c, ks, [np.asarray(x) for x in nl])
        o, npr = oj.sieve(p0, p1, datless=datless)
        want += [(int(x["p"]), int(x["k"]), int(x["n"]), b, c) for x in o]
    assert st["primes"] == npr
    assert got == sorted(want)
    assert len({(b, c) for *_, b, c in got}) == 3 if datless else len(got) >= 5


@pytest.mark.parametrize("window", ["sr745_default", "plain_1e9", "plain_2_33"])
def test_contains_reference_projection(rs, oracle_mod, sr745_text, kat, window):
    """Every factor line the reference executable would write (the oracle's
    reference projection: its probable primes, one report per prime, its Q=1
    fallback and x-window, kernel_v0.24.6.cu:288-620,1605-1732) is in the GPU's
    complete set on the same input and range, with and without -v."""
    import rsieve.synth as S

    if window == "sr745_default":
        text = sr745_text
        p0 = kat["default_range"]["low"]
        p1 = p0 + kat["default_range"]["width_per_scale"]
    else:
        b, s, ks, nl = S.plain_job(1)
        text = S.to_abcd(b, s, ks, nl)
        p0 = 10**9 if window == "plain_1e9" else _NEAR_2_33
        p1 = p0 + 2 * 10**6
    oj = oracle_mod.Job.from_abcd(text)
    for verify in (True, False):
        ref, _ = oj.sieve_ref(p0, p1, Qin=18, hash_m=8, verify=verify)
        with rs.Job(text, datless=int(not verify)) as job:
            g, st = job.sieve(p0, p1)
        got = set(_set(g))
        want = set(_set(ref))
        assert want <= got, sorted(want - got)[:5]
        if window == "sr745_default" and not verify:
            d = kat["datless"]
            assert (d["p"], d["k"], d["n"]) in want
        if window != "sr745_default":
            assert len(want) > 0
