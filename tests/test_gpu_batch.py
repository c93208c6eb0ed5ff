"""The batched form (rs_batch_*): many jobs' ranges sieved together, one
persistent BSGS launch per kernel variant per round, each round a CUDA graph.
Every item's factors and prime count equal the job's own rs_sieve_range on the
same range: warp-per-prime jobs of several variants (row mask, integers in V,
row ids, per-prime residues; several giant-lane widths), a CTA-per-prime job,
a job of two (base, sign) parts, Sierpinski, a window with factors on the
benchmark path, an empty range and ranges of a few primes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _key(f):
    return [(int(x["p"]), int(x["k"]), int(x["n"]), int(x["b"]), int(x["c"])) for x in f]


def _items(sr745_text):
    import rsieve.synth as S

    out = []
    b, s, ks, nl = S.plain_job(1)
    plain = S.to_abcd(b, s, ks, nl)
    out.append((plain, {}, 2**33 + 1, 2**33 + 10**7))                      # row mask, short baby product
    out.append((plain, {"datless": 1}, 10**9, 10**9 + 2 * 10**6))          # Shoup baby product, datless
    out.append((S.to_abcd(b, 1, ks, nl), {}, 2**33 + 1, 2**33 + 3 * 10**7))  # Sierpinski
    out.append((sr745_text, {"datless": 1}, 10**6, 10**6 + 2 * 10**6))     # Q = 18: per-prime residues
    for i in (4, 19, 48, 62, 20, 8):                                         # mask, mask, V, ids; CTA jobs
        (bb, ss, kk, nn), (p0, _) = S.batch_job(7, i)
        out.append((S.to_abcd(bb, ss, kk, nn), {"datless": 1}, 2**33 + 1, 2**33 + 10**6))
        out.append((S.to_abcd(bb, ss, kk, nn), {"datless": 1}, p0, p0 + 10**5))
    two = S.to_abcd(b, s, ks[:8], nl[:8]) + S.to_abcd(2, -1, ks[8:16], nl[8:16])
    out.append((two, {"datless": 1}, 2**33 + 1, 2**33 + 10**6))             # two parts: own path
    out.append((plain, {"Q": 2}, 10**12 + 10, 10**12 + 9))                  # empty range
    out.append((plain, {"Q": 1}, 10**9 + 7, 10**9 + 9))                     # one prime
    return out


def test_batch_matches_standalone(rs, sr745_text):
    specs = _items(sr745_text)
    want = []
    for text, opts, p0, p1 in specs:
        with rs.Job(text, **opts) as j:
            f, st = j.sieve(p0, p1)
        want.append((_key(f), st["primes"]))
    jobs = [rs.Job(text, mem_limit=256 << 20, **opts) for text, opts, _, _ in specs]
    with rs.Batch() as bt:
        items = [bt.add(j, p0, p1) for j, (_, _, p0, p1) in zip(jobs, specs)]
        tot = bt.run()
        for it, (wf, wp) in zip(items, want):
            f, st = bt.result(it)
            assert _key(f) == wf, it
            assert st["primes"] == wp, it
        # a second run of the same batch gives the same results (resident jobs)
        bt.run()
        for it, (wf, _) in zip(items, want):
            assert _key(bt.result(it)[0]) == wf
    for j in jobs:
        j.close()
    assert tot["factors"] == sum(len(w) for w, _ in want) > 100
    assert tot["bsgs_launches"] > 0
    # one launch per kernel variant and round, fewer than one per job and chunk
    assert tot["bsgs_launches"] < sum(1 for s in specs) * 2


def test_batch_rejects_a_job_twice(rs):
    import rsieve.synth as S

    b, s, ks, nl = S.plain_job(1)
    with rs.Job(base=b, sign=s, ks=ks, nlists=nl) as j, rs.Batch() as bt:
        bt.add(j, 10**9, 10**9 + 10**6)
        with pytest.raises(rs.RsieveError) as e:
            bt.add(j, 10**9 + 10**6, 10**9 + 2 * 10**6)
        assert e.value.code == rs.RS_ERR_INVALID


def test_batch_more_jobs_of_one_variant_than_one_launch_takes(rs):
    """300 jobs of one kernel variant and table size: the launch takes at most
    256 jobs, so each round runs two; every item still equals its own run."""
    import rsieve.synth as S

    b, s, ks, nl = S.plain_job(1)
    text = S.to_abcd(b, s, ks[:10], nl[:10])  # 44 datless factors over the 300 windows
    n = 300
    wins = [(2**33 + 1 + i * 40000, 2**33 + (i + 1) * 40000) for i in range(n)]
    jobs = [rs.Job(text, mem_limit=16 << 20, datless=1) for _ in range(n)]
    try:
        want = [_key(j.sieve(p0, p1)[0]) for j, (p0, p1) in zip(jobs, wins)]
        with rs.Batch() as bt:
            items = [bt.add(j, p0, p1) for j, (p0, p1) in zip(jobs, wins)]
            tot = bt.run()
            for it, w in zip(items, want):
                assert _key(bt.result(it)[0]) == w, it
        assert sum(len(w) for w in want) > 30
        assert tot["bsgs_launches"] >= 2
    finally:
        for j in jobs:
            j.close()
