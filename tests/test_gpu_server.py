"""The served form (rs_server_*): jobs submitted together run concurrently on
the GPU, and each job's factors are the same as when it runs alone through
rs_job_create_abcd + rs_sieve_range.  Admission by device memory (a job larger
than the budget runs alone, the charged bytes of running jobs never exceed
the budget otherwise), resident job state reused by later requests of the same
job, the queue limit (RS_ERR_BUSY) and the wait timeout (RS_ERR_TIMEOUT)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mix(sr745_text):
    import rsieve.synth as S

    jobs = []
    b, s, ks, nl = S.plain_job(1)
    plain = S.to_abcd(b, s, ks, nl)
    jobs.append((plain, 10**9, 10**9 + 2 * 10**7, {}))
    jobs.append((plain, 10**13, 10**13 + 3 * 10**8, {}))
    jobs.append((sr745_text, 5 * 10**12, 5 * 10**12 + 5 * 10**7, {}))
    jobs.append((sr745_text, 10**9, 10**9 + 10**7, {"datless": 1}))
    for i in range(4):
        (b, s, ks, nl), (p0, _) = S.batch_job(7, i)
        jobs.append((S.to_abcd(b, s, ks, nl), p0, p0 + 2 * 10**6, {"datless": 1}))
    b, s, ks, nl = S.wide_job(1)
    jobs.append((S.to_abcd(b, s, ks, nl), S.WIDE_RANGE[0], S.WIDE_RANGE[0] + 10**6, {}))
    return jobs


def _key(f):
    return [(int(x["p"]), int(x["k"]), int(x["n"])) for x in f]


def test_server_results_match_standalone(rs, sr745_text):
    jobs = _mix(sr745_text)
    alone = []
    for abcd, p0, p1, opts in jobs:
        with rs.Job(abcd, **opts) as j:
            f, st = j.sieve(p0, p1)
        alone.append((_key(f), st["primes"]))
    with rs.Server(slots=4) as srv:
        tickets = [srv.submit(abcd, p0, p1, **opts) for abcd, p0, p1, opts in jobs]
        # collect in reverse order of submission: completion order does not matter
        got = {}
        for t in reversed(tickets):
            f, rep = srv.wait(t)
            got[t] = (_key(f), rep)
    for t, (want, primes) in zip(tickets, alone):
        f, rep = got[t]
        assert f == want
        assert rep["status"] == rs.RS_OK and rep["factors"] == len(want) and rep["primes"] == primes
        assert rep["latency_ms"] >= rep["run_ms"] > 0
    assert sum(len(w) for w, _ in alone) > 0


def test_server_queue_limit_and_timeout(rs):
    import rsieve.synth as S

    b, s, ks, nl = S.plain_job(1)
    plain = S.to_abcd(b, s, ks, nl)
    with rs.Server(slots=1, queue_cap=1) as srv:
        long_job = srv.submit(plain, 10**13, 10**13 + 2 * 10**9)
        tickets, busy = [long_job], 0
        for _ in range(3):
            try:
                tickets.append(srv.submit(plain, 10**9, 10**9 + 10**6))
            except rs.RsieveError as e:
                assert e.code == rs.RS_ERR_BUSY
                busy += 1
        assert busy >= 1
        with pytest.raises(rs.RsieveError) as e:
            srv.wait(tickets[-1], timeout_ms=0)
        assert e.value.code == rs.RS_ERR_TIMEOUT
        for t in tickets:
            f, rep = srv.wait(t)
            assert rep["status"] == rs.RS_OK
        with pytest.raises(rs.RsieveError) as e:
            srv.wait(tickets[0])
        assert e.value.code == rs.RS_ERR_INVALID  # a ticket is released once collected


def test_server_reports_job_errors(rs):
    """A malformed job is refused at submit (it is parsed and planned there);
    a range the sieve refuses fails in the job's own status."""
    with rs.Server(slots=2) as srv:
        with pytest.raises(rs.RsieveError) as e:
            srv.submit("ABCD 3*2^$a-1 [x]\n", 10**9, 10**9 + 10**5)
        assert e.value.code == rs.RS_ERR_INVALID
        bad = srv.submit("ABCD 3*2^$a-1 [10]\n2\n4\n", 2**63 - 100, 2**63 + 100)
        good = srv.submit("ABCD 3*2^$a-1 [10]\n2\n4\n", 10**9, 10**9 + 10**5)
        with pytest.raises(rs.RsieveError) as e:
            srv.wait(bad)
        assert e.value.code == rs.RS_ERR_RANGE
        f, rep = srv.wait(good)
        assert rep["status"] == rs.RS_OK
        assert isinstance(f, np.ndarray)


def test_server_admits_by_memory(rs):
    """With a 768 MiB budget the wide job (its arrays alone exceed the budget)
    runs by itself, and the plain jobs run as many at a time as their
    footprints fit: the bytes charged to running jobs stay within the budget,
    whatever the slot count, and every result equals the standalone run."""
    import rsieve.synth as S

    budget = 768 << 20
    b, s, ks, nl = S.plain_job(1)
    plain = S.to_abcd(b, s, ks, nl)
    jobs = [(plain, 10**9 + i * 10**7, 10**9 + (i + 1) * 10**7, {}) for i in range(6)]
    bw, sw, kw, nw = S.wide_job(1)
    jobs.insert(2, (S.to_abcd(bw, sw, kw, nw), S.WIDE_RANGE[0], S.WIDE_RANGE[0] + 10**6, {}))
    alone = []
    for abcd, p0, p1, opts in jobs:
        with rs.Job(abcd, **opts) as j:
            f, _ = j.sieve(p0, p1)
        alone.append(_key(f))
    with rs.Server(slots=4, mem_budget=budget) as srv:
        tickets = [srv.submit(abcd, p0, p1, **opts) for abcd, p0, p1, opts in jobs]
        reps = []
        for t, want in zip(tickets, alone):
            f, rep = srv.wait(t)
            assert _key(f) == want
            reps.append(rep)
    wide = reps[2]
    assert wide["mem_bytes"] > budget and wide["mem_in_use"] == wide["mem_bytes"]  # alone
    others = [r for i, r in enumerate(reps) if i != 2]
    assert all(budget // 8 < r["mem_bytes"] < budget for r in others)
    assert all(r["mem_in_use"] <= budget for r in others)
    assert sum(r["mem_bytes"] for r in others) > budget  # the budget, not the slots, bounded concurrency


def test_server_keeps_job_state_resident(rs):
    """A second request of the same job (another p-window) runs on the arrays
    the first one left on the device: no parse, plan or upload, same factors
    as standalone; with room for one idle job, a different job evicts it."""
    import rsieve.synth as S

    b, s, ks, nl = S.plain_job(1)
    plain = S.to_abcd(b, s, ks, nl)
    b2, s2, ks2, nl2 = S.plain_job(2)
    other = S.to_abcd(b2, s2, ks2, nl2)
    w = [(10**9, 10**9 + 10**7), (10**9 + 10**7 + 1, 10**9 + 2 * 10**7)]
    want = []
    for p0, p1 in w:
        with rs.Job(plain) as j:
            want.append(_key(j.sieve(p0, p1)[0]))
    with rs.Server(slots=1, cache_jobs=1) as srv:
        f, r1 = srv.wait(srv.submit(plain, *w[0]))
        assert _key(f) == want[0] and r1["resident"] == 0 and r1["create_ms"] > 0
        f, r2 = srv.wait(srv.submit(plain, *w[1]))
        assert _key(f) == want[1] and r2["resident"] == 1 and r2["create_ms"] == 0
        _, r3 = srv.wait(srv.submit(other, *w[0]))
        assert r3["resident"] == 0
        f, r4 = srv.wait(srv.submit(plain, *w[0]))
        assert _key(f) == want[0] and r4["resident"] == 0  # evicted by the other job
        _, r5 = srv.wait(srv.submit(plain, *w[0], datless=1))
        assert r5["resident"] == 0  # other options: another job
