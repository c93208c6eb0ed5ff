"""The served form (rs_server_*): jobs submitted together run concurrently on
the GPU, and each job's factors are the same as when it runs alone through
rs_job_create_abcd + rs_sieve_range.  Also the queue limit (RS_ERR_BUSY) and
the wait timeout (RS_ERR_TIMEOUT)."""
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
    with rs.Server(slots=2) as srv:
        bad = srv.submit("ABCD 3*2^$a-1 [x]\n", 10**9, 10**9 + 10**5)
        good = srv.submit("ABCD 3*2^$a-1 [10]\n2\n4\n", 10**9, 10**9 + 10**5)
        with pytest.raises(rs.RsieveError) as e:
            srv.wait(bad)
        assert e.value.code == rs.RS_ERR_INVALID
        f, rep = srv.wait(good)
        assert rep["status"] == rs.RS_OK
        assert isinstance(f, np.ndarray)
