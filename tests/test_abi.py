"""The C ABI library: builds, loads, exports every declared symbol, and its
host-only logic (ABCD parsing, planning, argument checks) works without a GPU."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT


def _declared():
    text = open(os.path.join(ROOT, "include", "rsieve.h")).read()
    return sorted(set(re.findall(r"\b(rs_[a-z_0-9]+)\s*\(", text)))


def test_exports_match_header(rs):
    names = _declared()
    assert set(names) == set(rs.EXPORTS)
    lib = ctypes.CDLL(rs.LIB)
    for n in names:
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", rs.LIB], capture_output=True, text=True).stdout
    for n in names:
        assert re.search(r"\bT " + n + r"\b", out), n


def test_version(rs):
    assert "sm_103a" in rs.version()


def test_plan_sr745(rs, sr745_text):
    info = rs.plan_abcd(sr745_text)
    assert info["base"] == 745 and info["sign"] == -1
    assert info["num_k"] == 22 and info["num_candidates"] == 65111
    assert info["nmin"] == 182644 and info["nmax"] == 250000
    # the plan covers the whole x range: m*T >= X
    assert info["baby_steps"] * info["giant_steps"] >= info["x_range"]
    assert info["table_slots"] >= 2 * info["baby_steps"]
    forced = rs.plan_abcd(sr745_text, Q=18)
    assert forced["Q"] == 18 and forced["rows"] == 198 and forced["x_range"] == 3743


def test_plan_forced_m(rs, sr745_text):
    info = rs.plan_abcd(sr745_text, hash_m=6, Q=2)
    assert info["baby_steps"] <= 2 << 6
    assert info["baby_steps"] * info["giant_steps"] >= info["x_range"]


def test_plan_datless_rows(rs):
    txt = "ABCD 5*3^$a-1 [100]\n6\n6\n"
    assert rs.plan_abcd(txt, Q=6)["rows"] == 1
    assert rs.plan_abcd(txt, Q=6, datless=1)["rows"] == 6


@pytest.mark.parametrize("bad", [
    "12\n",
    "ABCD 3*2^$a-1 [10]\n0\n",
    "ABCD x*2^$a-1 [10]\n",
    "ABCD 3*2^$a-1 10\n",
    "",
])
def test_plan_rejects_malformed(rs, bad):
    with pytest.raises(rs.RsieveError) as e:
        rs.plan_abcd(bad)
    assert e.value.code == rs.RS_ERR_INVALID


def test_plan_sierpinski_and_crlf(rs):
    info = rs.plan_abcd("ABCD 7*2^$a+1 [10]\r\n2\r\n\r\n3\r\n")
    assert info["sign"] == 1 and info["num_candidates"] == 3 and info["nmax"] == 15


def _py_parse(text):
    """Plain restatement of the ABCD reading: per-k sorted, de-duplicated n."""
    seqs, cur, total = {}, None, 0
    for raw in text.split("\n"):
        ln = raw.strip(" \t\r")
        if not ln:
            continue
        if ln.startswith("ABCD"):
            k = int(ln[5:].split("*")[0])
            n0 = int(ln.split("[")[1].split("]")[0])
            cur, total = seqs.setdefault(k, set()), n0
            cur.add(n0)
        else:
            total += int(ln)
            cur.add(total)
    return {k: sorted(v) for k, v in seqs.items()}


@pytest.mark.parametrize("seed", range(6))
def test_abcd_parse_fuzz(rs, seed):
    """The reader (8-byte fast path for short delta lines, general path for the
    rest) against a plain restatement: deltas of 1 to 10 digits with leading
    zeros, CRLF endings, blanks, blank lines, header comments, repeated k, and
    files that end with or without a newline (the fast path needs 8 readable
    bytes)."""
    import numpy as np

    rng = np.random.default_rng(seed)
    parts = []
    for _ in range(int(rng.integers(1, 6))):
        k = int(rng.choice([3, 5, 7, 9, 11]))
        n = int(rng.integers(1, 1000))
        parts.append(f"ABCD {k}*2^$a-1 [{n}]" + (" // comment" if rng.random() < 0.3 else ""))
        for _ in range(int(rng.integers(0, 400))):
            nd = int(rng.choice([1, 1, 2, 2, 3, 4, 5, 6, 7, 8, 9, 10], p=None))
            d = int(rng.integers(1, 10 ** min(nd, 6)))
            if n + d > 2**31 - 1:
                break
            n += d
            s = str(d)
            if rng.random() < 0.1:
                s = "0" * int(rng.integers(1, 3)) + s
            if rng.random() < 0.05:
                s = s + " "
            if rng.random() < 0.05:
                s = s + "\r"
            parts.append(s)
            if rng.random() < 0.03:
                parts.append("")
    text = "\n".join(parts) + ("\n" if seed % 2 == 0 else "")
    want = _py_parse(text)
    out = rs.abcd_remove(text, [], 1)
    assert _py_parse(out) == want
    info = rs.plan_abcd(text)
    allv = [n for v in want.values() for n in v]
    assert info["num_k"] == len(want) and info["num_candidates"] == len(allv)
    assert (info["nmin"], info["nmax"]) == (min(allv), max(allv))


def test_abcd_parse_large_file(rs):
    """A file large enough to be read in pieces on several cores: the same
    sequences as the plain restatement, and an error in a late piece reports
    the line the serial reader reports."""
    import numpy as np

    rng = np.random.default_rng(5)
    parts = []
    for k in range(3, 3 + 2 * 600, 2):
        n = int(rng.integers(1, 1000))
        parts.append(f"ABCD {k}*5^$a-1 [{n}]")
        d = rng.integers(1, 200, size=int(rng.integers(3000, 9000)))
        parts.extend(map(str, d.tolist()))
        if k % 7 == 0:
            parts.append("")
    text = "\n".join(parts) + "\n"
    assert len(text) > 9 * 2**20
    want = _py_parse(text)
    allv = [n for v in want.values() for n in v]
    info = rs.plan_abcd(text)
    assert info["num_k"] == len(want) and info["num_candidates"] == len(allv)
    assert (info["nmin"], info["nmax"]) == (min(allv), max(allv))
    assert _py_parse(rs.abcd_remove(text, [], 1)) == want
    bad_line = len(parts) - 5
    broken = "\n".join(parts[: bad_line - 1] + ["x12"] + parts[bad_line:]) + "\n"
    with pytest.raises(rs.RsieveError) as e:
        rs.plan_abcd(broken)
    assert e.value.code == rs.RS_ERR_INVALID and f"line {bad_line}:" in str(e.value)


def test_no_cpu_fallback(rs):
    """Without a GPU the library refuses work instead of computing on the CPU."""
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("GPU present")
    except ImportError:
        pass
    with pytest.raises(rs.RsieveError) as e:
        rs.Job("ABCD 3*2^$a-1 [10]\n2\n")
    assert e.value.code == rs.RS_ERR_NODEVICE
    with pytest.raises(rs.RsieveError):
        rs.gpu_primes(3, 1000)
    with pytest.raises(rs.RsieveError) as e:
        rs.Server()
    assert e.value.code == rs.RS_ERR_NODEVICE


def test_cli_help(rs):
    out = subprocess.run([rs.CLI, "-h"], capture_output=True, text=True)
    assert out.returncode == 0 and "-Q Q" in out.stdout


def test_cli_rejects_odd_q(rs, tmp_path):
    out = subprocess.run([rs.CLI, "-Q", "3"], capture_output=True, text=True, cwd=tmp_path)
    assert out.returncode == 1 and "Q must be an even integer" in out.stdout


def test_abcd_remove_round_trip(rs, oracle_mod, sr745_text):
    """Sieve-file update: removed (k, n) disappear, everything else survives."""
    import numpy as np

    job = oracle_mod.Job.from_abcd(sr745_text)
    ks = job.ks
    removed = [(ks[0], int(job.nlist(0)[0])), (ks[0], int(job.nlist(0)[5])), (ks[3], int(job.nlist(3)[-1]))]
    # a k whose every candidate is removed disappears
    tiny = "ABCD 3*2^$a-1 [10]\n2\nABCD 5*2^$a-1 [11]\n"
    out_tiny = rs.abcd_remove(tiny, np.array([(0, 5, 11, 0, 0)], dtype=rs.FACTOR_DTYPE), 10**9)
    assert "5*2" not in out_tiny and out_tiny.startswith("ABCD 3*2^$a-1 [10] // Sieved to 1000000000\n2\n")
    f = np.array([(0, k, n, 0, 0) for k, n in removed], dtype=rs.FACTOR_DTYPE)
    out = rs.abcd_remove(sr745_text, f, 6 * 10**12)
    assert out.count("// Sieved to 6000000000000") == 22
    job2 = oracle_mod.Job.from_abcd(out)
    assert job2.ks == ks
    for i in range(len(ks)):
        want = set(job.nlist(i).tolist()) - {n for k, n in removed if k == ks[i]}
        assert set(job2.nlist(i).tolist()) == want
    # nothing removed: identical candidate sets
    job3 = oracle_mod.Job.from_abcd(rs.abcd_remove(sr745_text, [], 1))
    assert all(np.array_equal(job3.nlist(i), job.nlist(i)) for i in range(len(ks)))


def test_plan_layouts(rs):
    """The planner keeps the warp-per-prime layout for the plain job and picks a
    CTA per prime for the wide job, whose best table does not fit a warp."""
    import rsieve.synth as S

    d = rs.plan_abcd(S.to_abcd(*S.plain_job(1)))
    assert (d["Q"], d["baby_steps"], d["giant_steps"], d["warps_per_prime"]) == (2, 1152, 32, 1)
    # the wide job's shape: b=2, 1000 k, n in [1e6, 3e6] with every residue mod Q <= 48
    body = "\n".join(["1"] * 47 + [str(3 * 10**6 - 10**6 - 47)])
    wide = "".join(f"ABCD {k}*2^$a-1 [1000000]\n{body}\n" for k in range(3, 2003, 2))
    d = rs.plan_abcd(wide)
    assert d["warps_per_prime"] == 16 and d["baby_steps"] % 1024 == 0
    assert d["baby_steps"] * d["giant_steps"] >= d["x_range"]
    # expected false tag matches per prime stay well inside the CTA match list
    er = d["rows"] * (0.5 if d["Q"] % 2 == 0 else 0.75)
    assert er * d["giant_steps"] * d["baby_steps"] / (d["table_slots"] / 8) / 65536 <= 16
    # a CTA plan stays below 2^16 baby steps (a bucket's insert count is the low
    # half of its count word) at the largest -m values
    for hm in (12, 13, 14):
        d = rs.plan_abcd(wide, hash_m=hm)
        assert d["warps_per_prime"] == 1 or d["baby_steps"] < 65536


def test_plan_row_forms(rs, sr745_text):
    """Giant-step start values: an active-row mask for the plain job (44 rows,
    every k*745 < 2^32, a warp per prime), the integers k*b^r in the records
    for a warp-per-prime job with more than 64 rows, read by row id for the wide
    job and another CTA job with two giant steps per lane, per-prime residues for
    sr_745.abcd (Q = 18, so b^r is far above 2^32)."""
    import rsieve.synth as S

    assert rs.plan_abcd(S.to_abcd(*S.plain_job(1)))["row_form"] == 3
    (b, s, ks, nl), _ = S.batch_job(7, 48)
    d = rs.plan_abcd(S.to_abcd(b, s, ks, nl), datless=1)
    assert (d["row_form"], d["warps_per_prime"]) == (1, 1) and d["rows"] > 64
    body = "\n".join(["1"] * 47 + [str(3 * 10**6 - 10**6 - 47)])
    wide = "".join(f"ABCD {k}*2^$a-1 [1000000]\n{body}\n" for k in range(3, 2003, 2))
    d = rs.plan_abcd(wide)
    assert (d["row_form"], d["warps_per_prime"]) == (2, 16) and d["giant_steps"] >= 64
    (b, s, ks, nl), _ = S.batch_job(7, 8)
    d = rs.plan_abcd(S.to_abcd(b, s, ks, nl), datless=1)
    assert d["row_form"] == 2 and d["giant_steps"] >= 64
    d = rs.plan_abcd(sr745_text)
    assert d["Q"] > 2 and d["row_form"] == 0


def test_plan_per_sequence_bases(rs):
    """Headers with different bases and signs form parts (no longer an error)."""
    text = ("ABCD 3*2^$a-1 [10]\n2\n4\nABCD 5*10^$a+1 [7]\n3\nABCD 7*2^$a-1 [11]\n1\n"
            "ABCD 3*10^$a+1 [20]\n5\n")
    info = rs.plan_abcd(text)
    assert info["parts"] == 2 and info["num_k"] == 4 and info["num_candidates"] == 9
    assert (info["base"], info["sign"]) == (2, -1)


def test_abcd_remove_per_sequence_bases(rs):
    """Removal matches each factor's base and sign (b == 0 matches any)."""
    text = "ABCD 3*2^$a-1 [10]\n2\nABCD 3*10^$a-1 [10]\n2\n"
    f = np.array([(0, 3, 10, 2, -1)], dtype=rs.FACTOR_DTYPE)
    out = rs.abcd_remove(text, f, 10**9)
    assert "ABCD 3*2^$a-1 [12]" in out and "ABCD 3*10^$a-1 [10]" in out
    f = np.array([(0, 3, 10, 0, 0)], dtype=rs.FACTOR_DTYPE)
    out = rs.abcd_remove(text, f, 10**9)
    assert "ABCD 3*2^$a-1 [12]" in out and "ABCD 3*10^$a-1 [12]" in out
