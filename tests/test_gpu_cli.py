"""The rsieve CLI as a drop-in for the reference executable (GPU): the
reference's flags and factor-file format, datless KAT through the CLI,
checkpoint/resume and the sieve-file update."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

LINE = re.compile(r"^(\d+) \| (\d+)\*(\d+)\^(\d+)([-+])1$")


def _fnv1a(data: bytes) -> int:
    """The CLI's checkpoint hash of the input file's contents (64-bit FNV-1a)."""
    h = 1469598103934665603
    for c in data:
        h = ((h ^ c) * 1099511628211) & (2**64 - 1)
    return h


def _factors(path):
    out = []
    for line in open(path):
        m = LINE.match(line.rstrip("\n"))
        assert m, line
        out.append(tuple(int(m.group(i)) for i in (1, 2, 3, 4)) + (-1 if m.group(5) == "-" else 1,))
    return out


def test_cli_datless_kat_and_format(rs, oracle_mod, kat, tmp_path):
    d = kat["datless"]
    lo = kat["default_range"]["low"]
    abcd = os.path.join(GOLDEN, "sr_745.abcd")
    r = subprocess.run([rs.CLI, "-i", abcd, "-p", str(lo), "-P", str(lo + 2500000), "-v", "-O", "f.txt"],
                       capture_output=True, text=True, cwd=tmp_path, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Progress = 2500001 at" in r.stdout
    fac = _factors(tmp_path / "f.txt")
    assert (d["p"], d["k"], 745, d["n"], -1) in fac
    for p, k, b, n, sg in fac:
        assert lo <= p <= lo + 2500000 and oracle_mod.verify(p, k, b, n, sg)


def test_cli_checkpoint_resume_and_abcd_update(rs, oracle_mod, tmp_path):
    import rsieve.synth as S

    b, s, ks, nl = S.plain_job(4)
    (tmp_path / "job.abcd").write_text(S.to_abcd(b, s, ks, nl))
    lo, hi = 10**9, 10**9 + 30 * 10**6
    base = [rs.CLI, "-i", "job.abcd", "-p", str(lo), "-P", str(hi), "-b", "1", "-t", "1"]
    # one uninterrupted run
    r = subprocess.run(base + ["-O", "full.txt", "-w", "out.abcd"], capture_output=True, text=True, cwd=tmp_path,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    full = _factors(tmp_path / "full.txt")
    oj = oracle_mod.Job.from_arrays(b, s, ks, [np.asarray(x) for x in nl])
    want, _ = oj.sieve(lo, hi)
    assert [(p, k, n) for p, k, _, n, _ in full] == [tuple(map(int, x)) for x in want]
    assert len(full) > 0
    # resume from a checkpoint in the middle: only the second half is sieved
    mid = lo + 17 * 10**6 + 1
    h = _fnv1a((tmp_path / "job.abcd").read_bytes())
    # a checkpoint of other file contents (or another P0) is not resumed
    for bad in (f"low={lo}\nabcd_hash={h ^ 1:016x}\n", f"low={lo + 2}\nabcd_hash={h:016x}\n"):
        (tmp_path / "ck").write_text(f"next_p={mid}\nhigh={hi}\n{bad}abcd=job.abcd\n")
        r = subprocess.run(base + ["-O", "ignored.txt", "-C", "ck"], capture_output=True, text=True, cwd=tmp_path,
                           timeout=300)
        assert r.returncode == 0 and "Resuming" not in r.stdout and "another input" in r.stdout, r.stderr
    (tmp_path / "ck").write_text(f"next_p={mid}\nlow={lo}\nhigh={hi}\nabcd_hash={h:016x}\nabcd=job.abcd\n")
    r = subprocess.run(base + ["-O", "half.txt", "-C", "ck"], capture_output=True, text=True, cwd=tmp_path,
                       timeout=300)
    assert r.returncode == 0 and "Resuming from checkpoint" in r.stdout, r.stderr
    half = _factors(tmp_path / "half.txt") if os.path.exists(tmp_path / "half.txt") else []
    assert half == [f for f in full if f[0] >= mid]
    assert (tmp_path / "ck").read_text().startswith(f"next_p={hi + 1}\n")
    # a finished checkpoint sieves nothing more
    r = subprocess.run(base + ["-O", "again.txt", "-C", "ck"], capture_output=True, text=True, cwd=tmp_path,
                       timeout=300)
    assert r.returncode == 0 and not os.path.exists(tmp_path / "again.txt")
    # the updated sieve file lacks exactly the factored candidates
    oj2 = oracle_mod.Job.from_abcd((tmp_path / "out.abcd").read_text())
    removed = {(k, n) for _, k, _, n, _ in full}
    cand = {(int(k), int(n)) for k, ns in zip(ks, nl) for n in ns}
    left = {(k, int(n)) for i, k in enumerate(oj2.ks) for n in oj2.nlist(i)}
    assert left == cand - removed


def test_cli_autotune_same_factors(rs, tmp_path):
    """-A picks a layout by measurement; the factor file is the same as without it."""
    import rsieve.synth as S

    b, s, ks, nl = S.plain_job(4)
    (tmp_path / "job.abcd").write_text(S.to_abcd(b, s, ks, nl))
    lo, hi = 10**9, 10**9 + 20 * 10**6
    base = [rs.CLI, "-i", "job.abcd", "-p", str(lo), "-P", str(hi)]
    r1 = subprocess.run(base + ["-O", "plain.txt"], capture_output=True, text=True, cwd=tmp_path, timeout=300)
    r2 = subprocess.run(base + ["-A", "-O", "tuned.txt"], capture_output=True, text=True, cwd=tmp_path, timeout=300)
    assert r1.returncode == 0 and r2.returncode == 0, (r1.stderr, r2.stderr)
    assert "Autotuned on [" in r2.stdout
    assert sorted(_factors(tmp_path / "plain.txt")) == sorted(_factors(tmp_path / "tuned.txt"))
    assert _factors(tmp_path / "plain.txt")
