"""Regenerate the golden fixtures in tests/golden/ from the reference checkout.

Run with the path of the reference's "CUDA Riesel Sieve" directory, as an
argument or in the environment variable RSIEVE_REFERENCE_DIR:
    python tests/golden/make_golden.py "<checkout>/CUDA Riesel Sieve"

Writes
  sr_745.abcd  the reference's own test input ("CUDA Riesel Sieve/sr_745.abcd"),
               copied byte for byte (data, not source).
  kat.json     known-answer facts read from the reference's files:
     - negative: the header of sr_745.abcd says "Sieved to 5000000000000", so no
       candidate of the file has a factor below 5e12;
     - datless:  kernel_v0.24.6.cu:244 names the debug prime 102297149781479;
       it divides 18300*745^242670-1 (n=242670 is not a candidate of the file);
     - structure: the reference's planner (kernel_v0.24.6.cu:1086-1255) picks
       Q=18 with 198 rows and x-range 3743, tMin=19, tMax=28 at -m 8, and the
       row order of its selection sort; recomputed here with the oracle's
       restatement and cross-checked against an independent Python restatement.
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RSIEVE_REFERENCE_DIR", "")
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))


def py_ref_plan(text: str, Qin: int = 0, hash_elems: int = 512):
    """Independent pure-Python restatement of kernel_v0.24.6.cu:1086-1255."""
    ks, ns, minN, maxN = [], [], 2**31 - 1, 0
    for line in text.splitlines():
        tok = line.split(" ")[0].strip()
        if tok == "ABCD":
            rest = line.split(" ", 1)[1]
            k = int(rest.split("*")[0])
            n0 = int(rest.split("[")[1].split("]")[0])
            ks.append(k)
            ns.append([n0])
            minN = min(minN, n0)
        elif tok:
            ns[-1].append(ns[-1][-1] + int(tok))
            maxN = max(maxN, ns[-1][-1])
    rng = maxN - minN
    minWork, minSubs, minRange, minQ = len(ks) * rng, len(ks), rng, 1
    qs = range(Qin, Qin + 1) if Qin else range(2, 24, 2)
    for Q in qs:
        subs = len({(i, n % Q) for i in range(len(ks)) for n in ns[i]})
        r = maxN // Q - minN // Q + 1
        if subs * r < minWork:
            minQ, minWork, minSubs, minRange = Q, subs * r, subs, r
    shift = hash_elems.bit_length() - 1
    tmin = (minN // minQ) >> shift
    tmax = (((maxN // minQ) + 1) >> shift) + 1
    rows = []
    for i, k in enumerate(ks):
        for n in ns[i]:
            if (k, n % minQ) not in rows:
                rows.append((k, n % minQ))
    INT_MAX = 2**31 - 1
    M = [list(r) for r in rows]
    order = []
    for _ in range(len(M)):
        km = rm = INT_MAX
        idx = 0
        for j, (k, r) in enumerate(M):
            if k <= km and k != INT_MAX and r < rm:
                km, rm, idx = k, r, j
        order.append(tuple(M[idx]))
        M[idx][0] = INT_MAX
    return dict(Q=minQ, rows=minSubs, x_range=minRange, tmin=tmin, tmax=tmax, order=order)


def main() -> None:
    src = os.path.join(REF, "sr_745.abcd")
    dst = os.path.join(HERE, "sr_745.abcd")
    shutil.copyfile(src, dst)
    text = open(dst).read()
    digest = hashlib.sha256(open(dst, "rb").read()).hexdigest()
    header = text.splitlines()[0]
    sieved_to = int(re.search(r"Sieved to (\d+)", header).group(1))
    kern = open(os.path.join(REF, "kernel_v0.24.6.cu")).read().splitlines()
    dbg = re.search(r"\(unsigned int\)(\d+)\)", kern[243]).group(1)  # line 244
    plan = py_ref_plan(text, 0, 512)
    import oracle as O  # noqa: E402

    job = O.Job.from_abcd(text)
    op = job.ref_plan(0, 512)
    assert (op.Q, op.rows, op.x_range, op.tmin, op.tmax) == (plan["Q"], plan["rows"], plan["x_range"],
                                                             plan["tmin"], plan["tmax"])
    assert list(zip(op.row_k, op.row_r)) == plan["order"]
    p = int(dbg)
    hits = [(k, n) for k in job.ks for n in [242670] if pow(745, n, p) * k % p == 1]
    kat = {
        "sr_745_sha256": digest,
        "negative": {"file": "sr_745.abcd", "sieved_to": sieved_to,
                     "source": "sr_745.abcd:1 header"},
        "datless": {"p": p, "k": 18300, "b": 745, "n": 242670, "candidate": False,
                    "source": "kernel_v0.24.6.cu:244 (debug prime)", "check": hits},
        "structure": {"hash_elems": 512, "Q": plan["Q"], "rows": plan["rows"], "x_range": plan["x_range"],
                      "tmin": plan["tmin"], "tmax": plan["tmax"], "row_order": plan["order"],
                      "source": "kernel_v0.24.6.cu:1086-1255"},
        "default_range": {"low": 102297149770000, "width_per_scale": 2500000,
                          "source": "kernel_v0.24.6.cu:837-839"},
    }
    with open(os.path.join(HERE, "kat.json"), "w") as f:
        json.dump(kat, f, indent=1)
    print("wrote", dst, "and kat.json")


if __name__ == "__main__":
    if not REF or not os.path.isfile(os.path.join(REF, "kernel_v0.24.6.cu")):
        sys.exit("usage: make_golden.py <reference 'CUDA Riesel Sieve' directory> (or RSIEVE_REFERENCE_DIR)")
    main()
