"""Benchmark: p/sec of the plain sieve on the steady-state workload.

Workload ("plain_steady"): base 745, 22 seeded odd k in [3, 1e6], n in
[180000, 250000] kept at 5%, every prime p in [1e13, 1e13 + 1e11).  One step =
one 1e10-wide slice of that window through the hot path (device prime sieve ->
per-prime setup -> BSGS -> verify).  Step i sieves slice i mod 10, so the
default 10 timed steps cover the whole window once and more steps go round it
again: every sieved p lies inside the stated window.  Metric p/sec = width of
the p-interval sieved per second, the reference's definition
(kernel_v0.24.6.cu:1552-1554,1783).

  value  device time: summed CUDA-event time of each rs_sieve_range call, from
         its first kernel to its last, job resident in HBM.
  e2e    the same through the C ABI from host buffers, over the same steps and
         slices: per step, create the job from its ABCD text (H2D upload), sieve
         the slice, copy the factors back (D2H), destroy the job; host wall
         clock around it.

--workload wide / sr745 measure the wide job near 2^50 or the reference's own
file sr_745.abcd from the reference's default low bound instead.

Extra keys: roofline (the BSGS kernel against this GPU's measured integer
multiply throughput), cpu_baseline (the CPU oracle on a bounded sub-window),
clocks (nvidia-smi sampled during the timed region), gpu_launches.

--served runs the batched and served forms instead (see run_served).

--impl reference times the reference's CPU path for the same metric.  The
reference sieve (kernel_v0.24.6.cu) has no CPU implementation, so this arm runs
the project's scalar CPU oracle (oracle/), all host cores, a bounded
sub-window per step.

Multi-GPU (torchrun, N>1): weak scaling, rank r sieves its own slices
(step*N + r); no data-path collective, only a barrier and a max over ranks of
the elapsed time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "cuda-riesel-sieve_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "p/sec (b=745, 22 k, n 180k–250k)"
UNIT = "p/sec"
P_START = 10**13
WINDOW = 10**11
SLICE = 10**10
MONTMUL_MULS = 19  # 32-bit multiply-class PTX instructions per 64-bit Montgomery product
WORKLOAD = ("plain_steady: b=745, 22 seeded odd k in [3,1e6], n in [180000,250000] at 5% density, "
            "all primes p in [1e13, 1e13+1e11)")
JOB = "plain_job"

# Other workloads, measured on request (the default line is the plain
# steady-state workload):
#   wide   the wide-n, many-k job near 2^50
#   sr745  the reference's own file sr_745.abcd (the file its published p/sec
#          figures are quoted on, README.md:12-20) from the reference's default
#          low bound 102297149770000 (kernel_v0.24.6.cu:836)
WORKLOADS = {
    "wide": {
        "METRIC": "p/sec (b=2, 1000 k, n 1e6–3e6)", "P_START": 1 << 50, "WINDOW": 5 * 10**10, "SLICE": 5 * 10**9,
        "WORKLOAD": ("wide: b=2, 1000 seeded odd k in [3,1e7], n in [1e6,3e6] at 2% density, "
                     "all primes p in [2^50, 2^50+5e10)"),
        "JOB": "wide_job", "PROFILE": "bsgs_cta_kernel.wide.txt",
    },
    "sr745": {
        "METRIC": "p/sec (sr_745.abcd: b=745, 22 k, n 182644–250000)", "P_START": 102297149770000,
        "WINDOW": 10**11, "SLICE": 10**10,
        "WORKLOAD": ("sr745: the reference's sr_745.abcd (65111 candidates), all primes p in "
                     "[102297149770000, 102297149770000+1e11)"),
        "JOB": "sr745", "PROFILE": None,
    },
}
PROFILE = "bsgs_kernel.plain_steady.txt"  # committed ncu summary with the BSGS kernel's DRAM bytes per prime


def select_workload(name: str) -> None:
    if name in WORKLOADS:
        globals().update(WORKLOADS[name])


def workload_abcd() -> str:
    """The workload's job as ABCD text (seeded synthetic, or the reference's own file)."""
    if JOB == "sr745":
        with open(os.path.join(ROOT, "tests", "golden", "sr_745.abcd")) as f:
            return f.read()
    import rsieve.synth as S

    b, s, ks, nl = getattr(S, JOB)(1)
    return S.to_abcd(b, s, ks, nl)


def slice_start(idx: int, slice_w: int) -> int:
    """Start of slice idx, wrapped so that every slice lies inside [P_START, P_START + WINDOW)."""
    per = max(1, WINDOW // slice_w)
    return P_START + (idx % per) * slice_w


def bsgs_bytes_per_prime():
    """DRAM bytes per prime of the BSGS kernel from the committed ncu summary."""
    if not PROFILE:
        return None
    path = os.path.join(ROOT, "profiles", PROFILE)
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_prime:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Barrier and max-reduction across ranks (torch.distributed when N > 1)."""

    def __init__(self, world: int, local: int, backend: str):
        self.world = world
        self.pg = None
        if world > 1:
            import torch
            import torch.distributed as dist

            if backend == "nccl":
                torch.cuda.set_device(local)
            dist.init_process_group(backend=backend)
            self.pg = dist
            self.torch = torch

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        t = self.torch.tensor([v], dtype=self.torch.float64,
                              device="cuda" if self.pg.get_backend() == "nccl" else "cpu")
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if not self.pg:
            return v
        t = self.torch.tensor([v], dtype=self.torch.float64,
                              device="cuda" if self.pg.get_backend() == "nccl" else "cpu")
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(abcd: str, seconds: float = 12.0) -> dict:
    """The CPU oracle on a sub-window of the workload's window, all host threads."""
    import oracle

    oj = oracle.Job.from_abcd(abcd)
    threads = oracle.default_threads()
    w0 = 2 * 10**6
    t = time.perf_counter()
    oj.sieve(P_START, P_START + w0 - 1, threads=threads)
    dt = max(time.perf_counter() - t, 1e-3)
    width = int(min(5 * 10**8, max(w0, w0 * seconds / dt)))
    t = time.perf_counter()
    f, npr = oj.sieve(P_START + w0, P_START + w0 + width - 1, threads=threads)
    dt = time.perf_counter() - t
    return {"value": width / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"p in [{P_START}+{w0}, +{width}) ({npr} primes, {len(f)} factors), {dt:.1f} s"}


def run_reference(args, rank: int) -> None:
    """The reference arm: the CPU oracle (the reference's sieve is CUDA-only)."""
    if rank != 0:
        return
    import oracle

    oracle.build()
    oj = oracle.Job.from_abcd(workload_abcd())
    threads = oracle.default_threads()
    # per-step sample sized to ~3 s of CPU work
    w0 = 10**6
    t = time.perf_counter()
    oj.sieve(P_START, P_START + w0 - 1, threads=threads)
    dt = max(time.perf_counter() - t, 1e-3)
    width = int(min(2 * 10**8, max(w0, w0 * 3.0 / dt)))
    a = P_START + w0
    for _ in range(args.warmup):
        oj.sieve(a, a + width // 4 - 1, threads=threads)
        a += width // 4
    t = time.perf_counter()
    tot_f = tot_p = 0
    for _ in range(args.steps):
        f, npr = oj.sieve(a, a + width - 1, threads=threads)
        tot_f += len(f)
        tot_p += npr
        a += width
    dt = time.perf_counter() - t
    value = args.steps * width / dt
    sample = (f"{args.steps} steps of {width}-wide windows of the workload from {P_START} "
              f"({tot_p} primes, {tot_f} factors)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(1, args.steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded)", "config": {"workload": WORKLOAD, "sample_width": width},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": ("the reference sieve (kernel_v0.24.6.cu) has no CPU path; this arm is the scalar "
                 "CPU BSGS oracle restating it, all host threads"),
    }))


def run_served(args) -> None:
    """--served: the batched and served forms on the mixed-job stream.

    Jobs are drawn from the mixed-batch distribution (rsieve/synth.py
    batch_job: base in [2, 1024] without perfect powers, 1-1000 k, n windows
    of 1e4-2e6 at 1-10%, a p-window starting uniform in [1e12, 2^60]).  Each
    job's p-window is requested in --served-splits consecutive parts, all
    first parts before any second part, so that a job's later requests find
    its state resident on the device.  Three runs over the same requests:
    plain (one job after another through rs_job_create_abcd + rs_sieve_range,
    every part of a job on the same job object), batched (all requests
    submitted to an rs_server at once) and served (Poisson arrivals at a sweep
    of loads relative to the batched capacity, repeated --served-repeats
    times).  Beside them, the persistent batched launch (rs_batch: every job's
    whole window in one batch, one BSGS launch per kernel variant per round),
    and plain once more at the persistent run's chunk budget (1 GiB a job).
    Every request's factors in the batched, persistent and served runs are
    checked equal to the plain run.  Latencies are the server's own
    submit-to-finish times.
    """
    import threading

    import numpy as np

    import rsieve
    import rsieve.synth as S

    rsieve.build()
    n, width, splits = args.served_jobs, int(args.served_window), max(1, args.served_splits)
    jobs = []
    for i in range(n):
        (b, s, ks, nl), (p0, _) = S.batch_job(1, i)
        jobs.append((S.to_abcd(b, s, ks, nl), p0, p0 + width - 1))
    part = width // splits
    # requests (job, part): every job's first part, then every second part, ...
    reqs = [(i, q) for q in range(splits) for i in range(n)]

    def window(i, q):
        _, p0, p1 = jobs[i]
        a = p0 + q * part
        return a, (p1 if q == splits - 1 else a + part - 1)

    total_width = n * width

    def key(f):
        return [(int(x["p"]), int(x["k"]), int(x["n"])) for x in f]

    # warm-up: the shared sieving primes up to sqrt of the largest p, module load
    top = max(jobs, key=lambda j: j[2])
    with rsieve.Job(top[0]) as j:
        j.sieve(top[2] - 10**6, top[2])
    t0 = time.perf_counter()
    plain = {}
    t_create = gpu_plain = 0.0
    for i, (abcd, _, _) in enumerate(jobs):
        tc = time.perf_counter()
        with rsieve.Job(abcd) as j:
            t_create += time.perf_counter() - tc
            for q in range(splits):
                f, st = j.sieve(*window(i, q))
                gpu_plain += st["gpu_ms"] / 1e3
                plain[(i, q)] = key(f)
    t_plain = time.perf_counter() - t0

    def run_server(arrivals):
        """Submit request r at arrivals[r] seconds (None: all at once); return (reports, span, all equal)."""
        m = len(reqs)
        reps = [None] * m
        same = [True]
        with rsieve.Server(slots=args.slots) as srv:
            tickets = []
            lock = threading.Lock()
            ready = threading.Semaphore(0)

            def collect():
                for r in range(m):
                    ready.acquire()
                    with lock:
                        t = tickets[r]
                    f, rep = srv.wait(t)
                    reps[r] = rep
                    if key(f) != plain[reqs[r]]:
                        same[0] = False

            th = threading.Thread(target=collect)
            th.start()
            start = time.perf_counter()
            for r, (i, q) in enumerate(reqs):
                if arrivals is not None:
                    delay = start + arrivals[r] - time.perf_counter()
                    if delay > 0:
                        time.sleep(delay)
                t = srv.submit(jobs[i][0], *window(i, q))
                with lock:
                    tickets.append(t)
                ready.release()
            th.join()
            span = time.perf_counter() - start
        return reps, span, same[0]

    # the persistent batched launch (rs_batch): every job's whole window in one
    # batch, one BSGS launch per kernel variant per round, rounds as CUDA graphs
    t0 = time.perf_counter()
    bjobs = [rsieve.Job(abcd, mem_limit=1 << 30) for abcd, _, _ in jobs]  # 1 GiB of chunk buffers each
    t_bcreate = time.perf_counter() - t0
    with rsieve.Batch() as bt:
        for j, (_, p0, p1) in zip(bjobs, jobs):
            bt.add(j, p0, p1)
        bst = bt.run()
        ok_persist = True
        for i in range(n):
            f, _ = bt.result(i)
            got = key(f)
            want = sorted(x for q in range(splits) for x in plain[(i, q)])
            ok_persist &= got == want
    t_persist = time.perf_counter() - t0
    for j in bjobs:
        j.close()
    # plain again at the persistent run's chunk budget (1 GiB a job): the same
    # chunks, one job's launches after another
    t0 = time.perf_counter()
    gpu_plain_1g = 0.0
    for abcd, p0, p1 in jobs:
        with rsieve.Job(abcd, mem_limit=1 << 30) as j:
            gpu_plain_1g += j.sieve(p0, p1)[1]["gpu_ms"] / 1e3
    t_plain_1g = time.perf_counter() - t0

    reps, t_batch, ok_batch = run_server(None)
    capacity = len(reqs) / t_batch  # requests per second
    served = []
    ok_served = True
    for rep_i in range(max(1, args.served_repeats)):
        for load in args.served_loads:
            rng = np.random.default_rng(1000 + 7919 * rep_i + int(load * 100))
            arrivals = np.cumsum(rng.exponential(1.0 / (load * capacity), size=len(reqs))).tolist()
            reps_l, span, ok = run_server(arrivals)
            ok_served &= ok
            lat = sorted(r["latency_ms"] for r in reps_l)
            served.append({"load": load, "repeat": rep_i, "p50_ms": float(np.percentile(lat, 50)),
                           "p99_ms": float(np.percentile(lat, 99)), "p_per_s": total_width / span, "span_s": span,
                           "resident_requests": int(sum(r["resident"] for r in reps_l)),
                           "peak_mem_in_use_gib": max(r["mem_in_use"] for r in reps_l) / 2**30})
    at1 = [x for x in served if abs(x["load"] - 1.0) < 1e-9]
    p99_at1 = [x["p99_ms"] for x in at1]
    out = {
        "metric": "served p99 job latency (mixed jobs, Poisson arrivals at 1.0x batched capacity)",
        "value": float(np.median(p99_at1)) if p99_at1 else None, "unit": "ms", "higher_is_better": False,
        "n_gpus": 1, "dtype": "u64", "data": "synthetic (seeded)",
        "config": {"workload": (f"{n} jobs of rsieve.synth.batch_job(1, i), p-window {width} wide each, "
                                f"requested in {splits} parts ({len(reqs)} requests)"),
                   "slots": args.slots, "mem_budget_gib": 64, "queue_cap": 1024},
        # create_s: host parse + plan + upload; gpu_s: summed device time of the sieve calls
        "plain": {"p_per_s": total_width / t_plain, "wall_s": t_plain, "create_s": t_create, "gpu_s": gpu_plain},
        "persistent": {"p_per_s": total_width / t_persist, "wall_s": t_persist, "vs_plain": t_plain / t_persist,
                       "create_s": t_bcreate, "gpu_s": bst["gpu_ms"] / 1e3, "bsgs_launches": bst["bsgs_launches"],
                       "results_match_plain": bool(ok_persist),
                       # one job after another at the same 1 GiB chunk budget
                       "plain_same_budget": {"wall_s": t_plain_1g, "gpu_s": gpu_plain_1g,
                                             "vs_it_wall": t_plain_1g / t_persist,
                                             "vs_it_gpu": gpu_plain_1g / (bst["gpu_ms"] / 1e3)}},
        "batched": {"p_per_s": total_width / t_batch, "wall_s": t_batch, "vs_plain": t_plain / t_batch,
                    "requests_per_s": capacity, "gpu_s": sum(r["gpu_ms"] for r in reps) / 1e3,
                    "resident_requests": int(sum(r["resident"] for r in reps))},
        "served": served,
        "p99_at_1x_ms": p99_at1,
        "results_match_plain": bool(ok_batch and ok_served and ok_persist),
    }
    print(json.dumps(out))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--workload", default="plain", choices=["plain"] + sorted(WORKLOADS))
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--slice", type=float, default=None, help="p-width of one step (default: the workload's)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--Q", type=int, default=0, help="force the subsequence modulus (default: planner)")
    ap.add_argument("--hash-m", type=int, default=0, help="cap baby steps at 2<<M (default: planner)")
    ap.add_argument("--served", action="store_true",
                    help="instead: plain vs batched vs served runs of the mixed-job stream (one JSON line)")
    ap.add_argument("--served-jobs", type=int, default=64)
    ap.add_argument("--served-window", type=float, default=1e9, help="p-window width of each job")
    ap.add_argument("--served-splits", type=int, default=2, help="requests per job (consecutive parts of its window)")
    ap.add_argument("--served-repeats", type=int, default=2, help="repeats of the served load sweep")
    ap.add_argument("--served-loads", type=float, nargs="*", default=[0.25, 0.5, 1.0, 1.5])
    ap.add_argument("--slots", type=int, default=4, help="jobs running at once in the served form")
    args = ap.parse_args()
    select_workload(args.workload)
    if args.slice is None:
        args.slice = SLICE
    if args.served:
        run_served(args)
        return
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank)
        return

    import rsieve

    rsieve.build()
    dist = Dist(world, local, "nccl")
    dev = local
    slice_w = int(args.slice)
    abcd = workload_abcd()

    # roofline denominator: this GPU's measured rate of 64-bit modular products
    rates = rsieve.bench_products(dev)
    mul_ops = rates["mad_lo_u32"]
    modmul_per_s = max(rates["montmul"], rates["montmul_ptx"], rates["shoup"])

    job = rsieve.Job(abcd, device=dev, Q=args.Q, hash_m=args.hash_m)
    info = job.info
    # warm-up: slices just below the window
    for w in range(args.warmup):
        a = P_START - (w + 1) * (slice_w // 10)
        job.sieve(a, a + slice_w // 10 - 1)

    sampler = ClockSampler(dev)
    dist.barrier()
    sampler.start()
    t0 = time.perf_counter()
    gpu_ms = bsgs_ms = setup_ms = sieve_ms = exact_ms = 0.0
    primes = launches = bsgs_launches = factors = 0
    covered = set()
    for step in range(args.steps):
        idx = step * world + rank
        a = slice_start(idx, slice_w)
        covered.add(a)
        f, st = job.sieve(a, a + slice_w - 1)
        gpu_ms += st["gpu_ms"]
        bsgs_ms += st["bsgs_ms"]
        setup_ms += st["setup_ms"]
        sieve_ms += st["sieve_ms"]
        exact_ms += st["exact_ms"]
        primes += st["primes"]
        launches += st["launches"]
        bsgs_launches += st["bsgs_launches"]
        factors += len(f)
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    dist.barrier()
    job.close()
    t_max = dist.max(gpu_ms / 1e3)
    total_width = world * args.steps * slice_w
    value = total_width / t_max

    # roofline of the BSGS kernel: algorithmic multiply ops / BSGS kernel time
    alg_ops = primes * info["work_per_prime"] * MONTMUL_MULS
    achieved = alg_ops / (bsgs_ms / 1e3) / 1e12
    peak = modmul_per_s * MONTMUL_MULS / 1e12
    bpp = bsgs_bytes_per_prime()
    traffic = None if bpp is None or not bsgs_launches else bpp * primes / bsgs_launches

    e2e = None
    if not args.no_e2e:
        dist.barrier()
        t0 = time.perf_counter()
        h2d = d2h = 0
        e2e_steps = args.steps
        for step in range(e2e_steps):
            idx = step * world + rank
            a = slice_start(idx, slice_w)
            with rsieve.Job(abcd, device=dev, Q=args.Q, hash_m=args.hash_m) as j2:
                f, st = j2.sieve(a, a + slice_w - 1)
                h2d += j2.info["upload_bytes"] + st["h2d_bytes"]
                d2h += st["d2h_bytes"]
        e2e_t = dist.max(time.perf_counter() - t0)
        e2e = {"value": world * e2e_steps * slice_w / e2e_t, "unit": UNIT,
               "h2d_bytes_per_step": h2d // e2e_steps, "d2h_bytes_per_step": d2h // e2e_steps,
               "steps": e2e_steps}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(abcd)
    dist.close()
    if rank != 0:
        return
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": gpu_ms / max(1, args.steps), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded)",
        "config": {
            "workload": WORKLOAD, "slice_width": slice_w,
            "sieved": (f"{args.steps} slices of {slice_w} per rank, {len(covered)} distinct, all inside "
                       f"[{P_START}, {P_START + WINDOW})"),
            "plan": {
                k: info[k] for k in ("Q", "rows", "x_range", "baby_steps", "giant_steps", "table_slots",
                                     "primes_per_launch", "warps_per_prime")},
            "l2": ("no flush: each step streams the per-prime records of a fresh prime window (GBs, > 129 MB L2); "
                   "the job tables stay resident by design"),
            "parallelism": f"p-range shards x{world}, no collective",
        },
        "roofline": {
            "bound": "imad", "achieved": achieved, "peak": peak, "unit": "Tops/s", "frac": achieved / peak,
            "traffic": traffic,
            "traffic_unit": "DRAM bytes per BSGS launch (ncu dram__bytes_read+write per prime x primes per launch)",
            "what": ("32-bit multiply-class ops of the algorithmic BSGS work (2*sqrt(E[R]*X) Montgomery "
                     f"products per prime = {info['work_per_prime']:.0f}, x{MONTMUL_MULS} ops) per second of "
                     "BSGS kernel time"),
            "peak_source": ("measured this run by rs_bench_products: the fastest 64-bit modular product on "
                            "this GPU from independent chains, max(Montgomery in C "
                            f"{rates['montmul']:.3e}/s, Montgomery in inline PTX {rates['montmul_ptx']:.3e}/s, "
                            f"Shoup {rates['shoup']:.3e}/s) x{MONTMUL_MULS}; plain mad.lo.u32 peak "
                            f"{mul_ops / 1e12:.1f} Tops/s"),
            "product_rates": rates,
        },
        "e2e": e2e,
        "cpu_baseline": cpu,
        "clocks": clocks,
        "gpu_launches": launches,
        "detail": {"primes": primes, "factors": factors, "bsgs_ms": bsgs_ms, "gpu_ms": gpu_ms,
                   "setup_ms": setup_ms, "sieve_ms": sieve_ms, "exact_ms": exact_ms,
                   "wall_s": wall, "bsgs_launches": bsgs_launches,
                   "bsgs_share": bsgs_ms / gpu_ms if gpu_ms else None},
    }
    print(json.dumps(out))


if __name__ == "__main__":
    main()
