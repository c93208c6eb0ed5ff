"""Python binding of librsieve_gb300 (the C ABI in include/rsieve.h), via ctypes.

This is a thin mirror of the C entry points for tests and benchmarks; the
product is the shared library and the ``rsieve`` CLI.  There is no CPU path:
if the library is missing or no GPU is present, calls raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .build import BUILD, CLI, LIB, build  # noqa: F401

RS_OK = 0
RS_ERR_INVALID = 1
RS_ERR_CUDA = 2
RS_ERR_NOMEM = 3
RS_ERR_RANGE = 4
RS_ERR_NODEVICE = 5
RS_ERR_CAPACITY = 6
RS_ERR_INTERNAL = 7
RS_ERR_BUSY = 8
RS_ERR_TIMEOUT = 9

# rs_options.baby_step
BABY_AUTO, BABY_SHOUP, BABY_SHORT, BABY_HIGH = 0, 1, 2, 3
# rs_options.char_tables: when the per-k quadratic-character tables are built
TABLES_AUTO, TABLES_ALWAYS, TABLES_NEVER = 0, 1, 2

# rs_gpu_modmul_check operations
OPS = {"montmul": 0, "from_mont": 1, "shoup_const": 2, "shoup": 3, "shoup32": 4, "shoup_w32": 5,
       "mul_small": 6, "pinv": 7, "one": 8, "r2": 9, "pow": 10, "montmul_ptx": 11}
PRODUCT_RATES = ("mad_lo_u32", "montmul", "montmul_ptx", "shoup", "shoup32", "mul_small")

# rs_factor: p | k*b^n+c
FACTOR_DTYPE = np.dtype([("p", "<u8"), ("k", "<u4"), ("n", "<u4"), ("b", "<u4"), ("c", "<i4")])

# Every entry point declared in include/rsieve.h.
EXPORTS = (
    "rs_options_default", "rs_job_create_abcd", "rs_job_create", "rs_job_info_get",
    "rs_plan_abcd", "rs_job_destroy", "rs_sieve_range", "rs_write_factors", "rs_gpu_primes",
    "rs_bench_imad", "rs_gpu_arith_check", "rs_last_error", "rs_version", "rs_gpu_primes_static",
    "rs_abcd_remove", "rs_server_options_default", "rs_server_create", "rs_server_submit",
    "rs_server_wait", "rs_server_destroy", "rs_job_autotune", "rs_gpu_modmul_check", "rs_bench_products",
    "rs_batch_create", "rs_batch_add", "rs_batch_run", "rs_batch_result", "rs_batch_destroy",
)


class RsieveError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[rs error {code}] {msg}")
        self.code = code


class Options(ctypes.Structure):
    _fields_ = [
        ("Q", ctypes.c_int32),
        ("hash_m", ctypes.c_int32),
        ("block_scale", ctypes.c_int32),
        ("thread_scale", ctypes.c_int32),
        ("small_prime_scale", ctypes.c_int32),
        ("datless", ctypes.c_int32),
        ("host_verify", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("baby_step", ctypes.c_int32),
        ("char_tables", ctypes.c_int32),
        ("mem_limit", ctypes.c_uint64),
    ]


class JobInfo(ctypes.Structure):
    _fields_ = [
        ("base", ctypes.c_uint32),
        ("sign", ctypes.c_int32),
        ("num_k", ctypes.c_uint32),
        ("num_candidates", ctypes.c_uint32),
        ("nmin", ctypes.c_uint32),
        ("nmax", ctypes.c_uint32),
        ("Q", ctypes.c_uint32),
        ("rows", ctypes.c_uint32),
        ("x_range", ctypes.c_uint32),
        ("baby_steps", ctypes.c_uint32),
        ("giant_steps", ctypes.c_uint32),
        ("table_slots", ctypes.c_uint32),
        ("primes_per_launch", ctypes.c_uint32),
        ("work_per_prime", ctypes.c_double),
        ("upload_bytes", ctypes.c_uint64),
        ("warps_per_prime", ctypes.c_uint32),
        ("row_form", ctypes.c_uint32),
        ("parts", ctypes.c_uint32),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class Stats(ctypes.Structure):
    _fields_ = [
        ("primes", ctypes.c_uint64),
        ("raw_hits", ctypes.c_uint64),
        ("factors", ctypes.c_uint64),
        ("p_covered", ctypes.c_uint64),
        ("gpu_ms", ctypes.c_double),
        ("bsgs_ms", ctypes.c_double),
        ("sieve_ms", ctypes.c_double),
        ("setup_ms", ctypes.c_double),
        ("exact_ms", ctypes.c_double),
        ("launches", ctypes.c_uint32),
        ("bsgs_launches", ctypes.c_uint32),
        ("h2d_bytes", ctypes.c_uint64),
        ("d2h_bytes", ctypes.c_uint64),
        ("primes_by_step", ctypes.c_uint64 * 3),
        ("paired_primes", ctypes.c_uint64),
        ("exact_primes", ctypes.c_uint64),
    ]

    def as_dict(self) -> dict:
        d = {f: getattr(self, f) for f, _ in self._fields_}
        d["primes_by_step"] = {"shoup": d["primes_by_step"][0], "short": d["primes_by_step"][1],
                               "high": d["primes_by_step"][2]}
        return d


class ServerOptions(ctypes.Structure):
    _fields_ = [
        ("device", ctypes.c_int32),
        ("slots", ctypes.c_uint32),
        ("queue_cap", ctypes.c_uint32),
        ("cache_jobs", ctypes.c_uint32),
        ("mem_budget", ctypes.c_uint64),
    ]


class JobReport(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int32),
        ("resident", ctypes.c_uint32),
        ("primes", ctypes.c_uint64),
        ("factors", ctypes.c_uint64),
        ("p_covered", ctypes.c_uint64),
        ("queue_ms", ctypes.c_double),
        ("run_ms", ctypes.c_double),
        ("latency_ms", ctypes.c_double),
        ("gpu_ms", ctypes.c_double),
        ("create_ms", ctypes.c_double),
        ("mem_bytes", ctypes.c_uint64),
        ("mem_in_use", ctypes.c_uint64),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


_lib = None


def lib():
    """Load librsieve_gb300.so (building it first if needed)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        vp, u32, i32, u64, sz = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int32, ctypes.c_uint64, ctypes.c_size_t
        L.rs_options_default.argtypes = [ctypes.POINTER(Options)]
        L.rs_options_default.restype = None
        L.rs_job_create_abcd.argtypes = [ctypes.c_char_p, sz, ctypes.POINTER(Options), ctypes.POINTER(vp)]
        L.rs_job_create.argtypes = [u32, i32, u32, vp, vp, vp, ctypes.POINTER(Options), ctypes.POINTER(vp)]
        L.rs_job_info_get.argtypes = [vp, ctypes.POINTER(JobInfo)]
        L.rs_plan_abcd.argtypes = [ctypes.c_char_p, sz, ctypes.POINTER(Options), ctypes.POINTER(JobInfo)]
        L.rs_job_destroy.argtypes = [vp]
        L.rs_sieve_range.argtypes = [vp, u64, u64, vp, sz, ctypes.POINTER(sz), ctypes.POINTER(Stats)]
        L.rs_write_factors.argtypes = [vp, ctypes.c_char_p, vp, sz]
        L.rs_gpu_primes.argtypes = [u64, u64, vp, sz, ctypes.POINTER(sz), ctypes.c_int]
        L.rs_bench_imad.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                    ctypes.POINTER(ctypes.c_double)]
        L.rs_gpu_arith_check.argtypes = [vp, vp, vp, sz, vp, vp, ctypes.c_int]
        L.rs_gpu_modmul_check.argtypes = [i32, vp, vp, vp, vp, sz, vp, ctypes.c_int]
        L.rs_bench_products.argtypes = [ctypes.c_int, vp]
        L.rs_batch_create.argtypes = [ctypes.c_int, ctypes.POINTER(vp)]
        L.rs_batch_add.argtypes = [vp, vp, u64, u64, ctypes.POINTER(u32)]
        L.rs_batch_run.argtypes = [vp, ctypes.POINTER(Stats)]
        L.rs_batch_result.argtypes = [vp, u32, vp, sz, ctypes.POINTER(sz), ctypes.POINTER(Stats)]
        L.rs_batch_destroy.argtypes = [vp]
        L.rs_gpu_primes_static.argtypes = [u64, u64, vp, vp, u32, vp, u32, vp, vp]
        L.rs_abcd_remove.argtypes = [ctypes.c_char_p, sz, vp, sz, u64, vp, sz, ctypes.POINTER(sz)]
        L.rs_job_autotune.argtypes = [vp, u64, u64, u32, ctypes.POINTER(JobInfo)]
        L.rs_server_options_default.argtypes = [ctypes.POINTER(ServerOptions)]
        L.rs_server_options_default.restype = None
        L.rs_server_create.argtypes = [ctypes.POINTER(ServerOptions), ctypes.POINTER(vp)]
        L.rs_server_submit.argtypes = [vp, ctypes.c_char_p, sz, ctypes.POINTER(Options), u64, u64,
                                       ctypes.POINTER(u64)]
        L.rs_server_wait.argtypes = [vp, u64, i32, vp, sz, ctypes.POINTER(sz), ctypes.POINTER(JobReport)]
        L.rs_server_destroy.argtypes = [vp]
        L.rs_last_error.restype = ctypes.c_char_p
        L.rs_version.restype = ctypes.c_char_p
        _lib = L
    return _lib


def _check(rc: int) -> None:
    if rc != RS_OK:
        raise RsieveError(rc, lib().rs_last_error().decode(errors="replace"))


def make_options(**kw) -> Options:
    o = Options()
    lib().rs_options_default(ctypes.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise TypeError(f"unknown option {k}")
        setattr(o, k, int(v))
    return o


def version() -> str:
    return lib().rs_version().decode()


def plan_abcd(text: str | bytes, **opts) -> dict:
    """Parse and plan on the host only (no GPU needed)."""
    if isinstance(text, str):
        text = text.encode()
    info = JobInfo()
    _check(lib().rs_plan_abcd(text, len(text), ctypes.byref(make_options(**opts)), ctypes.byref(info)))
    return info.as_dict()


class Job:
    """A resident sieve job on one GPU."""

    def __init__(self, abcd: str | bytes | None = None, *, base: int | None = None, sign: int = -1,
                 ks=None, nlists=None, **opts):
        self._h = ctypes.c_void_p(None)
        o = make_options(**opts)
        if abcd is not None:
            if isinstance(abcd, str):
                abcd = abcd.encode()
            _check(lib().rs_job_create_abcd(abcd, len(abcd), ctypes.byref(o), ctypes.byref(self._h)))
            self.h2d_bytes = len(abcd)
        else:
            ks = np.ascontiguousarray(ks, dtype=np.uint32)
            noff = np.zeros(len(ks) + 1, dtype=np.uint32)
            noff[1:] = np.cumsum([len(x) for x in nlists])
            nv = np.ascontiguousarray(np.concatenate([np.asarray(x, dtype=np.uint32) for x in nlists]))
            _check(lib().rs_job_create(base, sign, len(ks), ks.ctypes.data, noff.ctypes.data, nv.ctypes.data,
                                       ctypes.byref(o), ctypes.byref(self._h)))
            self.h2d_bytes = ks.nbytes + noff.nbytes + nv.nbytes
        info = JobInfo()
        _check(lib().rs_job_info_get(self._h, ctypes.byref(info)))
        self.info = info.as_dict()

    def sieve(self, p0: int, p1: int):
        """All factors with p in [p0, p1]: (structured array (p,k,n), stats dict)."""
        cap = 1 << 12
        while True:
            out = np.zeros(cap, dtype=FACTOR_DTYPE)
            cnt = ctypes.c_size_t(0)
            st = Stats()
            rc = lib().rs_sieve_range(self._h, p0, p1, out.ctypes.data, cap, ctypes.byref(cnt), ctypes.byref(st))
            if rc == RS_ERR_CAPACITY:
                cap = cnt.value
                continue
            _check(rc)
            return out[: cnt.value], st.as_dict()

    def autotune(self, p0: int, p1: int, candidates: int = 3) -> dict:
        """Time the cheapest modelled layouts on [p0, p1], keep the fastest; returns the new plan."""
        info = JobInfo()
        _check(lib().rs_job_autotune(self._h, p0, p1, candidates, ctypes.byref(info)))
        self.info = info.as_dict()
        return self.info

    def write_factors(self, path: str, factors) -> None:
        f = np.ascontiguousarray(factors, dtype=FACTOR_DTYPE)
        _check(lib().rs_write_factors(self._h, path.encode(), f.ctypes.data, len(f)))

    def close(self) -> None:
        if self._h:
            lib().rs_job_destroy(self._h)
            self._h = ctypes.c_void_p(None)

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """The batched form (rs_batch_*): many jobs' ranges sieved together, one
    persistent BSGS launch per kernel variant per round, rounds as CUDA graphs."""

    def __init__(self, device: int = 0):
        self._h = ctypes.c_void_p(None)
        self._jobs = []  # keeps the added jobs alive
        _check(lib().rs_batch_create(device, ctypes.byref(self._h)))

    def add(self, job: "Job", p0: int, p1: int) -> int:
        item = ctypes.c_uint32(0)
        _check(lib().rs_batch_add(self._h, job._h, p0, p1, ctypes.byref(item)))
        self._jobs.append(job)
        return item.value

    def run(self) -> dict:
        st = Stats()
        _check(lib().rs_batch_run(self._h, ctypes.byref(st)))
        return st.as_dict()

    def result(self, item: int):
        """(factors, stats dict) of one item after run()."""
        cap = 1 << 12
        while True:
            out = np.zeros(cap, dtype=FACTOR_DTYPE)
            cnt = ctypes.c_size_t(0)
            st = Stats()
            rc = lib().rs_batch_result(self._h, item, out.ctypes.data, cap, ctypes.byref(cnt), ctypes.byref(st))
            if rc == RS_ERR_CAPACITY:
                cap = cnt.value
                continue
            _check(rc)
            return out[: cnt.value], st.as_dict()

    def close(self) -> None:
        if self._h:
            lib().rs_batch_destroy(self._h)
            self._h = ctypes.c_void_p(None)

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """A job server on one GPU (rs_server_*): jobs run concurrently in `slots`."""

    def __init__(self, device: int = 0, slots: int = 0, queue_cap: int = 0, mem_budget: int = 0,
                 cache_jobs: int = 0):
        self._h = ctypes.c_void_p(None)
        o = ServerOptions()
        lib().rs_server_options_default(ctypes.byref(o))
        o.device = device
        if slots:
            o.slots = slots
        if queue_cap:
            o.queue_cap = queue_cap
        if mem_budget:
            o.mem_budget = mem_budget
        if cache_jobs:
            o.cache_jobs = cache_jobs
        _check(lib().rs_server_create(ctypes.byref(o), ctypes.byref(self._h)))

    def submit(self, abcd: str | bytes, p0: int, p1: int, **opts) -> int:
        if isinstance(abcd, str):
            abcd = abcd.encode()
        t = ctypes.c_uint64(0)
        _check(lib().rs_server_submit(self._h, abcd, len(abcd), ctypes.byref(make_options(**opts)), p0, p1,
                                      ctypes.byref(t)))
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1):
        """(factors, report dict) of a finished job; raises RsieveError(RS_ERR_TIMEOUT) if still running."""
        cap = 1 << 12
        while True:
            out = np.zeros(cap, dtype=FACTOR_DTYPE)
            cnt = ctypes.c_size_t(0)
            rep = JobReport()
            rc = lib().rs_server_wait(self._h, ticket, timeout_ms, out.ctypes.data, cap, ctypes.byref(cnt),
                                      ctypes.byref(rep))
            if rc == RS_ERR_CAPACITY:
                cap = cnt.value
                continue
            _check(rc)
            return out[: cnt.value], rep.as_dict()

    def close(self) -> None:
        if self._h:
            lib().rs_server_destroy(self._h)
            self._h = ctypes.c_void_p(None)

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def abcd_remove(text: str | bytes, removed, sieved_to: int) -> str:
    """ABCD text with the (k, n) of `removed` (array with fields k, n) dropped (host only)."""
    if isinstance(text, str):
        text = text.encode()
    f = np.ascontiguousarray(removed, dtype=FACTOR_DTYPE) if len(removed) else np.zeros(0, FACTOR_DTYPE)
    cap = len(text) + 4096 + 64 * text.count(b"ABCD")
    while True:
        out = ctypes.create_string_buffer(cap)
        n = ctypes.c_size_t(0)
        rc = lib().rs_abcd_remove(text, len(text), f.ctypes.data, len(f), sieved_to, out, cap, ctypes.byref(n))
        if rc == RS_ERR_CAPACITY:
            cap = n.value
            continue
        _check(rc)
        return out.raw[: n.value].decode()


def gpu_primes(lo: int, hi: int, device: int = 0) -> np.ndarray:
    """Odd primes in [lo, hi] from the device sieve kernel."""
    cap = max(16, int((hi - lo) // 2 + 2)) if hi - lo < (1 << 24) else int((hi - lo) / max(2.0, np.log(max(lo, 3)) - 1.5)) + 4096
    while True:
        out = np.zeros(cap, dtype=np.uint64)
        cnt = ctypes.c_size_t(0)
        rc = lib().rs_gpu_primes(lo, hi, out.ctypes.data, cap, ctypes.byref(cnt), device)
        if rc == RS_ERR_CAPACITY:
            cap = cnt.value
            continue
        _check(rc)
        return out[: cnt.value]


def bench_imad(device: int = 0) -> tuple[float, float, float]:
    """(32-bit mad.lo ops/s, Montgomery products/s, Shoup products/s) on this GPU."""
    a, b, c = ctypes.c_double(0), ctypes.c_double(0), ctypes.c_double(0)
    _check(lib().rs_bench_imad(device, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
    return a.value, b.value, c.value


def arith_check(a, b, p, device: int = 0):
    a = np.ascontiguousarray(a, dtype=np.uint64)
    b = np.ascontiguousarray(b, dtype=np.uint64)
    p = np.ascontiguousarray(p, dtype=np.uint64)
    mm = np.zeros(len(a), dtype=np.uint64)
    jj = np.zeros(len(a), dtype=np.int32)
    _check(lib().rs_gpu_arith_check(a.ctypes.data, b.ctypes.data, p.ctypes.data, len(a), mm.ctypes.data,
                                    jj.ctypes.data, device))
    return mm, jj


def modmul_check(op: str, a, b, c, p, device: int = 0) -> np.ndarray:
    """out[i] = op(a[i], b[i], c[i], p[i]) on the GPU (rs_gpu_modmul_check); see include/rsieve.h."""
    arrs = [np.ascontiguousarray([int(x) for x in v], dtype=np.uint64) for v in (a, b, c, p)]
    out = np.zeros(len(arrs[0]), dtype=np.uint64)
    _check(lib().rs_gpu_modmul_check(OPS[op], arrs[0].ctypes.data, arrs[1].ctypes.data, arrs[2].ctypes.data,
                                     arrs[3].ctypes.data, len(out), out.ctypes.data, device))
    return out


def bench_products(device: int = 0) -> dict:
    """Measured rates of every product form (rs_bench_products): name -> operations per second."""
    r = (ctypes.c_double * len(PRODUCT_RATES))()
    _check(lib().rs_bench_products(device, r))
    return dict(zip(PRODUCT_RATES, list(r)))
