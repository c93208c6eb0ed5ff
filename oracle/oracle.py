"""ctypes binding of the CPU oracle (oracle/rs_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
as the checker and by ``bench.py``'s CPU baseline / reference arm.  The product
library never imports this module.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle_rs.so")


class _Job(ctypes.Structure):
    _fields_ = [
        ("base", ctypes.c_uint32),
        ("sign", ctypes.c_int32),
        ("nk", ctypes.c_uint32),
        ("k", ctypes.POINTER(ctypes.c_uint32)),
        ("noff", ctypes.POINTER(ctypes.c_uint32)),
        ("n", ctypes.POINTER(ctypes.c_uint32)),
        ("ref_minN", ctypes.c_int32),
        ("ref_maxN", ctypes.c_int32),
        ("nlines", ctypes.c_uint32),
    ]


class _RefPlan(ctypes.Structure):
    _fields_ = [
        ("minQ", ctypes.c_int32),
        ("minSubs", ctypes.c_int32),
        ("minRange", ctypes.c_int32),
        ("minWork", ctypes.c_int32),
        ("tMin", ctypes.c_int32),
        ("tMax", ctypes.c_int32),
        ("shift", ctypes.c_int32),
        ("minimum", ctypes.c_int32),
        ("rowoffset", ctypes.c_int32),
        ("row_k", ctypes.POINTER(ctypes.c_int32)),
        ("row_r", ctypes.POINTER(ctypes.c_int32)),
    ]


FACTOR_DTYPE = np.dtype([("p", "<u8"), ("k", "<u4"), ("n", "<u4")])

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle into oracle/_build/liboracle_rs.so (gcc, no CUDA)."""
    import subprocess

    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    src = os.path.join(HERE, "rs_oracle.c")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(os.path.join(HERE, "rs_oracle.h"))):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-o", tmp, src, "-lpthread", "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_parse_abcd.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(_Job),
                                     ctypes.c_char_p, ctypes.c_size_t]
        L.orc_job_from_arrays.argtypes = [ctypes.c_uint32, ctypes.c_int32, ctypes.c_uint32,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.POINTER(_Job)]
        L.orc_job_free.argtypes = [ctypes.POINTER(_Job)]
        L.orc_ref_plan.argtypes = [ctypes.POINTER(_Job), ctypes.c_int32, ctypes.c_int32,
                                   ctypes.POINTER(_RefPlan)]
        L.orc_refplan_free.argtypes = [ctypes.POINTER(_RefPlan)]
        L.orc_primes.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_size_t]
        L.orc_primes.restype = ctypes.c_size_t
        L.orc_sieve.argtypes = [ctypes.POINTER(_Job), ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int32,
                                ctypes.c_int32, ctypes.c_void_p, ctypes.c_size_t,
                                ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_uint64)]
        L.orc_verify.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                 ctypes.c_int32]
        L.orc_jacobi.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.orc_sieve_ref.argtypes = [ctypes.POINTER(_Job), ctypes.POINTER(_RefPlan), ctypes.c_int32, ctypes.c_int32,
                                    ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int32, ctypes.c_int32,
                                    ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t),
                                    ctypes.POINTER(ctypes.c_uint64)]
        L.orc_default_threads.restype = ctypes.c_int
        _lib = L
    return _lib


@dataclass
class RefPlan:
    Q: int
    rows: int
    x_range: int
    work: int
    tmin: int
    tmax: int
    row_k: list
    row_r: list


class Job:
    """An oracle-side sieve job (owns its C arrays)."""

    def __init__(self, cjob: _Job):
        self._j = cjob

    @classmethod
    def from_abcd(cls, text: str | bytes) -> "Job":
        if isinstance(text, str):
            text = text.encode()
        j = _Job()
        err = ctypes.create_string_buffer(256)
        rc = lib().orc_parse_abcd(text, len(text), ctypes.byref(j), err, 256)
        if rc:
            raise ValueError(err.value.decode())
        return cls(j)

    @classmethod
    def from_arrays(cls, base: int, sign: int, ks, nlists) -> "Job":
        ks = np.ascontiguousarray(ks, dtype=np.uint32)
        noff = np.zeros(len(ks) + 1, dtype=np.uint32)
        noff[1:] = np.cumsum([len(x) for x in nlists])
        n = (np.ascontiguousarray(np.concatenate(nlists), dtype=np.uint32)
             if len(nlists) else np.zeros(0, np.uint32))
        j = _Job()
        rc = lib().orc_job_from_arrays(base, sign, len(ks), ks.ctypes.data, noff.ctypes.data,
                                       n.ctypes.data, ctypes.byref(j))
        if rc:
            raise MemoryError("orc_job_from_arrays failed")
        return cls(j)

    def __del__(self):
        try:
            if self._j.k:
                lib().orc_job_free(ctypes.byref(self._j))
        except Exception:
            pass

    @property
    def base(self) -> int:
        return self._j.base

    @property
    def sign(self) -> int:
        return self._j.sign

    @property
    def ks(self) -> list:
        return [self._j.k[i] for i in range(self._j.nk)]

    def nlist(self, i: int) -> np.ndarray:
        a, b = self._j.noff[i], self._j.noff[i + 1]
        return np.ctypeslib.as_array(self._j.n, shape=(self._j.noff[self._j.nk],))[a:b].copy()

    @property
    def ncand(self) -> int:
        return self._j.noff[self._j.nk]

    def ref_plan(self, Qin: int = 0, hash_elems: int = 512) -> RefPlan:
        pl = _RefPlan()
        rc = lib().orc_ref_plan(ctypes.byref(self._j), Qin, hash_elems, ctypes.byref(pl))
        if rc:
            raise MemoryError("orc_ref_plan failed")
        try:
            rk = [pl.row_k[i] for i in range(pl.minSubs)]
            rr = [pl.row_r[i] for i in range(pl.minSubs)]
            return RefPlan(pl.minQ, pl.minSubs, pl.minRange, pl.minWork, pl.tMin, pl.tMax, rk, rr)
        finally:
            lib().orc_refplan_free(ctypes.byref(pl))

    def sieve_ref(self, p0: int, p1: int, Qin: int = 0, hash_m: int = 8, small_prime_scale: int = 256,
                  verify: bool = True, threads: int = 0):
        """Reference projection (orc_sieve_ref): the factor lines one run of the
        reference executable with -Q Qin -m hash_m -s small_prime_scale (and -v when
        verify is False) would write for [p0, p1].  Returns (structured array of
        (p,k,n), number of candidate q tested)."""
        hash_elems = 2 << hash_m
        pl = _RefPlan()
        rc = lib().orc_ref_plan(ctypes.byref(self._j), Qin, hash_elems, ctypes.byref(pl))
        if rc:
            raise MemoryError("orc_ref_plan failed")
        try:
            cap = 1 << 14
            while True:
                out = np.zeros(cap, dtype=FACTOR_DTYPE)
                cnt = ctypes.c_size_t(0)
                nc = ctypes.c_uint64(0)
                rc = lib().orc_sieve_ref(ctypes.byref(self._j), ctypes.byref(pl), hash_elems, small_prime_scale,
                                         p0, p1, int(verify), threads, out.ctypes.data, cap, ctypes.byref(cnt),
                                         ctypes.byref(nc))
                if rc:
                    raise ValueError("orc_sieve_ref: arguments outside its domain (Riesel, p0 > b, p0 > k)")
                if cnt.value <= cap:
                    return out[: cnt.value], nc.value
                cap = cnt.value
        finally:
            lib().orc_refplan_free(ctypes.byref(pl))

    def sieve(self, p0: int, p1: int, datless: bool = False, threads: int = 0):
        """Complete factor set; returns (structured array of (p,k,n), number of primes)."""
        cap = 1 << 16
        while True:
            out = np.zeros(cap, dtype=FACTOR_DTYPE)
            cnt = ctypes.c_size_t(0)
            npr = ctypes.c_uint64(0)
            rc = lib().orc_sieve(ctypes.byref(self._j), p0, p1, int(datless), threads, out.ctypes.data,
                                 cap, ctypes.byref(cnt), ctypes.byref(npr))
            if rc:
                raise RuntimeError(f"orc_sieve failed rc={rc}")
            if cnt.value <= cap:
                return out[: cnt.value], npr.value
            cap = cnt.value


def primes(lo: int, hi: int) -> np.ndarray:
    cap = max(16, int((hi - lo) // 2 + 2)) if hi - lo < 10**7 else int((hi - lo) / max(1.0, np.log(max(lo, 3)) - 1.2) * 1.3) + 1000
    out = np.zeros(cap, dtype=np.uint64)
    c = lib().orc_primes(lo, hi, out.ctypes.data, cap)
    if c > cap:
        out = np.zeros(c, dtype=np.uint64)
        c = lib().orc_primes(lo, hi, out.ctypes.data, c)
    return out[:c]


def verify(p: int, k: int, b: int, n: int, sign: int = -1) -> bool:
    return bool(lib().orc_verify(p, k, b, n, sign))


def jacobi(a: int, n: int) -> int:
    return int(lib().orc_jacobi(a, n))


def default_threads() -> int:
    return int(lib().orc_default_threads())
