"""rs_gpu_primes_static: the device prime sieve for callers that cannot allocate.

Hosts that run under a device-memory pool or budget, plug-ins whose host owns
all device memory, or code recording a CUDA graph cannot call cudaMalloc where
they want primes.  This entry point takes every buffer from the caller and
keeps its one scratch bitmap in a fixed array inside the library.  The test
calls it through the C ABI on caller-owned device buffers (allocated here with
PyTorch, standing in for the host's own memory) twice in a row and checks each
result against the allocating entry point rs_gpu_primes and against the CPU
oracle's primes, then at its edges: a window of exactly the largest size, one
odd number wider (refused), an output buffer smaller than the prime count, and
a sieving-prime list shorter than the primes below 65536.  This file is named
to run last, so a failure here comes after every other test has run.
"""
import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sieving_primes(hi: int):
    """Consecutive odd primes 3, 5, 7, ... up to sqrt(hi), and floor(2^64/q)."""
    r = math.isqrt(hi) + 1
    sieve = np.ones(r + 1, dtype=bool)
    sieve[:2] = False
    for q in range(2, math.isqrt(r) + 1):
        if sieve[q]:
            sieve[q * q::q] = False
    ps = np.nonzero(sieve)[0]
    ps = ps[ps > 2].astype(np.uint64)
    rcp = np.array([((1 << 64) - 1) // int(q) for q in ps], dtype=np.uint64)
    return ps.astype(np.uint32), rcp


def _device(arr, torch):
    view = {np.dtype(np.uint32): np.int32, np.dtype(np.uint64): np.int64}[arr.dtype]
    return torch.from_numpy(np.ascontiguousarray(arr).view(view)).to("cuda")


MAX_ODDS = 1 << 25  # odd numbers the static scratch bitmap covers


def _call(lib, lo, hi, d_sp, d_rcp, n_sp, d_out, cap, d_cnt):
    return lib.rs_gpu_primes_static(lo, hi, d_sp.data_ptr(), d_rcp.data_ptr(), n_sp, d_out.data_ptr(), cap,
                                    d_cnt.data_ptr(), None)


def test_static_sieve_matches_allocating_sieve(rs, oracle_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    lib = rs.lib()
    windows = [(10**13, 10**13 + 3 * 10**7), (10**9 + 1, 10**9 + 4 * 10**6)]
    sp, rcp = _sieving_primes(windows[0][1])
    d_sp, d_rcp = _device(sp, torch), _device(rcp, torch)
    cap = 2_000_000
    d_out = torch.zeros(cap, dtype=torch.int64, device="cuda")
    d_cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    for lo, hi in windows:  # two calls in a row on the same scratch array
        want = rs.gpu_primes(lo, hi)
        d_out.fill_(-1)
        rc = lib.rs_gpu_primes_static(lo, hi, d_sp.data_ptr(), d_rcp.data_ptr(), len(sp), d_out.data_ptr(), cap,
                                      d_cnt.data_ptr(), None)
        assert rc == 0, lib.rs_last_error().decode()
        torch.cuda.synchronize()
        n = int(d_cnt.item())
        assert n == len(want) and n <= cap
        got = np.sort(d_out[:n].cpu().numpy().view(np.uint64))
        assert np.array_equal(got, want)
        assert np.array_equal(got, oracle_mod.primes(lo, hi))


def test_static_sieve_edges(rs, oracle_mod):
    """The largest window (2^25 odd numbers) works and matches the oracle; one odd
    number more is refused; a small output buffer gets exactly cap primes and the
    full count; a short sieving-prime list (hi < 65536^2) works."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    lib = rs.lib()
    lo = 10**12 + 1
    hi = lo + 2 * (MAX_ODDS - 1)  # exactly MAX_ODDS odd numbers
    sp, rcp = _sieving_primes(hi + 2)
    d_sp, d_rcp = _device(sp, torch), _device(rcp, torch)
    cap = 3_000_000
    d_out = torch.full((cap + 64,), -1, dtype=torch.int64, device="cuda")
    d_cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = _call(lib, lo, hi, d_sp, d_rcp, len(sp), d_out, cap, d_cnt)
    assert rc == 0, lib.rs_last_error().decode()
    torch.cuda.synchronize()
    want = oracle_mod.primes(lo, hi)
    n = int(d_cnt.item())
    assert n == len(want) and n <= cap
    assert np.array_equal(np.sort(d_out[:n].cpu().numpy().view(np.uint64)), want)
    # one odd number past the limit
    rc = _call(lib, lo, hi + 2, d_sp, d_rcp, len(sp), d_out, cap, d_cnt)
    assert rc == rs.RS_ERR_RANGE and "window too wide" in lib.rs_last_error().decode()
    # output buffer smaller than the count: cap primes written, the rest untouched
    small = 1000
    d_out.fill_(-1)
    rc = _call(lib, lo, lo + 2 * 10**6, d_sp, d_rcp, len(sp), d_out, small, d_cnt)
    assert rc == 0, lib.rs_last_error().decode()
    torch.cuda.synchronize()
    want = oracle_mod.primes(lo, lo + 2 * 10**6)
    out = d_out.cpu().numpy()
    assert int(d_cnt.item()) == len(want) > small
    assert (out[small:] == -1).all()
    assert set(out[:small].view(np.uint64).tolist()) <= set(want.tolist())
    # fewer sieving primes than the 6541 odd primes below 65536 (hi < 65536^2)
    lo2, hi2 = 3 * 10**9 + 1, 3 * 10**9 + 4 * 10**6
    sp2, rcp2 = _sieving_primes(hi2)
    assert len(sp2) < 6541
    d_sp2, d_rcp2 = _device(sp2, torch), _device(rcp2, torch)
    rc = _call(lib, lo2, hi2, d_sp2, d_rcp2, len(sp2), d_out, cap, d_cnt)
    assert rc == 0, lib.rs_last_error().decode()
    torch.cuda.synchronize()
    n = int(d_cnt.item())
    assert np.array_equal(np.sort(d_out[:n].cpu().numpy().view(np.uint64)), oracle_mod.primes(lo2, hi2))


def test_static_sieve_rejects_wide_window(rs):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    lib = rs.lib()
    sp, rcp = _sieving_primes(10**12)
    d_sp, d_rcp = _device(sp, torch), _device(rcp, torch)
    d_out = torch.zeros(16, dtype=torch.int64, device="cuda")
    d_cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = lib.rs_gpu_primes_static(10**11, 10**11 + 10**9, d_sp.data_ptr(), d_rcp.data_ptr(), len(sp),
                                  d_out.data_ptr(), 16, d_cnt.data_ptr(), None)
    assert rc == rs.RS_ERR_RANGE
    assert "window too wide" in lib.rs_last_error().decode()
