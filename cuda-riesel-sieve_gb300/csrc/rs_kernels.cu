// rs_kernels.cu -- the sieve's device kernels for sm_103a.
//
//   sieve_large_kernel, sieve_small_kernel
//                  segmented Eratosthenes over odd numbers: primes >= 65536
//                  once per window into an L2-resident bitmap, smaller ones
//                  per 2^15-odd segment in shared memory, then compaction; the
//                  primes of a p-window go straight into HBM.  Replaces the
//                  host prime generator generateGPUPrimes
//                  (kernel_v0.24.6.cu:1838-1987), but is complete (every
//                  composite removed) where the reference leaves composites
//                  above smallP_max^2.
//   setup_kernel   one thread per prime: Montgomery constants, B = b^Q, the
//                  quadratic-character filter per (k, n mod Q) row
//                  (kernel_v0.24.6.cu:461-521), the per-row giant-step start
//                  values k*b^r*B^e0 (kernel_v0.24.6.cu:454-509,525-528) and the
//                  per-lane power tables the BSGS kernels start from.  For
//                  integer rows (every k*b^r < 2^32) B^e0 moves into the lane
//                  table and a start value is the integer k*b^r itself.
//   bsgs_kernel    one prime per warp: baby steps B^j (j < m) in 64 chains of
//                  consecutive exponents into a shared-memory table of 16-bit
//                  tags, then giant steps for every active row, 32 lanes per
//                  prime (kernel_v0.24.6.cu:365-620 is the per-thread,
//                  global-memory original).  Candidate hits are checked
//                  against the row bitmap on the device and appended with one
//                  atomic each.
//   bsgs_cta_kernel  the same with a CTA of 16 warps per prime and one large
//                  table, for jobs with many k or wide n ranges.  Both are
//                  instantiated per form of the start values (RM: per-prime
//                  residues, integers in the record, integers by row id).
//   bsgs_exact_kernel  the rare primes whose tag matches overflow the fast
//                  path's list, with an exact (tag, j) table.
//   verify_kernel  direct k*b^n check of every hit (kernel_v0.24.6.cu:1649-1671).
#include <cstdio>

#include "rs_arith.cuh"
#include "rs_internal.h"

namespace rs {

// ---------------------------------------------------------------------------
// Segmented sieve of Eratosthenes over the odd numbers of [lo, hi], lo odd.
// Bit x of the window stands for lo + 2x.  Sieving primes q >= 2*kSieveOdds hit a
// 2^15-odd segment at most once or twice, so they are applied once per window
// by sieve_large_kernel (one thread per prime, atomicOr into an L2-resident
// bitmap of the whole window); sieve_small_kernel then starts each segment from
// that bitmap, crosses off the small primes in shared memory and compacts.

__global__ void __launch_bounds__(256) sieve_large_kernel(uint64_t lo, uint64_t hi, const uint32_t *__restrict__ sp,
                                                          const uint64_t *__restrict__ sp_rcp, uint32_t first,
                                                          uint32_t nsp, uint32_t *__restrict__ gbits, uint64_t nodd) {
  const uint32_t t = first + blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nsp) return;
  const uint32_t q = sp[t];
  const uint64_t qq = (uint64_t)q * q;
  if (qq > hi) return;
  const uint64_t start = qq > lo ? qq : lo;
  const uint32_t r = mod_rcp(start, q, sp_rcp[t]);
  uint64_t f = r ? start + (q - r) : start;
  if (!(f & 1)) f += q;
#pragma unroll 1
  for (uint64_t x = (f - lo) >> 1; x < nodd; x += q) atomicOr(&gbits[x >> 5], 1u << (x & 31));
}

__global__ void __launch_bounds__(kSieveThreads)
sieve_small_kernel(uint64_t lo, uint64_t hi, const uint32_t *__restrict__ sp, const uint64_t *__restrict__ sp_rcp,
                   uint32_t nsmall, const uint32_t *__restrict__ gbits, uint64_t *__restrict__ out,
                   uint32_t *__restrict__ count, uint32_t cap) {
  __shared__ uint32_t bits[kSieveOdds / 32];
  __shared__ uint32_t warp_tot[kSieveThreads / 32];
  __shared__ uint32_t block_base;
  const uint64_t base = lo + 2ull * (uint64_t)kSieveOdds * blockIdx.x;  // odd
  if (base > hi) return;
  const uint64_t span = (hi - base) / 2 + 1;
  const uint32_t nodd = span < (uint64_t)kSieveOdds ? (uint32_t)span : (uint32_t)kSieveOdds;
  const uint64_t last = base + 2ull * (nodd - 1);
  const uint32_t tid = threadIdx.x;
  const uint32_t nwords = (nodd + 31) / 32;
  const uint32_t *gseg = gbits + (size_t)blockIdx.x * (kSieveOdds / 32);

  for (uint32_t w = tid; w < kSieveOdds / 32; w += kSieveThreads) bits[w] = w < nwords ? gseg[w] : 0u;
  __syncthreads();

  // Smallest primes: the whole CTA strides over the multiples of one prime.
  uint32_t t = 0;
#pragma unroll 1
  for (; t < nsmall; t++) {
    const uint32_t q = sp[t];
    if (q >= 2 * kSieveThreads) break;
    const uint64_t qq = (uint64_t)q * q;
    if (qq > last) break;
    const uint64_t start = qq > base ? qq : base;
    const uint32_t r = mod_rcp(start, q, sp_rcp[t]);
    uint64_t f = r ? start + (q - r) : start;
    if (!(f & 1)) f += q;
    for (uint64_t x = ((f - base) >> 1) + (uint64_t)tid * q; x < nodd; x += (uint64_t)kSieveThreads * q)
      atomicOr(&bits[x >> 5], 1u << (x & 31));
  }
  // Other small primes: one prime per thread.
#pragma unroll 1
  for (uint32_t u = t + tid; u < nsmall; u += kSieveThreads) {
    const uint32_t q = sp[u];
    const uint64_t qq = (uint64_t)q * q;
    if (qq > last) break;  // sp ascending
    const uint64_t start = qq > base ? qq : base;
    const uint32_t r = mod_rcp(start, q, sp_rcp[u]);
    uint64_t f = r ? start + (q - r) : start;
    if (!(f & 1)) f += q;
    for (uint64_t x = (f - base) >> 1; x < nodd; x += q) atomicOr(&bits[x >> 5], 1u << (x & 31));
  }
  __syncthreads();

  // Compaction: each thread owns a contiguous run of words.
  constexpr uint32_t WPT = kSieveOdds / 32 / kSieveThreads;
  uint32_t mine = 0;
  uint32_t wv[WPT];
#pragma unroll
  for (uint32_t i = 0; i < WPT; i++) {
    const uint32_t w = tid * WPT + i;
    uint32_t m = 0;
    if (w < nwords) {
      m = ~bits[w];
      const uint32_t valid = nodd - w * 32;
      if (valid < 32) m &= (1u << valid) - 1u;
    }
    wv[i] = m;
    mine += __popc(m);
  }
  const uint32_t lane = tid & 31, warp = tid >> 5;
  uint32_t incl = mine;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= (uint32_t)d) incl += y;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t v = lane < kSieveThreads / 32 ? warp_tot[lane] : 0;
    uint32_t s = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, s, d);
      if (lane >= (uint32_t)d) s += y;
    }
    if (lane < kSieveThreads / 32) warp_tot[lane] = s - v;  // exclusive
    if (lane == kSieveThreads / 32 - 1) block_base = atomicAdd(count, s);
  }
  __syncthreads();
  uint32_t pos = block_base + warp_tot[warp] + incl - mine;
#pragma unroll
  for (uint32_t i = 0; i < WPT; i++) {
    uint32_t m = wv[i];
    const uint64_t wbase = base + 2ull * 32ull * (tid * WPT + i);
    while (m) {
      const int b = __ffs(m) - 1;
      m &= m - 1;
      if (pos < cap) out[pos] = wbase + 2ull * (uint32_t)b;
      pos++;
    }
  }
}

uint64_t sieve_bitmap_words(uint64_t lo, uint64_t hi) {
  const uint64_t nodd = (hi - lo) / 2 + 1;
  const uint64_t segs = (nodd + kSieveOdds - 1) / kSieveOdds;
  return segs * (kSieveOdds / 32);
}

cudaError_t launch_sieve(uint64_t lo, uint64_t hi, const uint32_t *sp, const uint64_t *sp_rcp, uint32_t nsp,
                         uint32_t nsmall, uint32_t *gbits, uint64_t *out, uint32_t *count, uint32_t cap,
                         cudaStream_t st) {
  const uint64_t nodd = (hi - lo) / 2 + 1;
  const uint64_t blocks = (nodd + kSieveOdds - 1) / kSieveOdds;
  cudaError_t e = cudaMemsetAsync(gbits, 0, sieve_bitmap_words(lo, hi) * 4, st);
  if (e != cudaSuccess) return e;
  if (nsp > nsmall) {
    const uint32_t nl = nsp - nsmall;
    sieve_large_kernel<<<(nl + 255) / 256, 256, 0, st>>>(lo, hi, sp, sp_rcp, nsmall, nsp, gbits, nodd);
  }
  sieve_small_kernel<<<(unsigned)blocks, kSieveThreads, 0, st>>>(lo, hi, sp, sp_rcp, nsmall, gbits, out, count, cap);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Per-prime setup, one thread per prime.

__device__ __forceinline__ uint64_t &rec_el(const JobDev &J, const ChunkBufs &cb, uint32_t e, uint32_t i) {
  return cb.recs[(size_t)i * J.rec_elems + e];
}

// 16-byte store of elements e, e+1 (e even) of a record.
__device__ __forceinline__ void rec_st2(uint64_t *rec, uint32_t e, uint64_t a, uint64_t b) {
  *reinterpret_cast<uint4 *>(rec + e) = make_uint4((uint32_t)a, (uint32_t)(a >> 32), (uint32_t)b, (uint32_t)(b >> 32));
}

constexpr uint32_t kSetupRegQ = 8;  // Q up to this keeps the table of b^r*B^e0 in shared memory
constexpr uint32_t kTabChunks = 8;  // 16-byte value pairs per lane per staging round
constexpr uint32_t kTabPad = 33;    // chunk slots per staging row: 32 lanes + 1, so column reads are conflict-free

// Per-warp shared memory of the setup kernel: first the staging area of the
// lane tables, then (reused) the per-thread table of b^r*B^e0 and its Shoup
// constants.
union SetupWarpSmem {
  uint4 stage[kTabChunks][kTabPad];
  uint64_t hb[kSetupRegQ][2][32];
};

// Writes 16 consecutive table values of each of the warp's 32 records, starting
// at element e0: every lane has put its values (as pairs, chunk c = values 2c,
// 2c+1) into column `lane` of the staging area; the warp then stores whole
// record runs of 128 bytes (four records per instruction) instead of 32
// scattered 16-byte pieces.
__device__ __forceinline__ void flush_table_round(const SetupWarpSmem &S, uint64_t *recs, uint32_t rec_elems,
                                                  uint32_t i0, uint32_t n, uint32_t e0, uint32_t lane) {
  __syncwarp();
  const uint32_t c = lane & (kTabChunks - 1);
#pragma unroll
  for (uint32_t q = 0; q < 32; q += 32 / kTabChunks) {
    const uint32_t r = q + lane / kTabChunks;
    const uint4 v = S.stage[c][r];
    if (i0 + r < n) *reinterpret_cast<uint4 *>(recs + (size_t)(i0 + r) * rec_elems + e0 + 2 * c) = v;
  }
  __syncwarp();
}

// One thread per prime (a warp per 32 consecutive primes).  Lanes past the
// chunk's prime count compute on a stand-in prime and store nothing.
constexpr uint32_t kSetupKStage = 256;  // per-k records staged in shared memory (8 KB)

__global__ void __launch_bounds__(128) setup_kernel(JobDev J, ChunkBufs cb) {
  __shared__ SetupWarpSmem smem[4];
  __shared__ KInfo sk[kSetupKStage];
  // the per-k records, read by every thread of the block in the row loop
  const bool kstaged = J.nk <= kSetupKStage;
  if (kstaged)
    for (uint32_t c = threadIdx.x; c < J.nk; c += blockDim.x) sk[c] = J.kinfo[c];
  __syncthreads();
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  SetupWarpSmem &S = smem[warp];
  const uint32_t i0 = blockIdx.x * blockDim.x + warp * 32;
  const uint32_t i = i0 + lane;
  const uint32_t cnt = *cb.count;
  const uint32_t n = cnt < cb.cap ? cnt : cb.cap;
  if (i0 >= n) return;  // the whole warp
  const bool live = i < n;
  const uint64_t p = live ? cb.primes[i] : 1000000007ull;
  uint64_t *rec = cb.recs + (size_t)i * J.rec_elems;
  const uint64_t b0 = p > J.base ? (uint64_t)J.base : (uint64_t)J.base % p;
  const bool pb = b0 == 0;          // p | b: no k*b^n+-1 is divisible by p (nact = 0)
  const uint64_t bmod = pb ? 1 : b0;  // keeps the arithmetic below defined
  Mont M;
  M.p = p;
  M.pinv = mont_pinv(p);
  uint64_t one, r2;
  mont_consts(p, M.pinv, one, r2);
  const uint64_t bm = montmul(bmod, r2, M);        // b in Montgomery form
  const uint64_t bq = shoup_const(bm, M.pinv);     // Shoup constant of b
  const uint64_t B = mont_pow(bm, J.Q, one, M);    // b^Q
  const uint64_t e = J.e0 >= 0 ? (uint64_t)J.e0 : (p - 1) - (uint64_t)(-J.e0) % (p - 1);
  const uint64_t H = mont_pow(B, e, one, M);       // B^e0
  const uint64_t G = mont_pow(B, J.m, one, M);     // B^m
  const uint64_t Bc = mont_pow(B, J.chain_len, one, M);  // B^chain_len

  // Lane tables: B^(lane*chain_len) (baby chain starts) and G^(lane % tlanes + 1)
  // (giant multipliers), stepped with Shoup products by the fixed B^chain_len
  // and G, 16 values per round.
  uint64_t Bs, Gs = 0;
  {
    const uint64_t Bw = from_mont(Bc, p, M.pinv), Bq = shoup_const(Bc, M.pinv);
    uint64_t v = one;
#pragma unroll 1
    for (uint32_t h = 0; h < 2; h++) {
#pragma unroll 4
      for (uint32_t c = 0; c < kTabChunks; c++) {
        const uint64_t v1 = shoup_mul(v, Bw, Bq, p);
        S.stage[c][lane] = make_uint4((uint32_t)v, (uint32_t)(v >> 32), (uint32_t)v1, (uint32_t)(v1 >> 32));
        v = shoup_mul(v1, Bw, Bq, p);
      }
      flush_table_round(S, cb.recs, J.rec_elems, i0, n, J.el_tab + 16 * h, lane);
    }
    Bs = v;  // B^(32*chain_len)
    // value t of the G table is G^(t % tlanes + 1): the chain restarts at G
    // whenever t % tlanes wraps to 0 (tlanes divides 32)
    const uint64_t Gw = from_mont(G, p, M.pinv), Gq = shoup_const(G, M.pinv);
    // integer rows: the table holds Z_(t+1) = +-B^e0 * G^(t+1) times 2^128 instead
    uint64_t g0 = G;
    if (J.int_rows) {
      uint64_t h2 = montmul(H, r2, M);  // B^e0 times 2^128
      if (J.sign > 0 && h2) h2 = p - h2;
      g0 = shoup_mul(h2, Gw, Gq, p);
    }
    uint64_t g = g0;
    uint32_t k = 0;
#pragma unroll 1
    for (uint32_t h = 0; h < 2; h++) {
#pragma unroll 1
      for (uint32_t c = 0; c < kTabChunks; c++) {
        uint64_t pair[2];
#pragma unroll
        for (uint32_t u = 0; u < 2; u++) {
          pair[u] = g;
          if (++k == J.tlanes) {
            k = 0;
            g = g0;
          } else {
            g = shoup_mul(g, Gw, Gq, p);
          }
        }
        S.stage[c][lane] =
            make_uint4((uint32_t)pair[0], (uint32_t)(pair[0] >> 32), (uint32_t)pair[1], (uint32_t)(pair[1] >> 32));
        if (h == 1 && c == kTabChunks - 1) Gs = pair[1];  // G^32 when tlanes == 32
      }
      flush_table_round(S, cb.recs, J.rec_elems, i0, n, J.el_tab + 32 + 16 * h, lane);
    }
    if (J.tlanes != 32) {
      Gs = 0;
    } else if (J.int_rows) {  // the table's last entry is Z_32: G^32 by squaring
      Gs = G;
#pragma unroll 1
      for (uint32_t q = 0; q < 5; q++) Gs = montmul(Gs, Gs, M);
    }
  }

  // HB[r] = b^r * B^e0 (Montgomery form) with the Shoup constant of HB[r] taken
  // as an integer, so the start value of row (k, r) is the single product k*HB[r]
  // (not needed for integer rows).
  // Kept per thread in shared memory (indexed by r without a select chain); the
  // staging area is free again after the last flush.
  const bool regtab = J.Q <= kSetupRegQ;
  if (regtab && !J.int_rows) {
    uint64_t h = H;
#pragma unroll 1
    for (uint32_t r = 0; r < J.Q; r++) {
      S.hb[r][0][lane] = h;
      S.hb[r][1][lane] = shoup_const(montmul(h, r2, M), M.pinv);
      h = shoup_mul(h, bmod, bq, p);
    }
  }

  // Active rows (quadratic-character filter) and their giant-step start values
  // (the integers k*b^r for integer rows), written in pairs (V) and in groups of
  // eight (row ids) as 16-byte stores.
  const int chib = legendre_k_tab(p, J.b_odd, J.b_e2, J.b_rcp, J.b_jac, J.jac_bits);
  const int chim1 = ((uint32_t)p & 3u) == 1u ? 1 : -1;  // (-1/p)
  const bool qeven = (J.Q & 1u) == 0;
  uint32_t nact = 0;
  uint64_t vprev = 0, rp0 = 0, rp1 = 0;
  uint64_t rows_on = 0;  // row_mask: the active rows as bits
  // one active row: its start value V and its row id, packed into the record
  // (integer rows: the row id only, the kernels look up k*b^r by it; row_mask:
  // one bit)
  auto emit = [&](uint64_t V, uint32_t row) {
    if (J.row_mask) {
      rows_on |= 1ull << row;
      nact++;
      return;
    }
    if (nact & 1) {
      if (live && !J.row_ids_only) rec_st2(rec, J.el_v + nact - 1, vprev, V);
    } else {
      vprev = V;
    }
    const uint64_t rbits = (uint64_t)row << (16 * (nact & 3));
    if (nact & 4) rp1 |= rbits;
    else rp0 |= rbits;
    if ((nact & 7) == 7) {
      if (live) rec_st2(rec, J.el_row + (nact >> 2) - 1, rp0, rp1);
      rp0 = rp1 = 0;
    }
    nact++;
  };
  if (regtab) {
    // Q <= 8: the rows of k are its residues present (KInfo.rmask, r ascending),
    // the active ones follow from the two characters, and V = k * HB[r]; all
    // per-k data comes from one 32-byte record (shared memory when staged).
#pragma unroll 1
    for (uint32_t c0 = 0; c0 < J.nk; c0 += 4) {
      // the four characters first, so their table loads are in flight together;
      // kept as 2-bit fields (character + 1) so that no array goes to local memory
      uint32_t chpack = 0;
#pragma unroll
      for (uint32_t u = 0; u < 4; u++) {
        const uint32_t c = c0 + u;
        int ch = 0;
        if (c < J.nk) {
          const KInfo &ki = kstaged ? sk[c] : J.kinfo[c];
          ch = legendre_k_tab(p, ki.k_odd, ki.k_e2, ki.k_rcp, ki.k_jac, J.jac_bits);
        }
        chpack |= (uint32_t)(ch + 1) << (2 * u);
      }
#pragma unroll 1
      for (uint32_t u = 0; u < 4; u++) {
        const uint32_t c = c0 + u;
        int chik = (int)((chpack >> (2 * u)) & 3u) - 1;
        if (c >= J.nk) break;
        if (J.sign > 0) chik *= chim1;  // character of -k
        if (chik == 0) continue;        // p | k
        const KInfo ki = kstaged ? sk[c] : J.kinfo[c];
        uint32_t amask;
        if (qeven)  // even r: (k/p) = 1; odd r: (k/p)(b/p) = 1
          amask = (chik == 1 ? ki.rmask & 0x55555555u : 0u) | (chik * chib == 1 ? ki.rmask & 0xaaaaaaaau : 0u);
        else
          amask = (chib == -1 || chik == 1) ? ki.rmask : 0u;
        if (!amask) continue;
        const uint64_t kmod = p > ki.k_val ? (uint64_t)ki.k_val : (uint64_t)ki.k_val % p;
        const uint64_t kx = J.sign > 0 ? p - kmod : kmod;  // -k for k*b^n+1
#pragma unroll 1
        while (amask) {
          const uint32_t r = __ffs(amask) - 1;
          amask &= amask - 1;
          const uint32_t row = ki.row0 + __popc(ki.rmask & ((1u << r) - 1));
          emit(J.int_rows ? (J.row_ids_only || J.row_mask ? 0 : (uint64_t)__ldg(J.row_c + row))
                          : shoup_mul(kx, S.hb[r][0][lane], S.hb[r][1][lane], p),
               row);
        }
      }
    }
  } else {
#pragma unroll 1
    for (uint32_t c0 = 0; c0 < J.nk; c0 += 4) {
      uint32_t chpack = 0;
#pragma unroll
      for (uint32_t u = 0; u < 4; u++) {
        const uint32_t c = c0 + u;
        const int ch = c < J.nk ? legendre_k_tab(p, J.k_odd[c], J.k_e2[c], J.k_rcp[c], J.k_jac[c], J.jac_bits) : 0;
        chpack |= (uint32_t)(ch + 1) << (2 * u);
      }
#pragma unroll 1
      for (uint32_t u = 0; u < 4; u++) {
        const uint32_t c = c0 + u;
        int chik = (int)((chpack >> (2 * u)) & 3u) - 1;
        if (c >= J.nk) break;
        if (J.sign > 0) chik *= chim1;  // character of -k
        if (chik == 0) continue;        // p | k
        const uint32_t r0 = J.k_row0[c], r1 = J.k_row0[c + 1];
        const uint64_t kmod = p > J.k_val[c] ? (uint64_t)J.k_val[c] : (uint64_t)J.k_val[c] % p;
        const uint64_t kx = J.sign > 0 ? p - kmod : kmod;  // -k for k*b^n+1
        uint64_t V = 0;
        uint32_t cur = 0;
        bool have = false;
#pragma unroll 1
        for (uint32_t row = r0; row < r1; row++) {
          const uint32_t r = J.row_r[row];
          const bool act = qeven ? (chik * ((r & 1u) ? chib : 1) == 1) : (chib == -1 || chik == 1);
          if (!act) continue;
          if (J.int_rows) {
            emit(J.row_ids_only || J.row_mask ? 0 : (uint64_t)__ldg(J.row_c + row), row);
            continue;
          }
          if (!have) {
            V = montmul(montmul(kx, r2, M), H, M);
            have = true;
          }
#pragma unroll 1
          for (; cur < r; cur++) V = shoup_mul(V, bmod, bq, p);
          emit(V, row);
        }
      }
    }
  }
  if (!live) return;
  if (J.row_mask) {
    rec_st2(rec, J.el_v, rows_on, 0);
  } else {
    if ((nact & 1) && !J.row_ids_only) rec[J.el_v + nact - 1] = vprev;
    if (nact & 7) rec_st2(rec, J.el_row + ((nact >> 3) << 1), rp0, rp1);
  }
  rec_st2(rec, kElP, p, M.pinv);
  rec_st2(rec, kElBm, B, Gs);
  // floor(2^64/p) is the Shoup constant of 1, whose Montgomery form is `one`
  // With (b/p) = 1 and both residues of every k present, k's two rows are both
  // active or both not, so the active rows come in adjacent (k, 0), (k, 1) pairs
  // whose start values differ by the factor b.
  const uint64_t paired = (J.pairable && chib == 1) ? 1ull << 32 : 0ull;
  rec_st2(rec, kElNact, pb ? 0 : (nact | paired), shoup_const(one, M.pinv));
  // the strides in normal form with their Shoup constants, once per prime
  rec_st2(rec, kElStw, from_mont(B, p, M.pinv), shoup_const(B, M.pinv));
  rec_st2(rec, kElGw, from_mont(Gs, p, M.pinv), shoup_const(Gs, M.pinv));
  // chain offsets: warp w of a prime's group starts its chains at B^(32w*c),
  // and a thread's second chain is 32W chains after its first
  uint64_t off = Bs;  // B^(32*c)
  if (J.cta_warps > 1) {
    uint64_t o = one;
#pragma unroll 1
    for (uint32_t w = 0; w < J.cta_warps; w++) {
      rec_st2(rec, kElWoff + 2 * w, from_mont(o, p, M.pinv), shoup_const(o, M.pinv));
      o = montmul(o, Bs, M);
    }
    off = o;  // B^(32W*c)
  }
  rec_st2(rec, kElOfw, from_mont(off, p, M.pinv), shoup_const(off, M.pinv));
}

// Quadratic-character tables: word w of the table of odd k' holds bit t =
// ((32*w + t) / k') == +1 (Jacobi symbol), for 32*w + t < k'.  One launch
// builds the tables sel[0..nsel) of the job's list (odd parts kodd[], word
// offsets word_off[]); thread g writes word g - first[i] of table sel[i], where
// first[] are the running word counts of the selected tables.
__global__ void jacobi_table_kernel(const uint32_t *kodd, const uint32_t *word_off, const uint32_t *sel,
                                    const uint32_t *first, uint32_t nsel, uint32_t total_words, uint32_t *bits) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total_words) return;
  uint32_t lo = 0, hi = nsel;  // last selected table with first <= g
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) / 2;
    if (first[mid] <= g) lo = mid;
    else hi = mid;
  }
  const uint32_t t = sel[lo];
  const uint32_t k = kodd[t];
  const uint32_t w = g - first[lo];
  const uint32_t a0 = 32 * w;
  uint32_t out = 0;
  for (uint32_t b = 0; b < 32; b++) {
    const uint32_t a = a0 + b;
    if (a < k && jacobi32(a, k) == 1) out |= 1u << b;
  }
  bits[word_off[t] + w] = out;
}

cudaError_t launch_jacobi_tables(const uint32_t *kodd, const uint32_t *word_off, const uint32_t *sel,
                                 const uint32_t *first, uint32_t nsel, uint32_t total_words, uint32_t *bits,
                                 cudaStream_t st) {
  if (total_words == 0 || nsel == 0) return cudaSuccess;
  jacobi_table_kernel<<<(total_words + 255) / 256, 256, 0, st>>>(kodd, word_off, sel, first, nsel, total_words,
                                                                 bits);
  return cudaGetLastError();
}

cudaError_t launch_setup(const JobDev &job, const ChunkBufs &cb, cudaStream_t st) {
  const unsigned blocks = (cb.cap + 127) / 128;
  setup_kernel<<<blocks, 128, 0, st>>>(job, cb);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Baby-step giant-step, one prime per warp.

// Candidate check of x = e0 + m*s - j on row `row`, then one atomic append.
__device__ __forceinline__ void record_hit(const JobDev &J, const HitBufs &hb, uint64_t p, uint32_t row,
                                           uint32_t s, uint32_t j) {
  const int64_t x = J.e0 + (int64_t)J.m * (int64_t)s - (int64_t)j;
  if (x < (int64_t)J.x_lo || x > (int64_t)J.x_hi) return;
  const uint64_t n = (uint64_t)x * J.Q + J.row_r[row];
  if (n < J.nmin || n > J.nmax) return;
  const uint32_t bit = (uint32_t)(x - J.x_lo);
  if (!J.datless) {
    const uint32_t w = J.bitmap[(size_t)row * J.words_per_row + (bit >> 5)];
    if (!((w >> (bit & 31)) & 1u)) return;
  }
  const uint32_t idx = atomicAdd(hb.raw_count, 1u);
  if (idx < hb.cap) {
    Hit h;
    h.p = p;
    h.k = J.k_val[J.row_kidx[row]];
    h.n = (uint32_t)n;
    hb.raw[idx] = h;
  }
}

// Asynchronous copy of the first `elems` (even) elements of prime i's record
// into shared memory: 16-byte cp.async chunks, one group per lane.
__device__ __forceinline__ void stage_copy(uint64_t *dst, const JobDev &J, const ChunkBufs &cb, uint32_t i,
                                           uint32_t elems, uint32_t lane) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
  const uint64_t *src = cb.recs + (size_t)i * J.rec_elems;
#pragma unroll 1
  for (uint32_t e = 2 * lane; e < elems; e += 64)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d + 8 * e), "l"(src + e) : "memory");
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}

__device__ __forceinline__ void stage_commit_empty() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void stage_wait_prev() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void stage_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Index of the n-th (from 0) set bit of a row mask (row_mask records).
__device__ __forceinline__ uint32_t nth_row(uint64_t mask, uint32_t n) {
#pragma unroll 1
  for (uint32_t t = 0; t < n; t++) mask &= mask - 1;
  return (uint32_t)(__ffsll((long long)mask) - 1);
}

struct __align__(16) Match {
  uint64_t y;     // giant-step value whose tag matched
  uint32_t slot;  // active-row slot
  uint32_t s;     // giant index
};

// 16-bit tag of a residue: the high half of its low word (the bucket index
// uses the low log2(NB) <= 16 bits), raised to 1 if 0 (0 marks an empty slot).
// tag_pair gives it in both halves, t*0x10001: the high half copied to both
// halves, each raised to at least 1; its low half is the tag itself.
__device__ __forceinline__ uint32_t tag_pair(uint32_t lo) { return __vmaxu2(__byte_perm(lo, 0, 0x3232), 0x00010001u); }

// Nonzero iff some 16-bit half of x is zero: (x - 0x10001) & ~x sets bit 15 of
// the low half iff it is zero, and bit 15 of the high half iff it is zero or
// the low half borrowed (which only happens when the low half is zero).
__device__ __forceinline__ uint32_t zero_half(uint32_t x) { return (x - 0x00010001u) & ~x & 0x80008000u; }

// Bucket layout: 16 bytes = eight 16-bit tags (0 = empty).  True iff one of
// the 8 tags equals the tag pair T = t*0x10001.
__device__ __forceinline__ bool bucket_has(const uint4 &q, uint32_t T) {
  return zero_half(__vminu2(__vminu2(q.x ^ T, q.y ^ T), __vminu2(q.z ^ T, q.w ^ T))) != 0;
}

constexpr uint32_t kSlots = 8;  // tag slots per bucket

// Hash-table view of a prime's shared memory: NB buckets of tags and NB 32-bit
// insert counts, kept apart from the buckets so that the counts of a warp's 32
// random buckets spread over all 32 banks.  An insert takes slot c of its
// bucket from an atomic add on the bucket's count and writes its tag there with
// a plain 16-bit store.  Slots fill in order, so a bucket is full iff its slot 7
// holds a tag, and an entry overflows into the next bucket only when its bucket
// is full: a probe scans from the home bucket to the first bucket that is not
// full.  The home bucket comes from the low 16 bits of a residue's low word and
// the tag from the high 16 bits: the low bits masked when NB is a power of two
// (MUL false), else scaled, (lo16 * NB) >> 16 (MUL true; any NB <= 65536), which
// lets a CTA size its table to its shared memory instead of to a power of two.
//
// SIG: the bucket's count word also holds a 16-bit signature of its entries:
// the count in bits 0-15 (a bucket sees at most one increment per baby step,
// and the planner keeps CTA plans below 2^16 baby steps, so it never carries
// out), and bit 16 + sig(v) set (atomic OR) for every entry v
// stored there, sig(v) a 4-bit hash of v's high word.  A tag match counts only
// if the bucket holding the tag has the signature bit of the probed value, so
// with ~2 entries a bucket ~88% of the false 16-bit matches are rejected
// before they cost a pass over the baby steps; a true match always has its bit.
template <bool MUL, bool SIG = false>
struct TableT {
  uint4 *tab4;
  uint16_t *tab16;
  uint32_t *cnt32;
  uint32_t nb;     // buckets
  uint32_t bmask;  // nb - 1 (MUL false)

  __device__ __forceinline__ uint32_t home(uint32_t lo) const {
    return MUL ? (uint32_t)(((lo & 0xffffu) * nb) >> 16) : (lo & bmask);
  }
  __device__ __forceinline__ uint32_t next(uint32_t b) const {
    return MUL ? (b + 1 == nb ? 0u : b + 1) : ((b + 1) & bmask);
  }
  __device__ __forceinline__ static uint32_t sig_bit(uint64_t v) {
    return 1u << (16 + ((uint32_t)(v >> 32) * 0x9E3779B1u >> 28));
  }

  __device__ __forceinline__ uint32_t take(uint32_t b) const {
    const uint32_t c = atomicAdd(&cnt32[b], 1u);
    return SIG ? c & 0xffffu : c;
  }
  __device__ __forceinline__ void store(uint64_t v, uint32_t b, uint32_t c) const {
    tab16[b * kSlots + c] = (uint16_t)tag_pair((uint32_t)v);
    if (SIG) atomicOr(&cnt32[b], sig_bit(v));
  }

  // Insert continuing after bucket b, whose slots are all taken.
  __device__ __forceinline__ void insert_after(uint64_t v, uint32_t b) const {
    uint32_t c = kSlots;
#pragma unroll 1
    for (uint32_t g = 0; c >= kSlots && g + 1 < nb; g++) {
      b = next(b);
      c = take(b);
    }
    if (c < kSlots) store(v, b, c);
  }

  // Insert into the home bucket; false if it was full (the caller finishes the
  // insert later with insert_after, keeping the rare overflow off the hot loop).
  __device__ __forceinline__ bool insert_home(uint64_t v) const {
    const uint32_t b = home((uint32_t)v);
    const uint32_t c = take(b);
    if (c < kSlots) store(v, b, c);
    return c < kSlots;
  }

  // Home-bucket test: true if the tag of y is in y's home bucket or that bucket
  // is full (then only probe() can tell).
  __device__ __forceinline__ bool probe_home(uint64_t y) const {
    const uint32_t lo = (uint32_t)y;
    const uint4 q = tab4[home(lo)];
    const uint32_t T = tag_pair(lo);
    const uint32_t m = __vminu2(__vminu2(q.x ^ T, q.y ^ T), __vminu2(q.z ^ T, q.w ^ T));
    return (zero_half(m) | (q.w & 0xffff0000u)) != 0;  // a tag match, or slot 7 taken
  }

  // True iff some entry with the tag of y (and, SIG, the signature bit of y)
  // lies in y's probe sequence.
  __device__ __forceinline__ bool probe(uint64_t y) const {
    const uint32_t lo = (uint32_t)y;
    uint32_t b = home(lo);
    const uint32_t T = tag_pair(lo);
    const uint32_t sb = SIG ? sig_bit(y) : 0u;
    auto has = [&](const uint4 &q, uint32_t bk) { return bucket_has(q, T) && (!SIG || (cnt32[bk] & sb)); };
    uint4 q = tab4[b];
    bool hit = has(q, b);
    if (q.w >= 0x10000u) {  // the home bucket is full, continue scanning
#pragma unroll 1
      for (uint32_t g = 0; g + 1 < nb; g++) {
        b = next(b);
        q = tab4[b];
        hit |= has(q, b);
        if (q.w < 0x10000u) break;
      }
    }
    return hit;
  }
};
using WarpTable = TableT<false>;

struct MatchList {
  Match *list;
  uint32_t *count;
  uint32_t cap;  // matches the list holds; the baby phase's overflow values use the same space (2*cap)
  // Baby-phase use of the same space: up to 2*cap values to insert late.
  __device__ __forceinline__ void append(uint64_t *ovf, uint64_t v) const {
    const uint32_t idx = atomicAdd(count, 1u);
    if (idx < 2 * cap) ovf[idx] = v;
  }
  __device__ __forceinline__ void push(uint64_t y, uint32_t slot, uint32_t s) const {
    const uint32_t idx = atomicAdd(count, 1u);
    if (idx < cap) {
      Match mt;
      mt.y = y;
      mt.slot = slot;
      mt.s = s;
      list[idx] = mt;
    }
  }
};

// One chain step: the product by B, as Shoup's product by the full-size
// constant or, when the chunk allows it, as the short product by the integer b^Q.
struct StepShoup {
  uint64_t w, wq, p;
  __device__ __forceinline__ uint64_t operator()(uint64_t x) const { return shoup_mul(x, w, wq, p); }
};
struct StepSmall {
  uint32_t c, rc;
  uint64_t p;
  __device__ __forceinline__ uint64_t operator()(uint64_t x) const { return mul_small(x, c, rc, p); }
};
// b^Q * 2^32 < p (large primes): Shoup's product with a 32-bit constant.
struct StepHigh {
  uint32_t w, wq;
  uint64_t p;
  __device__ __forceinline__ uint64_t operator()(uint64_t x) const { return shoup_mul_w32(x, w, wq, p); }
};

// Baby steps of one lane: two chains of `len` steps from va and vb, of which
// the first na (nb) are inserted (all of them when FULL).  A value whose home bucket is full is
// appended to ovf and inserted after the loop.
template <bool FULL, class Step, class Table>
__device__ __forceinline__ void baby_chains(const Table &W, const MatchList &ML, uint64_t *ovf, uint64_t va,
                                            uint64_t vb, uint32_t na, uint32_t nb, uint32_t len, const Step &step) {
#pragma unroll 4
  for (uint32_t t = 0; t < len; t++) {
    const bool fa = (!FULL && t >= na) || W.insert_home(va);
    const bool fb = (!FULL && t >= nb) || W.insert_home(vb);
    if (!(fa && fb)) {
      if (!fa) ML.append(ovf, va);
      if (!fb) ML.append(ovf, vb);
    }
    va = step(va);
    vb = step(vb);
  }
}

// Giant steps with one step per row slot: lane (lane_row) multiplies the V of
// slots gi*RPI + lane_row and (gi+1)*RPI + lane_row by its G^(lane_t+1) and
// tests the home buckets; bit gi/2 of hA (hB) records a hit or full bucket.
// PAIRED (RPI == 1 only): slots gi, gi+1 hold a (k, 0), (k, 1) pair, so the
// second value is the first times the integer b (the short product).
// INT: integer rows with k*b^r in V (Shoup's product for a 32-bit operand).
template <uint32_t RPI, bool PAIRED = false, bool INT = false>
__device__ __forceinline__ void giant_home(const WarpTable &W, const uint64_t *__restrict__ Vs, uint32_t ngi,
                                           uint32_t nact, uint32_t lane_row, uint64_t Glw, uint64_t Glq, uint64_t p,
                                           uint32_t &hA, uint32_t &hB, uint32_t b = 0, uint32_t rc = 0) {
#pragma unroll 2
  for (uint32_t gi = 0; gi < ngi; gi += 2) {
    uint64_t va, vb;
    if (RPI == 1) {
      // slots gi, gi+1 are adjacent: one 16-byte load (gi even, V 16-byte
      // aligned).  Slot gi+1 may be past nact; its value (still inside the V
      // area) is discarded after the loop.
      const uint4 w = *reinterpret_cast<const uint4 *>(Vs + gi);
      va = ((uint64_t)w.y << 32) | w.x;
      vb = ((uint64_t)w.w << 32) | w.z;
    } else {
      const uint32_t sa = gi * RPI + lane_row;
      va = Vs[min(sa, nact - 1)];
      vb = Vs[min(sa + RPI, nact - 1)];
    }
    const uint64_t ya = INT ? shoup_mul32((uint32_t)va, Glw, Glq, p) : shoup_mul(va, Glw, Glq, p);
    const uint64_t yb = PAIRED ? mul_small(ya, b, rc, p)
                               : (INT ? shoup_mul32((uint32_t)vb, Glw, Glq, p) : shoup_mul(vb, Glw, Glq, p));
    const uint32_t bit = 1u << (gi >> 1);
    if (W.probe_home(ya)) hA |= bit;
    if (W.probe_home(yb)) hB |= bit;
  }
}

// The same for integer rows: slot gi holds a row id (16 bits), whose k*b^r is
// read from the job's table (read-only cache) and multiplied by the lane's Z
// with Shoup's product for a 32-bit operand.  A slot past nact (RPI == 1, nact
// odd) repeats slot gi; its outcome is discarded after the loop.
template <uint32_t RPI, bool PAIRED = false>
__device__ __forceinline__ void giant_home_int(const WarpTable &W, const uint16_t *__restrict__ Rs,
                                               const uint32_t *__restrict__ ctab, uint32_t ngi, uint32_t nact,
                                               uint32_t lane_row, uint64_t Glw, uint64_t Glq, uint64_t p, uint32_t &hA,
                                               uint32_t &hB, uint32_t b = 0, uint32_t rc = 0) {
#pragma unroll 2
  for (uint32_t gi = 0; gi < ngi; gi += 2) {
    uint32_t ra, rb;
    if (RPI == 1) {
      const uint32_t rr = *reinterpret_cast<const uint32_t *>(Rs + gi);  // slots gi, gi+1 (gi even)
      ra = rr & 0xffffu;
      rb = gi + 1 < nact ? rr >> 16 : ra;
    } else {
      const uint32_t sa = gi * RPI + lane_row;
      ra = Rs[min(sa, nact - 1)];
      rb = Rs[min(sa + RPI, nact - 1)];
    }
    const uint64_t ya = shoup_mul32(__ldg(ctab + ra), Glw, Glq, p);
    const uint64_t yb = PAIRED ? mul_small(ya, b, rc, p) : shoup_mul32(__ldg(ctab + rb), Glw, Glq, p);
    const uint32_t bit = 1u << (gi >> 1);
    if (W.probe_home(ya)) hA |= bit;
    if (W.probe_home(yb)) hB |= bit;
  }
}

// The work of one prime in the warp-per-prime layout, the whole warp together:
// baby steps into the table, giant steps with home-bucket tests, deferred
// probes, and the exact resolution of tag matches.  cur is the prime's staged
// record (header, and V or the row mask; nact != 0), Bl and Glm the lane's two
// table entries, c_lo / c_hi (row_mask) the lane's row constants; npaired
// counts the primes that took the row-pair path.  Shared by the single-job
// kernel and the multi-job kernel below.
template <int TL, int RM>
__device__ __forceinline__ void bsgs_prime(const JobDev &J, const ChunkBufs &cb, const HitBufs &hb,
                                           const WarpTable &W, const MatchList &ML, uint64_t *vbuf,
                                           const uint64_t *cur, uint32_t i, uint32_t nact, uint64_t Bl,
                                           uint64_t Glm, uint32_t lane, uint32_t c_lo, uint32_t c_hi,
                                           uint32_t &npaired) {
  constexpr uint32_t RPI = 32 / TL;  // row slots per lane-group pass
  const uint32_t lane_t = lane & (TL - 1);
  const uint32_t lane_row = lane / TL;
  const uint32_t spl = J.steps_per_lane;
  if constexpr (RM == kRowsMask) {  // V from the active-row mask
    const uint64_t am = cur[kElV];
    const uint32_t lo = (uint32_t)am, hi = (uint32_t)(am >> 32), below = (1u << lane) - 1u;
    if ((lo >> lane) & 1u) vbuf[__popc(lo & below)] = c_lo;
    if ((hi >> lane) & 1u) vbuf[__popc(lo) + __popc(hi & below)] = c_hi;
  }
  const uint64_t p = cur[kElP], pinv = cur[kElPinv];
  // Multipliers in normal form with their Shoup constants; the values
  // they multiply stay in Montgomery form, so products stay comparable.
  const uint64_t Stw = cur[kElStw], Stq = cur[kElStq];
  const uint64_t Gw = cur[kElGw], Gq = cur[kElGq];
  const uint64_t Glw = from_mont(Glm, p, pinv), Glq = shoup_const(Glm, pinv);
  // chain starts B^(lane*CL) and B^((lane+32)*CL); valid steps na, nb (j < m)
  const uint32_t CL = J.chain_len;
  const uint32_t ja0 = lane * CL, jb0 = ja0 + 32 * CL;
  const uint32_t na = J.m > ja0 ? min(CL, J.m - ja0) : 0;
  const uint32_t nb = J.m > jb0 ? min(CL, J.m - jb0) : 0;
  const uint64_t Blb = shoup_mul(Bl, cur[kElOfw], cur[kElOfq], p);
  // clear the table (tags and counts)
  const uint4 z4 = make_uint4(0, 0, 0, 0);
#pragma unroll 4
  for (uint32_t q = lane; q < W.nb + W.nb / 4; q += 32) W.tab4[q] = z4;
  if (lane == 0) *ML.count = 0;
  __syncwarp();

  // Baby steps: chain A owns j = ja0 + t, chain B j = jb0 + t.  Values whose
  // home bucket is full go to a short list (the match list's space, unused
  // until the giant steps) and are inserted after the loop.
  uint64_t *ovf = reinterpret_cast<uint64_t *>(ML.list);
  if (J.m == 64 * CL) {  // every chain full (the planner's usual choice of m)
    // (kStepHigh chunks take Shoup's product here: a third baby loop in this
    // kernel measured slower on the short-product path)
    if (cb.small_step == kStepSmall)
      baby_chains<true>(W, ML, ovf, Bl, Blb, na, nb, CL, StepSmall{J.bq_small, (uint32_t)cur[kElRcp], p});
    else
      baby_chains<true>(W, ML, ovf, Bl, Blb, na, nb, CL, StepShoup{Stw, Stq, p});
  } else {
    if (cb.small_step == kStepSmall)
      baby_chains<false>(W, ML, ovf, Bl, Blb, na, nb, CL, StepSmall{J.bq_small, (uint32_t)cur[kElRcp], p});
    else
      baby_chains<false>(W, ML, ovf, Bl, Blb, na, nb, CL, StepShoup{Stw, Stq, p});
  }
  __syncwarp();
  const uint32_t novf = *ML.count;
  if (novf > 2 * ML.cap) {  // pathological table: leave the prime to the exact path
    if (lane == 0) {
      const uint32_t r = atomicAdd(cb.redo_count, 1u);
      if (r < cb.cap) cb.redo[r] = i;
    }
    __syncwarp();
    return;
  }
  if (novf) {
    const uint64_t v = lane < novf ? ovf[lane] : 0;
    __syncwarp();
    if (lane == 0) *ML.count = 0;
    if (lane < novf) W.insert_after(v, W.home((uint32_t)v));
    __syncwarp();
  }

  // Giant steps: lane (lane_row, lane_t) takes row slots g*RPI + lane_row for
  // two consecutive passes g at a time, giant indices s = lane_t + 1 (+32).
  const uint32_t ngi = (nact + RPI - 1) / RPI;
  const uint64_t *Vs = J.stage_full ? cur + kElV : cb.recs + (size_t)i * J.rec_elems + kElV;
  // integer rows: the row ids (16 bits) of the staged or global record
  const uint16_t *Rs = reinterpret_cast<const uint16_t *>(
      J.stage_full ? cur + J.el_row : cb.recs + (size_t)i * J.rec_elems + J.el_row);
  // the giant value of slot sl (the general and the integer-row form)
  auto giant_val = [&](uint32_t sl) -> uint64_t {
    if constexpr (RM == kRowsIntId) return shoup_mul32(__ldg(J.row_c + Rs[sl]), Glw, Glq, p);
    else if constexpr (RM == kRowsIntV) return shoup_mul32((uint32_t)Vs[sl], Glw, Glq, p);
    else if constexpr (RM == kRowsMask) return shoup_mul32((uint32_t)vbuf[sl], Glw, Glq, p);
    else return shoup_mul(Vs[sl], Glw, Glq, p);
  };
  if (spl == 1 && ngi <= 64) {
    // One giant step per slot.  The loop only tests each value's home
    // bucket and collects the outcome as bits (pass gi of chain A or B ->
    // bit gi/2); tag hits and full home buckets are finished after it.
    // Separate calls for staged and global V keep each load's address
    // space known to the compiler.
    uint32_t hA = 0, hB = 0;
    const bool paired = RPI == 1 && cb.small_step == kStepSmall && (cur[kElNact] >> 32);
    npaired += paired && J.stage_full;
    if constexpr (RM == kRowsIntId) {
      const uint16_t *Rst = reinterpret_cast<const uint16_t *>(cur + J.el_row);
      if (paired && J.stage_full)
        giant_home_int<RPI, RPI == 1>(W, Rst, J.row_c, ngi, nact, lane_row, Glw, Glq, p, hA, hB, J.base,
                                      (uint32_t)cur[kElRcp]);
      else if (J.stage_full)
        giant_home_int<RPI>(W, Rst, J.row_c, ngi, nact, lane_row, Glw, Glq, p, hA, hB);
      else
        giant_home_int<RPI>(W, Rs, J.row_c, ngi, nact, lane_row, Glw, Glq, p, hA, hB);
    } else {
      constexpr bool INT = RM == kRowsIntV || RM == kRowsMask;
      const uint64_t *Vst = RM == kRowsMask ? vbuf : cur + kElV;  // V in shared memory
      if (paired && J.stage_full)
        giant_home<RPI, RPI == 1, INT>(W, Vst, ngi, nact, lane_row, Glw, Glq, p, hA, hB, J.base,
                                       (uint32_t)cur[kElRcp]);
      else if (J.stage_full)
        giant_home<RPI, false, INT>(W, Vst, ngi, nact, lane_row, Glw, Glq, p, hA, hB);
      else
        giant_home<RPI, false, INT>(W, Vs, ngi, nact, lane_row, Glw, Glq, p, hA, hB);
    }
    if (hA | hB) {
#pragma unroll 1
      for (uint32_t h = 0; h < 2; h++) {
        uint32_t bits = h ? hB : hA;
        while (bits) {
          const uint32_t g = 2 * (__ffs(bits) - 1) + h;
          bits &= bits - 1;
          const uint32_t sl = g * RPI + lane_row;
          if (sl < nact) {
            const uint64_t y = giant_val(sl);
            if (W.probe(y)) ML.push(y, sl, lane_t + 1);
          }
        }
      }
    }
  } else {
#pragma unroll 1
    for (uint32_t gi = 0; gi < ngi; gi += 2) {
      const uint32_t sa = gi * RPI + lane_row, sb = sa + RPI;
      const bool aa = sa < nact, ab = sb < nact;
      uint64_t ya = giant_val(min(sa, nact - 1));
      uint64_t yb = giant_val(min(sb, nact - 1));
      uint32_t s = lane_t + 1;
#pragma unroll 1
      for (uint32_t u = 0;; u++) {
        if (W.probe(ya) && aa) ML.push(ya, sa, s);
        if (W.probe(yb) && ab) ML.push(yb, sb, s);
        if (u + 1 >= spl) break;
        ya = shoup_mul(ya, Gw, Gq, p);
        yb = shoup_mul(yb, Gw, Gq, p);
        s += 32;
      }
    }
  }
  __syncwarp();

  // Tag matches: recompute the baby steps and compare full 64-bit values.
  const uint32_t mc = *ML.count;
  if (mc > (uint32_t)kMatchCap) {
    if (lane == 0) {
      const uint32_t r = atomicAdd(cb.redo_count, 1u);
      if (r < cb.cap) cb.redo[r] = i;
    }
  } else if (mc > 0) {
    uint64_t va = Bl, vb = Blb;
#pragma unroll 1
    for (uint32_t t = 0; t < CL; t++) {
#pragma unroll 1
      for (uint32_t h = 0; h < 2; h++) {
        const uint64_t v = h ? vb : va;
        if (t < (h ? nb : na)) {
#pragma unroll 1
          for (uint32_t q = 0; q < mc; q++) {
            const Match mt = ML.list[q];
            if (mt.y == v) {
              uint32_t row;
              if constexpr (RM == kRowsMask) {
                row = nth_row(cur[kElV], mt.slot);
              } else {
                const uint64_t pk = rec_el(J, cb, J.el_row + (mt.slot >> 2), i);
                row = (uint32_t)(pk >> (16 * (mt.slot & 3))) & 0xffffu;
              }
              record_hit(J, hb, p, row, mt.s, (h ? jb0 : ja0) + t);
            }
          }
        }
      }
      va = shoup_mul(va, Stw, Stq, p);
      vb = shoup_mul(vb, Stw, Stq, p);
    }
  }
}

// Per-warp shared memory of the fast kernel:
//   [NB buckets x 16 B][NB counts x 4 B][2 stages x stage_elems x 8 B]
//   ([kMaskRows V x 8 B], row_mask only)[kMatchCap matches][count, 16 B]
// The stages hold a record's header and V (double-buffered with cp.async); each
// lane's B^lane and G^(lane+1) entries are loaded into registers one prime ahead.
// With row_mask the stage holds the header and the active-row mask, and the
// warp writes V (the integers k*b^r of the active rows, in row order) into its
// own buffer from the constants of rows lane and lane + 32 that each lane keeps
// in registers.
//
// Each lane runs two independent product chains in both phases (baby steps
// j = lane + 64t and j = lane + 32 + 64t; giant steps on two row slots at a
// time) so that consecutive dependent Shoup products overlap.
// TL = giant steps handled side by side per row (min(T, 32)); RM = the form
// of the giant-step start values (kRowsV, kRowsIntV, kRowsIntId).
template <int TL, int RM>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, 4)
bsgs_kernel(JobDev J, ChunkBufs cb, HitBufs hb) {
  extern __shared__ uint4 smem4[];
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t NB = 1u << J.table_log2;
  uint8_t *base = reinterpret_cast<uint8_t *>(smem4) + (size_t)warp * J.warp_smem;
  WarpTable W;
  W.tab4 = reinterpret_cast<uint4 *>(base);
  W.tab16 = reinterpret_cast<uint16_t *>(base);
  W.cnt32 = reinterpret_cast<uint32_t *>(base + NB * 16);
  W.nb = NB;
  W.bmask = NB - 1;
  uint64_t *stage0 = reinterpret_cast<uint64_t *>(base + NB * 20);
  uint64_t *vbuf = stage0 + 2 * J.stage_elems;  // row_mask: V of the current prime
  MatchList ML;
  ML.list = reinterpret_cast<Match *>(vbuf + (RM == kRowsMask ? kMaskRows : 0));
  ML.count = reinterpret_cast<uint32_t *>(ML.list + kMatchCap);
  ML.cap = kMatchCap;
  const uint32_t total = *cb.count;
  const uint32_t n = total < cb.cap ? total : cb.cap;
  const uint32_t nwarps = gridDim.x * kWarpsPerBlock;
  const uint32_t first = blockIdx.x * kWarpsPerBlock + warp;
  const uint64_t *ltab = cb.recs + J.el_tab + lane;  // this lane's B^lane; G^(lane+1) 32 further

  uint64_t nBl = 0, nGl = 0;
  uint32_t npaired = 0;  // primes of this warp that took the row-pair path
  uint32_t c_lo = 0, c_hi = 0;  // row_mask: k*b^r of rows lane and lane + 32
  if constexpr (RM == kRowsMask) {
    c_lo = lane < J.nrows ? __ldg(J.row_c + lane) : 0u;
    c_hi = lane + 32 < J.nrows ? __ldg(J.row_c + lane + 32) : 0u;
  }
  if (first < n) {
    stage_copy(stage0, J, cb, first, J.stage_elems, lane);
    nBl = __ldg(ltab + (size_t)first * J.rec_elems);
    nGl = __ldg(ltab + (size_t)first * J.rec_elems + 32);
  } else {
    stage_commit_empty();
  }

#pragma unroll 1
  for (uint32_t it = 0;; it++) {
    const uint32_t i = first + it * nwarps;
    if (i >= n) break;
    const uint64_t *cur = stage0 + (it & 1) * J.stage_elems;
    uint64_t *nxt = stage0 + ((it + 1) & 1) * J.stage_elems;
    const uint64_t Bl = nBl, Glm = nGl;
    if (i + nwarps < n) {
      stage_copy(nxt, J, cb, i + nwarps, J.stage_elems, lane);
      nBl = __ldg(ltab + (size_t)(i + nwarps) * J.rec_elems);
      nGl = __ldg(ltab + (size_t)(i + nwarps) * J.rec_elems + 32);
    } else {
      stage_commit_empty();
    }
    stage_wait_prev();
    __syncwarp();
    const uint32_t nact = (uint32_t)cur[kElNact];
    if (nact != 0) bsgs_prime<TL, RM>(J, cb, hb, W, ML, vbuf, cur, i, nact, Bl, Glm, lane, c_lo, c_hi, npaired);
    __syncwarp();
  }
  stage_wait_all();
  if (lane == 0 && npaired) atomicAdd(&hb.stat[kStatPaired], (unsigned long long)npaired);
}

// The warp-per-prime BSGS over many jobs in one persistent launch (the batched
// form): the primes of every item's chunk form one index space, and each warp
// walks it with the grid stride, so the work of small and large jobs spreads
// over the whole GPU in one launch instead of one launch per job.  Every item
// has its own constants (JobDev, read from global memory), records, hit buffers
// and baby-step product; all items share the template's giant lanes TL and
// start-value form RM.  Per-warp shared memory, in fixed places whatever the
// item:
//   [2 stages x stage_max x 8 B]([kMaskRows V x 8 B], RM = kRowsMask)[kMatchCap matches][count, 16 B]
//   [the item's table: NB buckets x 16 B, NB counts x 4 B]
// The record of the warp's next prime (possibly another item's) is staged by
// cp.async while the current one runs, as in bsgs_kernel.
template <int TL, int RM>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, 4)
bsgs_batch_kernel(const BatchItem *__restrict__ items, uint32_t nitems, uint32_t warp_bytes, uint32_t stage_max) {
  extern __shared__ uint4 smem4[];
  __shared__ uint32_t start[kBatchMaxItems + 1];  // prefix sums of the items' prime counts
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // the items' prime counts, loaded in parallel, then their prefix sums
  for (uint32_t k = threadIdx.x; k < nitems; k += blockDim.x) {
    const uint32_t c = *items[k].cb.count, cap = items[k].cb.cap;
    start[k + 1] = c < cap ? c : cap;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    start[0] = 0;
    for (uint32_t k = 0; k < nitems; k++) start[k + 1] += start[k];
  }
  __syncthreads();
  const uint32_t total = start[nitems];
  uint8_t *base = reinterpret_cast<uint8_t *>(smem4) + (size_t)warp * warp_bytes;
  uint64_t *stage0 = reinterpret_cast<uint64_t *>(base);
  uint64_t *vbuf = stage0 + 2 * stage_max;
  MatchList ML;
  ML.list = reinterpret_cast<Match *>(vbuf + (RM == kRowsMask ? kMaskRows : 0));
  ML.count = reinterpret_cast<uint32_t *>(ML.list + kMatchCap);
  ML.cap = kMatchCap;
  uint8_t *tbase = reinterpret_cast<uint8_t *>(ML.count) + 16;
  const uint32_t nwarps = gridDim.x * kWarpsPerBlock;
  const uint32_t first = blockIdx.x * kWarpsPerBlock + warp;
  // the item of global index g, from the item of an earlier (smaller) index
  auto locate = [&](uint32_t g, uint32_t k) {
    while (k + 1 < nitems && g >= start[k + 1]) k++;
    return k;
  };

  uint64_t nBl = 0, nGl = 0;
  uint32_t nk = 0;               // item of the staged next prime
  uint32_t ck = 0xffffffffu;     // item whose row constants the lanes hold
  uint32_t c_lo = 0, c_hi = 0;
  uint32_t npaired = 0;          // paired primes of item ck not yet added to its counter
  auto prefetch = [&](uint32_t g, uint64_t *dst) {
    nk = locate(g, nk);
    const BatchItem &X = items[nk];
    const uint32_t i = g - start[nk];
    stage_copy(dst, X.J, X.cb, i, X.J.stage_elems, lane);
    const uint64_t *lt = X.cb.recs + (size_t)i * X.J.rec_elems + X.J.el_tab + lane;
    nBl = __ldg(lt);
    nGl = __ldg(lt + 32);
  };
  if (first < total) prefetch(first, stage0);
  else stage_commit_empty();

#pragma unroll 1
  for (uint32_t it = 0;; it++) {
    const uint32_t g = first + it * nwarps;
    if (g >= total) break;
    const uint32_t k = nk;
    const uint32_t i = g - start[k];
    const uint64_t *cur = stage0 + (it & 1) * stage_max;
    uint64_t *nxt = stage0 + ((it + 1) & 1) * stage_max;
    const uint64_t Bl = nBl, Glm = nGl;
    if (g + nwarps < total) prefetch(g + nwarps, nxt);
    else stage_commit_empty();
    const BatchItem &X = items[k];
    if (k != ck) {
      if (lane == 0 && npaired) atomicAdd(&items[ck].hb.stat[kStatPaired], (unsigned long long)npaired);
      npaired = 0;
      ck = k;
      if constexpr (RM == kRowsMask) {
        c_lo = lane < X.J.nrows ? __ldg(X.J.row_c + lane) : 0u;
        c_hi = lane + 32 < X.J.nrows ? __ldg(X.J.row_c + lane + 32) : 0u;
      }
    }
    stage_wait_prev();
    __syncwarp();
    const uint32_t nact = (uint32_t)cur[kElNact];
    if (nact != 0) {
      const uint32_t NB = 1u << X.J.table_log2;
      WarpTable W;
      W.tab4 = reinterpret_cast<uint4 *>(tbase);
      W.tab16 = reinterpret_cast<uint16_t *>(tbase);
      W.cnt32 = reinterpret_cast<uint32_t *>(tbase + NB * 16);
      W.nb = NB;
      W.bmask = NB - 1;
      bsgs_prime<TL, RM>(X.J, X.cb, X.hb, W, ML, vbuf, cur, i, nact, Bl, Glm, lane, c_lo, c_hi, npaired);
    }
    __syncwarp();
  }
  stage_wait_all();
  if (lane == 0 && npaired && ck < nitems) atomicAdd(&items[ck].hb.stat[kStatPaired], (unsigned long long)npaired);
}

typedef void (*BatchFn)(const BatchItem *, uint32_t, uint32_t, uint32_t);

template <int RM>
static BatchFn batch_fn_t(uint32_t tlanes) {
  switch (tlanes) {
    case 1: return bsgs_batch_kernel<1, RM>;
    case 2: return bsgs_batch_kernel<2, RM>;
    case 4: return bsgs_batch_kernel<4, RM>;
    case 8: return bsgs_batch_kernel<8, RM>;
    case 16: return bsgs_batch_kernel<16, RM>;
    default: return bsgs_batch_kernel<32, RM>;
  }
}

typedef void (*BsgsFn)(JobDev, ChunkBufs, HitBufs);

template <int RM>
static BsgsFn bsgs_fn_t(uint32_t tlanes) {
  switch (tlanes) {
    case 1: return bsgs_kernel<1, RM>;
    case 2: return bsgs_kernel<2, RM>;
    case 4: return bsgs_kernel<4, RM>;
    case 8: return bsgs_kernel<8, RM>;
    case 16: return bsgs_kernel<16, RM>;
    default: return bsgs_kernel<32, RM>;
  }
}

static int row_mode(const JobDev &job) {
  return job.row_mask ? kRowsMask : job.row_ids_only ? kRowsIntId : job.int_rows ? kRowsIntV : kRowsV;
}

static BsgsFn bsgs_fn(const JobDev &job) {
  switch (row_mode(job)) {
    case kRowsMask: return bsgs_fn_t<kRowsMask>(job.tlanes);
    case kRowsIntId: return bsgs_fn_t<kRowsIntId>(job.tlanes);
    case kRowsIntV: return bsgs_fn_t<kRowsIntV>(job.tlanes);
    default: return bsgs_fn_t<kRowsV>(job.tlanes);
  }
}


int bsgs_smem_bytes(const JobDev &job) {
  return job.cta_warps > 1 ? (int)job.warp_smem : kWarpsPerBlock * (int)job.warp_smem;
}

// Giant steps of the CTA kernel: warp w takes row slots w, w + W, ..., four at
// a time (four independent product chains per lane).  The loop tests home
// buckets only and records the outcome as bits (step u of slot k -> bit 4u + k,
// spl <= 8); tag hits and full buckets are finished after each pass.  RM: vst
// holds V (kRowsV), the integers k*b^r (kRowsIntV) or 16-bit row ids whose
// k*b^r come from the job's table ctab (kRowsIntId; CS: ctab is the CTA's
// shared-memory copy of it).  TWO (integer rows, spl == 2): the
// second value of a slot is also c times a lane multiplier, Z advanced by G^32
// (Glw2, Glq2), so both products are independent short ones.
template <int RM, bool TWO, bool CS, class Table>
__device__ __forceinline__ void cta_giants(const Table &W, const MatchList &ML, const uint64_t *vst, uint32_t nact,
                                           uint32_t warp, uint32_t lane, uint32_t spl, uint64_t Glw, uint64_t Glq,
                                           uint64_t Gw, uint64_t Gq, uint64_t p, const uint32_t *__restrict__ ctab,
                                           uint64_t Glw2 = 0, uint64_t Glq2 = 0) {
  const uint16_t *rid = reinterpret_cast<const uint16_t *>(vst);
  auto row_c = [&](uint32_t r) -> uint32_t { return CS ? ctab[r] : __ldg(ctab + r); };
#pragma unroll 1
  for (uint32_t s0 = warp; s0 < nact; s0 += 4 * kCtaWarps) {
    uint64_t y[4];
    uint32_t c[4];
    uint32_t valid = 0;
#pragma unroll
    for (uint32_t k = 0; k < 4; k++) {
      const uint32_t sl = s0 + k * kCtaWarps;
      valid |= (sl < nact ? 0x11111111u : 0u) << k;
      if (RM == kRowsIntId) {
        c[k] = row_c(rid[sl < nact ? sl : s0]);
        y[k] = shoup_mul32(c[k], Glw, Glq, p);
      } else if (RM == kRowsIntV) {
        c[k] = (uint32_t)vst[sl < nact ? sl : s0];
        y[k] = shoup_mul32(c[k], Glw, Glq, p);
      } else {
        y[k] = shoup_mul(vst[sl < nact ? sl : s0], Glw, Glq, p);
      }
    }
    uint32_t bits = 0;
    if (TWO) {
      uint64_t z[4];
#pragma unroll
      for (uint32_t k = 0; k < 4; k++) z[k] = shoup_mul32(c[k], Glw2, Glq2, p);
#pragma unroll
      for (uint32_t k = 0; k < 4; k++) {
        if (W.probe_home(y[k])) bits |= 1u << k;
        if (W.probe_home(z[k])) bits |= 1u << (4 + k);
      }
    } else {
#pragma unroll 1
      for (uint32_t u = 0;; u++) {
#pragma unroll
        for (uint32_t k = 0; k < 4; k++)
          if (W.probe_home(y[k])) bits |= 1u << (4 * u + k);
        if (u + 1 >= spl) break;
#pragma unroll
        for (uint32_t k = 0; k < 4; k++) y[k] = shoup_mul(y[k], Gw, Gq, p);
      }
    }
    bits &= valid;
    while (bits) {  // rare
      const uint32_t b = __ffs(bits) - 1;
      bits &= bits - 1;
      const uint32_t k = b & 3, u = b >> 2, sl = s0 + k * kCtaWarps;
      uint64_t v = RM == kRowsIntId  ? shoup_mul32(row_c(rid[sl]), Glw, Glq, p)
                   : RM == kRowsIntV ? shoup_mul32((uint32_t)vst[sl], Glw, Glq, p)
                                     : shoup_mul(vst[sl], Glw, Glq, p);
#pragma unroll 1
      for (uint32_t q = 0; q < u; q++) v = shoup_mul(v, Gw, Gq, p);
      if (W.probe(v)) ML.push(v, sl, lane + 1 + 32 * u);
    }
  }
}

// The CTA-per-prime kernel, for jobs whose best baby-step count needs a table
// larger than a warp's share of shared memory (many k, wide n ranges).  All
// kCtaWarps warps of a CTA work on one prime: thread t runs baby chains t and
// t + 32W into one table that fills most of the SM's shared memory, and warp w
// takes the giant steps of row slots w, w + W, ... (32 lanes per row, T/32
// steps per lane).  Shared memory:
//   [NB buckets x 16 B][NB count words x 4 B: insert count, entries' signature]
//   [V, max_act x 8 B][kCtaMatchCap matches][count, 16 B]([row table, nrows x 4 B])
// The row table (row ids only, when it fits) is copied once per launch.
// V is staged with cp.async during the baby steps.  Table operations, the
// deferred overflow inserts and the exact tag-match resolution are those of
// bsgs_kernel; hits are pushed where they are found (tag matches are rare).
template <int RM, bool MUL>
__global__ void __launch_bounds__(32 * kCtaWarps, 1) bsgs_cta_kernel(JobDev J, ChunkBufs cb, HitBufs hb) {
  extern __shared__ uint4 smem4[];
  constexpr uint32_t G = 32 * kCtaWarps;
  const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t NB = J.nbuckets;
  uint8_t *base = reinterpret_cast<uint8_t *>(smem4);
  TableT<MUL, true> W;
  W.tab4 = reinterpret_cast<uint4 *>(base);
  W.tab16 = reinterpret_cast<uint16_t *>(base);
  W.cnt32 = reinterpret_cast<uint32_t *>(base + NB * 16);
  W.nb = NB;
  W.bmask = NB - 1;
  uint64_t *vst = reinterpret_cast<uint64_t *>(base + NB * 20);
  const uint32_t vst_elems = RM == kRowsIntId ? 2 * ((J.max_act + 7) / 8) : (J.max_act + 1) & ~1u;
  MatchList ML;
  ML.list = reinterpret_cast<Match *>(vst + vst_elems);
  ML.count = reinterpret_cast<uint32_t *>(ML.list + kCtaMatchCap);
  ML.cap = kCtaMatchCap;
  uint64_t *ovf = reinterpret_cast<uint64_t *>(ML.list);
  const uint32_t total = *cb.count;
  const uint32_t n = total < cb.cap ? total : cb.cap;
  const uint32_t CL = J.chain_len, spl = J.steps_per_lane;
  const uint32_t ja0 = tid * CL, jb0 = (tid + G) * CL;  // the thread's chains; m == 2*G*CL
  const uint32_t vdst = (uint32_t)__cvta_generic_to_shared(vst);
  // the row table, copied once per launch (row ids, when it fits); the first
  // barrier of the prime loop orders these stores before any read
  uint32_t *cts = reinterpret_cast<uint32_t *>(reinterpret_cast<uint8_t *>(ML.count) + 16);
  if (RM == kRowsIntId && J.ctab_smem)
    for (uint32_t r = tid; r < J.nrows; r += G) cts[r] = __ldg(J.row_c + r);

#pragma unroll 1
  for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
    const uint64_t *rec = cb.recs + (size_t)i * J.rec_elems;
    const uint32_t nact = (uint32_t)rec[kElNact];
    if (nact == 0) continue;
    const uint64_t p = rec[kElP], pinv = rec[kElPinv];
    __syncthreads();  // the previous prime is done with the table, V and the list
    // V of the active rows (integer rows: their 16-bit row ids) into shared
    // memory, 16 bytes per copy
    constexpr bool IDS = RM == kRowsIntId;
    const uint32_t vn = IDS ? 2 * ((nact + 7) / 8) : (nact + 1) & ~1u;
    const uint64_t *vsrc = rec + (IDS ? J.el_row : J.el_v);
#pragma unroll 1
    for (uint32_t e = 2 * tid; e < vn; e += 2 * G)
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(vdst + 8 * e), "l"(vsrc + e)
                   : "memory");
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    const uint4 z4 = make_uint4(0, 0, 0, 0);
#pragma unroll 4
    for (uint32_t q = tid; q < NB + NB / 4; q += G) W.tab4[q] = z4;
    if (tid == 0) *ML.count = 0;
    __syncthreads();

    // Baby steps: chain starts B^(lane*c) times the warp's offset B^(32w*c)
    uint64_t Bl = rec[J.el_tab + lane];
    if (warp) Bl = shoup_mul(Bl, rec[kElWoff + 2 * warp], rec[kElWoff + 2 * warp + 1], p);
    const uint64_t Blb = shoup_mul(Bl, rec[kElOfw], rec[kElOfq], p);
    if (cb.small_step == kStepSmall)
      baby_chains<true>(W, ML, ovf, Bl, Blb, CL, CL, CL, StepSmall{J.bq_small, (uint32_t)rec[kElRcp], p});
    else if (cb.small_step == kStepHigh)
      baby_chains<true>(W, ML, ovf, Bl, Blb, CL, CL, CL, StepHigh{J.bq_small, (uint32_t)rec[kElStq], p});
    else
      baby_chains<true>(W, ML, ovf, Bl, Blb, CL, CL, CL, StepShoup{rec[kElStw], rec[kElStq], p});
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();
    const uint32_t novf = *ML.count;
    if (novf > 2 * ML.cap) {  // pathological table: leave the prime to the exact path
      if (tid == 0) {
        const uint32_t r = atomicAdd(cb.redo_count, 1u);
        if (r < cb.cap) cb.redo[r] = i;
      }
      continue;
    }
    if (novf) {
      const uint64_t v = tid < novf ? ovf[tid] : 0;
      __syncthreads();
      if (tid == 0) *ML.count = 0;
      if (tid < novf) W.insert_after(v, W.home((uint32_t)v));
      __syncthreads();
    }

    // Giant steps (cta_giants)
    const uint64_t Glm = rec[J.el_tab + 32 + lane];
    const uint64_t Glw = from_mont(Glm, p, pinv), Glq = shoup_const(Glm, pinv);
    const uint64_t Gw = rec[kElGw], Gq = rec[kElGq];
    if constexpr (RM == kRowsIntId) {
      if (spl == 2) {
        const uint64_t E2 = shoup_mul(Glm, Gw, Gq, p);  // Z advanced by G^32, times 2^128
        const uint64_t E2w = from_mont(E2, p, pinv), E2q = shoup_const(E2, pinv);
        if (J.ctab_smem)
          cta_giants<RM, true, true>(W, ML, vst, nact, warp, lane, spl, Glw, Glq, Gw, Gq, p, cts, E2w, E2q);
        else
          cta_giants<RM, true, false>(W, ML, vst, nact, warp, lane, spl, Glw, Glq, Gw, Gq, p, J.row_c, E2w, E2q);
      } else if (J.ctab_smem) {
        cta_giants<RM, false, true>(W, ML, vst, nact, warp, lane, spl, Glw, Glq, Gw, Gq, p, cts);
      } else {
        cta_giants<RM, false, false>(W, ML, vst, nact, warp, lane, spl, Glw, Glq, Gw, Gq, p, J.row_c);
      }
    } else if constexpr (RM == kRowsIntV) {
      if (spl == 2) {
        const uint64_t E2 = shoup_mul(Glm, Gw, Gq, p);  // Z advanced by G^32, times 2^128
        cta_giants<RM, true, false>(W, ML, vst, nact, warp, lane, spl, Glw, Glq, Gw, Gq, p, J.row_c,
                                    from_mont(E2, p, pinv), shoup_const(E2, pinv));
      } else {
        cta_giants<RM, false, false>(W, ML, vst, nact, warp, lane, spl, Glw, Glq, Gw, Gq, p, J.row_c);
      }
    } else {
      cta_giants<kRowsV, false, false>(W, ML, vst, nact, warp, lane, spl, Glw, Glq, Gw, Gq, p, J.row_c);
    }
    __syncthreads();

    // Tag matches: recompute the baby steps and compare full 64-bit values.
    const uint32_t mc = *ML.count;
    if (mc > ML.cap) {
      if (tid == 0) {
        const uint32_t r = atomicAdd(cb.redo_count, 1u);
        if (r < cb.cap) cb.redo[r] = i;
      }
    } else if (mc > 0) {
      // The first four matched values stay in registers (most primes have one
      // or two false tag matches); only a step whose value equals one of them
      // (or every step, with more than four matches) scans the list.
      const uint64_t y0 = ML.list[0].y;
      const uint64_t y1 = mc > 1 ? ML.list[1].y : y0;
      const uint64_t y2 = mc > 2 ? ML.list[2].y : y0;
      const uint64_t y3 = mc > 3 ? ML.list[3].y : y0;
      auto pass = [&](auto step) {
        uint64_t va = Bl, vb = Blb;
#pragma unroll 2
        for (uint32_t t = 0; t < CL; t++) {
          const bool in_a = va == y0 || va == y1 || va == y2 || va == y3;
          const bool in_b = vb == y0 || vb == y1 || vb == y2 || vb == y3;
          if (in_a || in_b || mc > 4) {
#pragma unroll 1
            for (uint32_t q = 0; q < mc; q++) {
              const Match mt = ML.list[q];
              if (mt.y == va || mt.y == vb) {  // both when B has a small order
                const uint64_t pk = rec_el(J, cb, J.el_row + (mt.slot >> 2), i);
                const uint32_t row = (uint32_t)(pk >> (16 * (mt.slot & 3))) & 0xffffu;
                if (mt.y == va) record_hit(J, hb, p, row, mt.s, ja0 + t);
                if (mt.y == vb) record_hit(J, hb, p, row, mt.s, jb0 + t);
              }
            }
          }
          va = step(va);
          vb = step(vb);
        }
      };
      if (cb.small_step == kStepSmall) pass(StepSmall{J.bq_small, (uint32_t)rec[kElRcp], p});
      else pass(StepShoup{rec[kElStw], rec[kElStq], p});
    }
  }
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// The exact path: a table of (tag << jbits) | j entries with linear probing per
// prime, for the primes whose tag matches overflowed the fast path's list.  WG
// warps share a prime (1 for warp-per-prime jobs, kCtaWarps for CTA jobs) with
// the same chain layout as the fast kernels.
template <int WG>
__global__ void __launch_bounds__(WG == 1 ? 32 * kWarpsPerBlock : 32 * WG, 1)
bsgs_exact_kernel(JobDev J, ChunkBufs cb, HitBufs hb) {
  extern __shared__ uint4 smem4[];
  constexpr uint32_t G = 32 * WG;                           // threads per prime
  constexpr uint32_t NG = WG == 1 ? kWarpsPerBlock : 1;     // primes per block
  const uint32_t grp = threadIdx.x / G, gt = threadIdx.x % G, wig = gt >> 5, lane = threadIdx.x & 31;
  const uint32_t S = 1u << J.exact_log2;
  const uint32_t tmask = S - 1;
  // the table in shared memory, or (tables larger than shared memory) in this
  // CTA's slice of the chunk's global scratch
  uint32_t *tab = (J.exact_global ? cb.exact_tab + (size_t)blockIdx.x * NG * S : reinterpret_cast<uint32_t *>(smem4)) +
                  (size_t)grp * S;
  const uint32_t jbits = J.jbits;
  const uint32_t jmask = (1u << jbits) - 1u;
  const uint32_t tagmask = (1u << (32 - jbits)) - 1u;
  const uint32_t tl = J.exact_log2;
  const uint32_t lane_t = lane & (J.tlanes - 1);
  const uint32_t lane_row = lane / J.tlanes;
  const uint32_t rows_pass = J.rows_per_it * WG;  // row slots per pass of the group
  const uint32_t rc = *cb.redo_count;
  const uint32_t nr = rc < cb.cap ? rc : cb.cap;
  const uint32_t ngroups = gridDim.x * NG;
  if (blockIdx.x == 0 && threadIdx.x == 0 && nr) atomicAdd(&hb.stat[kStatExact], (unsigned long long)nr);
#pragma unroll 1
  for (uint32_t r = blockIdx.x * NG + grp; r < nr; r += ngroups) {
    const uint32_t i = cb.redo[r];
    const uint64_t p = rec_el(J, cb, kElP, i), pinv = rec_el(J, cb, kElPinv, i);
    const uint32_t nact = (uint32_t)rec_el(J, cb, kElNact, i);
    const uint64_t Gs = rec_el(J, cb, kElGs, i);
    const uint64_t Stw = rec_el(J, cb, kElStw, i), Stq = rec_el(J, cb, kElStq, i);
    if (WG == 1) __syncwarp();
    else __syncthreads();
    for (uint32_t q = gt; q < S; q += G) tab[q] = kEmpty;
    if (WG == 1) __syncwarp();
    else __syncthreads();
    // the thread's two baby chains, j = (gt + G*c)*chain_len + t
    uint64_t Bl = rec_el(J, cb, J.el_tab + lane, i);
    if (WG > 1 && wig) Bl = shoup_mul(Bl, rec_el(J, cb, kElWoff + 2 * wig, i), rec_el(J, cb, kElWoff + 2 * wig + 1, i), p);
#pragma unroll 1
    for (uint32_t c = 0; c < 2; c++) {
      const uint32_t j0 = (gt + G * c) * J.chain_len;
      uint64_t v = c ? shoup_mul(Bl, rec_el(J, cb, kElOfw, i), rec_el(J, cb, kElOfq, i), p) : Bl;
#pragma unroll 1
      for (uint32_t j = j0; j < J.m && j < j0 + J.chain_len; j++) {
        uint32_t h = (uint32_t)v & tmask;
        const uint32_t e = ((((uint32_t)(v >> tl)) & tagmask) << jbits) | j;
#pragma unroll 1
        for (uint32_t t = 0; t < S; t++) {
          if (atomicCAS(&tab[h], kEmpty, e) == kEmpty) break;
          h = (h + 1) & tmask;
        }
        v = shoup_mul(v, Stw, Stq, p);
      }
    }
    if (WG == 1) __syncwarp();
    else __syncthreads();
    const uint64_t Gl = rec_el(J, cb, J.el_tab + 32 + lane, i);
    const uint32_t ngi = (nact + rows_pass - 1) / rows_pass;
#pragma unroll 1
    for (uint32_t gi = 0; gi < ngi; gi++) {
      const uint32_t slot = gi * rows_pass + wig * J.rows_per_it + lane_row;
      if (slot < nact) {
        const uint32_t row = J.row_mask ? nth_row(rec_el(J, cb, J.el_v, i), slot)
                                        : (uint32_t)(rec_el(J, cb, J.el_row + (slot >> 2), i) >> (16 * (slot & 3))) &
                                              0xffffu;
        // integer rows: montmul(k*b^r, Z * 2^128) is the Montgomery form of the giant value
        uint64_t y = montmul(J.row_ids_only || J.row_mask ? (uint64_t)__ldg(J.row_c + row)
                                                          : rec_el(J, cb, J.el_v + slot, i),
                             Gl, p, pinv);
        uint32_t s = lane_t + 1;
#pragma unroll 1
        for (uint32_t u = 0; u < J.steps_per_lane; u++) {
          uint32_t h = (uint32_t)y & tmask;
          const uint32_t tag = ((uint32_t)(y >> tl)) & tagmask;
#pragma unroll 1
          for (uint32_t q = 0; q < S; q++) {
            const uint32_t e = tab[h];
            if (e == kEmpty) break;
            if ((e >> jbits) == tag) record_hit(J, hb, p, row, s, e & jmask);
            h = (h + 1) & tmask;
          }
          if (u + 1 < J.steps_per_lane) {
            y = montmul(y, Gs, p, pinv);
            s += 32;
          }
        }
      }
    }
  }
}

int bsgs_exact_smem_bytes(const JobDev &job) {
  return job.exact_global ? 0 : (job.cta_warps > 1 ? 1 : kWarpsPerBlock) * (4 << job.exact_log2);
}

uint64_t bsgs_exact_scratch_bytes(const JobDev &job, int exact_grid) {
  if (!job.exact_global) return 0;
  return (uint64_t)exact_grid * (job.cta_warps > 1 ? 1 : kWarpsPerBlock) * (4ull << job.exact_log2);
}

static cudaError_t configure_one(const void *fn, int smem, int threads, int device, int *grid_out) {
  // The limit is a property of the kernel shared by every job in the process,
  // so it is set to the device maximum (the same value from every thread)
  // rather than to this job's size, which a concurrent job could lower.
  int max_smem = 0;
  cudaError_t e = cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  if (e != cudaSuccess) return e;
  cudaFuncAttributes fa;
  e = cudaFuncGetAttributes(&fa, fn);
  if (e != cudaSuccess) return e;
  max_smem -= (int)fa.sharedSizeBytes;  // the kernel's static shared memory counts against the same limit
  if (smem > max_smem) return cudaErrorInvalidValue;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
  if (e != cudaSuccess) return e;
  int sms = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  *grid_out = per_sm * sms;
  return cudaSuccess;
}

static int bsgs_threads(const JobDev &job) { return job.cta_warps > 1 ? 32 * kCtaWarps : 32 * kWarpsPerBlock; }

template <bool MUL>
static BsgsFn bsgs_cta_fn_t(const JobDev &job) {
  switch (row_mode(job)) {
    case kRowsIntId: return bsgs_cta_kernel<kRowsIntId, MUL>;
    case kRowsIntV: return bsgs_cta_kernel<kRowsIntV, MUL>;
    default: return bsgs_cta_kernel<kRowsV, MUL>;
  }
}

static BsgsFn bsgs_cta_fn(const JobDev &job) {
  const bool pow2 = (job.nbuckets & (job.nbuckets - 1)) == 0;
  return pow2 ? bsgs_cta_fn_t<false>(job) : bsgs_cta_fn_t<true>(job);
}

static const void *bsgs_fast_fn(const JobDev &job) {
  if (job.cta_warps > 1) return (const void *)bsgs_cta_fn(job);
  return (const void *)bsgs_fn(job);
}

static const void *bsgs_exact_fn(const JobDev &job) {
  return job.cta_warps > 1 ? (const void *)bsgs_exact_kernel<kCtaWarps> : (const void *)bsgs_exact_kernel<1>;
}

cudaError_t bsgs_configure(const JobDev &job, int device, int *grid_out, int *exact_grid_out) {
  cudaError_t e = configure_one(bsgs_fast_fn(job), bsgs_smem_bytes(job), bsgs_threads(job), device, grid_out);
  if (e != cudaSuccess) return e;
  e = configure_one(bsgs_exact_fn(job), bsgs_exact_smem_bytes(job), bsgs_threads(job), device, exact_grid_out);
  if (e != cudaSuccess) return e;
  if (job.exact_global) {  // one CTA per SM keeps the global scratch small (the exact path is rare)
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess && sms > 0 && *exact_grid_out > sms) *exact_grid_out = sms;
  }
  return e;
}

cudaError_t launch_bsgs(const JobDev &job, const ChunkBufs &cb, const HitBufs &hb, int grid,
                        cudaStream_t st) {
  if (job.cta_warps > 1)
    bsgs_cta_fn(job)<<<grid, 32 * kCtaWarps, bsgs_smem_bytes(job), st>>>(job, cb, hb);
  else
    bsgs_fn(job)<<<grid, 32 * kWarpsPerBlock, bsgs_smem_bytes(job), st>>>(job, cb, hb);
  return cudaGetLastError();
}

static BatchFn batch_fn(const JobDev &rep) {
  switch (row_mode(rep)) {
    case kRowsMask: return batch_fn_t<kRowsMask>(rep.tlanes);
    case kRowsIntId: return batch_fn_t<kRowsIntId>(rep.tlanes);
    case kRowsIntV: return batch_fn_t<kRowsIntV>(rep.tlanes);
    default: return batch_fn_t<kRowsV>(rep.tlanes);
  }
}

uint32_t batch_warp_bytes(uint32_t stage_max, uint32_t table_log2_max, bool row_mask) {
  const uint32_t b = 16 * stage_max + (row_mask ? 8 * kMaskRows : 0) + 16 * kMatchCap + 16 + (20u << table_log2_max);
  return (b + 15) & ~15u;
}

cudaError_t batch_configure(const JobDev &rep, uint32_t warp_bytes, int device, int *grid_out) {
  return configure_one((const void *)batch_fn(rep), kWarpsPerBlock * (int)warp_bytes, 32 * kWarpsPerBlock, device,
                       grid_out);
}

cudaError_t launch_bsgs_batch(const JobDev &rep, const BatchItem *items, uint32_t nitems, uint32_t stage_max,
                              uint32_t warp_bytes, int grid, cudaStream_t st) {
  if (nitems == 0) return cudaSuccess;
  if (nitems > kBatchMaxItems) return cudaErrorInvalidValue;
  batch_fn(rep)<<<grid, 32 * kWarpsPerBlock, kWarpsPerBlock * warp_bytes, st>>>(items, nitems, warp_bytes, stage_max);
  return cudaGetLastError();
}

cudaError_t launch_bsgs_exact(const JobDev &job, const ChunkBufs &cb, const HitBufs &hb, int grid,
                              cudaStream_t st) {
  if (job.cta_warps > 1)
    bsgs_exact_kernel<kCtaWarps><<<grid, 32 * kCtaWarps, bsgs_exact_smem_bytes(job), st>>>(job, cb, hb);
  else
    bsgs_exact_kernel<1><<<grid, 32 * kWarpsPerBlock, bsgs_exact_smem_bytes(job), st>>>(job, cb, hb);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Direct verification of every candidate hit.

__global__ void verify_kernel(JobDev J, HitBufs hb) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t cnt = *hb.raw_count;
  const uint32_t n = cnt < hb.cap ? cnt : hb.cap;
  if (i >= n) return;
  const Hit h = hb.raw[i];
  const uint64_t p = h.p;
  Mont M;
  M.p = p;
  M.pinv = mont_pinv(p);
  uint64_t one, r2;
  mont_consts(p, M.pinv, one, r2);
  const uint64_t bmod = p > J.base ? (uint64_t)J.base : (uint64_t)J.base % p;
  const uint64_t bm = montmul(bmod, r2, M);
  const uint64_t x = mont_pow(bm, h.n, one, M);
  const uint64_t km = montmul((uint64_t)h.k, r2, M);
  const uint64_t y = montmul(montmul(x, km, M), 1, M);  // k*b^n mod p, normal form
  const uint64_t want = J.sign < 0 ? 1 : p - 1;
  if (y == want) {
    const uint32_t idx = atomicAdd(hb.fac_count, 1u);
    if (idx < hb.cap) hb.fac[idx] = h;
  }
}

cudaError_t launch_verify(const JobDev &job, const HitBufs &hb, cudaStream_t st) {
  const unsigned blocks = (hb.cap + 255) / 256;
  verify_kernel<<<blocks, 256, 0, st>>>(job, hb);
  return cudaGetLastError();
}

}  // namespace rs
