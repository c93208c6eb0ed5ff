// rs_kernels.cu -- the sieve's device kernels for sm_103a.
//
//   sieve_kernel   segmented Eratosthenes over odd numbers; one 2^18-odd
//                  segment per CTA in shared memory; writes the primes of a
//                  p-window straight into HBM.  Replaces the host prime
//                  generator generateGPUPrimes (kernel_v0.24.6.cu:1838-1987),
//                  but is complete (every composite removed) where the
//                  reference leaves composites above smallP_max^2.
//   setup_kernel   one thread per prime: Montgomery constants, B = b^Q, the
//                  quadratic-character filter per (k, n mod Q) row
//                  (kernel_v0.24.6.cu:461-521), the per-row giant-step start
//                  values k*b^r*B^e0 (kernel_v0.24.6.cu:454-509,525-528) and the
//                  per-lane power tables the BSGS kernel starts from.
//   bsgs_kernel    one prime per warp: baby steps B^j (j < m) into a
//                  shared-memory open-addressing table, then giant steps for
//                  every active row, 32 lanes sharing each prime
//                  (kernel_v0.24.6.cu:365-620 is the per-thread, global-memory
//                  original).  Candidate hits are checked against the row
//                  bitmap on the device and appended with one atomic each.
//   verify_kernel  direct k*b^n check of every hit (kernel_v0.24.6.cu:1649-1671).
#include <cstdio>

#include "rs_arith.cuh"
#include "rs_internal.h"

namespace rs {

// ---------------------------------------------------------------------------
// Segmented sieve.

__global__ void __launch_bounds__(kSieveThreads)
sieve_kernel(uint64_t lo, uint64_t hi, const uint32_t *__restrict__ sp,
             const uint64_t *__restrict__ sp_rcp, uint32_t nsp, uint64_t *__restrict__ out,
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

  for (uint32_t w = tid; w < kSieveOdds / 32; w += kSieveThreads) bits[w] = 0;
  __syncthreads();

  // Small primes: the whole CTA strides over the multiples of one prime.
  uint32_t t = 0;
#pragma unroll 1
  for (; t < nsp; t++) {
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
  // Larger primes: one prime per thread.
#pragma unroll 1
  for (uint32_t u = t + tid; u < nsp; u += kSieveThreads) {
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
  const uint32_t nwords = (nodd + 31) / 32;
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

cudaError_t launch_sieve(uint64_t lo, uint64_t hi, const uint32_t *sp, const uint64_t *sp_rcp,
                         uint32_t nsp, uint64_t *out, uint32_t *count, uint32_t cap,
                         cudaStream_t st) {
  const uint64_t nodd = (hi - lo) / 2 + 1;
  const uint64_t blocks = (nodd + kSieveOdds - 1) / kSieveOdds;
  sieve_kernel<<<(unsigned)blocks, kSieveThreads, 0, st>>>(lo, hi, sp, sp_rcp, nsp, out, count, cap);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Per-prime setup, one thread per prime.

__global__ void __launch_bounds__(128) setup_kernel(JobDev J, ChunkBufs cb) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t cnt = *cb.count;
  const uint32_t n = cnt < cb.cap ? cnt : cb.cap;
  if (i >= n) return;
  const uint64_t p = cb.primes[i];
  PrimeRec rec;
  rec.p = p;
  rec.pinv = 0;
  rec.Bstride = 0;
  rec.Gstride = 0;
  rec.nact = 0;
  rec.flags = 0;
  rec.pad = 0;
  const uint64_t bmod = p > J.base ? (uint64_t)J.base : (uint64_t)J.base % p;
  if (bmod == 0) {  // p | b: no k*b^n+-1 is divisible by p
    cb.rec[i] = rec;
    return;
  }
  Mont M;
  M.p = p;
  M.pinv = mont_pinv(p);
  uint64_t one, r2;
  mont_consts(p, M.pinv, one, r2);
  const uint64_t bm = montmul(bmod, r2, M);        // b in Montgomery form
  const uint64_t B = mont_pow(bm, J.Q, one, M);    // b^Q
  const uint64_t e = J.e0 >= 0 ? (uint64_t)J.e0 : (p - 1) - (uint64_t)(-J.e0) % (p - 1);
  const uint64_t H = mont_pow(B, e, one, M);       // B^e0
  const uint64_t G = mont_pow(B, J.m, one, M);     // B^m

  // Lane tables: B^lane (baby starts) and G^(lane % tlanes + 1) (giant multipliers).
  uint64_t *vb = cb.vecB + (size_t)i * 32;
  uint64_t v = one;
#pragma unroll 1
  for (int l = 0; l < 32; l++) {
    vb[l] = v;
    v = montmul(v, B, M);
  }
  rec.Bstride = v;  // B^32
  uint64_t *vg = cb.vecG + (size_t)i * 32;
  uint64_t g = G;
#pragma unroll 1
  for (uint32_t l = 0; l < J.tlanes; l++) {
    vg[l] = g;
    if (l == 31) rec.Gstride = g;  // G^32
    g = montmul(g, G, M);
  }
#pragma unroll 1
  for (uint32_t l = J.tlanes; l < 32; l++) vg[l] = vg[l & (J.tlanes - 1)];

  // Active rows and their giant-step start values.
  const int chib = legendre_k(p, J.b_odd, J.b_e2, J.b_rcp);
  const int chim1 = ((uint32_t)p & 3u) == 1u ? 1 : -1;  // (-1/p)
  const bool qeven = (J.Q & 1u) == 0;
  uint64_t *aV = cb.actV + (size_t)i * J.max_act;
  uint32_t *aR = cb.actRow + (size_t)i * J.max_act;
  uint32_t nact = 0;
#pragma unroll 1
  for (uint32_t c = 0; c < J.nk; c++) {
    int chik = legendre_k(p, J.k_odd[c], J.k_e2[c], J.k_rcp[c]);
    if (J.sign > 0) chik *= chim1;  // character of -k
    if (chik == 0) continue;        // p | k
    const uint32_t r0 = J.k_row0[c], r1 = J.k_row0[c + 1];
    uint64_t V = 0;
    uint32_t cur = 0;
    bool have = false;
#pragma unroll 1
    for (uint32_t row = r0; row < r1; row++) {
      const uint32_t r = J.row_r[row];
      const bool act = qeven ? (chik * ((r & 1u) ? chib : 1) == 1) : (chib == -1 || chik == 1);
      if (!act) continue;
      if (!have) {
        uint64_t km = montmul((uint64_t)J.k_val[c], r2, M);  // k R mod p
        if (J.sign > 0) km = km ? p - km : 0;
        V = montmul(km, H, M);
        have = true;
      }
#pragma unroll 1
      for (; cur < r; cur++) V = montmul(V, bm, M);
      aV[nact] = V;
      aR[nact] = row;
      nact++;
    }
  }
  rec.pinv = M.pinv;
  rec.nact = nact;
  cb.rec[i] = rec;
}

cudaError_t launch_setup(const JobDev &job, const ChunkBufs &cb, cudaStream_t st) {
  const unsigned blocks = (cb.cap + 127) / 128;
  setup_kernel<<<blocks, 128, 0, st>>>(job, cb);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Baby-step giant-step, one prime per warp.

__device__ __forceinline__ void record_hit(const JobDev &J, const ChunkBufs &cb, const HitBufs &hb,
                                           uint32_t i, uint64_t p, uint32_t slot, uint32_t s,
                                           uint32_t j) {
  const int64_t x = J.e0 + (int64_t)J.m * (int64_t)s - (int64_t)j;
  if (x < (int64_t)J.x_lo || x > (int64_t)J.x_hi) return;
  const uint32_t row = cb.actRow[(size_t)i * J.max_act + slot];
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

__global__ void __launch_bounds__(32 * kWarpsPerBlock)
bsgs_kernel(JobDev J, ChunkBufs cb, HitBufs hb) {
  extern __shared__ uint4 smem4[];
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t S = 1u << J.table_log2;
  const uint32_t tmask = S - 1;
  uint32_t *tab = reinterpret_cast<uint32_t *>(smem4) + (size_t)warp * S;
  uint4 *tab4 = smem4 + (size_t)warp * (S / 4);
  const uint32_t jbits = J.jbits;
  const uint32_t jmask = (1u << jbits) - 1u;
  const uint32_t tagmask = (1u << (32 - jbits)) - 1u;  // jbits >= 1
  const uint32_t tl = J.table_log2;
  const uint32_t lane_t = lane & (J.tlanes - 1);
  const uint32_t lane_row = lane / J.tlanes;
  const uint32_t cnt = *cb.count;
  const uint32_t n = cnt < cb.cap ? cnt : cb.cap;
  const uint32_t nwarps = gridDim.x * kWarpsPerBlock;

#pragma unroll 1
  for (uint32_t i = blockIdx.x * kWarpsPerBlock + warp; i < n; i += nwarps) {
    const PrimeRec rec = cb.rec[i];
    if (rec.nact == 0) continue;
    const uint64_t p = rec.p, pinv = rec.pinv;
    const uint4 empty4 = make_uint4(kEmpty, kEmpty, kEmpty, kEmpty);
    for (uint32_t s = lane; s < S / 4; s += 32) tab4[s] = empty4;
    __syncwarp();

    // Baby steps: lane handles j = lane, lane+32, ...
    uint64_t v = cb.vecB[(size_t)i * 32 + lane];
#pragma unroll 1
    for (uint32_t j = lane; j < J.m; j += 32) {
      uint32_t h = (uint32_t)v & tmask;
      const uint32_t e = ((((uint32_t)(v >> tl)) & tagmask) << jbits) | j;
#pragma unroll 1
      for (uint32_t it = 0; it < S; it++) {
        if (atomicCAS(&tab[h], kEmpty, e) == kEmpty) break;
        h = (h + 1) & tmask;
      }
      v = montmul(v, rec.Bstride, p, pinv);
    }
    __syncwarp();

    // Giant steps: lanes (lane_row, lane_t) take row slot it*rows_per_it+lane_row,
    // giant indices s = lane_t+1 (+32 per extra step).
    const uint64_t Gl = cb.vecG[(size_t)i * 32 + lane];
    const uint32_t nit = (rec.nact + J.rows_per_it - 1) / J.rows_per_it;
#pragma unroll 1
    for (uint32_t it = 0; it < nit; it++) {
      const uint32_t slot = it * J.rows_per_it + lane_row;
      if (slot < rec.nact) {
        uint64_t y = montmul(cb.actV[(size_t)i * J.max_act + slot], Gl, p, pinv);
        uint32_t s = lane_t + 1;
#pragma unroll 1
        for (uint32_t u = 0; u < J.steps_per_lane; u++) {
          uint32_t h = (uint32_t)y & tmask;
          const uint32_t tag = ((uint32_t)(y >> tl)) & tagmask;
#pragma unroll 1
          for (uint32_t q = 0; q < S; q++) {
            const uint32_t e = tab[h];
            if (e == kEmpty) break;
            if ((e >> jbits) == tag) record_hit(J, cb, hb, i, p, slot, s, e & jmask);
            h = (h + 1) & tmask;
          }
          if (u + 1 < J.steps_per_lane) {
            y = montmul(y, rec.Gstride, p, pinv);
            s += 32;
          }
        }
      }
    }
    __syncwarp();
  }
}

int bsgs_smem_bytes(const JobDev &job) { return kWarpsPerBlock * (4 << job.table_log2); }

cudaError_t bsgs_configure(const JobDev &job, int device, int *grid_out) {
  const int smem = bsgs_smem_bytes(job);
  cudaError_t e = cudaFuncSetAttribute(bsgs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(bsgs_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                           cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bsgs_kernel, 32 * kWarpsPerBlock, smem);
  if (e != cudaSuccess) return e;
  int sms = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  *grid_out = per_sm * sms;
  return cudaSuccess;
}

cudaError_t launch_bsgs(const JobDev &job, const ChunkBufs &cb, const HitBufs &hb, int grid,
                        cudaStream_t st) {
  bsgs_kernel<<<grid, 32 * kWarpsPerBlock, bsgs_smem_bytes(job), st>>>(job, cb, hb);
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

// ---------------------------------------------------------------------------
// Integer-multiply pipe microbenchmarks (roofline denominators).

__global__ void __launch_bounds__(256) imad_kernel(uint32_t iters, uint32_t seed, uint32_t *sink) {
  uint32_t x0 = seed ^ threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  uint32_t x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  const uint32_t a = 0x9E3779B9u | 1u, c = seed | 1u;
#pragma unroll 1
  for (uint32_t i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 16; u++) {
      asm volatile("mad.lo.u32 %0, %0, %8, %9;\n\t"
                   "mad.lo.u32 %1, %1, %8, %9;\n\t"
                   "mad.lo.u32 %2, %2, %8, %9;\n\t"
                   "mad.lo.u32 %3, %3, %8, %9;\n\t"
                   "mad.lo.u32 %4, %4, %8, %9;\n\t"
                   "mad.lo.u32 %5, %5, %8, %9;\n\t"
                   "mad.lo.u32 %6, %6, %8, %9;\n\t"
                   "mad.lo.u32 %7, %7, %8, %9;\n\t"
                   : "+r"(x0), "+r"(x1), "+r"(x2), "+r"(x3), "+r"(x4), "+r"(x5), "+r"(x6), "+r"(x7)
                   : "r"(a), "r"(c));
    }
  }
  const uint32_t r = x0 ^ x1 ^ x2 ^ x3 ^ x4 ^ x5 ^ x6 ^ x7;
  if (r == 0x12345678u) sink[0] = r;
}

__global__ void __launch_bounds__(256) montmul_kernel(uint32_t iters, uint64_t p, uint64_t pinv,
                                                      uint64_t *sink) {
  const uint64_t t = blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t x0 = (t * 0x9E3779B97F4A7C15ull) % p, x1 = (x0 + 1) % p, x2 = (x0 + 2) % p, x3 = (x0 + 3) % p;
  const uint64_t c = (p >> 1) + 12345;
#pragma unroll 1
  for (uint32_t i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 8; u++) {
      x0 = montmul(x0, c, p, pinv);
      x1 = montmul(x1, c, p, pinv);
      x2 = montmul(x2, c, p, pinv);
      x3 = montmul(x3, c, p, pinv);
    }
  }
  const uint64_t r = x0 ^ x1 ^ x2 ^ x3;
  if (r == 0x123456789ull) sink[0] = r;
}

static uint64_t host_pinv(uint64_t p) {
  uint64_t x = p;
  for (int i = 0; i < 5; i++) x *= 2 - p * x;
  return (uint64_t)0 - x;
}

cudaError_t run_imad_bench(int device, double *mul_ops_per_s, double *montmul_per_s) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return e;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  void *sink = nullptr;
  e = cudaMalloc(&sink, 64);
  if (e != cudaSuccess) return e;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const int blocks = sms * 8, threads = 256;
  float best1 = 1e30f, best2 = 1e30f;
  const uint32_t it1 = 2048, it2 = 256;
  for (int rep = 0; rep < 4; rep++) {
    cudaEventRecord(a);
    imad_kernel<<<blocks, threads>>>(it1, 7u + rep, (uint32_t *)sink);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    if (rep && ms < best1) best1 = ms;
    const uint64_t p = 10000000000037ull;  // a prime near 1e13
    cudaEventRecord(a);
    montmul_kernel<<<blocks, threads>>>(it2, p, host_pinv(p), (uint64_t *)sink);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    cudaEventElapsedTime(&ms, a, b);
    if (rep && ms < best2) best2 = ms;
  }
  e = cudaGetLastError();
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(sink);
  if (e != cudaSuccess) return e;
  const double n1 = (double)blocks * threads * it1 * 16 * 8;
  const double n2 = (double)blocks * threads * it2 * 8 * 4;
  *mul_ops_per_s = n1 / (best1 * 1e-3);
  *montmul_per_s = n2 / (best2 * 1e-3);
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// Arithmetic self-test.

__global__ void arith_kernel(const uint64_t *a, const uint64_t *b, const uint64_t *p, size_t n,
                             uint64_t *out_mm, int32_t *out_j) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t P = p[i];
  Mont M;
  M.p = P;
  M.pinv = mont_pinv(P);
  uint64_t one, r2;
  mont_consts(P, M.pinv, one, r2);
  const uint64_t am = montmul(a[i], r2, M), bm = montmul(b[i], r2, M);
  out_mm[i] = montmul(montmul(am, bm, M), 1, M);
  // character of the low 32 bits of a with respect to P
  uint32_t k = (uint32_t)a[i];
  if (k == 0) {
    out_j[i] = 0;
    return;
  }
  uint32_t e2 = __ffs(k) - 1;
  uint32_t kodd = k >> e2;
  const uint64_t rcp = kodd > 1 ? (~0ull) / kodd : 0;  // floor((2^64-1)/kodd) == floor(2^64/kodd) for kodd odd > 1
  out_j[i] = legendre_k(P, kodd, e2, rcp);
}

cudaError_t run_arith_check(const uint64_t *a, const uint64_t *b, const uint64_t *p, size_t n,
                            uint64_t *out_mm, int32_t *out_j) {
  arith_kernel<<<(unsigned)((n + 255) / 256), 256>>>(a, b, p, n, out_mm, out_j);
  return cudaGetLastError();
}

}  // namespace rs
