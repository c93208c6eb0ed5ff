// rs_selftest.cu -- measured throughput of the modular products (the roofline
// denominators of the BSGS kernels) and device self-tests of the arithmetic in
// rs_arith.cuh, which the parity tests compare against exact integer results.
#include "rs_arith.cuh"
#include "rs_internal.h"
#include "rsieve.h"

namespace rs {

// ---------------------------------------------------------------------------
// Throughput microbenchmarks: every thread runs four (eight for mad.lo)
// independent dependency chains of one operation, so the rate is set by the
// pipes, not by the latency of one chain.

enum BenchOp { kBenchMad = 0, kBenchMont, kBenchMontPtx, kBenchShoup, kBenchShoup32, kBenchSmall, kBenchOps };

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

// Four chains of one 64-bit modular product by a fixed multiplier c:
// Montgomery (both forms), Shoup by a full-size constant, Shoup of a 32-bit
// operand (its chains restart from 32-bit values each step), the short product.
template <int OP>
__global__ void __launch_bounds__(256) product_kernel(uint32_t iters, uint64_t p, uint64_t pinv, uint64_t c,
                                                      uint64_t cq, uint32_t small, uint32_t rcp, uint64_t *sink) {
  const uint64_t t = blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t x0 = (t * 0x9E3779B97F4A7C15ull) % p, x1 = (x0 + 1) % p, x2 = (x0 + 2) % p, x3 = (x0 + 3) % p;
  auto step = [&](uint64_t x) -> uint64_t {
    if (OP == kBenchMont) return montmul(x, c, p, pinv);
    if (OP == kBenchMontPtx) return montmul_ptx(x, c, p, pinv);
    if (OP == kBenchShoup) return shoup_mul(x, c, cq, p);
    if (OP == kBenchShoup32) return shoup_mul32((uint32_t)(x ^ (x >> 32)), c, cq, p);
    return mul_small(x, small, rcp, p);
  };
#pragma unroll 1
  for (uint32_t i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 8; u++) {
      x0 = step(x0);
      x1 = step(x1);
      x2 = step(x2);
      x3 = step(x3);
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

// rates[kBenchOps]: mad.lo.u32 per second, then modular products per second of
// each BenchOp, the best of three timed launches after one warm-up.
cudaError_t run_product_bench(int device, double *rates) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return e;
  int sms = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return e;
  void *sink = nullptr;
  e = cudaMalloc(&sink, 64);
  if (e != cudaSuccess) return e;
  cudaStream_t st;
  e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    cudaFree(sink);
    return e;
  }
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const int blocks = sms * 8, threads = 256;
  const uint32_t it_mad = 2048, it_mod = 256;
  const uint64_t p = 10000000000037ull;  // a prime near 1e13 (p > 2^33, so the short product applies)
  const uint64_t c = (p >> 1) + 12345;
  const uint64_t cq = (uint64_t)(((unsigned __int128)c << 64) / p);
  const uint32_t small = 555025;          // 745^2
  const uint32_t rcp = (uint32_t)(~0ull / p);
  float best[kBenchOps];
  for (int op = 0; op < kBenchOps; op++) best[op] = 1e30f;
  for (int rep = 0; rep < 4; rep++) {
    for (int op = 0; op < kBenchOps; op++) {
      float ms = 0;
      cudaEventRecord(a, st);
      switch (op) {
        case kBenchMad: imad_kernel<<<blocks, threads, 0, st>>>(it_mad, 7u + rep, (uint32_t *)sink); break;
        case kBenchMont:
          product_kernel<kBenchMont><<<blocks, threads, 0, st>>>(it_mod, p, host_pinv(p), c, cq, small, rcp,
                                                                 (uint64_t *)sink);
          break;
        case kBenchMontPtx:
          product_kernel<kBenchMontPtx><<<blocks, threads, 0, st>>>(it_mod, p, host_pinv(p), c, cq, small, rcp,
                                                                    (uint64_t *)sink);
          break;
        case kBenchShoup:
          product_kernel<kBenchShoup><<<blocks, threads, 0, st>>>(it_mod, p, host_pinv(p), c, cq, small, rcp,
                                                                  (uint64_t *)sink);
          break;
        case kBenchShoup32:
          product_kernel<kBenchShoup32><<<blocks, threads, 0, st>>>(it_mod, p, host_pinv(p), c, cq, small, rcp,
                                                                    (uint64_t *)sink);
          break;
        default:
          product_kernel<kBenchSmall><<<blocks, threads, 0, st>>>(it_mod, p, host_pinv(p), c, cq, small, rcp,
                                                                  (uint64_t *)sink);
          break;
      }
      cudaEventRecord(b, st);
      cudaEventSynchronize(b);
      cudaEventElapsedTime(&ms, a, b);
      if (rep && ms < best[op]) best[op] = ms;
    }
  }
  e = cudaGetLastError();
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaStreamDestroy(st);
  cudaFree(sink);
  if (e != cudaSuccess) return e;
  const double n_mad = (double)blocks * threads * it_mad * 16 * 8;
  const double n_mod = (double)blocks * threads * it_mod * 8 * 4;
  for (int op = 0; op < kBenchOps; op++) rates[op] = (op == kBenchMad ? n_mad : n_mod) / (best[op] * 1e-3);
  return cudaSuccess;
}

cudaError_t run_imad_bench(int device, double *mul_ops_per_s, double *montmul_per_s, double *shoup_per_s) {
  double r[kBenchOps];
  const cudaError_t e = run_product_bench(device, r);
  if (e != cudaSuccess) return e;
  *mul_ops_per_s = r[kBenchMad];
  *montmul_per_s = r[kBenchMont] > r[kBenchMontPtx] ? r[kBenchMont] : r[kBenchMontPtx];
  *shoup_per_s = r[kBenchShoup];
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// Arithmetic self-tests.

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

// One operation of rs_gpu_modmul_check per thread, each function of
// rs_arith.cuh called exactly as the kernels call it.
__global__ void modmul_kernel(int op, const uint64_t *a, const uint64_t *b, const uint64_t *c, const uint64_t *p,
                              size_t n, uint64_t *out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t P = p[i], A = a[i], B = b[i], C = c[i];
  const uint64_t pinv = mont_pinv(P);
  uint64_t r = 0;
  switch (op) {
    case RS_OP_MONTMUL: r = montmul(A, B, P, pinv); break;
    case RS_OP_MONTMUL_PTX: r = montmul_ptx(A, B, P, pinv); break;
    case RS_OP_FROM_MONT: r = from_mont(A, P, pinv); break;
    case RS_OP_SHOUP_CONST: r = shoup_const(A, pinv); break;
    case RS_OP_SHOUP: r = shoup_mul(A, B, C, P); break;
    case RS_OP_SHOUP32: r = shoup_mul32((uint32_t)A, B, C, P); break;
    case RS_OP_SHOUP_W32: r = shoup_mul_w32(A, (uint32_t)B, (uint32_t)C, P); break;
    case RS_OP_MUL_SMALL: r = mul_small(A, (uint32_t)B, (uint32_t)C, P); break;
    case RS_OP_PINV: r = pinv; break;
    case RS_OP_ONE:
    case RS_OP_R2: {
      uint64_t one, r2;
      mont_consts(P, pinv, one, r2);
      r = op == RS_OP_ONE ? one : r2;
      break;
    }
    case RS_OP_POW: {  // a^b in normal form, through Montgomery form as the setup kernel computes powers
      Mont M;
      M.p = P;
      M.pinv = pinv;
      uint64_t one, r2;
      mont_consts(P, pinv, one, r2);
      r = from_mont(mont_pow(montmul(A, r2, M), B, one, M), P, pinv);
      break;
    }
    default: r = 0; break;
  }
  out[i] = r;
}

cudaError_t run_modmul_check(int op, const uint64_t *a, const uint64_t *b, const uint64_t *c, const uint64_t *p,
                             size_t n, uint64_t *out) {
  modmul_kernel<<<(unsigned)((n + 255) / 256), 256>>>(op, a, b, c, p, n, out);
  return cudaGetLastError();
}

}  // namespace rs
