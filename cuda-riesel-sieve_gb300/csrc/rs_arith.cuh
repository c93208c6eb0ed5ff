// rs_arith.cuh -- 64-bit modular arithmetic for sm_103a, written in inline PTX.
//
// Montgomery multiplication with R = 2^64 on 32-bit limbs (the reference's
// montmul, kernel_v0.24.6.cu:182-270, computes the same product a*b*R^-1 mod p
// for p < 2^63).  This implementation is exact for every input: the carry out
// of the lowest column is derived from t0 != 0 with one add instead of the
// reference's unconditional "+1" into the second column, which drops a carry
// whenever that column holds 0xFFFFFFFF.
//
// Constraints: p odd, p < 2^63; a < 2^64, b < p  ->  result in [0, p).
#pragma once
#include <cstdint>

namespace rs {

struct Mont {
  uint64_t p;     // modulus
  uint64_t pinv;  // -p^-1 mod 2^64
};

__device__ __forceinline__ uint32_t lo32(uint64_t x) { return (uint32_t)x; }
__device__ __forceinline__ uint32_t hi32(uint64_t x) { return (uint32_t)(x >> 32); }

// a*b*2^-64 mod p.  19 multiply-class PTX instructions.
#pragma nv_diag_suppress 550  // the asm's scratch outputs are intentionally unread
__device__ __forceinline__ uint64_t montmul(uint64_t a, uint64_t b, uint64_t p, uint64_t pinv) {
  uint32_t a0 = lo32(a), a1 = hi32(a), b0 = lo32(b), b1 = hi32(b);
  uint32_t p0 = lo32(p), p1 = hi32(p), q0 = lo32(pinv), q1 = hi32(pinv);
  uint32_t t0, t1, t2, t3, m0, m1, z;
  asm("{\n\t"
      // t = a*b (128 bits: t3 t2 t1 t0)
      "mul.lo.u32     %0, %7, %9;\n\t"
      "mul.hi.u32     %1, %7, %9;\n\t"
      "mul.lo.u32     %2, %8, %10;\n\t"
      "mul.hi.u32     %3, %8, %10;\n\t"
      "mad.lo.cc.u32  %1, %7, %10, %1;\n\t"
      "madc.hi.cc.u32 %2, %7, %10, %2;\n\t"
      "addc.u32       %3, %3, 0;\n\t"
      "mad.lo.cc.u32  %1, %8, %9, %1;\n\t"
      "madc.hi.cc.u32 %2, %8, %9, %2;\n\t"
      "addc.u32       %3, %3, 0;\n\t"
      // m = (t mod 2^64) * pinv mod 2^64
      "mul.lo.u32     %4, %0, %13;\n\t"
      "mul.hi.u32     %5, %0, %13;\n\t"
      "mad.lo.u32     %5, %0, %14, %5;\n\t"
      "mad.lo.u32     %5, %1, %13, %5;\n\t"
      // (t + m*p) >> 64.  Column 0 sums to 0 mod 2^32 and carries iff t0 != 0.
      "add.cc.u32     %6, %0, 0xffffffff;\n\t"
      "madc.hi.cc.u32 %1, %4, %11, %1;\n\t"
      "madc.hi.cc.u32 %2, %4, %12, %2;\n\t"
      "madc.hi.u32    %3, %5, %12, %3;\n\t"
      "mad.lo.cc.u32  %1, %4, %12, %1;\n\t"
      "madc.hi.cc.u32 %2, %5, %11, %2;\n\t"
      "addc.u32       %3, %3, 0;\n\t"
      "mad.lo.cc.u32  %1, %5, %11, %1;\n\t"
      "madc.lo.cc.u32 %2, %5, %12, %2;\n\t"
      "addc.u32       %3, %3, 0;\n\t"
      "}"
      : "=&r"(t0), "=&r"(t1), "=&r"(t2), "=&r"(t3), "=&r"(m0), "=&r"(m1), "=&r"(z)
      : "r"(a0), "r"(a1), "r"(b0), "r"(b1), "r"(p0), "r"(p1), "r"(q0), "r"(q1));
  uint64_t u = ((uint64_t)t3 << 32) | t2;
  return u >= p ? u - p : u;
}
#pragma nv_diag_default 550

__device__ __forceinline__ uint64_t montmul(uint64_t a, uint64_t b, const Mont &m) {
  return montmul(a, b, m.p, m.pinv);
}

// -p^-1 mod 2^64 by Newton iteration (p*p == 1 mod 8 gives 3 correct bits).
__device__ __forceinline__ uint64_t mont_pinv(uint64_t p) {
  uint64_t x = p;
#pragma unroll
  for (int i = 0; i < 5; i++) x *= 2 - p * x;
  return (uint64_t)0 - x;
}

// 2^64 mod p and 2^128 mod p by doubling (p odd, 3 <= p < 2^63).
__device__ __forceinline__ void mont_consts(uint64_t p, uint64_t pinv, uint64_t &one, uint64_t &r2) {
  int L = 64 - __clzll((long long)p);      // bit length, p in [2^(L-1), 2^L)
  uint64_t x = (uint64_t)1 << (L - 1);      // < p
  int e = L - 1;
  one = 0;
#pragma unroll 1
  for (; e < 96; e++) {
    if (e == 64) one = x;
    x <<= 1;
    if (x >= p) x -= p;
  }
  // x = 2^96 mod p; montmul(2^96, 2^96) = 2^128 mod p
  r2 = montmul(x, x, p, pinv);
}

__device__ __forceinline__ uint64_t mont_pow(uint64_t base_m, uint64_t e, uint64_t one, const Mont &m) {
  uint64_t r = one;
  if (e == 0) return r;
  int top = 63 - __clzll((long long)e);
#pragma unroll 1
  for (int i = top; i >= 0; i--) {
    r = montmul(r, r, m);
    if ((e >> i) & 1) r = montmul(r, base_m, m);
  }
  return r;
}

// x mod d for 64-bit x and 32-bit d >= 1 with rcp = floor(2^64 / d)
// (rcp = 0 encodes d == 1).
__device__ __forceinline__ uint32_t mod_rcp(uint64_t x, uint32_t d, uint64_t rcp) {
  if (d == 1) return 0;
  uint64_t q = __umul64hi(x, rcp);
  uint64_t r = x - q * d;
  while (r >= d) r -= d;
  return (uint32_t)r;
}

// Jacobi symbol (a/n) for n odd; returns +1, -1 or 0 (binary algorithm).
__device__ __forceinline__ int jacobi32(uint32_t a, uint32_t n) {
  uint32_t t = 0;
#pragma unroll 1
  while (a != 0) {
    int z = __ffs(a) - 1;
    a >>= z;
    t ^= (uint32_t)z & ((n >> 1) ^ (n >> 2)) & 1u;  // (2/n)^z: n mod 8 in {3,5}
    if (a < n) {
      t ^= (a & n & 2u) >> 1;                         // both 3 mod 4
      uint32_t tmp = a;
      a = n;
      n = tmp;
    }
    a -= n;
  }
  return n == 1 ? (t ? -1 : 1) : 0;
}

// Quadratic character of an odd-part/2-adic decomposed k with respect to prime p:
// (k/p) with k = 2^e2 * kodd, via reciprocity (kodd/p) = (p mod kodd / kodd) * s.
__device__ __forceinline__ int legendre_k(uint64_t p, uint32_t kodd, uint32_t e2, uint64_t rcp) {
  int s = 1;
  if (e2 & 1) {
    uint32_t p8 = (uint32_t)p & 7u;
    if (p8 == 3 || p8 == 5) s = -s;
  }
  if (kodd == 1) return s;
  uint32_t a = mod_rcp(p, kodd, rcp);
  int j = jacobi32(a, kodd);
  if ((kodd & 3u) == 3u && ((uint32_t)p & 3u) == 3u) j = -j;
  return s * j;
}

}  // namespace rs
