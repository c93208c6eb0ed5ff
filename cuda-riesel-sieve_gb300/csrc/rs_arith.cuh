// rs_arith.cuh -- 64-bit modular arithmetic for sm_103a.
//
// Montgomery multiplication with R = 2^64 (the reference's montmul,
// kernel_v0.24.6.cu:182-270, computes the same a*b*R^-1 mod p for p < 2^63 in
// 32-bit PTX limbs).  Here the 128-bit products come from __umul64hi and the
// carry out of the discarded low word is (t_lo != 0): the low 64 bits of
// t + m*p are zero by construction, so they carry exactly when t_lo is nonzero.
// This is exact for every input; the reference's "+1" into its second 32-bit
// column drops a carry whenever that column holds 0xFFFFFFFF.  On GB300 this
// form measured ~10% faster than a hand-scheduled 32-bit PTX carry chain.
//
// Constraints: p odd, p < 2^63; a < 2^64, b < p  ->  result in [0, p).
#pragma once
#include <cstdint>

namespace rs {

struct Mont {
  uint64_t p;     // modulus
  uint64_t pinv;  // -p^-1 mod 2^64
};

// a*b*2^-64 mod p.
__device__ __forceinline__ uint64_t montmul(uint64_t a, uint64_t b, uint64_t p, uint64_t pinv) {
  const uint64_t tlo = a * b;
  const uint64_t thi = __umul64hi(a, b);
  const uint64_t m = tlo * pinv;
  uint64_t u = thi + __umul64hi(m, p) + (tlo != 0 ? 1u : 0u);  // < 2p
  u -= p;
  u += p & (uint64_t)((int64_t)u >> 63);
  return u;
}

__device__ __forceinline__ uint64_t montmul(uint64_t a, uint64_t b, const Mont &m) {
  return montmul(a, b, m.p, m.pinv);
}

// The same product as a hand-scheduled inline-PTX chain of 32-bit limbs
// (mul/mad(c).lo/hi with carry flags, the instruction form of the reference's
// montmul, kernel_v0.24.6.cu:205-237): t = a*b in four limbs, m = t_lo*pinv mod
// 2^64 in two, the high half of m*p in two, u = hi(m*p) + t_hi + (t_lo != 0),
// one masked subtraction.  19 multiply-class instructions.  Same domain and
// result as montmul(); kept for the measured comparison of the two forms
// (rs_bench_products) and tested against exact arithmetic (RS_OP_MONTMUL_PTX).
__device__ __forceinline__ uint64_t montmul_ptx(uint64_t a, uint64_t b, uint64_t p, uint64_t pinv) {
  uint32_t u0, u1;
  asm("{\n\t"
      ".reg .u32 a0, a1, b0, b1, p0, p1, q0, q1, t0, t1, t2, t3, m0, m1, x1, x2, x3, c, v0, v1;\n\t"
      ".reg .pred nz, neg;\n\t"
      "mov.b64 {a0, a1}, %2;\n\t"
      "mov.b64 {b0, b1}, %3;\n\t"
      "mov.b64 {p0, p1}, %4;\n\t"
      "mov.b64 {q0, q1}, %5;\n\t"
      // t = a*b
      "mul.lo.u32 t0, a0, b0;\n\t"
      "mul.hi.u32 t1, a0, b0;\n\t"
      "mad.lo.cc.u32 t1, a0, b1, t1;\n\t"
      "madc.hi.u32 t2, a0, b1, 0;\n\t"
      "mad.lo.cc.u32 t1, a1, b0, t1;\n\t"
      "madc.hi.cc.u32 t2, a1, b0, t2;\n\t"
      "madc.hi.u32 t3, a1, b1, 0;\n\t"
      "mad.lo.cc.u32 t2, a1, b1, t2;\n\t"
      "addc.u32 t3, t3, 0;\n\t"
      // m = t_lo * pinv mod 2^64
      "mul.lo.u32 m0, t0, q0;\n\t"
      "mul.hi.u32 m1, t0, q0;\n\t"
      "mad.lo.u32 m1, t0, q1, m1;\n\t"
      "mad.lo.u32 m1, t1, q0, m1;\n\t"
      // (x3:x2) = high half of m*p (limb 1 only for its carry)
      "mul.hi.u32 x1, m0, p0;\n\t"
      "mad.lo.cc.u32 x1, m0, p1, x1;\n\t"
      "madc.hi.u32 x2, m0, p1, 0;\n\t"
      "mad.lo.cc.u32 x1, m1, p0, x1;\n\t"
      "madc.hi.cc.u32 x2, m1, p0, x2;\n\t"
      "madc.hi.u32 x3, m1, p1, 0;\n\t"
      "mad.lo.cc.u32 x2, m1, p1, x2;\n\t"
      "addc.u32 x3, x3, 0;\n\t"
      // the low halves of t and m*p sum to 0 or 2^64: carry (t_lo != 0)
      "or.b32 c, t0, t1;\n\t"
      "setp.ne.u32 nz, c, 0;\n\t"
      "selp.u32 c, 1, 0, nz;\n\t"
      "add.cc.u32 x2, x2, t2;\n\t"
      "addc.u32 x3, x3, t3;\n\t"
      "add.cc.u32 x2, x2, c;\n\t"
      "addc.u32 x3, x3, 0;\n\t"
      // u < 2p: subtract p unless that goes negative
      "sub.cc.u32 v0, x2, p0;\n\t"
      "subc.u32 v1, x3, p1;\n\t"
      "setp.lt.s32 neg, v1, 0;\n\t"
      "selp.u32 %0, x2, v0, neg;\n\t"
      "selp.u32 %1, x3, v1, neg;\n\t"
      "}"
      : "=r"(u0), "=r"(u1)
      : "l"(a), "l"(b), "l"(p), "l"(pinv));
  return ((uint64_t)u1 << 32) | u0;
}

// x*2^-64 mod p for x < p (leaving Montgomery form): the Montgomery product by 1
// with its zero high word dropped.  With m = x*pinv mod 2^64, m*p == -x (mod 2^64),
// so x + m*p = umulhi(m, p)*2^64 + 2^64 when x != 0: the result is
// umulhi(m, p) + 1, already below p (it equals p only for x == 0 mod p).
__device__ __forceinline__ uint64_t from_mont(uint64_t x, uint64_t p, uint64_t pinv) {
  return x ? __umul64hi(x * pinv, p) + 1 : 0;
}

// Shoup's product x*w mod p for a fixed multiplier w < p with
// wq = floor(w * 2^64 / p); any x < 2^64; p < 2^63.  The quotient estimate
// umulhi(x, wq) is at most one short, so r = x*w - q*p lies in [0, 2p) and one
// masked subtraction finishes.  Measured on GB300: ~1.4x the throughput of the
// Montgomery product above.
__device__ __forceinline__ uint64_t shoup_mul(uint64_t x, uint64_t w, uint64_t wq, uint64_t p) {
  const uint64_t q = __umul64hi(x, wq);
  const uint64_t r = x * w + q * (0 - p);  // x*w - q*p, a multiply-add chain
  const uint64_t t = r - p;
  return (int64_t)t < 0 ? r : t;
}

// Shoup's product for a 32-bit x: c*w mod p with wq = floor(w * 2^64 / p).
// The bound is the one above (x < 2^64), and the quotient estimate
// floor(c * wq / 2^64) <= c*w/p < c fits 32 bits, so the high product is two
// 32x32 multiply-adds and q*p one: about ten instructions against sixteen.
__device__ __forceinline__ uint64_t shoup_mul32(uint32_t c, uint64_t w, uint64_t wq, uint64_t p) {
  const uint64_t t = (uint64_t)c * (uint32_t)wq;
  const uint64_t u = (uint64_t)c * (uint32_t)(wq >> 32) + (t >> 32);
  const uint32_t q = (uint32_t)(u >> 32);
  const uint64_t r = (uint64_t)c * w + (uint64_t)q * (0 - p);
  const uint64_t s = r - p;
  return (int64_t)s < 0 ? r : s;
}

// Shoup's product by a small fixed multiplier: x*w mod p for w < 2^32 with
// w * 2^32 < p, so that wq = floor(w * 2^64 / p) < 2^32.  The quotient
// estimate floor(x * wq / 2^64) < wq then needs two 32x32 multiply-adds, and
// the bound is Shoup's (any x < 2^64, r in [0, 2p)).
__device__ __forceinline__ uint64_t shoup_mul_w32(uint64_t x, uint32_t w, uint32_t wq, uint64_t p) {
  const uint64_t t = (uint64_t)(uint32_t)x * wq;
  const uint64_t u = (x >> 32) * (uint64_t)wq + (t >> 32);
  const uint32_t q = (uint32_t)(u >> 32);
  const uint64_t r = x * (uint64_t)w + (uint64_t)q * (0 - p);
  const uint64_t s = r - p;
  return (int64_t)s < 0 ? r : s;
}

// x*c mod p for a small integer multiplier c, with rc = floor(2^64 / p).
// Requires x < p, 2^33 < p and c*p < 2^63.  Then P = x*c < 2^63 and the
// quotient estimate q' = floor(hi32(P) * rc / 2^32) satisfies
//   P/p - 1 - (hi32(P)/2^32 + 2^32/p) < q' <= P/p,
// where the bracket is below 1/2 + 1/2, so q' is floor(P/p) or one less and
// r = P - q'*p lies in [0, 2p): one masked subtraction finishes.  Two 32x32
// products form P, one high product forms q', and one multiply-add forms r,
// against ten multiplies for Shoup's product by a full-size constant.  The
// product of a Montgomery-form x by an integer is the Montgomery form of the
// product, so x may be in either form.
__device__ __forceinline__ uint64_t mul_small(uint64_t x, uint32_t c, uint32_t rc, uint64_t p) {
  const uint64_t P = x * (uint64_t)c;
  const uint32_t q = __umulhi((uint32_t)(P >> 32), rc);
  const uint64_t r = P + (uint64_t)q * (0 - p);
  const uint64_t t = r - p;
  return (int64_t)t < 0 ? r : t;
}

// floor(w * 2^64 / p) from the Montgomery form wm = w * 2^64 mod p: since
// w * 2^64 = wq * p + wm, wq == -wm * p^-1 == wm * pinv (mod 2^64), and
// wq < 2^64 because w < p.  One 64-bit multiply instead of a 128/64 division.
__device__ __forceinline__ uint64_t shoup_const(uint64_t wm, uint64_t pinv) { return wm * pinv; }

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

// (k/p) as above, reading (p mod kodd / kodd) from a precomputed bit table when
// one exists (table word offset `jac`) and p > kodd, so that gcd(p, kodd) = 1.
__device__ __forceinline__ int legendre_k_tab(uint64_t p, uint32_t kodd, uint32_t e2, uint64_t rcp,
                                              uint32_t jac, const uint32_t *bits) {
  int s = 1;
  if (e2 & 1) {
    uint32_t p8 = (uint32_t)p & 7u;
    if (p8 == 3 || p8 == 5) s = -s;
  }
  if (kodd == 1) return s;
  const uint32_t a = mod_rcp(p, kodd, rcp);
  int j;
  if (jac != 0xffffffffu && p > kodd) j = ((__ldg(bits + jac + (a >> 5)) >> (a & 31)) & 1u) ? 1 : -1;
  else j = jacobi32(a, kodd);
  if ((kodd & 3u) == 3u && ((uint32_t)p & 3u) == 3u) j = -j;
  return s * j;
}

}  // namespace rs
