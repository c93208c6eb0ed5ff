/*
 * rs_oracle.h -- CPU oracle for the Riesel/Sierpinski sieve hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code.  It is used by tests/, by __graft_entry__.smoke() as the
 * checker, and by bench.py's cpu_baseline leg / reference arm (the reference's
 * own sieve path is CUDA-only and has no CPU implementation to time).
 *
 * What it restates from rob147147/CUDA-Riesel-Sieve, "CUDA Riesel Sieve/kernel_v0.24.6.cu":
 *   - ABCD parsing                       kernel_v0.24.6.cu:938-1083
 *   - subsequence modulus Q choice,
 *     tMin/tMax, row build + sort        kernel_v0.24.6.cu:1086-1255
 *   - factor verification by modexp      kernel_v0.24.6.cu:1649-1671
 *   - the sieve contract itself          kernel_v0.24.6.cu:273-684
 *     (p | k*b^n-1  <=>  k*b^n == 1 mod p), restated as a textbook
 *     baby-step/giant-step search that is structurally unlike the GPU kernel.
 *   - the reference run's observable output (reference projection):
 *     its probable primes, one report per prime, Q=1 fallback, x-window
 *     and host filter                    kernel_v0.24.6.cu:288-620,1605-1732,
 *                                        1271-1303,1838-1987
 *
 * Parity pins (tests/test_oracle.py): the structural facts of the reference's
 * own test file sr_745.abcd (Q=18, 198 rows, x-range 3743, tMin=19, tMax=28
 * at -m 8), the datless factor 102297149781479 | 18300*745^242670-1 named in
 * kernel_v0.24.6.cu:244, and the negative KAT "Sieved to 5000000000000"
 * (sr_745.abcd:1): no candidate of that file has a factor below 5e12.
 */
#ifndef RS_ORACLE_H
#define RS_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  uint64_t p;
  uint32_t k;
  uint32_t n;
} orc_factor;

/* A parsed sieve job: candidates k*b^n+sign, n lists sorted ascending (CSR). */
typedef struct {
  uint32_t base;
  int32_t sign;   /* -1: Riesel k*b^n-1, +1: Sierpinski k*b^n+1 */
  uint32_t nk;
  uint32_t *k;    /* [nk] in file order */
  uint32_t *noff; /* [nk+1] */
  uint32_t *n;    /* [noff[nk]] */
  /* reference quirk (kernel_v0.24.6.cu:1039-1043): maxN is only updated on
   * delta lines, minN only on header lines.  Kept for the reference planner. */
  int32_t ref_minN, ref_maxN;
  uint32_t nlines;  /* number of text lines, as counted by countKs */
} orc_job;

/* Returns 0 on success, nonzero on malformed input; err gets a message. */
int orc_parse_abcd(const char *text, size_t len, orc_job *out, char *err, size_t errlen);
/* Build a job from arrays (n lists need not be sorted; duplicates merged). */
int orc_job_from_arrays(uint32_t base, int32_t sign, uint32_t nk, const uint32_t *k,
                        const uint32_t *noff, const uint32_t *n, orc_job *out);
void orc_job_free(orc_job *job);

/* The reference's planner (kernel_v0.24.6.cu:1086-1255). */
typedef struct {
  int32_t minQ, minSubs, minRange, minWork;
  int32_t tMin, tMax, shift, minimum, rowoffset;
  int32_t *row_k; /* [minSubs] in the reference's sorted order */
  int32_t *row_r; /* [minSubs] */
} orc_refplan;
/* Qin = 0 for auto (Q in 2..22 even), else a forced even Q.
 * hash_elems = the reference's hashTableSize (2<<M for -m M). */
int orc_ref_plan(const orc_job *job, int32_t Qin, int32_t hash_elems, orc_refplan *out);
void orc_refplan_free(orc_refplan *pl);

/* All odd primes in [lo, hi] (inclusive), ascending.  Returns the count
 * (which may exceed cap; only cap are written). */
size_t orc_primes(uint64_t lo, uint64_t hi, uint64_t *out, size_t cap);

/* The complete sieve: every (p,k,n) with p an odd prime in [p0,p1],
 * p < 2^63, n a candidate of k (or, datless, any n in [nmin,nmax]) and
 * p | k*b^n+sign.  Sorted by (p,k,n).  Returns 0 on success; *count may
 * exceed cap (only cap written).  nthreads <= 0 means all cores. */
int orc_sieve(const orc_job *job, uint64_t p0, uint64_t p1, int32_t datless, int32_t nthreads,
              orc_factor *out, size_t cap, size_t *count, uint64_t *nprimes);

/* Reference projection: the factor lines one run of the reference executable
 * would write for [p0, p1] with its plan pl (orc_ref_plan with the same
 * hash_elems = 2<<M for -m M), -s small_prime_scale and verify (1, or 0 for
 * -v): at most one (k, n) per candidate q, q from its probable-prime source
 * (odd numbers free of the first 4096*s odd primes, composites included above
 * that bound), chosen and filtered as kernel_v0.24.6.cu:288-620 and
 * 1605-1732 do.  Riesel jobs only, p0 > b and p0 > every k.  Sorted by
 * (p, k, n); *ncand = candidates q tested.  Returns 0, or 1 for arguments
 * outside that domain. */
int orc_sieve_ref(const orc_job *job, const orc_refplan *pl, int32_t hash_elems, int32_t small_prime_scale,
                  uint64_t p0, uint64_t p1, int32_t verify, int32_t nthreads, orc_factor *out, size_t cap,
                  size_t *count, uint64_t *ncand);

/* Direct check p | k*b^n+sign by square-and-multiply (kernel_v0.24.6.cu:1649-1671). */
int orc_verify(uint64_t p, uint32_t k, uint32_t b, uint32_t n, int32_t sign);

/* Jacobi symbol (a/n), n odd positive.  Returns -1, 0 or 1. */
int orc_jacobi(uint64_t a, uint64_t n);

/* Number of host threads orc_sieve uses for nthreads <= 0. */
int orc_default_threads(void);

#ifdef __cplusplus
}
#endif
#endif
