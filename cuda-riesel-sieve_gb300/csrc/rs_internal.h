// rs_internal.h -- types shared by the kernels (rs_kernels.cu) and the host
// driver (rs_host.cu).  Not part of the public C ABI.
#pragma once
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "rsieve.h"

namespace rs {

// BSGS fast path: per-prime hash of 16-bit tags, kBucket tags per 16-byte bucket.
constexpr int kBucket = 8;
constexpr int kMatchCap = 15;       // deferred tag matches per prime before the exact path (15 keeps
                                    // the benchmark job at five 4-warp CTAs per SM)
// BSGS exact path (rare primes): 32-bit entries (tag << jbits) | j, linear probing.
// j <= m-1 <= 2^jbits - 2, so a real entry is never all ones.
constexpr uint32_t kEmpty = 0xffffffffu;
constexpr int kWarpsPerBlock = 4;   // BSGS kernels: one prime per warp
constexpr int kSieveOdds = 1 << 15; // odd numbers per sieve segment (4 KB of bits)
constexpr int kSieveThreads = 256;
constexpr uint32_t kNoTable = 0xffffffffu;  // no quadratic-character table for this k

// Per-prime records, written by the setup kernel and read by the BSGS kernel:
// rec_elems (even) 64-bit elements per prime, contiguous, element e of prime i
// at recs[i * rec_elems + e].  The BSGS kernel stages the header and V (the
// first el_row elements) into shared memory with 16-byte cp.async copies and
// loads each lane's own table entries straight into registers.
//
// Baby steps run in 64*W chains of chain_len consecutive exponents, W the
// warps that share one prime (1 in the warp-per-prime kernel, kCtaWarps in the
// CTA-per-prime kernel): chain c covers j = c*chain_len + t, each step a
// product by B = b^Q.  Thread t of the prime's group (t = 32*warp + lane) owns
// chains t and t + 32W.  Element map:
//   0 p, 1 pinv, 2 B, 3 G^32 (spare: the kernels use 10,11), 4 nact (low word; high word 1 if the
//   active rows come in (k, 0), (k, 1) pairs, see pairable), 5 floor(2^64 / p),
//   6,7 B in normal form and its Shoup constant (the chain step),
//   8,9 B^(32W*chain_len) likewise (chain t -> chain t+32W), 10,11 G^32 likewise,
//   W > 1 only: 12.. B^(32w*chain_len) for w < W likewise (pairs; warp w's offset),
//   el_v.. V[max_act] (giant-step start per active row), el_row.. row ids (u16,
//   4 per element), el_tab.. B^(lane*chain_len) (32 elements, the chain starts
//   of warp 0), el_tab+32.. G^(lane % tlanes + 1) (32 elements).
// Residues are in Montgomery form unless marked normal.
//
// Integer rows (JobDev::int_rows, every row's k*b^r below 2^32): the giant value
// of row (k, r) at step s is c*Z_s with the integer c = k*b^r and
// Z_s = +-B^e0 * G^s (the sign of k*b^n+-1 folded in).  Then V[] holds the
// integers c, and el_tab+32.. holds Z_(lane % tlanes + 1) times 2^128 mod p
// instead of G^(lane % tlanes + 1) times 2^64: the kernels' normal-form
// multiplier from_mont(entry) is then Z's Montgomery form, so Shoup's product
// c*from_mont(entry), and equally montmul(c, entry), is the Montgomery form of
// the giant value, as V*G^s is in the general layout.  With row_ids_only the
// record has no V at all (el_row == el_v) and the kernels read c from row_c by
// the row id; this halves the setup kernel's scattered stores for jobs whose V
// would not be staged whole anyway.  With row_mask (integer rows, a warp per
// prime, at most 64 rows) the record keeps neither V nor row ids but one 64-bit
// mask of the active rows at el_v (el_v+1 spare, el_tab = el_v + 2); the warp
// kernel expands it into V (the integers c of the set bits, in row order) in
// shared memory from row constants its lanes hold in registers.
constexpr uint32_t kElP = 0, kElPinv = 1, kElBm = 2, kElGs = 3, kElNact = 4, kElRcp = 5;
constexpr uint32_t kElStw = 6, kElStq = 7, kElOfw = 8, kElOfq = 9, kElGw = 10, kElGq = 11;
constexpr uint32_t kElWoff = 12;   // warp offsets (W > 1)
constexpr uint32_t kElV = 12;      // V in the warp-per-prime layout (W == 1)
constexpr uint32_t kStepShoup = 0, kStepSmall = 1, kStepHigh = 2;  // ChunkBufs::small_step
// Giant-step start values of the fast kernels (template argument): V in
// Montgomery form, the integers k*b^r in V, k*b^r read by row id, or k*b^r of
// the rows of an active-row mask.
constexpr int kRowsV = 0, kRowsIntV = 1, kRowsIntId = 2, kRowsMask = 3;
constexpr uint32_t kMaskRows = 64;  // rows a row_mask record can describe
constexpr int kCtaWarps = 16;      // warps sharing one prime in the CTA-per-prime kernel
constexpr uint32_t kCtaSmemMax = 232448;  // shared memory a CTA may opt into (227 KB)
constexpr int kCtaMatchCap = 64;   // deferred tag matches per prime there

// Per-k data of the setup kernel's row loop, 32 bytes: odd part of k, its 2-adic
// valuation, the offset of its character table (kNoTable if none), k, its first
// row, the residues mod Q that have rows (bit r; Q <= 32), floor(2^64 / odd part).
struct __align__(16) KInfo {
  uint32_t k_odd, k_e2, k_jac, k_val, row0, rmask;
  uint64_t k_rcp;
};

// Job constants, passed by value to every kernel (lives in the constant bank).
struct JobDev {
  uint32_t base;
  int32_t sign;          // -1 Riesel, +1 Sierpinski
  uint32_t Q;
  uint32_t m;            // baby steps per prime
  uint32_t chain_len;    // baby steps per chain, m / (64 * cta_warps)
  uint32_t cta_warps;    // warps per prime: 1 (bsgs_kernel) or kCtaWarps (bsgs_cta_kernel)
  uint32_t el_v;         // first element of V (kElV, or kElWoff + 2*cta_warps)
  uint32_t bq_small;     // b^Q as an integer when below 2^32, else 0
  uint32_t pairable;     // Q == 2, a warp per prime and every k has rows for both residues
  uint32_t int_rows;     // every row's k*b^r < 2^32: V holds these integers (see the record layout)
  uint32_t row_ids_only; // integer rows whose records keep no V: the kernels read k*b^r by row id
  uint32_t row_mask;     // integer rows whose records keep only a mask of the active rows (see above)
  uint32_t T;            // giant steps per row
  uint32_t tlanes;       // min(T, 32): lanes sharing one row
  uint32_t rows_per_it;  // 32 / tlanes
  uint32_t steps_per_lane;  // max(1, T / 32)
  uint32_t table_log2;   // warp kernel: fast-path buckets per prime = 1 << table_log2
  uint32_t nbuckets;     // fast-path buckets per prime (the CTA kernel: any multiple of 64)
  uint32_t jbits;        // bits of j in an exact-path table entry
  uint32_t nrows, nk;
  int64_t e0;            // x = e0 + m*s - j for giant index s in [1, T]
  uint32_t x_lo, x_hi;   // x range of every row
  uint32_t nmin, nmax;
  uint32_t words_per_row;  // candidate bitmap words per row
  uint32_t datless;
  uint32_t max_act;      // capacity of the per-prime active-row arrays (= nrows)
  uint32_t rec_elems;    // 64-bit elements per prime record
  uint32_t el_row;       // first element of the row-id array
  uint32_t el_tab;       // first element of the per-lane tables (B^lane, then G^(lane % tlanes + 1))
  uint32_t stage_elems;  // elements staged per record by bsgs_kernel: header + V (el_row), or the header (el_v)
  uint32_t stage_full;   // 1 if V and row ids are read from the staged copy
  uint32_t warp_smem;    // shared-memory bytes per warp (bsgs_kernel) or per CTA (bsgs_cta_kernel)
  uint32_t exact_log2;   // slots of the exact kernel's table = 1 << exact_log2
  uint32_t exact_global; // that table exceeds shared memory: it lives in ChunkBufs::exact_tab
  uint32_t ctab_smem;    // CTA kernel, row ids: the table k*b^r of every row is copied into shared memory
  // device arrays
  const uint32_t *row_r;     // [nrows] n mod Q of each row
  const uint32_t *row_kidx;  // [nrows] index of the row's k
  const uint32_t *row_c;     // [nrows] k*b^r (meaningful when int_rows)
  const uint32_t *k_val;     // [nk]
  const uint32_t *k_odd;     // [nk] odd part of k
  const uint32_t *k_e2;      // [nk] 2-adic valuation of k
  const uint64_t *k_rcp;     // [nk] floor(2^64 / k_odd) (0 if k_odd == 1)
  const uint32_t *k_row0;    // [nk+1] rows of k are k_row0[i] .. k_row0[i+1]-1, r ascending
  const uint32_t *bitmap;    // [nrows * words_per_row], bit (x - x_lo) of row
  const uint32_t *jac_bits;  // quadratic-character tables: bit a of table k' = (a/k') == +1
  const uint32_t *k_jac;     // [nk] word offset of k's table, or kNoTable
  const KInfo *kinfo;        // [nk] the same per-k data packed for the setup kernel
  uint32_t b_odd, b_e2;
  uint64_t b_rcp;
  uint32_t b_jac;
};

struct Hit {
  uint64_t p;
  uint32_t k;
  uint32_t n;
};

// Buffers of one chunk of primes.
struct ChunkBufs {
  uint64_t *primes;     // [cap]
  uint32_t *count;      // [1] primes found by the sieve (may exceed cap)
  uint64_t *recs;       // [cap * rec_elems] records
  uint32_t *redo;       // [cap] primes handed to the exact BSGS kernel
  uint32_t *redo_count; // [1]
  uint32_t *exact_tab;  // exact-kernel tables of jobs whose table exceeds shared memory (else null)
  uint32_t cap;
  // The baby step of the chunk: kStepSmall if every prime p of the chunk has
  // p > 2^33 and b^Q * p < 2^63 (the short product by the integer b^Q,
  // mul_small), kStepHigh if b^Q < 2^32 and b^Q * 2^32 < p (Shoup's product
  // with a 32-bit constant), else kStepShoup (Shoup's product).
  uint32_t small_step;
};

struct HitBufs {
  Hit *raw;            // [cap] candidates from the BSGS kernel
  uint32_t *raw_count; // [1]
  Hit *fac;            // [cap] verified factors
  uint32_t *fac_count; // [1]
  uint32_t cap;
  unsigned long long *stat;  // [kStatCount] counters of one rs_sieve_range call, zeroed at its start
};
constexpr int kStatPaired = 0;  // primes whose giant loop took the (k, 0), (k, 1) row-pair path
constexpr int kStatExact = 1;   // primes finished by the exact kernel
constexpr int kStatCount = 2;

// One job's chunk in a multi-job BSGS launch (the batched form): its constants,
// its chunk of primes and records, its hit buffers.  Items of one launch share
// the warp-per-prime layout, the giant lanes (tlanes) and the start-value form.
struct BatchItem {
  JobDev J;
  ChunkBufs cb;
  HitBufs hb;
};
constexpr uint32_t kBatchMaxItems = 256;  // items of one multi-job launch

// Launchers (rs_kernels.cu).  All enqueue on `st` and return the launch status.
// Odd primes of [lo, hi] (lo odd) appended to out[] (count may exceed cap).
// sp: odd primes up to sqrt(hi), ascending, with rcp = floor(2^64/q); the first
// nsmall of them are below 2*kSieveOdds.  gbits: sieve_bitmap_words(lo, hi) words.
uint64_t sieve_bitmap_words(uint64_t lo, uint64_t hi);
cudaError_t launch_sieve(uint64_t lo, uint64_t hi, const uint32_t *sp, const uint64_t *sp_rcp, uint32_t nsp,
                         uint32_t nsmall, uint32_t *gbits, uint64_t *out, uint32_t *count, uint32_t cap,
                         cudaStream_t st);
cudaError_t launch_setup(const JobDev &job, const ChunkBufs &cb, cudaStream_t st);
cudaError_t launch_bsgs(const JobDev &job, const ChunkBufs &cb, const HitBufs &hb, int grid,
                        cudaStream_t st);
cudaError_t launch_bsgs_exact(const JobDev &job, const ChunkBufs &cb, const HitBufs &hb, int grid,
                              cudaStream_t st);
cudaError_t launch_verify(const JobDev &job, const HitBufs &hb, cudaStream_t st);
int bsgs_smem_bytes(const JobDev &job);
int bsgs_exact_smem_bytes(const JobDev &job);
uint64_t bsgs_exact_scratch_bytes(const JobDev &job, int exact_grid);
cudaError_t bsgs_configure(const JobDev &job, int device, int *grid_out, int *exact_grid_out);
// Multi-job launch over `nitems` items in device memory that share rep's kernel
// variant (rep: any of them); stage_max and table_log2_max are the largest over
// the items; row_mask: the variant builds V from an active-row mask.
// batch_configure gives its per-warp shared memory and grid.
uint32_t batch_warp_bytes(uint32_t stage_max, uint32_t table_log2_max, bool row_mask);
cudaError_t batch_configure(const JobDev &rep, uint32_t warp_bytes, int device, int *grid_out);
cudaError_t launch_bsgs_batch(const JobDev &rep, const BatchItem *items, uint32_t nitems, uint32_t stage_max,
                              uint32_t warp_bytes, int grid, cudaStream_t st);

// Build the character tables sel[0..nsel) of a job's list (odd parts kodd[],
// word offsets word_off[] into bits); first[] are the running word counts of
// the selected tables, total_words their sum.
cudaError_t launch_jacobi_tables(const uint32_t *kodd, const uint32_t *word_off, const uint32_t *sel,
                                 const uint32_t *first, uint32_t nsel, uint32_t total_words, uint32_t *bits,
                                 cudaStream_t st);
// Record an error for rs_last_error() and return code (rs_host.cu).
int set_error(int code, const char *fmt, ...);

// Served-form helpers (rs_host.cu, used by rs_server.cu).
// Device bytes a job from this ABCD text will hold, from a host-only plan:
// its arrays (character tables included) and its chunk buffers per prime of
// a launch (prime, count share and record).
struct JobFootprint {
  uint64_t arrays = 0;
  uint64_t per_prime = 0;
  uint32_t parts = 0;
};
int job_footprint(const char *text, size_t len, const rs_options &opt, JobFootprint *fp);
uint64_t job_resident_bytes(const rs_job *j);          // device bytes of its arrays
void job_set_mem_limit(rs_job *j, uint64_t bytes);     // chunk-buffer budget for later calls
void job_release_buffers(rs_job *j);                   // free its per-launch buffers, keep its arrays

cudaError_t run_imad_bench(int device, double *mul_ops_per_s, double *montmul_per_s, double *shoup_per_s);
// rates[6]: mad.lo.u32 per second, then 64-bit modular products per second by
// montmul, montmul_ptx, shoup_mul, shoup_mul32 and mul_small (rs_selftest.cu).
constexpr int kProductRates = 6;
cudaError_t run_product_bench(int device, double *rates);
cudaError_t run_modmul_check(int op, const uint64_t *a, const uint64_t *b, const uint64_t *c, const uint64_t *p,
                             size_t n, uint64_t *out);
cudaError_t run_arith_check(const uint64_t *a, const uint64_t *b, const uint64_t *p, size_t n,
                            uint64_t *out_mm, int32_t *out_j);

}  // namespace rs
