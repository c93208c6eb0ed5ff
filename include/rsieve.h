/*
 * rsieve.h -- C ABI of the GB300 Riesel/Sierpinski sieve (librsieve_gb300.so).
 *
 * The reference (rob147147/CUDA-Riesel-Sieve, "CUDA Riesel Sieve/kernel_v0.24.6.cu")
 * exposes no library API: its boundary is the executable's command line plus
 * the ABCD input file and the factor output file.  Each entry point below
 * replaces one step of that program, cited as kernel_v0.24.6.cu:LINE, so that
 * a host (the bundled `rsieve` CLI, a ctypes/cgo/JNI binding) can drive the
 * sieve without the process-global state the reference keeps
 * (kernel_v0.24.6.cu:37-52).
 *
 * Conventions
 *   - Every call returns an int status (RS_OK == 0).  On failure,
 *     rs_last_error() returns a message for the calling thread.
 *   - A job is caller-owned and immutable once created; device memory belongs
 *     to the job and is freed by rs_job_destroy().  Calls on one job are
 *     serialised internally (a mutex per job); distinct jobs may be used from
 *     distinct threads.
 *   - Only odd primes 3 <= p < 2^63 are sieved (the reference's arithmetic
 *     bound is p < 2^63, kernel_v0.24.6.cu:156-157,197).
 *   - The factor set is COMPLETE: every (p,k,n) with p prime in [p0,p1],
 *     n a candidate of k (or, with datless, any n in [nmin,nmax]) and
 *     p | k*b^n+sign.  The reference reports at most one factor per prime.
 */
#ifndef RSIEVE_H
#define RSIEVE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RS_OK 0
#define RS_ERR_INVALID 1   /* bad argument or malformed ABCD input */
#define RS_ERR_CUDA 2      /* CUDA runtime error (message has the CUDA text) */
#define RS_ERR_NOMEM 3     /* host or device allocation failed */
#define RS_ERR_RANGE 4     /* p range outside 3 <= p < 2^63 */
#define RS_ERR_NODEVICE 5  /* no CUDA device (the library has no CPU path) */
#define RS_ERR_CAPACITY 6  /* output buffer too small; *count holds the size needed */
#define RS_ERR_INTERNAL 7  /* a reported factor failed host re-verification */
#define RS_ERR_BUSY 8      /* server queue full: retry later */
#define RS_ERR_TIMEOUT 9   /* rs_server_wait: the job has not finished yet */

typedef struct rs_job rs_job;

/* rs_options.baby_step: the product by B = b^Q that advances a baby-step chain. */
#define RS_BABY_AUTO 0   /* the cheapest valid form below */
#define RS_BABY_SHOUP 1  /* Shoup's product by a full-size constant: valid for every prime */
#define RS_BABY_SHORT 2  /* the short product by the integer b^Q: p > 2^33 and b^Q * p < 2^63 */
#define RS_BABY_HIGH 3   /* Shoup's product by a 32-bit constant: b^Q * 2^32 < p, CTA-per-prime
                            layout only (the warp layout then takes RS_BABY_SHOUP) */

/* rs_options.char_tables: the quadratic character (k/p) of every k is read
 * from a bit table of (a/k') over a in [0, k'), k' the odd part of k, when the
 * table exists, else computed (a Jacobi symbol per prime and k).  A table costs
 * one Jacobi symbol per entry to build on the device, so it pays once the job
 * has sieved more primes than k'. */
#define RS_TABLES_AUTO 0    /* build each table when the primes the job has sieved, with
                               those of the range about to be sieved, reach its k' */
#define RS_TABLES_ALWAYS 1  /* build every table when the job is created */
#define RS_TABLES_NEVER 2   /* no tables: compute every character */

/* One removed candidate: p | k*b^n+c. */
typedef struct {
  uint64_t p;
  uint32_t k;
  uint32_t n;
  uint32_t b;  /* the sequence's base (each ABCD header carries its own) */
  int32_t c;   /* -1 (Riesel, k*b^n-1) or +1 (Sierpinski, k*b^n+1) */
} rs_factor;

/* Controls of the reference CLI (kernel_v0.24.6.cu:705-786), with AUTO = 0. */
typedef struct {
  int32_t Q;            /* -Q: subsequence modulus; 0 = chosen by the cost model.
                           A forced Q is always honoured (the reference only adopts
                           it when cheaper than Q=1, kernel_v0.24.6.cu:1089-1141). */
  int32_t hash_m;       /* -m M: at most 2<<M baby steps per prime; 0 = auto. */
  int32_t block_scale;  /* -b B: primes per launch = 128*2^(B-1) * 128*2^(T-1);   */
  int32_t thread_scale; /* -t T: 0 = auto (kernel_v0.24.6.cu:817-851).            */
  int32_t small_prime_scale; /* -s S: accepted for compatibility.  The device sieve
                           is complete up to sqrt(p1), so S changes nothing. */
  int32_t datless;      /* -v: report every n in [nmin,nmax] (kernel_v0.24.6.cu:1718-1723) */
  int32_t host_verify;  /* re-verify every factor on the host with 128-bit
                           arithmetic (kernel_v0.24.6.cu:1649-1671); default 1 */
  int32_t device;       /* CUDA device ordinal (the reference hard-codes 0) */
  int32_t baby_step;    /* form of the baby-step product (no counterpart in the
                           reference, whose only form is its montmul): RS_BABY_AUTO
                           picks, per launch, the cheapest form valid for every
                           prime of it; the others force a form where it is valid
                           (else AUTO) -- results are identical, only speed differs */
  int32_t char_tables;  /* RS_TABLES_*: when the per-k character tables are built (no
                           counterpart; results are identical, only speed differs) */
  uint64_t mem_limit;   /* device bytes for the job's per-launch buffers, which set the
                           primes per launch when -b/-t are not given; 0 = 3 GiB */
} rs_options;

/* The plan a job runs with. */
typedef struct {
  uint32_t base;
  int32_t sign;
  uint32_t num_k;
  uint32_t num_candidates;
  uint32_t nmin, nmax;
  uint32_t Q;            /* subsequence modulus */
  uint32_t rows;         /* (k, n mod Q) subsequences with candidates */
  uint32_t x_range;      /* floor(nmax/Q) - floor(nmin/Q) + 1 */
  uint32_t baby_steps;   /* m */
  uint32_t giant_steps;  /* T (per row) */
  uint32_t table_slots;  /* shared-memory hash slots per prime */
  uint32_t primes_per_launch;
  double work_per_prime; /* algorithmic montmuls per prime: 2*sqrt(E[R]*X) */
  uint64_t upload_bytes; /* host->device bytes copied when the job was created */
  uint32_t warps_per_prime; /* 1: a warp per prime; 16: a CTA per prime (large tables) */
  uint32_t row_form;     /* giant-step start values: 0 per-prime residues, 1 the integers
                            k*b^r (all < 2^32) in the records, 2 k*b^r read by row id,
                            3 k*b^r of the rows of a per-prime active-row mask (at most
                            64 rows, a warp per prime) */
  uint32_t parts;        /* (base, sign) groups of the input, each planned and searched as
                            its own part over the same primes; the plan fields above
                            describe the first part, num_k and num_candidates count all */
} rs_job_info;

/* Counters and device-timed durations of the last rs_sieve_range call. */
typedef struct {
  uint64_t primes;       /* primes sieved */
  uint64_t raw_hits;     /* hash matches that passed the candidate check */
  uint64_t factors;      /* verified factors */
  uint64_t p_covered;    /* width of the p-interval covered */
  double gpu_ms;         /* CUDA-event time from first to last kernel of the call */
  double bsgs_ms;        /* summed CUDA-event time of the BSGS kernel launches */
  double sieve_ms;       /* summed time of the prime-sieve kernel launches */
  double setup_ms;       /* summed time of the per-prime setup kernel launches */
  double exact_ms;       /* summed time of the exact-path BSGS launches (rare primes) */
  uint32_t launches;     /* kernels launched by the call */
  uint32_t bsgs_launches;
  uint64_t h2d_bytes;    /* host->device bytes the call copied */
  uint64_t d2h_bytes;    /* device->host bytes the call copied */
  uint64_t primes_by_step[3]; /* primes whose baby steps used RS_BABY_SHOUP, _SHORT, _HIGH
                            (index = form - 1) */
  uint64_t paired_primes; /* primes whose active rows came in (k, 0), (k, 1) pairs, the
                            second giant value of each pair formed by the short product by b */
  uint64_t exact_primes; /* primes finished by the exact (tag, j) table path */
} rs_stats;

void rs_options_default(rs_options *opt);

/* Parse an ABCD text (kernel_v0.24.6.cu:938-1083), plan the job
 * (kernel_v0.24.6.cu:1086-1255) and upload it (kernel_v0.24.6.cu:1367-1512).
 * Every header's base and sign are honoured: sequences are grouped by (base,
 * sign) into parts that share the prime windows (the reference takes the base
 * of the first header for every k, kernel_v0.24.6.cu:1009-1016). */
int rs_job_create_abcd(const char *text, size_t len, const rs_options *opt, rs_job **job);

/* Same from arrays: n lists in CSR form (n_offsets[num_k+1]); sign -1 or +1. */
int rs_job_create(uint32_t base, int32_t sign, uint32_t num_k, const uint32_t *k,
                  const uint32_t *n_offsets, const uint32_t *n_values, const rs_options *opt,
                  rs_job **job);

int rs_job_info_get(const rs_job *job, rs_job_info *info);

/* Parse and plan only, no device needed (the reference's planner step,
 * kernel_v0.24.6.cu:1086-1158, run on the host). */
int rs_plan_abcd(const char *text, size_t len, const rs_options *opt, rs_job_info *info);
int rs_job_destroy(rs_job *job);

/* Sieve p in [p0, p1] (inclusive; the reference's while(low < high) loop,
 * kernel_v0.24.6.cu:1537-1770, without its overshoot past P1).  Factors are
 * sorted by (p, k, n, b, c).  If more than cap are found, returns RS_ERR_CAPACITY
 * with *count = the number found (none written).  stats may be NULL. */
int rs_sieve_range(rs_job *job, uint64_t p0, uint64_t p1, rs_factor *out, size_t cap,
                   size_t *count, rs_stats *stats);

/* Measured autotuning (the reference has hand-set -b/-m/-s/-Q instead): sieve
 * [p0, p1] with each of the `candidates` (0: 3) cheapest layouts of the
 * planner's cost model (subsequence modulus Q, baby steps m, giant steps T,
 * warp or CTA per prime) and keep the fastest by device time for all later
 * calls.  The window should be representative of the job's range, large
 * enough to fill a few launches, and is not reported: sieve it again for its
 * factors, which are the same under every layout.  *chosen (may be NULL)
 * receives the resulting plan. */
int rs_job_autotune(rs_job *job, uint64_t p0, uint64_t p1, uint32_t candidates, rs_job_info *chosen);

/* Append factors in the reference's format "%llu | %d*%d^%d-1\n"
 * (kernel_v0.24.6.cu:1830-1835), with each factor's own base and sign ("+1"
 * for a Sierpinski sequence). */
int rs_write_factors(const rs_job *job, const char *path, const rs_factor *f, size_t count);

/* Sieve-file update (srsieve workflow; the reference only appends factor lines,
 * kernel_v0.24.6.cu:1830-1835): the ABCD text with every (k, n) in `removed`
 * dropped (matching the sequence's base and sign too, unless the factor's b is
 * 0), sequences with no candidate left omitted, and "// Sieved to <sieved_to>"
 * on each header.  Host only.  RS_ERR_CAPACITY with *out_len = bytes needed when
 * cap is too small. */
int rs_abcd_remove(const char *text, size_t len, const rs_factor *removed, size_t count, uint64_t sieved_to,
                   char *out, size_t cap, size_t *out_len);

/* The device prime sieve alone: odd primes in [lo, hi], ascending (replaces the
 * host generateGPUPrimes, kernel_v0.24.6.cu:1838-1987).  Returns
 * RS_ERR_CAPACITY with *count = needed when cap is too small. */
int rs_gpu_primes(uint64_t lo, uint64_t hi, uint64_t *out, size_t cap, size_t *count, int device);

/* The device prime sieve for callers that cannot allocate device memory (no
 * counterpart in the reference).  Code that runs under a device-memory budget or
 * pool that forbids new allocations, a plug-in whose host owns all device memory,
 * or a caller recording work for a CUDA graph cannot call cudaMalloc at this
 * point; this entry point allocates nothing.  The caller passes every buffer as
 * device memory it owns:
 *   sieve_primes  every odd prime up to sqrt(hi), ascending (best: the
 *                 consecutive odd primes 3, 5, 7, ...), n_sieve of them
 *   sieve_rcp     floor(2^64 / sieve_primes[i]) for each of them
 *   out, cap      the odd primes of [lo, hi], in no particular order
 *   count         the number found (may exceed cap; then only cap are written)
 * The one scratch buffer, the window's large-prime bitmap, is a fixed 4 MB array
 * in the library's device image that every GPU loading the library holds until
 * the process exits.  It limits a call to windows of at most 2^25 odd numbers
 * (hi - lo < about 6.7e7); wider windows return RS_ERR_RANGE, so split the range.
 * All calls share that array and every call clears it first: calls whose work
 * overlaps on the GPU (different streams, or threads sharing a device) race on it
 * and must be serialised by the caller.  The call is asynchronous on `stream`
 * (a cudaStream_t; NULL for the legacy default stream) on the current device;
 * results are valid once the stream has reached this point.  The first call on
 * each device looks up the array's device address (cudaGetSymbolAddress) with
 * that device current; make that first call before any stream capture.  The
 * address is looked up again on the first call after the device's context has
 * changed (a cudaDeviceReset), so that call too belongs before any capture. */
int rs_gpu_primes_static(uint64_t lo, uint64_t hi, const uint32_t *sieve_primes, const uint64_t *sieve_rcp,
                         uint32_t n_sieve, uint64_t *out, uint32_t cap, uint32_t *count, void *stream);

/* Measured throughput of the integer-multiply pipe on this GPU: plain 32-bit
 * mad.lo operations per second, and 64-bit modular products per second in the
 * two forms the kernels use (Montgomery, and Shoup's product by a fixed
 * multiplier), each from independent dependency chains.  No counterpart in the
 * reference; the roofline of the BSGS kernel is stated against it. */
int rs_bench_imad(int device, double *mul_ops_per_s, double *montmul_per_s, double *shoup_per_s);

/* The same measurement for every product form, rates[RS_BENCH_RATES]: 32-bit
 * mad.lo per second, then 64-bit modular products per second by the Montgomery
 * product in 64-bit C (__umul64hi), the same as an inline-PTX 32-bit-limb
 * carry chain (the reference's instruction form, kernel_v0.24.6.cu:205-237),
 * Shoup's product by a full-size constant, Shoup's product of a 32-bit operand,
 * and the short product by a 32-bit integer.  No counterpart in the reference. */
#define RS_BENCH_RATES 6
int rs_bench_products(int device, double *rates);

/* Device arithmetic self-test: n Montgomery products and Jacobi symbols on the
 * GPU for the given inputs (results written to out_*), used by the parity
 * tests against the oracle.  a, b < p < 2^63, p odd. */
int rs_gpu_arith_check(const uint64_t *a, const uint64_t *b, const uint64_t *p, size_t n,
                       uint64_t *out_mulmod, int32_t *out_jacobi_ap, int device);

/* Device self-test of the modular arithmetic the kernels are built from, one
 * operation per call on n inputs: out[i] = op(a[i], b[i], c[i], p[i]), p odd,
 * 3 <= p < 2^63.  No counterpart in the reference, whose montmul
 * (kernel_v0.24.6.cu:182-270) and modul64 (kernel_v0.24.6.cu:150-179) these
 * generalise.  The caller keeps every input inside the operation's domain (the
 * parity tests compare against exact integer arithmetic at the domain edges): */
#define RS_OP_MONTMUL 0     /* a*b*2^-64 mod p; a < 2^64, b < p */
#define RS_OP_FROM_MONT 1   /* a*2^-64 mod p; a < p */
#define RS_OP_SHOUP_CONST 2 /* floor(w*2^64/p) from a = w*2^64 mod p */
#define RS_OP_SHOUP 3       /* a*b mod p with c = floor(b*2^64/p); a < 2^64, b < p */
#define RS_OP_SHOUP32 4     /* (a mod 2^32)*b mod p with c = floor(b*2^64/p); b < p */
#define RS_OP_SHOUP_W32 5   /* a*b mod p with c = floor(b*2^64/p); a < 2^64, b*2^32 < p */
#define RS_OP_MUL_SMALL 6   /* a*b mod p with c = floor(2^64/p); a < p, 2^33 < p, b*p < 2^63 */
#define RS_OP_PINV 7        /* -p^-1 mod 2^64 */
#define RS_OP_ONE 8         /* 2^64 mod p */
#define RS_OP_R2 9          /* 2^128 mod p */
#define RS_OP_POW 10        /* a^b mod p; a < p */
#define RS_OP_MONTMUL_PTX 11 /* RS_OP_MONTMUL by the 32-bit-limb inline-PTX carry chain */
int rs_gpu_modmul_check(int32_t op, const uint64_t *a, const uint64_t *b, const uint64_t *c, const uint64_t *p,
                        size_t n, uint64_t *out, int device);

const char *rs_last_error(void);
const char *rs_version(void);

/* ------------------------------------------------------------------------
 * Batched form (no counterpart in the reference, which runs one job per
 * process): the p-ranges of many created jobs sieved together, round by round.
 * A round sieves and sets up every job's next chunk of primes, then runs the
 * BSGS of all warp-per-prime jobs that share a kernel variant (giant lanes and
 * start-value form) in ONE persistent launch over all their primes, so that
 * small jobs do not leave the GPU idle; jobs of the CTA-per-prime layout run
 * their own launch in the same round.  Each round is recorded as a CUDA graph
 * and launched as one: the jobs' sieve and setup launches, and then the BSGS
 * launches, sit on parallel branches of the graph (the graph instantiated for a
 * round is updated in place for the next when its shape allows).  A job of several (base, sign) parts is
 * sieved after the rounds through its own rs_sieve_range path.  Every item's
 * factors equal those of rs_sieve_range on the same job and range.  A job may
 * be in one item of a batch at a time; the jobs stay the caller's, and each
 * holds its own chunk buffers (sized by its rs_options.mem_limit) while the
 * batch runs, so many jobs in one batch want a modest mem_limit each.
 * ------------------------------------------------------------------------ */
typedef struct rs_batch rs_batch;

int rs_batch_create(int device, rs_batch **batch);
/* Add job's range [p0, p1]; *item (may be NULL) numbers it for rs_batch_result. */
int rs_batch_add(rs_batch *batch, rs_job *job, uint64_t p0, uint64_t p1, uint32_t *item);
/* Sieve every item.  stats (may be NULL) receives the whole run: gpu_ms from the
 * first round to the last verification, launches, primes and factors summed. */
int rs_batch_run(rs_batch *batch, rs_stats *stats);
/* An item's factors (sorted by (p, k, n, b, c)) and counters after rs_batch_run;
 * RS_ERR_CAPACITY with *count = the number found when cap is too small. */
int rs_batch_result(const rs_batch *batch, uint32_t item, rs_factor *out, size_t cap, size_t *count,
                    rs_stats *stats);
int rs_batch_destroy(rs_batch *batch);

/* ------------------------------------------------------------------------
 * Serving (no counterpart in the reference, which runs one job per process).
 * A server owns a device and runs submitted jobs concurrently on `slots`
 * worker threads.  Admission is by device memory: at submit a job's footprint
 * is computed on the host (its arrays plus per-launch buffers sized for its
 * p-window), and the oldest waiting job starts when a slot is free and its
 * footprint fits mem_budget next to the running jobs (a job larger than the
 * budget runs when no other does).  Finished jobs keep their arrays resident
 * (rows, per-k data, candidate bitmaps, character tables): a later request
 * with the same ABCD text and options takes them over and skips parsing,
 * planning and upload.  Idle resident jobs count against the budget and are
 * evicted least recently used first.  Results are identical to running each
 * job alone through rs_job_create_abcd + rs_sieve_range (the same kernels on
 * the same inputs).
 * ------------------------------------------------------------------------ */
typedef struct rs_server rs_server;

typedef struct {
  int32_t device;       /* CUDA device ordinal */
  uint32_t slots;       /* jobs running at once; 0 = 4 */
  uint32_t queue_cap;   /* jobs waiting for a slot before submit returns RS_ERR_BUSY; 0 = 1024 */
  uint32_t cache_jobs;  /* idle jobs kept resident at most; 0 = 64 */
  uint64_t mem_budget;  /* device bytes for running and resident jobs; 0 = 64 GiB */
} rs_server_options;

/* Timing and counters of one served job (host clock unless noted). */
typedef struct {
  int32_t status;       /* the job's rs_* status */
  uint32_t resident;    /* 1 if it ran on the resident arrays of an earlier request */
  uint64_t primes;      /* primes sieved */
  uint64_t factors;     /* factors found */
  uint64_t p_covered;   /* width of the p-interval covered */
  double queue_ms;      /* submit -> admitted to a slot */
  double run_ms;        /* admitted -> finished (job creation unless resident, sieve, release) */
  double latency_ms;    /* submit -> finished */
  double gpu_ms;        /* CUDA-event time of the job's kernels */
  double create_ms;     /* parse, plan and upload (0 when resident) */
  uint64_t mem_bytes;   /* device bytes charged to the job while it ran */
  uint64_t mem_in_use;  /* bytes charged to all running jobs just after its admission */
} rs_job_report;

void rs_server_options_default(rs_server_options *opt);
int rs_server_create(const rs_server_options *opt, rs_server **server);
/* Queue a job: the ABCD text (copied), its options (mem_limit, -b and -t are
 * set by the server) and the range [p0, p1].  The text is parsed and planned
 * here, unless the same job was submitted before, so a malformed job fails at
 * submit.  *ticket identifies it to rs_server_wait.  RS_ERR_BUSY when
 * queue_cap jobs are already waiting. */
int rs_server_submit(rs_server *server, const char *abcd, size_t len, const rs_options *opt, uint64_t p0,
                     uint64_t p1, uint64_t *ticket);
/* Wait up to timeout_ms (< 0: no limit) for a job.  RS_ERR_TIMEOUT if it has
 * not finished.  When it has: its factors (sorted by (p, k, n)) go to out and
 * *count, the report to *report (may be NULL), the ticket is released and the
 * job's own status is returned (its message via rs_last_error).  If more than
 * cap factors were found, RS_ERR_CAPACITY with *count = the number found; the
 * ticket stays valid for another call. */
int rs_server_wait(rs_server *server, uint64_t ticket, int32_t timeout_ms, rs_factor *out, size_t cap,
                   size_t *count, rs_job_report *report);
/* Let running jobs finish, drop waiting ones, stop the workers, free.  No
 * rs_server_wait may be in progress or follow (the tickets die with it). */
int rs_server_destroy(rs_server *server);

#ifdef __cplusplus
}
#endif
#endif
