// rs_internal.h -- types shared by the kernels (rs_kernels.cu) and the host
// driver (rs_host.cu).  Not part of the public C ABI.
#pragma once
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace rs {

// Empty slot of the per-prime baby-step table.  An entry is (tag << jbits) | j
// with j <= m-1 <= 2^jbits - 2, so a real entry is never all ones.
constexpr uint32_t kEmpty = 0xffffffffu;
constexpr int kWarpsPerBlock = 4;   // BSGS kernel: one prime per warp
constexpr int kSieveOdds = 1 << 18; // odd numbers per sieve segment (32 KB of bits)
constexpr int kSieveThreads = 512;

// Job constants, passed by value to every kernel (lives in the constant bank).
struct JobDev {
  uint32_t base;
  int32_t sign;          // -1 Riesel, +1 Sierpinski
  uint32_t Q;
  uint32_t m;            // baby steps per prime
  uint32_t T;            // giant steps per row
  uint32_t tlanes;       // min(T, 32): lanes sharing one row
  uint32_t rows_per_it;  // 32 / tlanes
  uint32_t steps_per_lane;  // max(1, T / 32)
  uint32_t table_log2;   // slots per prime = 1 << table_log2
  uint32_t jbits;        // bits of j in a table entry
  uint32_t nrows, nk;
  int64_t e0;            // x = e0 + m*s - j for giant index s in [1, T]
  uint32_t x_lo, x_hi;   // x range of every row
  uint32_t nmin, nmax;
  uint32_t words_per_row;  // candidate bitmap words per row
  uint32_t datless;
  uint32_t max_act;      // stride of the per-prime active-row arrays (= nrows)
  // device arrays
  const uint32_t *row_r;     // [nrows] n mod Q of each row
  const uint32_t *row_kidx;  // [nrows] index of the row's k
  const uint32_t *k_val;     // [nk]
  const uint32_t *k_odd;     // [nk] odd part of k
  const uint32_t *k_e2;      // [nk] 2-adic valuation of k
  const uint64_t *k_rcp;     // [nk] floor(2^64 / k_odd) (0 if k_odd == 1)
  const uint32_t *k_row0;    // [nk+1] rows of k are k_row0[i] .. k_row0[i+1]-1, r ascending
  const uint32_t *bitmap;    // [nrows * words_per_row], bit (x - x_lo) of row
  uint32_t b_odd, b_e2;
  uint64_t b_rcp;
};

// Per-prime record written by the setup kernel, read by the BSGS kernel.
struct __align__(16) PrimeRec {
  uint64_t p;
  uint64_t pinv;
  uint64_t Bstride;   // B^32 in Montgomery form (baby-step stride)
  uint64_t Gstride;   // G^32 (giant stride when T > 32)
  uint32_t nact;      // active rows
  uint32_t flags;
  uint64_t pad;
};

struct Hit {
  uint64_t p;
  uint32_t k;
  uint32_t n;
};

// Buffers of one chunk of primes.
struct ChunkBufs {
  uint64_t *primes;    // [cap]
  uint32_t *count;     // [1] primes found by the sieve (may exceed cap)
  PrimeRec *rec;       // [cap]
  uint64_t *vecB;      // [cap * 32]  B^lane
  uint64_t *vecG;      // [cap * 32]  G^(lane % tlanes + 1)
  uint64_t *actV;      // [cap * max_act]
  uint32_t *actRow;    // [cap * max_act]
  uint32_t cap;
};

struct HitBufs {
  Hit *raw;            // [cap] candidates from the BSGS kernel
  uint32_t *raw_count; // [1]
  Hit *fac;            // [cap] verified factors
  uint32_t *fac_count; // [1]
  uint32_t cap;
};

// Launchers (rs_kernels.cu).  All enqueue on `st` and return the launch status.
cudaError_t launch_sieve(uint64_t lo, uint64_t hi, const uint32_t *sp, const uint64_t *sp_rcp,
                         uint32_t nsp, uint64_t *out, uint32_t *count, uint32_t cap,
                         cudaStream_t st);
cudaError_t launch_setup(const JobDev &job, const ChunkBufs &cb, cudaStream_t st);
cudaError_t launch_bsgs(const JobDev &job, const ChunkBufs &cb, const HitBufs &hb, int grid,
                        cudaStream_t st);
cudaError_t launch_verify(const JobDev &job, const HitBufs &hb, cudaStream_t st);
int bsgs_smem_bytes(const JobDev &job);
cudaError_t bsgs_configure(const JobDev &job, int device, int *grid_out);

cudaError_t run_imad_bench(int device, double *mul_ops_per_s, double *montmul_per_s);
cudaError_t run_arith_check(const uint64_t *a, const uint64_t *b, const uint64_t *p, size_t n,
                            uint64_t *out_mm, int32_t *out_j);

}  // namespace rs
