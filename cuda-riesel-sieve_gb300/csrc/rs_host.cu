// rs_host.cu -- host side of librsieve_gb300: ABCD input, planner, device
// resources, the p-range driver loop and the C ABI declared in include/rsieve.h.
//
// Reference counterparts (rob147147/CUDA-Riesel-Sieve, kernel_v0.24.6.cu):
//   ABCD reader            938-1083   -> parse_abcd
//   Q choice / rows        1086-1255  -> make_plan (cost model instead of rows*range)
//   device setup, upload   1367-1512  -> upload_job / ensure_chunk_buffers
//   driver loop            1537-1770  -> rs_sieve_range (no overshoot past P1,
//                                        chunks pipelined on one stream, one sync)
//   verify + write         1600-1732, 1830-1835 -> verify kernel, host_verify,
//                                        rs_write_factors
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "rs_internal.h"
#include "rsieve.h"

using namespace rs;

// ---------------------------------------------------------------------------
// Errors

static thread_local std::string g_err;

static int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int rs::set_error(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CUDA_TRY(expr)                                                                   \
  do {                                                                                   \
    cudaError_t _e = (expr);                                                             \
    if (_e != cudaSuccess)                                                               \
      return fail(_e == cudaErrorMemoryAllocation ? RS_ERR_NOMEM : RS_ERR_CUDA, "%s: %s", \
                  #expr, cudaGetErrorString(_e));                                        \
  } while (0)

static int check_device(int device) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n <= 0)
    return fail(RS_ERR_NODEVICE, "no CUDA device available (%s); this library has no CPU path",
                e != cudaSuccess ? cudaGetErrorString(e) : "count 0");
  if (device < 0 || device >= n) return fail(RS_ERR_INVALID, "device %d out of range [0,%d)", device, n);
  CUDA_TRY(cudaSetDevice(device));
  return RS_OK;
}

// ---------------------------------------------------------------------------
// ABCD input (kernel_v0.24.6.cu:938-1083): "ABCD k*b^$a-1 [n0]" headers followed
// by positive n deltas.  Unlike the reference this rejects malformed lines,
// takes the base and the sign from each header (the reference uses the first
// header's base for every k, kernel_v0.24.6.cu:1009-1016, and assumes -1) and
// merges repeated sequences.

// Sequences of one job part: one base and one sign.  While a file is parsed,
// seq_base / seq_sign hold each sequence's own base and sign (split_parts then
// groups the sequences into parts).
struct Seqs {
  uint32_t base = 0;
  int32_t sign = 0;
  std::vector<uint32_t> k;
  std::vector<std::vector<uint32_t>> n;
  std::vector<uint32_t> seq_base;
  std::vector<int32_t> seq_sign;
};

// One n-delta line "d..d\n" of 1 to 7 digits, read eight bytes at a time: the
// digit count from the first non-digit byte (a byte b is a digit iff b - '0'
// neither borrows nor exceeds 9), the value by Lemire's three-multiply decimal
// conversion with the digits right-aligned among eight (leading zeros).
// Borrows and carries only move towards later bytes, so every byte up to the
// first non-digit is exact.  Needs 8 readable bytes at p and a little-endian
// host.  Returns false for anything else (the general path handles it).
static_assert(__BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__, "the 8-byte delta reader assumes little-endian loads");
static inline bool delta8(const char *p, uint32_t &val, uint32_t &ndig) {
  uint64_t w;
  memcpy(&w, p, 8);
  const uint64_t t = w - 0x3030303030303030ull;
  const uint64_t nd = (t | (t + 0x7676767676767676ull)) & 0x8080808080808080ull;
  if (!nd) return false;  // eight digits: longer than this reader takes
  const uint32_t L = (uint32_t)__builtin_ctzll(nd) >> 3;
  if (L == 0 || ((w >> (8 * L)) & 0xffu) != '\n') return false;
  uint64_t d = t << (8 * (8 - L));  // the digits in the top L bytes, zeros below
  d = d * 10 + (d >> 8);            // digit pairs
  d = ((d & 0x000000FF000000FFull) * (100 + (1000000ull << 32)) +
       ((d >> 16) & 0x000000FF000000FFull) * (1 + (10000ull << 32))) >> 32;
  val = (uint32_t)d;
  ndig = L;
  return true;
}

static int parse_abcd_serial(const char *text, size_t len, Seqs &out) {
  size_t i = 0;
  long line = 0;
  uint64_t total = 0;
  while (i < len) {
    line++;
    if (!out.k.empty() && i + 8 <= len) {
      // runs of short delta lines, the bulk of a file
      std::vector<uint32_t> &v = out.n.back();
      uint32_t d, L;
      bool first = true;
      while (i + 8 <= len && delta8(text + i, d, L)) {
        if (!first) line++;
        first = false;
        if (d == 0) return fail(RS_ERR_INVALID, "ABCD line %ld: bad n delta", line);
        total += d;
        if (total > 0x7fffffffull) return fail(RS_ERR_INVALID, "ABCD line %ld: n exceeds 2^31-1", line);
        v.push_back((uint32_t)total);
        i += L + 1;
      }
      if (!first) continue;
    }
    if (text[i] >= '0' && text[i] <= '9' && !out.k.empty()) {
      // the common line, a decimal n delta: digits, optional trailing blanks, newline
      uint64_t d = 0;
      size_t c = i;
      while (c < len && c - i < 11 && (unsigned)(text[c] - '0') < 10u) d = d * 10 + (uint64_t)(text[c++] - '0');
      size_t c2 = c;
      while (c2 < len && (text[c2] == '\r' || text[c2] == ' ' || text[c2] == '\t')) c2++;
      if (c - i <= 10 && (c2 == len || text[c2] == '\n')) {
        if (d == 0) return fail(RS_ERR_INVALID, "ABCD line %ld: bad n delta", line);
        total += d;
        if (total > 0x7fffffffull) return fail(RS_ERR_INVALID, "ABCD line %ld: n exceeds 2^31-1", line);
        out.n.back().push_back((uint32_t)total);
        i = c2 + 1;
        continue;
      }
    }
    size_t e = i;
    while (e < len && text[e] != '\n') e++;
    size_t a = i, z = e;
    i = e + 1;
    while (z > a && (text[z - 1] == '\r' || text[z - 1] == ' ' || text[z - 1] == '\t')) z--;
    while (a < z && (text[a] == ' ' || text[a] == '\t')) a++;
    if (a == z) continue;
    if (text[a] >= '0' && text[a] <= '9' && z - a <= 10 && !out.k.empty()) {
      // the common line: a plain decimal n delta, parsed in place
      uint64_t d = 0;
      size_t c = a;
      for (; c < z && text[c] >= '0' && text[c] <= '9'; c++) d = d * 10 + (uint64_t)(text[c] - '0');
      if (c == z) {
        if (d == 0) return fail(RS_ERR_INVALID, "ABCD line %ld: bad n delta", line);
        total += d;
        if (total > 0x7fffffffull) return fail(RS_ERR_INVALID, "ABCD line %ld: n exceeds 2^31-1", line);
        out.n.back().push_back((uint32_t)total);
        continue;
      }
    }
    std::string s(text + a, z - a);
    if (s.compare(0, 4, "ABCD") == 0 && s.size() > 4 && (s[4] == ' ' || s[4] == '\t')) {
      const char *c = s.c_str() + 5;
      while (*c == ' ' || *c == '\t') c++;
      char *end;
      unsigned long long kv = strtoull(c, &end, 10);
      if (end == c || *end != '*' || kv == 0 || kv > 0xffffffffull)
        return fail(RS_ERR_INVALID, "ABCD line %ld: bad k in header", line);
      c = end + 1;
      unsigned long long bv = strtoull(c, &end, 10);
      if (end == c || *end != '^' || bv < 2 || bv > 0xffffffffull)
        return fail(RS_ERR_INVALID, "ABCD line %ld: bad base in header", line);
      const char *dol = strstr(end, "$a");
      if (!dol) return fail(RS_ERR_INVALID, "ABCD line %ld: expected $a exponent", line);
      int32_t sg;
      if (dol[2] == '-' && dol[3] == '1') sg = -1;
      else if (dol[2] == '+' && dol[3] == '1') sg = +1;
      else return fail(RS_ERR_INVALID, "ABCD line %ld: expected -1 or +1", line);
      const char *lb = strchr(dol, '[');
      if (!lb) return fail(RS_ERR_INVALID, "ABCD line %ld: missing [n0]", line);
      long long n0 = strtoll(lb + 1, &end, 10);
      if (end == lb + 1 || *end != ']' || n0 < 0 || n0 > 0x7fffffffll)
        return fail(RS_ERR_INVALID, "ABCD line %ld: bad [n0]", line);
      if (out.base == 0) {
        out.base = (uint32_t)bv;
        out.sign = sg;
      }
      out.seq_base.push_back((uint32_t)bv);
      out.seq_sign.push_back(sg);
      out.k.push_back((uint32_t)kv);
      out.n.emplace_back();
      out.n.back().push_back((uint32_t)n0);
      total = (uint64_t)n0;
    } else {
      if (out.k.empty())
        return fail(RS_ERR_INVALID, "ABCD line %ld: data before the first ABCD header", line);
      char *end;
      long long d = strtoll(s.c_str(), &end, 10);
      if (end == s.c_str() || d <= 0) return fail(RS_ERR_INVALID, "ABCD line %ld: bad n delta", line);
      total += (uint64_t)d;
      if (total > 0x7fffffffull) return fail(RS_ERR_INVALID, "ABCD line %ld: n exceeds 2^31-1", line);
      out.n.back().push_back((uint32_t)total);
    }
  }
  if (out.k.empty()) return fail(RS_ERR_INVALID, "no ABCD header found");
  return RS_OK;
}

// Large files are parsed in pieces on the host's cores: the text is cut at
// "ABCD" header lines into contiguous ranges of about equal size, each range is
// read by the serial reader into its own sequence list, and the lists are
// concatenated in order.  Any error re-runs the serial reader on the whole
// text, so messages and line numbers are those of the serial reader.
static int parse_abcd(const char *text, size_t len, Seqs &out) {
  constexpr size_t kPieceBytes = 4u << 20;
  unsigned nthr = std::thread::hardware_concurrency();
  if (nthr > 16) nthr = 16;
  if (len < 2 * kPieceBytes || nthr < 2) return parse_abcd_serial(text, len, out);
  if (len / kPieceBytes < nthr) nthr = (unsigned)(len / kPieceBytes);
  // cut points: the first header line at or after len*t/nthr
  std::vector<size_t> cut{0};
  for (unsigned t = 1; t < nthr; t++) {
    size_t q = std::max(cut.back() + 1, len * t / nthr);
    bool found = false;
    while (q + 5 < len) {
      const void *nl = memchr(text + q, '\n', len - q);
      if (!nl) break;
      q = (size_t)((const char *)nl - text) + 1;
      if (q + 4 <= len && memcmp(text + q, "ABCD", 4) == 0) {
        found = true;
        break;
      }
    }
    if (!found) break;
    cut.push_back(q);
  }
  cut.push_back(len);
  const size_t np = cut.size() - 1;
  if (np < 2) return parse_abcd_serial(text, len, out);
  std::vector<Seqs> part(np);
  std::vector<int> rc(np, RS_OK);
  auto piece = [&](size_t t) { rc[t] = parse_abcd_serial(text + cut[t], cut[t + 1] - cut[t], part[t]); };
  std::vector<std::thread> th;
  size_t started = 0;
  try {
    for (; started < np; started++) th.emplace_back(piece, started);
  } catch (...) {  // no more threads: the rest run here
  }
  for (size_t t = started; t < np; t++) piece(t);
  for (auto &x : th) x.join();
  bool ok = true;
  for (size_t t = 0; t < np; t++) ok = ok && rc[t] == RS_OK;
  if (!ok) {
    out = Seqs();
    return parse_abcd_serial(text, len, out);
  }
  out.base = part[0].base;
  out.sign = part[0].sign;
  size_t nk = 0;
  for (auto &p : part) nk += p.k.size();
  out.k.reserve(nk);
  out.n.reserve(nk);
  out.seq_base.reserve(nk);
  out.seq_sign.reserve(nk);
  for (auto &p : part) {
    out.k.insert(out.k.end(), p.k.begin(), p.k.end());
    out.seq_base.insert(out.seq_base.end(), p.seq_base.begin(), p.seq_base.end());
    out.seq_sign.insert(out.seq_sign.end(), p.seq_sign.begin(), p.seq_sign.end());
    for (auto &v : p.n) out.n.push_back(std::move(v));
  }
  return RS_OK;
}

// Group parsed sequences by (base, sign), in order of first appearance: each
// group is planned and sieved as one part of the job.
static std::vector<Seqs> split_parts(Seqs &&all) {
  std::vector<Seqs> parts;
  if (all.seq_base.size() != all.k.size()) {  // built from arrays: one base and sign
    all.seq_base.clear();
    all.seq_sign.clear();
    parts.push_back(std::move(all));
    return parts;
  }
  for (size_t i = 0; i < all.k.size(); i++) {
    size_t g = 0;
    for (; g < parts.size(); g++)
      if (parts[g].base == all.seq_base[i] && parts[g].sign == all.seq_sign[i]) break;
    if (g == parts.size()) {
      parts.emplace_back();
      parts.back().base = all.seq_base[i];
      parts.back().sign = all.seq_sign[i];
    }
    parts[g].k.push_back(all.k[i]);
    parts[g].n.push_back(std::move(all.n[i]));
  }
  return parts;
}

// Merge repeated k, sort and de-duplicate every n list (sequences of one part).
static void normalise(Seqs &s) {
  Seqs o;
  o.base = s.base;
  o.sign = s.sign;
  for (size_t i = 0; i < s.k.size(); i++) {
    size_t j = 0;
    for (; j < o.k.size(); j++)
      if (o.k[j] == s.k[i]) break;
    if (j == o.k.size()) {
      o.k.push_back(s.k[i]);
      o.n.push_back(std::move(s.n[i]));
    } else {
      o.n[j].insert(o.n[j].end(), s.n[i].begin(), s.n[i].end());
    }
  }
  for (auto &v : o.n) {
    if (std::adjacent_find(v.begin(), v.end(), [](uint32_t x, uint32_t y) { return x >= y; }) == v.end())
      continue;  // already strictly increasing (positive deltas)
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
  }
  s = std::move(o);
}

// ---------------------------------------------------------------------------
// Planner.  The reference picks the even Q in [2,22] minimising rows*range and
// keeps Q=1 unless strictly cheaper (kernel_v0.24.6.cu:1086-1146).  Here the
// cost is the per-lane Montgomery-product count of the warp-per-prime kernel;
// Q, the giant steps per row T and the baby steps m are chosen together.

struct Plan {
  uint32_t Q = 0, nrows = 0, X = 0, x_lo = 0, x_hi = 0, m = 0, T = 0;
  uint32_t tlanes = 0, rows_per_it = 0, steps_per_lane = 0, table_log2 = 0, jbits = 0, bucket_log2 = 0;
  uint32_t nbuckets = 0;  // fast-path buckets (1 << bucket_log2 for the warp kernel; a multiple of 64 for a CTA)
  bool cta = false;  // one CTA of kCtaWarps warps per prime (bsgs_cta_kernel)
  uint32_t nmin = 0, nmax = 0, ncand = 0, words_per_row = 0;
  int64_t e0 = 0;
  double cost = 0, work_per_prime = 0;
  std::vector<uint32_t> row_r, row_kidx, k_row0;
  std::vector<uint32_t> bitmap;
};

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

static uint32_t ilog2_ceil(uint64_t v) {
  uint32_t b = 0;
  while (((uint64_t)1 << b) < v) b++;
  return b;
}

static constexpr uint32_t kMaxTableLog2 = 13;  // 8192 slots = 32 KB per warp

static int count_rows(const Seqs &s, uint32_t Q, bool datless) {
  if (datless) return (int)(s.k.size() * Q);
  int rows = 0;
  std::vector<char> seen(Q);
  for (size_t i = 0; i < s.k.size(); i++) {
    std::fill(seen.begin(), seen.end(), 0);
    uint32_t got = 0;
    for (uint32_t n : s.n[i]) {
      if (!seen[n % Q]) {
        seen[n % Q] = 1;
        if (++got == Q) break;  // every residue present: the rest of the list adds nothing
      }
    }
    rows += (int)got;
  }
  return rows;
}

// One point of the planner's search: the parameters that define a plan, and its modelled cost.
struct PlanChoice {
  uint32_t Q = 0, T = 0, m = 0;
  bool cta = false;
  double cost = 0;
  uint32_t nb = 0;  // fast-path buckets
};

// Plan a job.  With `force`, take exactly that choice (it must be feasible);
// with `ranked`, also return every feasible choice, cheapest first.
static int make_plan(const Seqs &s, const rs_options &opt, Plan &pl, bool with_bitmap = true,
                     const PlanChoice *force = nullptr, std::vector<PlanChoice> *ranked = nullptr) {
  uint32_t nmin = 0xffffffffu, nmax = 0, ncand = 0;
  for (auto &v : s.n) {
    if (v.empty()) continue;
    nmin = std::min(nmin, v.front());
    nmax = std::max(nmax, v.back());
    ncand += (uint32_t)v.size();
  }
  if (ncand == 0) return fail(RS_ERR_INVALID, "job has no candidates");
  const bool datless = opt.datless != 0;
  const double K = (double)s.k.size();
  std::vector<uint32_t> Qs;
  if (opt.Q > 0) {
    Qs.push_back((uint32_t)opt.Q);
  } else {
    Qs.push_back(1);
    for (uint32_t q = 2; q <= 48; q += 2) Qs.push_back(q);
  }
  uint64_t mcap = 65534;
  if (opt.hash_m > 0) {
    if (opt.hash_m > 14) return fail(RS_ERR_INVALID, "-m %d too large (at most 14)", opt.hash_m);
    mcap = std::min<uint64_t>(mcap, (uint64_t)2 << opt.hash_m);
  }
  // Shared memory of an SM, and the warps per SM the warp-per-prime kernel
  // reaches with small tables (registers allow 5 CTAs of 4 warps).
  constexpr double kSmemPerSm = 233472.0, kFullWarps = 20.0;
  // A giant step (Shoup product + probe) costs about 1.4 baby steps (a short or
  // Shoup product + insert), measured on the benchmark job.
  constexpr double kGiantWeight = 1.4;
  // Setup-kernel cost per (k, n mod Q) row, in the same units.
  constexpr double kRowCost = 0.18;
  // A step of the CTA kernel costs more than one of the warp kernel (block-wide
  // barriers, per-prime tag-match passes); fitted with rs_job_autotune on mixed jobs.
  constexpr double kCtaStepCost = 1.25;
  double best = 1e300;
  for (uint32_t Q : Qs) {
    const uint32_t X = nmax / Q - nmin / Q + 1;
    const int rows = count_rows(s, Q, datless);
    const double ER = rows * ((Q & 1) ? 0.75 : 0.5);
    // every row's k*b^r below 2^32 (integer rows; see plan_row_form)
    bool ints_q = true;
    {
      uint64_t kmax = 0;
      for (uint32_t k : s.k) kmax = std::max<uint64_t>(kmax, k);
      uint64_t c = kmax;
      for (uint32_t e = 1; e < Q && c < (1ull << 32); e++) c *= s.base;
      ints_q = c < (1ull << 32);
    }
    auto consider = [&](bool cta, uint64_t T, uint64_t m, uint32_t blog, uint32_t nb, uint32_t slog, double cost) {
      if (ranked) ranked->push_back(PlanChoice{Q, (uint32_t)T, (uint32_t)m, cta, cost, nb});
      if (force) {
        if (force->Q != Q || force->T != T || force->m != m || force->cta != cta || force->nb != nb) return;
        cost = -1.0;  // the forced choice wins
      }
      if (cost < best) {
        best = cost;
        pl.Q = Q;
        pl.nrows = (uint32_t)rows;
        pl.X = X;
        pl.m = (uint32_t)m;
        pl.T = (uint32_t)T;
        pl.tlanes = (uint32_t)std::min<uint64_t>(T, 32);
        pl.rows_per_it = 32 / pl.tlanes;
        pl.steps_per_lane = (uint32_t)std::max<uint64_t>(1, T / 32);
        pl.table_log2 = slog;
        pl.bucket_log2 = blog;
        pl.nbuckets = nb;
        pl.cta = cta;
        pl.cost = cost;
        pl.work_per_prime = 2.0 * std::sqrt(ER * (double)X);
      }
    };
    for (uint32_t tl = 0; tl <= 20; tl++) {
      const uint64_t T = (uint64_t)1 << tl;
      const uint64_t m0 = (X + T - 1) / T;
      const uint32_t tlanes = (uint32_t)std::min<uint64_t>(T, 32);
      const uint32_t rpi = 32 / tlanes;
      const uint32_t spl = (uint32_t)std::max<uint64_t>(1, T / 32);
      // Costs are in warp-steps per prime: one baby or giant step of 32 lanes
      // (a product plus a table operation), the table clear, the per-prime
      // setup kernel (grows with the rows), the expected tag-match
      // resolution (one pass over the baby steps), and a penalty for fewer
      // resident warps when the tables are large.
      {  // warp per prime: whole chains of 64 when that stays within the cap
        uint64_t m = m0;
        if (m > 64 && ((m + 63) & ~63ull) <= mcap) m = (m + 63) & ~63ull;
        const uint32_t slog = std::max<uint32_t>(7, ilog2_ceil(2 * m));  // exact-path table
        if (m <= mcap && m * T >= X && slog <= kMaxTableLog2) {
          const uint32_t blog = std::max<uint32_t>(4, ilog2_ceil((2 * m + kBucket - 1) / kBucket));
          const double nb = (double)(1u << blog);
          // the kernel's shared memory per warp and per CTA (128-byte granules, 1 KB reserved)
          const uint64_t stage = kElV + ((rows + 1) & ~1u);
          const uint64_t wsm = align_up((20u << blog) + 16 * (stage * 8 <= 2048 ? stage : kElV) + 16 * kMatchCap + 16, 16);
          const double cta_bytes = (double)align_up(4 * wsm, 128) + 1024.0;
          const double warps = std::min(kFullWarps, 4.0 * std::floor(kSmemPerSm / cta_bytes));
          const double fp = ER * (double)T * ((double)m / nb) / 65536.0;  // expected tag matches per prime
          // (a prime with more than kMatchCap matches takes the slow exact path)
          if (warps >= 4 && fp <= 2.0) {
            const double cost = (std::ceil((double)m / 32.0) + kGiantWeight * std::ceil(ER / rpi) * spl +
                                 nb * 8 / 1024.0 + 3.7 + kRowCost * rows + std::min(1.0, fp) * (double)m / 32.0) *
                                std::sqrt(kFullWarps / warps);
            consider(false, T, m, blog, 1u << blog, slog, cost);
          }
        }
      }
      if (T >= 32 && T <= 256) {  // a CTA per prime: 64 * kCtaWarps chains share a table of up to ~220 KB
        const uint64_t chains = 64 * kCtaWarps;
        const uint64_t m = (m0 + chains - 1) / chains * chains;
        // exact-path table (rare primes): shared memory up to 2^15 slots, else global scratch
        const uint32_t slog = std::max<uint32_t>(7, ilog2_ceil(2 * m));
        // V staging: the integers k*b^r read by row id (two bytes a row) when a lane takes
        // two or more giant steps, else eight bytes a row (the row form of plan_row_form)
        const double vbytes = (ints_q && T >= 64 ? 2.0 : 8.0) * (rows + 2) + 16.0;
        // buckets: a power of two with at most ~2 entries each, or, when that table does
        // not fit the shared memory, the smallest multiple of 64 with at most ~2 each.
        // (Tables at ~3 entries a bucket measured slower on the wide job, 183-216 against
        // 174 ns per prime: more full buckets and more false tag matches.)
        const uint32_t blog = std::max<uint32_t>(4, ilog2_ceil((m + 1) / 2));
        const uint32_t nb_opts[2] = {1u << blog, (uint32_t)std::max<uint64_t>(64, ((m + 1) / 2 + 63) / 64 * 64)};
        for (int o = 0; o < 2; o++) {
          const uint32_t nbk = nb_opts[o];
          const double nb = (double)nbk;
          const double smem = 20.0 * nb + vbytes + 16.0 * (kCtaMatchCap + 1);
          if (o == 1 && (nbk >= nb_opts[0] || nbk > 65536 || 20.0 * nb_opts[0] + vbytes + 16.0 * (kCtaMatchCap + 1) <= kCtaSmemMax))
            continue;
          const double fp = ER * (double)T * ((double)m / nb) / 65536.0;
          // (m < 2^16: a bucket's insert count is the low half of its count word)
          if (m <= mcap && m < 65536 && m * T >= X && slog <= 17 && smem <= kCtaSmemMax && fp <= 16.0) {
            const double cost = ((double)m / 32.0 + kGiantWeight * kCtaWarps * std::ceil(ER / kCtaWarps) * spl +
                                 nb * 8 / 1024.0 + 3.7 + kRowCost * rows + std::min(1.0, fp) * (double)m / 32.0) *
                                std::sqrt(kFullWarps / kCtaWarps) * kCtaStepCost;
            consider(true, T, m, blog, nbk, slog, cost);
          }
        }
      }
    }
  }
  if (ranked)
    std::sort(ranked->begin(), ranked->end(), [](const PlanChoice &a, const PlanChoice &b) { return a.cost < b.cost; });
  if (pl.Q == 0) return fail(RS_ERR_INVALID, "no feasible plan (n range too wide for the -m limit)");
  pl.nmin = nmin;
  pl.nmax = nmax;
  pl.ncand = ncand;
  pl.x_lo = nmin / pl.Q;
  pl.x_hi = nmax / pl.Q;
  pl.e0 = (int64_t)pl.x_lo - 1;
  pl.jbits = 1;
  while (((uint64_t)1 << pl.jbits) < (uint64_t)pl.m + 1) pl.jbits++;
  pl.words_per_row = (pl.X + 31) / 32;
  // rows: k in input order, r ascending (the residues present: scan until all
  // Q have been seen)
  const uint32_t Q = pl.Q;
  const size_t nk = s.k.size();
  pl.k_row0.assign(nk + 1, 0);
  std::vector<char> seen(Q);
  for (size_t i = 0; i < nk; i++) {
    pl.k_row0[i] = (uint32_t)pl.row_r.size();
    if (datless) {
      std::fill(seen.begin(), seen.end(), 1);
    } else {
      std::fill(seen.begin(), seen.end(), 0);
      uint32_t got = 0;
      for (uint32_t n : s.n[i])
        if (!seen[n % Q]) {
          seen[n % Q] = 1;
          if (++got == Q) break;
        }
    }
    for (uint32_t r = 0; r < Q; r++)
      if (seen[r]) {
        pl.row_r.push_back(r);
        pl.row_kidx.push_back((uint32_t)i);
      }
  }
  pl.k_row0[nk] = (uint32_t)pl.row_r.size();
  pl.nrows = (uint32_t)pl.row_r.size();
  if (pl.nrows > 65535) return fail(RS_ERR_INVALID, "too many (k, n mod Q) rows (%u > 65535)", pl.nrows);
  if (datless) {
    pl.bitmap.assign(1, 0);
  } else if (with_bitmap) {
    // candidate bitmap rows (bit x - x_lo of row (k, n mod Q)); the k are
    // independent, so large jobs fill them on several host threads
    pl.bitmap.assign((size_t)pl.nrows * pl.words_per_row, 0);
    auto fill = [&](size_t k0, size_t k1) {
      std::vector<uint32_t> local(Q);
      for (size_t i = k0; i < k1; i++) {
        for (uint32_t row = pl.k_row0[i]; row < pl.k_row0[i + 1]; row++) local[pl.row_r[row]] = row;
        uint32_t *bm = pl.bitmap.data();
        const uint32_t wpr = pl.words_per_row, xlo = pl.x_lo;
        if (Q == 1) {
          uint32_t *rowp = bm + (size_t)pl.k_row0[i] * wpr;
          for (uint32_t n : s.n[i]) rowp[(n - xlo) >> 5] |= 1u << ((n - xlo) & 31);
        } else {
          for (uint32_t n : s.n[i]) {
            const uint32_t x = n / Q, r = n - x * Q, bit = x - xlo;
            bm[(size_t)local[r] * wpr + (bit >> 5)] |= 1u << (bit & 31);
          }
        }
      }
    };
    size_t ncand = 0;
    for (auto &v : s.n) ncand += v.size();
    unsigned nthr = std::min<unsigned>(16, std::max(1u, std::thread::hardware_concurrency()));
    if (ncand < (2u << 20) || nk < 2 * nthr) nthr = 1;
    if (nthr == 1) {
      fill(0, nk);
    } else {
      // k ranges of about equal candidate counts
      std::vector<std::pair<size_t, size_t>> ranges;
      size_t k0 = 0, acc = 0;
      for (size_t i = 0; i < nk; i++) {
        acc += s.n[i].size();
        if (acc * nthr >= ncand * (ranges.size() + 1) || i + 1 == nk) {
          ranges.emplace_back(k0, i + 1);
          k0 = i + 1;
        }
      }
      std::vector<std::thread> th;
      size_t started = 0;
      try {
        for (; started < ranges.size(); started++) th.emplace_back(fill, ranges[started].first, ranges[started].second);
      } catch (...) {  // no more threads: the rest run here
      }
      for (size_t t = started; t < ranges.size(); t++) fill(ranges[t].first, ranges[t].second);
      for (auto &x : th) x.join();
    }
  }
  return RS_OK;
}

// ---------------------------------------------------------------------------
// The job.

// Sieving primes of one device: odd primes <= limit with floor(2^64/q), shared
// by every job on that device (a job keeps the set it started with alive).
struct DevPrimes {
  int device = 0;
  uint64_t limit = 0;
  uint32_t n = 0, nsmall = 0;
  uint32_t *d_sp = nullptr;
  uint64_t *d_rcp = nullptr;
  ~DevPrimes() {
    int cur = 0;
    if (cudaGetDevice(&cur) != cudaSuccess) return;
    cudaSetDevice(device);
    if (d_sp) cudaFree(d_sp);
    if (d_rcp) cudaFree(d_rcp);
    cudaSetDevice(cur);
  }
};

// One part of a job: the sequences of one base and one sign, with their own
// plan, device arrays, kernel configuration and hit buffers.  A job's parts
// share its stream, sieving primes, prime windows and chunk buffers: each
// chunk of primes is sieved once and then set up and searched for every part.
struct Part {
  std::vector<PlanChoice> ranked;  // the planner's feasible choices, cheapest first (for rs_job_autotune)
  Seqs seqs;
  Plan plan;
  JobDev dev{};
  void *d_job = nullptr;  // job arrays
  size_t job_bytes = 0;   // bytes uploaded into them
  size_t dev_bytes = 0;   // their device size (with the character tables built on the device)
  HitBufs hb{};
  void *d_hits = nullptr;
  int bsgs_grid = 0;
  int exact_grid = 0;
  // Quadratic-character tables (rs_options.char_tables): the odd parts k' with
  // a table and their word offsets in the job arrays, which of them are built,
  // each k's table (index into tab_k, or -1) and the base's, the host copies of
  // the per-k table offsets and records that go to the device as tables are
  // built, and the primes the part has sieved (estimated from its ranges).
  std::vector<uint32_t> tab_k, tab_off;
  std::vector<uint8_t> tab_built;
  std::vector<int32_t> ktab;
  int32_t btab = -1;
  std::vector<uint32_t> kjac_host;
  std::vector<KInfo> kinfo_host;
  const uint32_t *d_tab_k = nullptr, *d_tab_off = nullptr;
  uint32_t *d_jac_bits = nullptr, *d_kjac = nullptr;
  KInfo *d_kinfo = nullptr;
  double primes_seen = 0;
};

struct rs_job {
  std::mutex mu;
  std::shared_ptr<DevPrimes> primes;  // sieving primes in use (d_sp, d_sp_rcp below point into it)
  rs_options opt;
  std::vector<std::unique_ptr<Part>> parts;
  int device = 0;
  cudaStream_t st = nullptr;
  // sieving primes (odd primes <= sp_limit)
  uint64_t sp_limit = 0;
  uint32_t nsp = 0;
  uint32_t nsp_small = 0;        // sieving primes below 2*kSieveOdds
  uint32_t *d_gbits = nullptr;   // window bitmap of the large-prime sieve pass
  uint64_t gbits_words = 0;
  uint32_t *d_sp = nullptr;
  uint64_t *d_sp_rcp = nullptr;
  // chunk buffers (records sized for the largest part)
  ChunkBufs cb{};
  void *d_chunk = nullptr;
  uint32_t *h_counts = nullptr;  // pinned, one slot per chunk + 2
  size_t h_counts_cap = 0;
  uint32_t chunk_cap = 0;
  uint32_t chunk_rec_elems = 0;  // record elements the chunk buffers were sized for
  uint64_t chunk_exact_bytes = 0;  // exact-kernel scratch they hold
  uint32_t max_rec_elems() const {
    uint32_t r = 0;
    for (auto &pt : parts) r = std::max(r, pt->dev.rec_elems);
    return r;
  }
};


// Pinned host blocks for the per-chunk prime counts, kept for reuse by later
// jobs: freeing pinned memory synchronises the whole device, which would stall
// the other jobs of a server.  Device buffers are stream-ordered
// (cudaMallocAsync / cudaFreeAsync on the job's stream) for the same reason.
static std::mutex g_pin_mu;
static std::vector<std::pair<void *, size_t>> g_pin_free;

static void *pinned_get(size_t bytes) {
  bytes = align_up(bytes, 4096);
  {
    std::lock_guard<std::mutex> lock(g_pin_mu);
    for (size_t i = 0; i < g_pin_free.size(); i++)
      if (g_pin_free[i].second == bytes) {
        void *p = g_pin_free[i].first;
        g_pin_free.erase(g_pin_free.begin() + i);
        return p;
      }
  }
  void *p = nullptr;
  return cudaMallocHost(&p, bytes) == cudaSuccess ? p : nullptr;
}

static void pinned_put(void *p, size_t bytes) {
  std::lock_guard<std::mutex> lock(g_pin_mu);
  g_pin_free.push_back({p, align_up(bytes, 4096)});
}

// Form of the giant-step start values (rs_job_info.row_form): kRowsV (V in
// Montgomery form per active row), kRowsIntV (the integers k*b^r, all below
// 2^32, in V) or kRowsIntId (no V: the kernels read k*b^r by row id).  The last
// when the warp kernel could not stage header + V whole anyway, or when the CTA
// kernel takes two or more giant steps per lane from each start value: there
// the lookup costs less than the setup kernel's V stores (measured on mixed
// jobs).  row_c receives k*b^r per row.
static uint32_t plan_row_form(const Plan &pl, const Seqs &s, std::vector<uint32_t> *row_c) {
  if (row_c) row_c->assign(pl.row_r.size(), 0);
  bool ints = !pl.row_r.empty();
  for (size_t r = 0; r < pl.row_r.size() && ints; r++) {
    uint64_t c = s.k[pl.row_kidx[r]];
    for (uint32_t e = 0; e < pl.row_r[r] && c < (1ull << 32); e++) c *= s.base;
    if (c >= (1ull << 32)) ints = false;
    else if (row_c) (*row_c)[r] = (uint32_t)c;
  }
  if (!ints) return kRowsV;
  if (!pl.cta && pl.nrows <= kMaskRows) return kRowsMask;
  const uint32_t vslots = (std::max<uint32_t>(1, pl.nrows) + 1) & ~1u;
  const uint32_t el_v = pl.cta ? kElWoff + 2 * kCtaWarps : kElV;
  const bool ids = pl.cta ? pl.steps_per_lane >= 2 : (el_v + vslots) * 8 > 2048;
  return ids ? kRowsIntId : kRowsIntV;
}

// First element of the lane tables in a record (el_tab; a record has el_tab + 64
// elements), from the plan and the row form, as upload_part lays it out.
static uint32_t record_el_tab(const Plan &pl, uint32_t form) {
  const uint32_t el_v = pl.cta ? kElWoff + 2 * kCtaWarps : kElV;
  if (form == kRowsMask) return el_v + 2;
  const uint32_t max_act = std::max<uint32_t>(1, pl.nrows);
  const uint32_t el_row = el_v + (form == kRowsIntId ? 0u : ((max_act + 1) & ~1u));
  return el_row + 2 * ((max_act + 7) / 8);
}

// Device bytes of a part's job arrays (upload_part's single allocation,
// character tables included), from a plan made without the bitmap.
static uint64_t part_array_bytes(const Plan &pl, const Seqs &s, bool datless) {
  const uint64_t nk = s.k.size(), nr = pl.nrows;
  uint64_t b = 3 * nr * 4 + nk * (4 + 4 + 4 + 8 + 4 + sizeof(KInfo)) + (nk + 1) * 4;
  b += datless ? 4 : nr * (uint64_t)pl.words_per_row * 4;
  std::vector<uint32_t> odd;
  for (uint32_t k : s.k) {
    while (!(k & 1)) k >>= 1;
    if (k > 1) odd.push_back(k);
  }
  uint32_t bo = s.base;
  while (!(bo & 1)) bo >>= 1;
  if (bo > 1) odd.push_back(bo);
  std::sort(odd.begin(), odd.end());
  odd.erase(std::unique(odd.begin(), odd.end()), odd.end());
  uint64_t words = 0;
  for (uint32_t k : odd) words += (k + 31) / 32;
  if (words <= (256ull << 20)) b += words * 4 + odd.size() * 8;
  return b + 20 * 256;  // section alignment
}

// Primes in [a, b], estimated (b - a + 1) / ln b.
static double primes_estimate(uint64_t a, uint64_t b) {
  if (b < a) return 0.0;
  return (double)(b - a + 1) / std::log((double)std::max<uint64_t>(b, 16));
}

// Build the character tables of a part that pay for themselves: every table
// when `all`, else those whose k' is at most the primes the part has sieved,
// counting `primes_more` (the estimate of the range about to be sieved) -- a
// table costs one Jacobi symbol per entry, and saves one per prime sieved.
// The per-k table offsets on the device (and the base's, in the part's
// JobDev) follow, on the job's stream, ahead of the setup launches.
static int build_char_tables(rs_job *j, Part &pt, double primes_more, bool all) {
  if (pt.tab_k.empty()) return RS_OK;
  pt.primes_seen += primes_more;
  std::vector<uint32_t> sel, first;
  uint64_t words = 0;
  for (size_t t = 0; t < pt.tab_k.size(); t++)
    if (!pt.tab_built[t] && (all || (double)pt.tab_k[t] <= pt.primes_seen)) {
      sel.push_back((uint32_t)t);
      first.push_back((uint32_t)words);
      words += (pt.tab_k[t] + 31) / 32;
    }
  if (sel.empty()) return RS_OK;
  std::vector<uint32_t> args(sel);
  args.insert(args.end(), first.begin(), first.end());
  uint32_t *d_args = nullptr;
  CUDA_TRY(cudaMallocAsync((void **)&d_args, args.size() * 4, j->st));
  cudaError_t e = cudaMemcpyAsync(d_args, args.data(), args.size() * 4, cudaMemcpyHostToDevice, j->st);
  if (e == cudaSuccess)
    e = launch_jacobi_tables(pt.d_tab_k, pt.d_tab_off, d_args, d_args + sel.size(), (uint32_t)sel.size(),
                             (uint32_t)words, pt.d_jac_bits, j->st);
  cudaFreeAsync(d_args, j->st);
  if (e != cudaSuccess) return fail(RS_ERR_CUDA, "character tables: %s", cudaGetErrorString(e));
  for (uint32_t t : sel) pt.tab_built[t] = 1;
  const size_t nk = pt.ktab.size();
  for (size_t i = 0; i < nk; i++) {
    const int32_t t = pt.ktab[i];
    const uint32_t off = t >= 0 && pt.tab_built[t] ? pt.tab_off[t] : kNoTable;
    pt.kjac_host[i] = off;
    pt.kinfo_host[i].k_jac = off;
  }
  if (pt.btab >= 0 && pt.tab_built[pt.btab]) pt.dev.b_jac = pt.tab_off[pt.btab];
  CUDA_TRY(cudaMemcpyAsync(pt.d_kjac, pt.kjac_host.data(), nk * 4, cudaMemcpyHostToDevice, j->st));
  CUDA_TRY(cudaMemcpyAsync(pt.d_kinfo, pt.kinfo_host.data(), nk * sizeof(KInfo), cudaMemcpyHostToDevice, j->st));
  return RS_OK;
}

static int upload_part(rs_job *j, Part &pt) {
  const Plan &pl = pt.plan;
  const Seqs &s = pt.seqs;
  const uint32_t nk = (uint32_t)s.k.size();
  std::vector<uint32_t> kodd(nk), ke2(nk);
  std::vector<uint64_t> krcp(nk);
  for (uint32_t i = 0; i < nk; i++) {
    uint32_t k = s.k[i], e = 0;
    while (!(k & 1)) {
      k >>= 1;
      e++;
    }
    kodd[i] = k;
    ke2[i] = e;
    krcp[i] = k > 1 ? (~0ull) / k : 0;
  }
  // one allocation, 256-byte aligned sections
  size_t off = 0;
  auto sec = [&](size_t bytes) {
    size_t o = off;
    off = align_up(off + bytes, 256);
    return o;
  };
  std::vector<uint32_t> row_c;
  const uint32_t form = plan_row_form(pl, s, &row_c);
  const size_t o_rr = sec(pl.row_r.size() * 4), o_rk = sec(pl.row_kidx.size() * 4), o_rc = sec(row_c.size() * 4);
  const size_t o_kv = sec(nk * 4), o_ko = sec(nk * 4), o_ke = sec(nk * 4), o_kr = sec(nk * 8);
  const size_t o_k0 = sec((nk + 1) * 4), o_bm = sec(pl.bitmap.size() * 4);
  // Quadratic-character tables, one per distinct odd part > 1 of k and b, room
  // for all of them when they fit in 1 GB; each is built on the device when it
  // pays (build_char_tables), until then the setup kernel computes (k/p).
  std::vector<uint32_t> &tab_k = pt.tab_k, &tab_off = pt.tab_off;  // odd parts and their word offsets
  tab_k.clear();
  tab_off.clear();
  pt.ktab.assign(nk, -1);
  pt.btab = -1;
  uint64_t twords = 0;
  if (j->opt.char_tables != RS_TABLES_NEVER) {
    uint32_t bo = s.base;
    while (!(bo & 1)) bo >>= 1;
    std::unordered_map<uint32_t, int32_t> index;
    auto find_or_add = [&](uint32_t ko) -> int32_t {
      if (ko <= 1) return -1;
      const auto f = index.find(ko);
      if (f != index.end()) return f->second;
      tab_k.push_back(ko);
      tab_off.push_back((uint32_t)twords);
      twords += (ko + 31) / 32;
      return index[ko] = (int32_t)tab_k.size() - 1;
    };
    for (uint32_t i = 0; i < nk; i++) pt.ktab[i] = find_or_add(kodd[i]);
    pt.btab = find_or_add(bo);
    if (twords > (256ull << 20)) {  // too large: compute the symbols instead
      std::fill(pt.ktab.begin(), pt.ktab.end(), -1);
      pt.btab = -1;
      tab_k.clear();
      tab_off.clear();
      twords = 0;
    }
  }
  pt.tab_built.assign(tab_k.size(), 0);
  pt.primes_seen = 0;
  std::vector<uint32_t> &kjac = pt.kjac_host;  // no table built yet
  kjac.assign(nk, kNoTable);
  const uint32_t bjac = kNoTable;
  const size_t o_kj = sec(nk * 4), o_ki = sec(nk * sizeof(KInfo)), o_tk = sec(tab_k.size() * 4);
  const size_t o_to = sec(tab_off.size() * 4);
  const size_t o_jb = sec(twords * 4);
  pt.job_bytes = o_jb;  // bytes uploaded (the character tables are built on the device)
  std::vector<uint8_t> host(o_jb, 0);
  memcpy(host.data() + o_rr, pl.row_r.data(), pl.row_r.size() * 4);
  memcpy(host.data() + o_rk, pl.row_kidx.data(), pl.row_kidx.size() * 4);
  memcpy(host.data() + o_rc, row_c.data(), row_c.size() * 4);
  memcpy(host.data() + o_kv, s.k.data(), nk * 4);
  memcpy(host.data() + o_ko, kodd.data(), nk * 4);
  memcpy(host.data() + o_ke, ke2.data(), nk * 4);
  memcpy(host.data() + o_kr, krcp.data(), nk * 8);
  memcpy(host.data() + o_k0, pl.k_row0.data(), (nk + 1) * 4);
  memcpy(host.data() + o_bm, pl.bitmap.data(), pl.bitmap.size() * 4);
  memcpy(host.data() + o_kj, kjac.data(), nk * 4);
  {
    std::vector<KInfo> &ki = pt.kinfo_host;
    ki.assign(nk, KInfo{});
    for (uint32_t i = 0; i < nk; i++) {
      ki[i].k_odd = kodd[i];
      ki[i].k_e2 = ke2[i];
      ki[i].k_jac = kjac[i];
      ki[i].k_val = s.k[i];
      ki[i].row0 = pl.k_row0[i];
      ki[i].k_rcp = krcp[i];
      uint32_t mask = 0;
      if (pl.Q <= 32)
        for (uint32_t row = pl.k_row0[i]; row < pl.k_row0[i + 1]; row++) mask |= 1u << pl.row_r[row];
      ki[i].rmask = mask;
    }
    memcpy(host.data() + o_ki, ki.data(), nk * sizeof(KInfo));
  }
  memcpy(host.data() + o_tk, tab_k.data(), tab_k.size() * 4);
  memcpy(host.data() + o_to, tab_off.data(), tab_off.size() * 4);
  CUDA_TRY(cudaMallocAsync(&pt.d_job, off, j->st));
  pt.dev_bytes = off;
  CUDA_TRY(cudaMemcpyAsync(pt.d_job, host.data(), o_jb, cudaMemcpyHostToDevice, j->st));
  uint8_t *b = (uint8_t *)pt.d_job;
  pt.d_tab_k = (const uint32_t *)(b + o_tk);
  pt.d_tab_off = (const uint32_t *)(b + o_to);
  pt.d_jac_bits = (uint32_t *)(b + o_jb);
  pt.d_kjac = (uint32_t *)(b + o_kj);
  pt.d_kinfo = (KInfo *)(b + o_ki);
  JobDev &d = pt.dev;
  d.base = s.base;
  d.sign = s.sign;
  d.Q = pl.Q;
  d.m = pl.m;
  d.cta_warps = pl.cta ? kCtaWarps : 1;
  {
    bool all_both = pl.Q == 2;
    for (size_t i = 0; all_both && i < s.k.size(); i++) all_both = pl.k_row0[i + 1] - pl.k_row0[i] == 2;
    d.pairable = all_both && d.cta_warps == 1 ? 1u : 0u;
  }
  d.chain_len = (pl.m + 64 * d.cta_warps - 1) / (64 * d.cta_warps);
  {
    uint64_t bq = 1;
    for (uint32_t q = 0; q < pl.Q && bq; q++) bq = (bq * s.base < (1ull << 32)) ? bq * s.base : 0;
    d.bq_small = (uint32_t)bq;
  }
  d.T = pl.T;
  d.tlanes = pl.tlanes;
  d.rows_per_it = pl.rows_per_it;
  d.steps_per_lane = pl.steps_per_lane;
  d.table_log2 = pl.bucket_log2;
  d.nbuckets = pl.nbuckets;
  d.exact_log2 = pl.table_log2;
  d.jbits = pl.jbits;
  d.nrows = pl.nrows;
  d.nk = nk;
  d.e0 = pl.e0;
  d.x_lo = pl.x_lo;
  d.x_hi = pl.x_hi;
  d.nmin = pl.nmin;
  d.nmax = pl.nmax;
  d.words_per_row = pl.words_per_row;
  d.datless = j->opt.datless ? 1u : 0u;
  d.max_act = std::max<uint32_t>(1, pl.nrows);
  d.int_rows = form != kRowsV ? 1u : 0u;
  d.row_ids_only = form == kRowsIntId ? 1u : 0u;  // no V in the record
  d.row_mask = form == kRowsMask ? 1u : 0u;       // neither V nor row ids: an active-row mask
  d.el_v = d.cta_warps > 1 ? kElWoff + 2 * d.cta_warps : kElV;
  if (d.row_mask) {
    d.el_row = d.el_v;
    d.el_tab = d.el_v + 2;
  } else {
    d.el_row = d.el_v + (d.row_ids_only ? 0u : ((d.max_act + 1) & ~1u));  // even: row ids are written 16 bytes at a time
    d.el_tab = d.el_row + 2 * ((d.max_act + 7) / 8);  // even, row ids in 16-byte groups
  }
  d.rec_elems = d.el_tab + 64;
  // the warp kernel's staged part of a record: header + V (header + row ids
  // without V, header + mask with row_mask) when it fits 2 KB; else the header alone
  const uint32_t staged = d.row_ids_only || d.row_mask ? d.el_tab : d.el_row;
  if (staged * 8 <= 2048) {
    d.stage_full = 1;
    d.stage_elems = staged;
  } else {
    d.stage_full = 0;
    d.stage_elems = d.el_v;
  }
  d.ctab_smem = 0;
  if (d.cta_warps > 1) {  // bytes per CTA: table, counts, V (or row ids), match list (, row table)
    d.warp_smem = (uint32_t)align_up(20u * d.nbuckets +
                                         (d.row_ids_only ? 16 * ((d.max_act + 7) / 8) : 8 * ((d.max_act + 1) & ~1u)) +
                                         kCtaMatchCap * 16 + 16,
                                     16);
    // row ids: the kernel reads k*b^r of each row from a shared-memory copy of
    // the job's row table when it fits beside the rest
    const uint32_t ctab_bytes = (uint32_t)align_up(4ull * d.nrows, 16);
    if (d.row_ids_only && d.warp_smem + ctab_bytes <= kCtaSmemMax) {
      d.ctab_smem = 1;
      d.warp_smem += ctab_bytes;
    }
  } else  // bytes per warp: table, counts, two record stages, (V of a row mask,) match list
    d.warp_smem = (uint32_t)align_up((20u << d.table_log2) + 16 * d.stage_elems + (d.row_mask ? 8 * kMaskRows : 0) +
                                         kMatchCap * 16 + 16,
                                     16);
  d.row_r = (const uint32_t *)(b + o_rr);
  d.row_kidx = (const uint32_t *)(b + o_rk);
  d.row_c = (const uint32_t *)(b + o_rc);
  d.k_val = (const uint32_t *)(b + o_kv);
  d.k_odd = (const uint32_t *)(b + o_ko);
  d.k_e2 = (const uint32_t *)(b + o_ke);
  d.k_rcp = (const uint64_t *)(b + o_kr);
  d.k_row0 = (const uint32_t *)(b + o_k0);
  d.bitmap = (const uint32_t *)(b + o_bm);
  d.jac_bits = (const uint32_t *)(b + o_jb);
  d.k_jac = (const uint32_t *)(b + o_kj);
  d.kinfo = (const KInfo *)(b + o_ki);
  d.b_jac = bjac;
  uint32_t bb = s.base, be = 0;
  while (!(bb & 1)) {
    bb >>= 1;
    be++;
  }
  d.b_odd = bb;
  d.b_e2 = be;
  d.b_rcp = bb > 1 ? (~0ull) / bb : 0;
  if (j->opt.char_tables == RS_TABLES_ALWAYS) {
    const int rc = build_char_tables(j, pt, 0.0, true);
    if (rc) return rc;
  }
  CUDA_TRY(cudaStreamSynchronize(j->st));
  return RS_OK;
}

// Odd primes <= limit by a simple sieve (the reference builds its small-prime
// table on the host too, kernel_v0.24.6.cu:1271-1303).  One set per device is
// kept for the life of the process and grown when a job needs a larger limit,
// so jobs after the first (a server's stream of jobs, a CLI resuming) reuse it.
static std::mutex g_primes_mu;
static std::shared_ptr<DevPrimes> g_primes[64];

static int ensure_sieving_primes(rs_job *j, uint64_t hi, uint64_t *h2d = nullptr) {
  uint64_t r = (uint64_t)std::sqrt((long double)hi);
  while (r * r > hi) r--;
  while ((r + 1) * (r + 1) <= hi) r++;
  if (j->primes && r <= j->primes->limit) return RS_OK;
  if (j->device < 0 || j->device >= 64) return fail(RS_ERR_INVALID, "device ordinal %d", j->device);
  std::lock_guard<std::mutex> lock(g_primes_mu);
  std::shared_ptr<DevPrimes> &slot = g_primes[j->device];
  if (!slot || slot->limit < r) {
    const uint64_t limit = std::max<uint64_t>(r, std::min<uint64_t>(2 * r, 1ull << 22));
    std::vector<uint8_t> comp(limit / 2 + 1, 0);
    std::vector<uint32_t> ps;
    std::vector<uint64_t> rc;
    for (uint64_t i = 3; i <= limit; i += 2) {
      if (comp[i / 2]) continue;
      ps.push_back((uint32_t)i);
      rc.push_back((~0ull) / i);
      for (uint64_t q = i * i; q <= limit; q += 2 * i) comp[q / 2] = 1;
    }
    auto dp = std::make_shared<DevPrimes>();
    dp->device = j->device;
    dp->limit = limit;
    CUDA_TRY(cudaMalloc(&dp->d_sp, std::max<size_t>(1, ps.size()) * 4));
    CUDA_TRY(cudaMalloc(&dp->d_rcp, std::max<size_t>(1, rc.size()) * 8));
    CUDA_TRY(cudaMemcpyAsync(dp->d_sp, ps.data(), ps.size() * 4, cudaMemcpyHostToDevice, j->st));
    CUDA_TRY(cudaMemcpyAsync(dp->d_rcp, rc.data(), rc.size() * 8, cudaMemcpyHostToDevice, j->st));
    CUDA_TRY(cudaStreamSynchronize(j->st));
    dp->n = (uint32_t)ps.size();
    dp->nsmall = (uint32_t)(std::lower_bound(ps.begin(), ps.end(), (uint32_t)(2 * kSieveOdds)) - ps.begin());
    if (h2d) *h2d += ps.size() * 12;
    slot = dp;
  }
  j->primes = slot;
  j->d_sp = slot->d_sp;
  j->d_sp_rcp = slot->d_rcp;
  j->nsp = slot->n;
  j->nsp_small = slot->nsmall;
  j->sp_limit = slot->limit;
  return RS_OK;
}

static int ensure_gbits(rs_job *j, uint64_t words) {
  if (j->d_gbits && j->gbits_words >= words) return RS_OK;
  if (j->d_gbits) cudaFreeAsync(j->d_gbits, j->st);
  j->d_gbits = nullptr;
  CUDA_TRY(cudaMallocAsync(&j->d_gbits, words * 4, j->st));
  j->gbits_words = words;
  return RS_OK;
}

static size_t chunk_bytes_per_prime(const rs_job *j) { return 8 + 4 + 8 * (size_t)j->max_rec_elems(); }

static uint64_t exact_scratch_bytes(const rs_job *j) {
  uint64_t b = 0;
  for (auto &pt : j->parts) b = std::max(b, bsgs_exact_scratch_bytes(pt->dev, pt->exact_grid));
  return b;
}

static int ensure_chunk_buffers(rs_job *j, uint32_t cap) {
  const uint32_t rec = j->max_rec_elems();
  const uint64_t xs = exact_scratch_bytes(j);
  if (j->d_chunk && j->chunk_cap >= cap && j->chunk_rec_elems >= rec && j->chunk_exact_bytes >= xs) return RS_OK;
  if (j->d_chunk) cudaFreeAsync(j->d_chunk, j->st);
  j->d_chunk = nullptr;
  size_t off = 0;
  auto sec = [&](size_t bytes) {
    size_t o = off;
    off = align_up(off + bytes, 256);
    return o;
  };
  const size_t o_pr = sec((size_t)cap * 8), o_ct = sec(16), o_rec = sec((size_t)cap * 8 * rec);
  const size_t o_rd = sec((size_t)cap * 4), o_rc = sec(16), o_xt = sec(xs);
  CUDA_TRY(cudaMallocAsync(&j->d_chunk, off, j->st));
  uint8_t *b = (uint8_t *)j->d_chunk;
  j->cb.primes = (uint64_t *)(b + o_pr);
  j->cb.count = (uint32_t *)(b + o_ct);
  j->cb.recs = (uint64_t *)(b + o_rec);
  j->cb.redo = (uint32_t *)(b + o_rd);
  j->cb.redo_count = (uint32_t *)(b + o_rc);
  j->cb.exact_tab = xs ? (uint32_t *)(b + o_xt) : nullptr;
  j->cb.cap = cap;
  j->chunk_cap = cap;
  j->chunk_rec_elems = rec;
  j->chunk_exact_bytes = xs;
  return RS_OK;
}

static int ensure_hit_buffers(rs_job *j, Part &pt, uint32_t cap) {
  if (pt.d_hits && pt.hb.cap >= cap) return RS_OK;
  if (pt.d_hits) cudaFreeAsync(pt.d_hits, j->st);
  pt.d_hits = nullptr;
  size_t off = 0;
  auto sec = [&](size_t bytes) {
    size_t o = off;
    off = align_up(off + bytes, 256);
    return o;
  };
  const size_t o_raw = sec((size_t)cap * sizeof(Hit)), o_rc = sec(16);
  const size_t o_fac = sec((size_t)cap * sizeof(Hit)), o_fc = sec(16);
  const size_t o_st = sec(kStatCount * sizeof(unsigned long long));
  CUDA_TRY(cudaMallocAsync(&pt.d_hits, off, j->st));
  uint8_t *b = (uint8_t *)pt.d_hits;
  pt.hb.raw = (Hit *)(b + o_raw);
  pt.hb.raw_count = (uint32_t *)(b + o_rc);
  pt.hb.fac = (Hit *)(b + o_fac);
  pt.hb.fac_count = (uint32_t *)(b + o_fc);
  pt.hb.stat = (unsigned long long *)(b + o_st);
  pt.hb.cap = cap;
  return RS_OK;
}

static void free_part_device(rs_job *j, Part &pt) {
  if (pt.d_job) cudaFreeAsync(pt.d_job, j->st);
  if (pt.d_hits) cudaFreeAsync(pt.d_hits, j->st);
  pt.d_job = nullptr;
  pt.d_hits = nullptr;
}

static void free_job(rs_job *j) {
  if (!j) return;
  if (j->st) cudaStreamSynchronize(j->st);
  if (j->st) {
    for (auto &pt : j->parts) free_part_device(j, *pt);
    if (j->d_chunk) cudaFreeAsync(j->d_chunk, j->st);
    if (j->d_gbits) cudaFreeAsync(j->d_gbits, j->st);
    cudaStreamSynchronize(j->st);
  }
  if (j->h_counts) pinned_put(j->h_counts, j->h_counts_cap * 4);
  if (j->st) cudaStreamDestroy(j->st);
  delete j;
}

// Primes per launch: -b/-t as in the reference (128*2^(b-1) blocks of
// 128*2^(t-1) threads, one prime each), else a memory budget of 3 GiB for the
// chunk buffers (larger launches measured 0.6% faster on the benchmark job
// than 2 GiB).
static void set_chunk_cap(rs_job *j) {
  const rs_options &opt = j->opt;
  uint64_t cap;
  if (opt.block_scale > 0 || opt.thread_scale > 0) {
    const int bs = opt.block_scale > 0 ? opt.block_scale : 1, ts = opt.thread_scale > 0 ? opt.thread_scale : 1;
    cap = (uint64_t)128 << (bs - 1);
    cap *= (uint64_t)128 << (ts - 1);
  } else {
    const uint64_t budget = opt.mem_limit ? opt.mem_limit : (3ull << 30);
    cap = budget / chunk_bytes_per_prime(j);
  }
  cap = std::max<uint64_t>(cap, 4096);
  cap = std::min<uint64_t>(cap, 1u << 23);
  j->cb.cap = (uint32_t)cap;
}

// Upload and configure one planned part.
static int make_part(rs_job *j, std::unique_ptr<Part> &pt) {
  int rc = upload_part(j, *pt);
  if (!rc) {  // an exact-path table larger than the shared memory of a CTA lives in global scratch
    int max_smem = 0;
    cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, j->device);
    pt->dev.exact_global = 0;
    pt->dev.exact_global = bsgs_exact_smem_bytes(pt->dev) > max_smem ? 1u : 0u;
  }
  if (!rc) {
    const cudaError_t e = bsgs_configure(pt->dev, j->device, &pt->bsgs_grid, &pt->exact_grid);
    if (e != cudaSuccess) rc = fail(RS_ERR_CUDA, "bsgs_configure: %s", cudaGetErrorString(e));
  }
  if (rc) free_part_device(j, *pt);
  return rc;
}

// A job from parsed sequences: one part per (base, sign).  `force` (a single
// part only) takes exactly that plan choice.
static int create_job(Seqs &&all, const rs_options *optp, rs_job **out, const PlanChoice *force = nullptr) {
  if (!out) return fail(RS_ERR_INVALID, "job pointer is NULL");
  *out = nullptr;
  rs_options opt;
  if (optp) opt = *optp;
  else rs_options_default(&opt);
  std::vector<Seqs> groups = split_parts(std::move(all));
  for (Seqs &g : groups) {
    normalise(g);
    if (g.sign != -1 && g.sign != 1) return fail(RS_ERR_INVALID, "sign must be -1 or +1");
    if (g.base < 2) return fail(RS_ERR_INVALID, "base must be >= 2");
  }
  if (groups.empty()) return fail(RS_ERR_INVALID, "job has no sequences");
  if (force && groups.size() != 1) return fail(RS_ERR_INTERNAL, "a forced plan needs a single-part job");
  if (opt.Q < 0 || opt.Q > 4096) return fail(RS_ERR_INVALID, "Q must be in [0, 4096]");
  if (opt.block_scale < 0 || opt.block_scale > 31 || opt.thread_scale < 0 || opt.thread_scale > 31)
    return fail(RS_ERR_INVALID, "-b/-t scale must be in [1, 31]");
  if (opt.baby_step < RS_BABY_AUTO || opt.baby_step > RS_BABY_HIGH)
    return fail(RS_ERR_INVALID, "baby_step must be one of RS_BABY_AUTO/SHOUP/SHORT/HIGH");
  // plan every part on the host first: a bad input fails before any device work
  std::vector<std::unique_ptr<Part>> parts;
  for (Seqs &g : groups) {
    auto pt = std::make_unique<Part>();
    const int rc = make_plan(g, opt, pt->plan, true, force, &pt->ranked);
    if (rc) return rc;
    pt->seqs = std::move(g);
    parts.push_back(std::move(pt));
  }
  int rc = check_device(opt.device);
  if (rc) return rc;
  rs_job *j = new rs_job();
  j->opt = opt;
  j->device = opt.device;
  cudaError_t e = cudaStreamCreateWithFlags(&j->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete j;
    return fail(RS_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
  }
  for (auto &pt : parts) {
    rc = make_part(j, pt);
    if (rc) {
      free_job(j);
      return rc;
    }
    j->parts.push_back(std::move(pt));
  }
  j->chunk_cap = 0;
  set_chunk_cap(j);
  *out = j;
  return RS_OK;
}

// ---------------------------------------------------------------------------
// Host re-verification, 128-bit arithmetic (kernel_v0.24.6.cu:1649-1671).

static bool host_verify(uint64_t p, uint32_t k, uint32_t b, uint32_t n, int32_t sign) {
  typedef unsigned __int128 u128;
  u128 val = 1;
  const uint64_t bb = b % p;
  for (int z = 31; z >= 0; --z) {
    val = (val * val) % p;
    if (n & (1u << z)) val = (val * bb) % p;
  }
  val = (val * (k % p)) % p;
  return (uint64_t)val == (sign < 0 ? 1 % p : p - 1);
}

// ---------------------------------------------------------------------------
// C ABI

extern "C" {

void rs_options_default(rs_options *opt) {
  if (!opt) return;
  memset(opt, 0, sizeof(*opt));
  opt->host_verify = 1;
}

const char *rs_last_error(void) { return g_err.c_str(); }

const char *rs_version(void) { return "rsieve-gb300 0.1.0 (sm_103a)"; }

int rs_job_create_abcd(const char *text, size_t len, const rs_options *opt, rs_job **job) {
  if (!text) return fail(RS_ERR_INVALID, "ABCD text is NULL");
  Seqs s;
  int rc = parse_abcd(text, len, s);
  if (rc) return rc;
  return create_job(std::move(s), opt, job);
}

int rs_job_create(uint32_t base, int32_t sign, uint32_t num_k, const uint32_t *k,
                  const uint32_t *n_offsets, const uint32_t *n_values, const rs_options *opt,
                  rs_job **job) {
  if (num_k == 0 || !k || !n_offsets || !n_values) return fail(RS_ERR_INVALID, "empty job");
  Seqs s;
  s.base = base;
  s.sign = sign;
  for (uint32_t i = 0; i < num_k; i++) {
    if (k[i] == 0) return fail(RS_ERR_INVALID, "k must be positive");
    if (n_offsets[i + 1] < n_offsets[i]) return fail(RS_ERR_INVALID, "n_offsets not ascending");
    s.k.push_back(k[i]);
    s.n.emplace_back(n_values + n_offsets[i], n_values + n_offsets[i + 1]);
    for (uint32_t v : s.n.back())
      if (v > 0x7fffffffu) return fail(RS_ERR_INVALID, "n exceeds 2^31-1");
  }
  return create_job(std::move(s), opt, job);
}

int rs_job_info_get(const rs_job *j, rs_job_info *info) {
  if (!j || !info) return fail(RS_ERR_INVALID, "NULL argument");
  const Part &p0 = *j->parts[0];
  const Plan &pl = p0.plan;
  memset(info, 0, sizeof(*info));
  info->base = p0.seqs.base;
  info->sign = p0.seqs.sign;
  for (auto &pt : j->parts) {
    info->num_k += (uint32_t)pt->seqs.k.size();
    info->num_candidates += pt->plan.ncand;
    info->upload_bytes += pt->job_bytes;
  }
  info->parts = (uint32_t)j->parts.size();
  info->nmin = pl.nmin;
  info->nmax = pl.nmax;
  info->Q = pl.Q;
  info->rows = pl.nrows;
  info->x_range = pl.X;
  info->baby_steps = pl.m;
  info->giant_steps = pl.T;
  info->table_slots = (uint32_t)kBucket * pl.nbuckets;
  info->primes_per_launch = j->cb.cap;
  info->work_per_prime = pl.work_per_prime;
  info->warps_per_prime = pl.cta ? kCtaWarps : 1;
  info->row_form = plan_row_form(pl, p0.seqs, nullptr);
  return RS_OK;
}

int rs_job_destroy(rs_job *j) {
  if (!j) return RS_OK;
  cudaSetDevice(j->device);
  free_job(j);
  return RS_OK;
}

}  // extern "C"

static constexpr int kRetryHits = -1;

// The baby-step product of a chunk [a, b] for one part (ChunkBufs::small_step).
// The short product by the integer b^Q needs p > 2^33 and b^Q * p < 2^63 for
// every p of the chunk; Shoup's product with a 32-bit constant needs
// b^Q * 2^32 < p and exists only in the CTA-per-prime kernel; Shoup's full
// product is always valid.  rs_options.baby_step may prefer a valid form over
// the cheapest.
static uint32_t chunk_step_form(const rs_job *j, const Part &pt, uint64_t a, uint64_t b) {
  const uint64_t bq = pt.dev.bq_small;
  const bool small_ok = bq != 0 && a > (1ull << 33) && (unsigned __int128)bq * b < ((unsigned __int128)1 << 63);
  const bool high_ok = bq != 0 && pt.dev.cta_warps > 1 && (bq << 32) < a;
  switch (j->opt.baby_step) {
    case RS_BABY_SHOUP: return kStepShoup;
    case RS_BABY_SHORT:
      if (small_ok) return kStepSmall;
      break;
    case RS_BABY_HIGH:
      if (high_ok) return kStepHigh;
      break;
    default: break;
  }
  return small_ok ? kStepSmall : high_ok ? kStepHigh : kStepShoup;
}

// Chunks [a, b] of [lo, hi] (lo odd) with an expected prime count of ~0.8*C each.
struct Chunk {
  uint64_t a, b;
};
static std::vector<Chunk> plan_chunks(uint64_t lo, uint64_t hi, uint32_t C) {
  std::vector<Chunk> todo;
  uint64_t a = lo;
  while (a <= hi) {
    const double la = std::log((double)a);
    double w = la > 3.0 ? 0.8 * (double)C * (la - 1.2) : 1.6 * (double)C;
    if (w < 64) w = 64;
    if (w > 64.0 * (double)C) w = 64.0 * (double)C;
    uint64_t width = (uint64_t)w & ~1ull;
    uint64_t b = (hi - a < width) ? hi : a + width - 1;  // a odd, width even -> b even or hi
    todo.push_back({a, b});
    if (b >= hi) break;
    a = b + 1;
    if (!(a & 1)) a++;
  }
  return todo;
}

// One pass over [p0, p1]; returns kRetryHits after growing a part's hit
// buffers when more candidate hits arrived than they could hold.
//
// Per chunk of primes, on the job's stream: the device sieve writes the
// chunk's primes, then every part runs its setup, BSGS and exact kernels on
// them (the chunk buffers are shared, so the parts follow one another).  After
// the last chunk each part verifies its candidate hits on the device.
static int sieve_range_impl(rs_job *j, uint64_t p0, uint64_t p1, rs_factor *out, size_t cap,
                            size_t *count, rs_stats *stats) {
  *count = 0;
  rs_stats st;
  memset(&st, 0, sizeof(st));
  if (p1 >= (1ull << 63)) return fail(RS_ERR_RANGE, "p1 must be < 2^63");
  uint64_t lo = p0 < 3 ? 3 : p0;
  if (!(lo & 1)) lo++;
  const uint64_t hi = p1;
  if (lo > hi) {
    if (stats) *stats = st;
    return RS_OK;
  }
  CUDA_TRY(cudaSetDevice(j->device));
  int rc = ensure_sieving_primes(j, hi, &st.h2d_bytes);
  if (rc) return rc;
  rc = ensure_chunk_buffers(j, j->cb.cap);
  if (rc) return rc;
  const size_t P = j->parts.size();
  for (auto &pt : j->parts) {
    if (!pt->d_hits) {
      rc = ensure_hit_buffers(j, *pt, P == 1 ? 1u << 20 : 1u << 16);
      if (rc) return rc;
    }
    rc = build_char_tables(j, *pt, primes_estimate(lo, hi), false);
    if (rc) return rc;
  }
  const uint32_t C = j->cb.cap;

  std::vector<Chunk> todo = plan_chunks(lo, hi, C);

  // timing events per chunk: before and after the sieve, then before setup,
  // before BSGS, before the exact kernel and after it, for every part
  const size_t EV = 2 + 4 * P;
  cudaEvent_t ev0, ev1;
  CUDA_TRY(cudaEventCreate(&ev0));
  CUDA_TRY(cudaEventCreate(&ev1));
  std::vector<cudaEvent_t> evs;
  auto cleanup_events = [&]() {
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    for (auto e : evs) cudaEventDestroy(e);
  };
  bool first_pass = true;
  uint64_t total_primes = 0;
  for (int attempt = 0; attempt < 8 && !todo.empty(); attempt++) {
    if (j->h_counts_cap < todo.size() + 2) {
      if (j->h_counts) pinned_put(j->h_counts, j->h_counts_cap * 4);
      j->h_counts = nullptr;
      j->h_counts_cap = todo.size() + 2;
      j->h_counts = (uint32_t *)pinned_get(j->h_counts_cap * 4);
      if (!j->h_counts) {
        cleanup_events();
        return fail(RS_ERR_NOMEM, "cudaMallocHost failed");
      }
    }
    while (evs.size() < todo.size() * EV) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) break;
      evs.push_back(e);
    }
    const bool timed = evs.size() >= todo.size() * EV;
    if (first_pass) {
      for (auto &pt : j->parts) {
        cudaMemsetAsync(pt->hb.raw_count, 0, 4, j->st);
        cudaMemsetAsync(pt->hb.fac_count, 0, 4, j->st);
        cudaMemsetAsync(pt->hb.stat, 0, kStatCount * sizeof(unsigned long long), j->st);
      }
      cudaEventRecord(ev0, j->st);
    }
    std::vector<uint32_t> forms(todo.size() * P);
    for (size_t c = 0; c < todo.size(); c++) {
      cudaEvent_t *ce = timed ? &evs[EV * c] : nullptr;
      cudaMemsetAsync(j->cb.count, 0, 4, j->st);
      if (ce) cudaEventRecord(ce[0], j->st);
      cudaError_t e = cudaSuccess;
      {
        const int grc = ensure_gbits(j, sieve_bitmap_words(todo[c].a, todo[c].b));
        if (grc) {
          cleanup_events();
          return grc;
        }
      }
      e = launch_sieve(todo[c].a, todo[c].b, j->d_sp, j->d_sp_rcp, j->nsp, j->nsp_small, j->d_gbits,
                       j->cb.primes, j->cb.count, C, j->st);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(&j->h_counts[c], j->cb.count, 4, cudaMemcpyDeviceToHost, j->st);
      if (ce) cudaEventRecord(ce[1], j->st);
      st.launches += j->nsp > j->nsp_small ? 2 : 1;
      for (size_t q = 0; q < P && e == cudaSuccess; q++) {
        Part &pt = *j->parts[q];
        const uint32_t form = chunk_step_form(j, pt, todo[c].a, todo[c].b);
        forms[c * P + q] = form;
        j->cb.small_step = form;
        if (ce) cudaEventRecord(ce[2 + 4 * q], j->st);
        e = launch_setup(pt.dev, j->cb, j->st);
        if (e == cudaSuccess) e = cudaMemsetAsync(j->cb.redo_count, 0, 4, j->st);
        if (ce) cudaEventRecord(ce[3 + 4 * q], j->st);
        if (e == cudaSuccess) e = launch_bsgs(pt.dev, j->cb, pt.hb, pt.bsgs_grid, j->st);
        if (ce) cudaEventRecord(ce[4 + 4 * q], j->st);
        if (e == cudaSuccess) e = launch_bsgs_exact(pt.dev, j->cb, pt.hb, pt.exact_grid, j->st);
        if (ce) cudaEventRecord(ce[5 + 4 * q], j->st);
        st.launches += 3;
        st.bsgs_launches += 1;
      }
      if (e != cudaSuccess) {
        cleanup_events();
        return fail(RS_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e));
      }
    }
    cudaError_t e = cudaStreamSynchronize(j->st);
    if (e != cudaSuccess) {
      cleanup_events();
      return fail(RS_ERR_CUDA, "sieve kernels: %s", cudaGetErrorString(e));
    }
    st.d2h_bytes += 4 * todo.size();
    if (timed) {
      for (size_t c = 0; c < todo.size(); c++) {
        const cudaEvent_t *ce = &evs[EV * c];
        float ms = 0;
        cudaEventElapsedTime(&ms, ce[0], ce[1]);
        st.sieve_ms += ms;
        for (size_t q = 0; q < P; q++) {
          cudaEventElapsedTime(&ms, ce[2 + 4 * q], ce[3 + 4 * q]);
          st.setup_ms += ms;
          cudaEventElapsedTime(&ms, ce[3 + 4 * q], ce[4 + 4 * q]);
          st.bsgs_ms += ms;
          cudaEventElapsedTime(&ms, ce[4 + 4 * q], ce[5 + 4 * q]);
          st.exact_ms += ms;
        }
      }
    }
    std::vector<Chunk> redo;
    for (size_t c = 0; c < todo.size(); c++) {
      const uint32_t n = j->h_counts[c];
      if (n > C) {
        // more primes than the buffer holds: split the chunk and run it again
        if (todo[c].b - todo[c].a < 8) {
          cleanup_events();
          return fail(RS_ERR_INTERNAL, "prime buffer overflow on a tiny chunk");
        }
        const uint64_t mid = (todo[c].a + (todo[c].b - todo[c].a) / 2) | 1ull;  // odd, > a
        redo.push_back({todo[c].a, mid - 1});
        redo.push_back({mid, todo[c].b});
      } else {
        total_primes += n;
        for (size_t q = 0; q < P; q++) {
          const uint32_t f = forms[c * P + q];
          st.primes_by_step[f == kStepShoup ? 0 : f == kStepSmall ? 1 : 2] += n;
        }
      }
    }
    todo.swap(redo);
    first_pass = false;
  }
  if (!todo.empty()) {
    cleanup_events();
    return fail(RS_ERR_INTERNAL, "prime buffer overflow could not be resolved");
  }
  // verify every part's candidates on the device, then read the counts
  cudaError_t e = cudaSuccess;
  for (auto &pt : j->parts) {
    if (e == cudaSuccess) e = launch_verify(pt->dev, pt->hb, j->st);
    st.launches += 1;
  }
  cudaEventRecord(ev1, j->st);
  std::vector<uint32_t> counts(2 * P, 0);
  std::vector<unsigned long long> dstat(kStatCount * P, 0);
  for (size_t q = 0; q < P; q++) {
    const Part &pt = *j->parts[q];
    if (e == cudaSuccess) e = cudaMemcpyAsync(&counts[2 * q], pt.hb.raw_count, 4, cudaMemcpyDeviceToHost, j->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&counts[2 * q + 1], pt.hb.fac_count, 4, cudaMemcpyDeviceToHost, j->st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&dstat[kStatCount * q], pt.hb.stat, kStatCount * sizeof(unsigned long long),
                          cudaMemcpyDeviceToHost, j->st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(j->st);
  if (e != cudaSuccess) {
    cleanup_events();
    return fail(RS_ERR_CUDA, "verify: %s", cudaGetErrorString(e));
  }
  st.d2h_bytes += P * (8 + kStatCount * sizeof(unsigned long long));
  {
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0, ev1);
    st.gpu_ms = ms;
  }
  cleanup_events();
  bool regrow = false;
  for (size_t q = 0; q < P; q++) {
    Part &pt = *j->parts[q];
    if (counts[2 * q] > pt.hb.cap) {
      const uint64_t need = std::min<uint64_t>((uint64_t)counts[2 * q] * 2, 1u << 30);
      rc = ensure_hit_buffers(j, pt, (uint32_t)need);
      if (rc) return rc;
      regrow = true;
    }
  }
  if (regrow) return kRetryHits;
  struct Fac {
    uint64_t p;
    uint32_t k, n, b;
    int32_t c;
  };
  std::vector<Fac> fac;
  uint64_t raw = 0;
  for (size_t q = 0; q < P; q++) {
    const Part &pt = *j->parts[q];
    raw += counts[2 * q];
    st.paired_primes += dstat[kStatCount * q + kStatPaired];
    st.exact_primes += dstat[kStatCount * q + kStatExact];
    const uint32_t nf = counts[2 * q + 1];
    if (!nf) continue;
    std::vector<Hit> h(nf);
    CUDA_TRY(cudaMemcpy(h.data(), pt.hb.fac, nf * sizeof(Hit), cudaMemcpyDeviceToHost));
    st.d2h_bytes += nf * sizeof(Hit);
    for (const Hit &x : h) fac.push_back(Fac{x.p, x.k, x.n, pt.seqs.base, pt.seqs.sign});
  }
  std::sort(fac.begin(), fac.end(), [](const Fac &a, const Fac &b) {
    return std::tie(a.p, a.k, a.n, a.b, a.c) < std::tie(b.p, b.k, b.n, b.b, b.c);
  });
  fac.erase(std::unique(fac.begin(), fac.end(),
                        [](const Fac &a, const Fac &b) {
                          return a.p == b.p && a.k == b.k && a.n == b.n && a.b == b.b && a.c == b.c;
                        }),
            fac.end());
  if (j->opt.host_verify) {
    for (const Fac &h : fac)
      if (!host_verify(h.p, h.k, h.b, h.n, h.c))
        return fail(RS_ERR_INTERNAL, "factor %llu | %u*%u^%u%+d failed host verification",
                    (unsigned long long)h.p, h.k, h.b, h.n, h.c);
  }
  st.primes = total_primes;
  st.raw_hits = raw;
  st.factors = fac.size();
  st.p_covered = hi - lo + 1;
  if (stats) *stats = st;
  *count = fac.size();
  if (fac.size() > cap) return fail(RS_ERR_CAPACITY, "%zu factors found, buffer holds %zu", fac.size(), cap);
  for (size_t i = 0; i < fac.size(); i++) {
    out[i].p = fac[i].p;
    out[i].k = fac[i].k;
    out[i].n = fac[i].n;
    out[i].b = fac[i].b;
    out[i].c = fac[i].c;
  }
  return RS_OK;
}

extern "C" int rs_sieve_range(rs_job *j, uint64_t p0, uint64_t p1, rs_factor *out, size_t cap,
                              size_t *count, rs_stats *stats) {
  if (!j || !count) return fail(RS_ERR_INVALID, "NULL argument");
  if (!out && cap) return fail(RS_ERR_INVALID, "NULL output with nonzero capacity");
  std::lock_guard<std::mutex> lock(j->mu);
  for (int attempt = 0; attempt < 4; attempt++) {
    const int rc = sieve_range_impl(j, p0, p1, out, cap, count, stats);
    if (rc != kRetryHits) return rc;
  }
  return fail(RS_ERR_INTERNAL, "candidate-hit buffer overflow could not be resolved");
}

// Measured autotuning, part by part: each of the part's cheapest distinct
// layouts (its own plan first) is built as a single-part job, timed on [p0, p1]
// by device events, and the fastest part replaces the job's.
extern "C" int rs_job_autotune(rs_job *j, uint64_t p0, uint64_t p1, uint32_t candidates, rs_job_info *chosen) {
  if (!j) return fail(RS_ERR_INVALID, "NULL job");
  if (candidates == 0) candidates = 3;
  std::lock_guard<std::mutex> lock(j->mu);
  std::vector<rs_factor> out(1 << 16);
  for (size_t q = 0; q < j->parts.size(); q++) {
    Part &cur = *j->parts[q];
    std::vector<PlanChoice> cand;
    for (const PlanChoice &c : cur.ranked) {
      bool dup = false;
      for (const PlanChoice &d : cand) dup |= d.Q == c.Q && d.T == c.T && d.m == c.m && d.cta == c.cta && d.nb == c.nb;
      if (!dup) cand.push_back(c);
      if (cand.size() >= candidates) break;
    }
    if (cand.size() < 2) continue;
    double best_ms = 0;
    rs_job *best = nullptr;
    for (size_t c = 0; c < cand.size(); c++) {
      rs_job *t = nullptr;
      Seqs copy = cur.seqs;
      int rc = create_job(std::move(copy), &j->opt, &t, &cand[c]);
      if (rc) {
        if (best) free_job(best);
        return rc;
      }
      rs_stats st{};
      size_t cnt = 0;
      for (int attempt = 0; attempt < 4; attempt++) {
        rc = sieve_range_impl(t, p0, p1, out.data(), out.size(), &cnt, &st);
        if (rc != kRetryHits) break;
      }
      if (rc == RS_ERR_CAPACITY) rc = RS_OK;  // the timing is what counts here
      if (rc) {
        free_job(t);
        if (best) free_job(best);
        return rc;
      }
      if (!best || st.gpu_ms < best_ms) {
        if (best) free_job(best);
        best = t;
        best_ms = st.gpu_ms;
      } else {
        free_job(t);
      }
    }
    // the winner's part (planned, uploaded and configured on this device)
    // moves into the job; its device memory was allocated on the temporary
    // job's stream, which is synchronised before it is destroyed
    cudaStreamSynchronize(best->st);
    std::swap(j->parts[q], best->parts[0]);
    free_job(best);  // frees the part that was replaced
  }
  if (j->d_chunk && j->chunk_rec_elems < j->max_rec_elems()) {
    cudaFreeAsync(j->d_chunk, j->st);
    j->d_chunk = nullptr;
    j->chunk_cap = 0;
  }
  set_chunk_cap(j);
  if (chosen) return rs_job_info_get(j, chosen);
  return RS_OK;
}

// ---------------------------------------------------------------------------
// Batched form: many jobs' ranges in rounds, one persistent BSGS launch per
// kernel variant per round, each round recorded as a CUDA graph.

// Branches of a round's graph: the jobs' sieve and setup launches, then the
// kernel variants' BSGS launches, are spread over this many captured streams so
// that the graph runs them side by side.
constexpr int kBatchBranches = 8;

struct rs_batch {
  int device = 0;
  cudaStream_t st = nullptr;               // the captured origin stream
  cudaStream_t side[kBatchBranches] = {};  // branch streams (forked from st in each capture)
  cudaEvent_t fork[2] = {}, join[2][kBatchBranches] = {};
  struct Item {
    rs_job *job = nullptr;
    uint64_t p0 = 0, p1 = 0;
    std::vector<rs_factor> out;
    rs_stats st{};
    int status = RS_OK;
    std::string err;
  };
  std::vector<Item> items;
  bool ran = false;
};

extern "C" int rs_batch_create(int device, rs_batch **out) {
  if (!out) return fail(RS_ERR_INVALID, "rs_batch_create: NULL argument");
  *out = nullptr;
  int rc = check_device(device);
  if (rc) return rc;
  rs_batch *b = new rs_batch();
  b->device = device;
  cudaError_t e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
  for (int s = 0; s < kBatchBranches && e == cudaSuccess; s++) e = cudaStreamCreateWithFlags(&b->side[s], cudaStreamNonBlocking);
  for (int h = 0; h < 2 && e == cudaSuccess; h++) {
    e = cudaEventCreateWithFlags(&b->fork[h], cudaEventDisableTiming);
    for (int s = 0; s < kBatchBranches && e == cudaSuccess; s++)
      e = cudaEventCreateWithFlags(&b->join[h][s], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    rs_batch_destroy(b);
    return fail(RS_ERR_CUDA, "rs_batch_create: %s", cudaGetErrorString(e));
  }
  *out = b;
  return RS_OK;
}

extern "C" int rs_batch_add(rs_batch *b, rs_job *job, uint64_t p0, uint64_t p1, uint32_t *item) {
  if (!b || !job) return fail(RS_ERR_INVALID, "rs_batch_add: NULL argument");
  if (job->device != b->device) return fail(RS_ERR_INVALID, "rs_batch_add: job on device %d, batch on %d", job->device,
                                            b->device);
  for (auto &it : b->items)
    if (it.job == job) return fail(RS_ERR_INVALID, "rs_batch_add: the job is already in this batch");
  if (b->items.size() >= 4096) return fail(RS_ERR_INVALID, "rs_batch_add: at most 4096 items");
  if (p1 >= (1ull << 63)) return fail(RS_ERR_RANGE, "p1 must be < 2^63");
  rs_batch::Item it;
  it.job = job;
  it.p0 = p0;
  it.p1 = p1;
  b->items.push_back(std::move(it));
  b->ran = false;
  if (item) *item = (uint32_t)(b->items.size() - 1);
  return RS_OK;
}

// Kernel variant of a warp-per-prime part: items of one multi-job launch share it.
static uint32_t batch_variant(const JobDev &d) {
  const uint32_t rm = d.row_mask ? kRowsMask : d.row_ids_only ? kRowsIntId : d.int_rows ? kRowsIntV : kRowsV;
  return d.tlanes * 8 + rm;
}

extern "C" int rs_batch_run(rs_batch *B, rs_stats *stats) {
  if (!B) return fail(RS_ERR_INVALID, "rs_batch_run: NULL batch");
  CUDA_TRY(cudaSetDevice(B->device));
  rs_stats tot{};
  // jobs locked for the whole run, in address order (a job is in one item only)
  std::vector<rs_job *> order;
  for (auto &it : B->items) order.push_back(it.job);
  std::sort(order.begin(), order.end());
  std::vector<std::unique_lock<std::mutex>> locks;
  for (rs_job *j : order) locks.emplace_back(j->mu);

  struct Run {  // a batched item: its chunks and their outcome
    size_t item;
    rs_job *j;
    Part *pt;
    uint64_t lo, hi;
    std::vector<Chunk> chunks;
    std::vector<uint32_t> forms;
    size_t count0 = 0;  // first slot of its chunks in the pinned count array
    bool own = false;   // BSGS through the job's own launch (CTA layout, or no batch kernel fits)
  };
  std::vector<Run> runs;
  std::vector<size_t> alone;  // items sieved through their own path (several parts)
  for (size_t q = 0; q < B->items.size(); q++) {
    auto &it = B->items[q];
    it.out.clear();
    it.st = rs_stats{};
    it.status = RS_OK;
    it.err.clear();
    if (it.job->parts.size() != 1) {
      alone.push_back(q);
      continue;
    }
    uint64_t lo = it.p0 < 3 ? 3 : it.p0;
    if (!(lo & 1)) lo++;
    if (lo > it.p1) continue;
    Run r;
    r.item = q;
    r.j = it.job;
    r.pt = it.job->parts[0].get();
    r.lo = lo;
    r.hi = it.p1;
    runs.push_back(std::move(r));
  }
  // device resources of every batched job, allocated before any recording
  size_t nslots = 0;
  for (Run &r : runs) {
    rs_job *j = r.j;
    int rc = ensure_sieving_primes(j, r.hi, &tot.h2d_bytes);
    if (!rc) rc = ensure_chunk_buffers(j, j->cb.cap);
    if (!rc && !r.pt->d_hits) rc = ensure_hit_buffers(j, *r.pt, 1u << 20);
    if (!rc) rc = build_char_tables(j, *r.pt, primes_estimate(r.lo, r.hi), false);
    if (rc) return rc;
    r.chunks = plan_chunks(r.lo, r.hi, j->cb.cap);
    uint64_t words = 0;
    r.forms.resize(r.chunks.size());
    for (size_t c = 0; c < r.chunks.size(); c++) {
      words = std::max(words, sieve_bitmap_words(r.chunks[c].a, r.chunks[c].b));
      r.forms[c] = chunk_step_form(j, *r.pt, r.chunks[c].a, r.chunks[c].b);
    }
    rc = ensure_gbits(j, words);
    if (rc) return rc;
    CUDA_TRY(cudaStreamSynchronize(j->st));
    r.count0 = nslots;
    nslots += r.chunks.size();
  }
  size_t rounds = 0;
  for (Run &r : runs) rounds = std::max(rounds, r.chunks.size());
  // groups of warp-per-prime runs sharing a kernel variant and a table size (the
  // per-warp shared memory of a launch is sized for its largest table), at most
  // kBatchMaxItems runs each, and their launch shape; a group whose shape fits
  // no launch runs its jobs' own launches, as CTA-layout jobs do
  struct Group {
    uint32_t variant, table_log2;
    std::vector<size_t> runs;
    uint32_t stage_max = 0, warp_bytes = 0;
    int grid = 0;
  };
  std::vector<Group> groups;
  for (size_t r = 0; r < runs.size(); r++) {
    const JobDev &d = runs[r].pt->dev;
    if (d.cta_warps > 1) {
      runs[r].own = true;
      continue;
    }
    const uint32_t v = batch_variant(d);
    size_t g = 0;
    for (; g < groups.size() && (groups[g].variant != v || groups[g].table_log2 != d.table_log2 ||
                                 groups[g].runs.size() >= kBatchMaxItems);
         g++) {
    }
    if (g == groups.size()) groups.push_back(Group{v, d.table_log2, {}});
    groups[g].runs.push_back(r);
    groups[g].stage_max = std::max(groups[g].stage_max, d.stage_elems);
  }
  for (size_t g = 0; g < groups.size();) {
    Group &G = groups[g];
    G.warp_bytes = batch_warp_bytes(G.stage_max, G.table_log2, runs[G.runs[0]].pt->dev.row_mask != 0);
    if (batch_configure(runs[G.runs[0]].pt->dev, G.warp_bytes, B->device, &G.grid) == cudaSuccess) {
      g++;
      continue;
    }
    cudaGetLastError();
    for (size_t r : G.runs) runs[r].own = true;
    groups.erase(groups.begin() + (std::ptrdiff_t)g);
  }
  // the launch items of every (round, group), written once and copied to the device once
  std::vector<std::vector<size_t>> goff(rounds, std::vector<size_t>(groups.size(), 0));
  std::vector<std::vector<uint32_t>> gn(rounds, std::vector<uint32_t>(groups.size(), 0));
  std::vector<BatchItem> hitems;
  for (size_t rd = 0; rd < rounds; rd++)
    for (size_t g = 0; g < groups.size(); g++) {
      goff[rd][g] = hitems.size();
      for (size_t r : groups[g].runs) {
        Run &R = runs[r];
        if (rd >= R.chunks.size()) continue;
        BatchItem x;
        x.J = R.pt->dev;
        x.cb = R.j->cb;
        x.cb.small_step = R.forms[rd];
        x.hb = R.pt->hb;
        hitems.push_back(x);
        gn[rd][g]++;
      }
      if (gn[rd][g] > kBatchMaxItems) return fail(RS_ERR_INVALID, "rs_batch_run: more than %u jobs of one kernel variant",
                                                  kBatchMaxItems);
    }
  BatchItem *d_items = nullptr;
  uint32_t *h_counts = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaGraphExec_t exec = nullptr;
  auto cleanup = [&]() {
    if (exec) cudaGraphExecDestroy(exec);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (d_items) cudaFreeAsync(d_items, B->st);
    if (h_counts) pinned_put(h_counts, (nslots + 1) * 4);
    cudaStreamSynchronize(B->st);
  };
  h_counts = (uint32_t *)pinned_get((nslots + 1) * 4);
  if (!h_counts) return fail(RS_ERR_NOMEM, "cudaMallocHost failed");
  if (!hitems.empty()) {
    if (cudaMallocAsync(&d_items, hitems.size() * sizeof(BatchItem), B->st) != cudaSuccess ||
        cudaMemcpyAsync(d_items, hitems.data(), hitems.size() * sizeof(BatchItem), cudaMemcpyHostToDevice, B->st) !=
            cudaSuccess) {
      cleanup();
      return fail(RS_ERR_CUDA, "rs_batch_run: batch item upload failed");
    }
    tot.h2d_bytes += hitems.size() * sizeof(BatchItem);
  }
  cudaEventCreate(&ev0);
  cudaEventCreate(&ev1);
  for (Run &R : runs) {
    cudaMemsetAsync(R.pt->hb.raw_count, 0, 4, B->st);
    cudaMemsetAsync(R.pt->hb.fac_count, 0, 4, B->st);
    cudaMemsetAsync(R.pt->hb.stat, 0, kStatCount * sizeof(unsigned long long), B->st);
  }
  cudaEventRecord(ev0, B->st);
  // the rounds, each recorded as one graph of two forked phases: every job's
  // sieve and setup (jobs spread over the branch streams), then every kernel
  // variant's persistent BSGS launch followed by its jobs' exact-path launches,
  // and every CTA-layout job's own BSGS and exact launches (again spread over
  // the branches).  Each job's launches stay in order on one branch; the
  // branches run side by side.
  auto fork = [&](int h) {
    cudaEventRecord(B->fork[h], B->st);
    for (int s = 0; s < kBatchBranches; s++) cudaStreamWaitEvent(B->side[s], B->fork[h], 0);
  };
  auto join = [&](int h) {
    for (int s = 0; s < kBatchBranches; s++) {
      cudaEventRecord(B->join[h][s], B->side[s]);
      cudaStreamWaitEvent(B->st, B->join[h][s], 0);
    }
  };
  cudaError_t e = cudaSuccess;
  for (size_t rd = 0; rd < rounds && e == cudaSuccess; rd++) {
    e = cudaStreamBeginCapture(B->st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) break;
    fork(0);
    size_t br = 0;
    for (Run &R : runs) {
      if (rd >= R.chunks.size()) continue;
      const cudaStream_t s = B->side[br++ % kBatchBranches];
      rs_job *j = R.j;
      const Chunk &c = R.chunks[rd];
      cudaMemsetAsync(j->cb.count, 0, 4, s);
      launch_sieve(c.a, c.b, j->d_sp, j->d_sp_rcp, j->nsp, j->nsp_small, j->d_gbits, j->cb.primes, j->cb.count,
                   j->cb.cap, s);
      cudaMemcpyAsync(&h_counts[R.count0 + rd], j->cb.count, 4, cudaMemcpyDeviceToHost, s);
      ChunkBufs cb = j->cb;
      cb.small_step = R.forms[rd];
      launch_setup(R.pt->dev, cb, s);
      cudaMemsetAsync(j->cb.redo_count, 0, 4, s);
      tot.launches += (j->nsp > j->nsp_small ? 2 : 1) + 1;
    }
    join(0);
    fork(1);
    br = 0;
    for (size_t g = 0; g < groups.size(); g++) {
      if (!gn[rd][g]) continue;
      const cudaStream_t s = B->side[br++ % kBatchBranches];
      launch_bsgs_batch(runs[groups[g].runs[0]].pt->dev, d_items + goff[rd][g], gn[rd][g], groups[g].stage_max,
                        groups[g].warp_bytes, groups[g].grid, s);
      tot.launches++;
      tot.bsgs_launches++;
      for (size_t r : groups[g].runs) {
        Run &R = runs[r];
        if (rd >= R.chunks.size()) continue;
        ChunkBufs cb = R.j->cb;
        cb.small_step = R.forms[rd];
        launch_bsgs_exact(R.pt->dev, cb, R.pt->hb, R.pt->exact_grid, s);
        tot.launches++;
      }
    }
    for (Run &R : runs) {
      if (rd >= R.chunks.size() || !R.own) continue;
      const cudaStream_t s = B->side[br++ % kBatchBranches];
      ChunkBufs cb = R.j->cb;
      cb.small_step = R.forms[rd];
      launch_bsgs(R.pt->dev, cb, R.pt->hb, R.pt->bsgs_grid, s);
      launch_bsgs_exact(R.pt->dev, cb, R.pt->hb, R.pt->exact_grid, s);
      tot.launches += 2;
      tot.bsgs_launches++;
    }
    join(1);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(B->st, &graph);
    if (e != cudaSuccess) break;
    if (exec) {
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(exec, graph, &info) != cudaSuccess) {
        cudaGetLastError();
        cudaGraphExecDestroy(exec);
        exec = nullptr;
      }
    }
    if (!exec) e = cudaGraphInstantiate(&exec, graph, 0);
    if (e == cudaSuccess) e = cudaGraphLaunch(exec, B->st);
    cudaGraphDestroy(graph);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(B->st);
  if (e != cudaSuccess) {
    cleanup();
    return fail(RS_ERR_CUDA, "rs_batch_run rounds: %s", cudaGetErrorString(e));
  }
  // verification, then every batched item's factors
  for (Run &R : runs) {
    e = launch_verify(R.pt->dev, R.pt->hb, B->st);
    tot.launches++;
    if (e != cudaSuccess) break;
  }
  cudaEventRecord(ev1, B->st);
  std::vector<uint32_t> counts(2 * runs.size());
  std::vector<unsigned long long> dstat(kStatCount * runs.size());
  for (size_t r = 0; r < runs.size() && e == cudaSuccess; r++) {
    const HitBufs &hb = runs[r].pt->hb;
    e = cudaMemcpyAsync(&counts[2 * r], hb.raw_count, 4, cudaMemcpyDeviceToHost, B->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&counts[2 * r + 1], hb.fac_count, 4, cudaMemcpyDeviceToHost, B->st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&dstat[kStatCount * r], hb.stat, kStatCount * sizeof(unsigned long long),
                          cudaMemcpyDeviceToHost, B->st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(B->st);
  if (e != cudaSuccess) {
    cleanup();
    return fail(RS_ERR_CUDA, "rs_batch_run verify: %s", cudaGetErrorString(e));
  }
  {
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0, ev1);
    tot.gpu_ms = ms;
  }
  for (size_t r = 0; r < runs.size(); r++) {
    Run &R = runs[r];
    auto &it = B->items[R.item];
    rs_job *j = R.j;
    rs_stats &st = it.st;
    // chunks with more primes than the buffer held are sieved again through the
    // job's own path; so is the whole item when its hit buffer overflowed
    std::vector<Chunk> again;
    for (size_t c = 0; c < R.chunks.size(); c++) {
      const uint32_t n = h_counts[R.count0 + c];
      if (n > j->cb.cap) {
        again.push_back(R.chunks[c]);
      } else {
        st.primes += n;
        const uint32_t f = R.forms[c];
        st.primes_by_step[f == kStepShoup ? 0 : f == kStepSmall ? 1 : 2] += n;
      }
    }
    if (counts[2 * r] > R.pt->hb.cap) {
      again.assign(1, Chunk{R.lo, R.hi});
      st = rs_stats{};
    } else {
      st.raw_hits = counts[2 * r];
      st.paired_primes = dstat[kStatCount * r + kStatPaired];
      st.exact_primes = dstat[kStatCount * r + kStatExact];
      const uint32_t nf = counts[2 * r + 1];
      std::vector<Hit> h(nf);
      if (nf) {
        e = cudaMemcpy(h.data(), R.pt->hb.fac, nf * sizeof(Hit), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
          cleanup();
          return fail(RS_ERR_CUDA, "rs_batch_run factors: %s", cudaGetErrorString(e));
        }
        tot.d2h_bytes += nf * sizeof(Hit);
      }
      const uint32_t base = R.pt->seqs.base;
      const int32_t sign = R.pt->seqs.sign;
      for (const Hit &x : h) it.out.push_back(rs_factor{x.p, x.k, x.n, base, sign});
    }
    for (const Chunk &c : again) {  // rare: through the job's own path
      std::vector<rs_factor> more(1 << 12);
      size_t cnt = 0;
      rs_stats s2{};
      int rc = kRetryHits;
      for (int attempt = 0; attempt < 4 && (rc == kRetryHits || rc == RS_ERR_CAPACITY); attempt++) {
        rc = sieve_range_impl(j, c.a, c.b, more.data(), more.size(), &cnt, &s2);
        if (rc == RS_ERR_CAPACITY) more.resize(cnt);
      }
      if (rc) {
        it.status = rc;
        it.err = rs_last_error();
        break;
      }
      it.out.insert(it.out.end(), more.begin(), more.begin() + cnt);
      st.primes += s2.primes;
      st.raw_hits += s2.raw_hits;
      for (int f = 0; f < 3; f++) st.primes_by_step[f] += s2.primes_by_step[f];
      st.paired_primes += s2.paired_primes;
      st.exact_primes += s2.exact_primes;
      tot.launches += s2.launches;
    }
    std::sort(it.out.begin(), it.out.end(), [](const rs_factor &a, const rs_factor &b) {
      return std::tie(a.p, a.k, a.n, a.b, a.c) < std::tie(b.p, b.k, b.n, b.b, b.c);
    });
    it.out.erase(std::unique(it.out.begin(), it.out.end(),
                             [](const rs_factor &a, const rs_factor &b) {
                               return a.p == b.p && a.k == b.k && a.n == b.n && a.b == b.b && a.c == b.c;
                             }),
                 it.out.end());
    if (it.status == RS_OK && j->opt.host_verify)
      for (const rs_factor &f : it.out)
        if (!host_verify(f.p, f.k, f.b, f.n, f.c)) {
          it.status = RS_ERR_INTERNAL;
          it.err = "a factor failed host verification";
          break;
        }
    st.factors = it.out.size();
    st.p_covered = R.hi - R.lo + 1;
  }
  cleanup();
  // jobs of several parts: their own path
  for (size_t q : alone) {
    auto &it = B->items[q];
    std::vector<rs_factor> out(1 << 12);
    size_t cnt = 0;
    int rc = kRetryHits;
    for (int attempt = 0; attempt < 4 && (rc == kRetryHits || rc == RS_ERR_CAPACITY); attempt++) {
      rc = sieve_range_impl(it.job, it.p0, it.p1, out.data(), out.size(), &cnt, &it.st);
      if (rc == RS_ERR_CAPACITY) out.resize(cnt);
    }
    if (rc) {
      it.status = rc;
      it.err = rs_last_error();
    } else {
      it.out.assign(out.begin(), out.begin() + cnt);
      tot.gpu_ms += it.st.gpu_ms;
      tot.launches += it.st.launches;
    }
  }
  for (auto &it : B->items) {
    tot.primes += it.st.primes;
    tot.factors += it.out.size();
    tot.raw_hits += it.st.raw_hits;
    tot.p_covered += it.st.p_covered;
    for (int f = 0; f < 3; f++) tot.primes_by_step[f] += it.st.primes_by_step[f];
    tot.paired_primes += it.st.paired_primes;
    tot.exact_primes += it.st.exact_primes;
  }
  if (stats) *stats = tot;
  B->ran = true;
  for (auto &it : B->items)
    if (it.status != RS_OK) return fail(it.status, "rs_batch_run: an item failed: %s", it.err.c_str());
  return RS_OK;
}

extern "C" int rs_batch_result(const rs_batch *B, uint32_t item, rs_factor *out, size_t cap, size_t *count,
                               rs_stats *stats) {
  if (!B || !count || (!out && cap)) return fail(RS_ERR_INVALID, "rs_batch_result: NULL argument");
  if (item >= B->items.size()) return fail(RS_ERR_INVALID, "rs_batch_result: no item %u", item);
  if (!B->ran) return fail(RS_ERR_INVALID, "rs_batch_result: the batch has not run");
  const auto &it = B->items[item];
  if (stats) *stats = it.st;
  *count = it.out.size();
  if (it.status != RS_OK) return fail(it.status, "%s", it.err.c_str());
  if (it.out.size() > cap) return fail(RS_ERR_CAPACITY, "%zu factors, buffer holds %zu", it.out.size(), cap);
  if (!it.out.empty()) memcpy(out, it.out.data(), it.out.size() * sizeof(rs_factor));
  return RS_OK;
}

extern "C" int rs_batch_destroy(rs_batch *B) {
  if (!B) return RS_OK;
  if (B->st) {
    cudaStreamSynchronize(B->st);
    cudaStreamDestroy(B->st);
  }
  for (int s = 0; s < kBatchBranches; s++)
    if (B->side[s]) cudaStreamDestroy(B->side[s]);
  for (int h = 0; h < 2; h++) {
    if (B->fork[h]) cudaEventDestroy(B->fork[h]);
    for (int s = 0; s < kBatchBranches; s++)
      if (B->join[h][s]) cudaEventDestroy(B->join[h][s]);
  }
  delete B;
  return RS_OK;
}

extern "C" int rs_write_factors(const rs_job *j, const char *path, const rs_factor *f, size_t count) {
  if (!j || !path || (!f && count)) return fail(RS_ERR_INVALID, "NULL argument");
  FILE *fp = fopen(path, "a");
  if (!fp) return fail(RS_ERR_INVALID, "cannot open %s for appending", path);
  for (size_t i = 0; i < count; i++)
    fprintf(fp, "%llu | %u*%u^%u%s\n", (unsigned long long)f[i].p, f[i].k, f[i].b ? f[i].b : j->parts[0]->seqs.base,
            f[i].n, (f[i].b ? f[i].c : j->parts[0]->seqs.sign) < 0 ? "-1" : "+1");
  const int bad = ferror(fp);
  fclose(fp);
  if (bad) return fail(RS_ERR_INVALID, "write error on %s", path);
  return RS_OK;
}

extern "C" int rs_plan_abcd(const char *text, size_t len, const rs_options *optp, rs_job_info *info) {
  if (!text || !info) return fail(RS_ERR_INVALID, "NULL argument");
  Seqs all;
  int rc = parse_abcd(text, len, all);
  if (rc) return rc;
  std::vector<Seqs> groups = split_parts(std::move(all));
  rs_options opt;
  if (optp) opt = *optp;
  else rs_options_default(&opt);
  memset(info, 0, sizeof(*info));
  Plan pl;
  for (size_t g = 0; g < groups.size(); g++) {
    normalise(groups[g]);
    Plan pg;
    rc = make_plan(groups[g], opt, pg, false);  // the plan's parameters only
    if (rc) return rc;
    info->num_k += (uint32_t)groups[g].k.size();
    info->num_candidates += pg.ncand;
    if (g == 0) pl = std::move(pg);
  }
  const Seqs &s = groups[0];
  info->parts = (uint32_t)groups.size();
  info->base = s.base;
  info->sign = s.sign;
  info->nmin = pl.nmin;
  info->nmax = pl.nmax;
  info->Q = pl.Q;
  info->rows = pl.nrows;
  info->x_range = pl.X;
  info->baby_steps = pl.m;
  info->giant_steps = pl.T;
  info->table_slots = (uint32_t)kBucket * pl.nbuckets;
  info->work_per_prime = pl.work_per_prime;
  info->warps_per_prime = pl.cta ? kCtaWarps : 1;
  info->row_form = plan_row_form(pl, s, nullptr);
  return RS_OK;
}

extern "C" int rs_gpu_primes(uint64_t lo, uint64_t hi, uint64_t *out, size_t cap, size_t *count,
                             int device) {
  if (!count || (!out && cap)) return fail(RS_ERR_INVALID, "NULL argument");
  *count = 0;
  if (hi >= (1ull << 63)) return fail(RS_ERR_RANGE, "hi must be < 2^63");
  if (lo < 3) lo = 3;
  if (!(lo & 1)) lo++;
  if (lo > hi) return RS_OK;
  int rc = check_device(device);
  if (rc) return rc;
  // a throwaway job-less context: sieving primes + output buffer
  rs_job tmp;
  tmp.device = device;
  CUDA_TRY(cudaStreamCreateWithFlags(&tmp.st, cudaStreamNonBlocking));
  struct Guard {
    rs_job &t;
    uint64_t *d_out = nullptr;
    uint32_t *d_cnt = nullptr;
    ~Guard() {
      if (d_out) cudaFree(d_out);
      if (d_cnt) cudaFree(d_cnt);
      if (t.d_gbits && t.st) cudaFreeAsync(t.d_gbits, t.st);
      if (t.st) {
        cudaStreamSynchronize(t.st);
        cudaStreamDestroy(t.st);
      }
      t.d_gbits = nullptr;
      t.d_sp = nullptr;
      t.d_sp_rcp = nullptr;
      t.st = nullptr;
    }
  } g{tmp};
  rc = ensure_sieving_primes(&tmp, hi);
  if (rc) return rc;
  const uint64_t odds = (hi - lo) / 2 + 1;
  if (odds > (1ull << 31)) return fail(RS_ERR_RANGE, "rs_gpu_primes: window wider than 2^32");
  const uint32_t dcap = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(odds, std::max<size_t>(cap, 1)));
  CUDA_TRY(cudaMalloc(&g.d_out, (size_t)dcap * 8));
  CUDA_TRY(cudaMalloc(&g.d_cnt, 4));
  CUDA_TRY(cudaMemsetAsync(g.d_cnt, 0, 4, tmp.st));
  rc = ensure_gbits(&tmp, sieve_bitmap_words(lo, hi));
  if (rc) return rc;
  CUDA_TRY(launch_sieve(lo, hi, tmp.d_sp, tmp.d_sp_rcp, tmp.nsp, tmp.nsp_small, tmp.d_gbits, g.d_out, g.d_cnt,
                        dcap, tmp.st));
  uint32_t n = 0;
  CUDA_TRY(cudaMemcpyAsync(&n, g.d_cnt, 4, cudaMemcpyDeviceToHost, tmp.st));
  CUDA_TRY(cudaStreamSynchronize(tmp.st));
  *count = n;
  if (n > cap) return fail(RS_ERR_CAPACITY, "%u primes, buffer holds %zu", n, cap);
  CUDA_TRY(cudaMemcpy(out, g.d_out, (size_t)n * 8, cudaMemcpyDeviceToHost));
  std::sort(out, out + n);  // segments finish in any order
  return RS_OK;
}

extern "C" int rs_bench_imad(int device, double *mul_ops_per_s, double *montmul_per_s,
                             double *shoup_per_s) {
  if (!mul_ops_per_s || !montmul_per_s || !shoup_per_s) return fail(RS_ERR_INVALID, "NULL argument");
  int rc = check_device(device);
  if (rc) return rc;
  CUDA_TRY(run_imad_bench(device, mul_ops_per_s, montmul_per_s, shoup_per_s));
  return RS_OK;
}

extern "C" int rs_bench_products(int device, double *rates) {
  if (!rates) return fail(RS_ERR_INVALID, "NULL argument");
  int rc = check_device(device);
  if (rc) return rc;
  CUDA_TRY(run_product_bench(device, rates));
  return RS_OK;
}

extern "C" int rs_gpu_modmul_check(int32_t op, const uint64_t *a, const uint64_t *b, const uint64_t *c,
                                   const uint64_t *p, size_t n, uint64_t *out, int device) {
  if (!a || !b || !c || !p || !out) return fail(RS_ERR_INVALID, "NULL argument");
  if (op < RS_OP_MONTMUL || op > RS_OP_MONTMUL_PTX) return fail(RS_ERR_INVALID, "unknown operation %d", op);
  for (size_t i = 0; i < n; i++)
    if (!(p[i] & 1) || p[i] < 3 || p[i] >= (1ull << 63))
      return fail(RS_ERR_INVALID, "modmul check modulus %zu out of range", i);
  if (n == 0) return RS_OK;
  int rc = check_device(device);
  if (rc) return rc;
  void *d = nullptr;
  CUDA_TRY(cudaMalloc(&d, n * 8 * 5));
  uint64_t *da = (uint64_t *)d, *db = da + n, *dc = db + n, *dp = dc + n, *dout = dp + n;
  cudaError_t e = cudaMemcpy(da, a, n * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(db, b, n * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dc, c, n * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dp, p, n * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = run_modmul_check(op, da, db, dc, dp, n, dout);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(out, dout, n * 8, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return fail(RS_ERR_CUDA, "modmul check: %s", cudaGetErrorString(e));
  return RS_OK;
}

extern "C" int rs_gpu_arith_check(const uint64_t *a, const uint64_t *b, const uint64_t *p, size_t n,
                                  uint64_t *out_mulmod, int32_t *out_jacobi_ap, int device) {
  if (!a || !b || !p || !out_mulmod || !out_jacobi_ap) return fail(RS_ERR_INVALID, "NULL argument");
  for (size_t i = 0; i < n; i++)
    if (!(p[i] & 1) || p[i] < 3 || p[i] >= (1ull << 63) || a[i] >= p[i] || b[i] >= p[i])
      return fail(RS_ERR_INVALID, "arith check input %zu out of range", i);
  if (n == 0) return RS_OK;
  int rc = check_device(device);
  if (rc) return rc;
  void *d = nullptr;
  CUDA_TRY(cudaMalloc(&d, n * (8 * 4 + 4)));
  uint64_t *da = (uint64_t *)d, *db = da + n, *dp = db + n, *dm = dp + n;
  int32_t *dj = (int32_t *)(dm + n);
  cudaError_t e = cudaMemcpy(da, a, n * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(db, b, n * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dp, p, n * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = run_arith_check(da, db, dp, n, dm, dj);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(out_mulmod, dm, n * 8, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(out_jacobi_ap, dj, n * 4, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return fail(RS_ERR_CUDA, "arith check: %s", cudaGetErrorString(e));
  return RS_OK;
}

// ---------------------------------------------------------------------------
// Helpers of the served form (rs_server.cu; declared in rs_internal.h).

int rs::job_footprint(const char *text, size_t len, const rs_options &opt, JobFootprint *fp) {
  Seqs all;
  int rc = parse_abcd(text, len, all);
  if (rc) return rc;
  std::vector<Seqs> groups = split_parts(std::move(all));
  *fp = JobFootprint{};
  fp->parts = (uint32_t)groups.size();
  uint32_t rec = 0;
  for (Seqs &g : groups) {
    normalise(g);
    Plan pl;
    rc = make_plan(g, opt, pl, false);
    if (rc) return rc;
    fp->arrays += part_array_bytes(pl, g, opt.datless != 0);
    rec = std::max(rec, record_el_tab(pl, plan_row_form(pl, g, nullptr)) + 64);
  }
  fp->per_prime = 8 + 4 + 8 * (uint64_t)rec;
  return RS_OK;
}

uint64_t rs::job_resident_bytes(const rs_job *j) {
  uint64_t b = 0;
  for (auto &pt : j->parts) b += pt->dev_bytes;
  return b;
}

void rs::job_set_mem_limit(rs_job *j, uint64_t bytes) {
  std::lock_guard<std::mutex> lock(j->mu);
  j->opt.mem_limit = bytes;
  j->opt.block_scale = j->opt.thread_scale = 0;
  set_chunk_cap(j);
}

void rs::job_release_buffers(rs_job *j) {
  std::lock_guard<std::mutex> lock(j->mu);
  cudaSetDevice(j->device);
  if (j->d_chunk) cudaFreeAsync(j->d_chunk, j->st);
  j->d_chunk = nullptr;
  j->chunk_cap = 0;
  j->chunk_rec_elems = 0;
  j->chunk_exact_bytes = 0;
  for (auto &pt : j->parts) {
    if (pt->d_hits) cudaFreeAsync(pt->d_hits, j->st);
    pt->d_hits = nullptr;
    pt->hb = HitBufs{};
  }
  if (j->d_gbits) cudaFreeAsync(j->d_gbits, j->st);
  j->d_gbits = nullptr;
  j->gbits_words = 0;
  cudaStreamSynchronize(j->st);
}

// ---------------------------------------------------------------------------
// Sieve-file update: the ABCD text with the removed candidates dropped.  The
// reference only appends factor lines (kernel_v0.24.6.cu:1830-1835); srsieve
// workflows continue from an updated ABCD file, which this writes.

extern "C" int rs_abcd_remove(const char *text, size_t len, const rs_factor *removed, size_t count,
                              uint64_t sieved_to, char *out, size_t cap, size_t *out_len) {
  if (!text || !out_len || (!removed && count) || (!out && cap)) return fail(RS_ERR_INVALID, "NULL argument");
  Seqs all;
  int rc = parse_abcd(text, len, all);
  if (rc) return rc;
  std::vector<Seqs> groups = split_parts(std::move(all));
  // removed (k, n) keyed by base and sign; b == 0 matches every sequence of that k
  typedef std::tuple<uint32_t, int32_t, uint32_t, uint32_t> Key;  // (b, c, k, n)
  std::vector<Key> rm(count);
  for (size_t i = 0; i < count; i++)
    rm[i] = Key{removed[i].b, removed[i].b ? (removed[i].c < 0 ? -1 : 1) : 0, removed[i].k, removed[i].n};
  std::sort(rm.begin(), rm.end());
  std::string o;
  char buf[160];
  for (Seqs &s : groups) {
    normalise(s);
    for (size_t i = 0; i < s.k.size(); i++) {
      std::vector<uint32_t> keep;
      for (uint32_t n : s.n[i])
        if (!std::binary_search(rm.begin(), rm.end(), Key{s.base, s.sign, s.k[i], n}) &&
            !std::binary_search(rm.begin(), rm.end(), Key{0u, 0, s.k[i], n}))
          keep.push_back(n);
      if (keep.empty()) continue;
      snprintf(buf, sizeof(buf), "ABCD %u*%u^$a%s [%u] // Sieved to %llu\n", s.k[i], s.base,
               s.sign < 0 ? "-1" : "+1", keep[0], (unsigned long long)sieved_to);
      o += buf;
      for (size_t t = 1; t < keep.size(); t++) {
        snprintf(buf, sizeof(buf), "%u\n", keep[t] - keep[t - 1]);
        o += buf;
      }
    }
  }
  *out_len = o.size();
  if (o.size() > cap) return fail(RS_ERR_CAPACITY, "output needs %zu bytes, buffer holds %zu", o.size(), cap);
  memcpy(out, o.data(), o.size());
  return RS_OK;
}
