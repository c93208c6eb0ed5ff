/*
 * rs_oracle.c -- CPU oracle for the Riesel/Sierpinski sieve hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see rs_oracle.h): the product library never
 * links or calls this file.  It is the checker for the CUDA path.
 *
 * The complete-mode search below is deliberately a different algorithm from
 * the GPU kernel: Q = 1 (no subsequences), no quadratic-character filter,
 * giant steps by the inverse of b^m, a full-64-bit-key hash with stamps, and
 * per-k targets from one batched modular inversion.  Everything it reports is
 * re-checked by orc_verify (unsigned __int128 arithmetic with '%').
 */
#define _GNU_SOURCE
#include "rs_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

typedef unsigned __int128 u128;

/* ------------------------------------------------------------------------ */
/* Plain modular arithmetic ('%' on 128-bit products).                       */

static inline uint64_t mulmod(uint64_t a, uint64_t b, uint64_t p) {
  return (uint64_t)(((u128)a * b) % p);
}

static uint64_t powmod(uint64_t b, uint64_t e, uint64_t p) {
  uint64_t r = 1 % p;
  b %= p;
  while (e) {
    if (e & 1) r = mulmod(r, b, p);
    b = mulmod(b, b, p);
    e >>= 1;
  }
  return r;
}

/* Inverse of a mod p (gcd(a,p) = 1) by the extended Euclidean algorithm. */
static uint64_t invmod(uint64_t a, uint64_t p) {
  __int128 t = 0, newt = 1;
  uint64_t r = p, newr = a % p;
  while (newr) {
    uint64_t q = r / newr;
    __int128 tmp = t - (__int128)q * newt;
    t = newt;
    newt = tmp;
    uint64_t tr = r - q * newr;
    r = newr;
    newr = tr;
  }
  if (t < 0) t += p;
  return (uint64_t)t;
}

int orc_verify(uint64_t p, uint32_t k, uint32_t b, uint32_t n, int32_t sign) {
  /* Square-and-multiply from the most significant bit of n, as
   * kernel_v0.24.6.cu:1649-1663 does, then k*b^n compared with -sign. */
  if (p < 2) return 0;
  u128 val = 1;
  uint64_t bb = b % p;
  for (int z = 31; z >= 0; --z) {
    val = (val * val) % p;
    if (n & (1u << z)) val = (val * bb) % p;
  }
  val = (val * (k % p)) % p;
  uint64_t want = sign < 0 ? 1 % p : (p - 1) % p;
  return (uint64_t)val == want;
}

int orc_jacobi(uint64_t a, uint64_t n) {
  /* Binary Jacobi symbol; n odd positive. */
  if (!(n & 1)) return 0;
  a %= n;
  int t = 1;
  while (a) {
    while (!(a & 1)) {
      a >>= 1;
      uint64_t r = n & 7;
      if (r == 3 || r == 5) t = -t;
    }
    uint64_t tmp = a;
    a = n;
    n = tmp;
    if ((a & 3) == 3 && (n & 3) == 3) t = -t;
    a %= n;
  }
  return n == 1 ? t : 0;
}

/* ------------------------------------------------------------------------ */
/* Montgomery arithmetic (R = 2^64), used only to make the oracle's inner     */
/* loops fast enough for second-scale runs; cross-checked against mulmod in   */
/* the oracle's own tests.  Requires p odd, p < 2^63.                        */

typedef struct {
  uint64_t p, pinv, r1, r2;
} mctx;

static void mctx_init(mctx *c, uint64_t p) {
  c->p = p;
  uint64_t x = p; /* p*p == 1 mod 8: 3 correct bits */
  for (int i = 0; i < 6; i++) x *= 2 - p * x;
  c->pinv = (uint64_t)0 - x; /* -p^-1 mod 2^64 */
  c->r1 = (uint64_t)(((u128)1 << 64) % p);
  c->r2 = mulmod(c->r1, c->r1, p);
}

static inline uint64_t mmul(const mctx *c, uint64_t a, uint64_t b) {
  u128 t = (u128)a * b;
  uint64_t m = (uint64_t)t * c->pinv;
  u128 u = (t + (u128)m * c->p) >> 64;
  uint64_t r = (uint64_t)u;
  return r >= c->p ? r - c->p : r;
}

static inline uint64_t to_m(const mctx *c, uint64_t a) { return mmul(c, a % c->p, c->r2); }

/* ------------------------------------------------------------------------ */
/* ABCD parsing (kernel_v0.24.6.cu:938-1083).                                */

typedef struct {
  uint32_t k;
  uint32_t *n;
  size_t cnt, cap;
} kseq;

static int cmp_u32(const void *a, const void *b) {
  uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
  return x < y ? -1 : x > y;
}

static void seterr(char *err, size_t errlen, const char *msg, long line) {
  if (err && errlen) snprintf(err, errlen, "ABCD line %ld: %s", line, msg);
}

static int push_n(kseq *s, uint32_t n) {
  if (s->cnt == s->cap) {
    size_t nc = s->cap ? s->cap * 2 : 64;
    uint32_t *nn = (uint32_t *)realloc(s->n, nc * sizeof(uint32_t));
    if (!nn) return -1;
    s->n = nn;
    s->cap = nc;
  }
  s->n[s->cnt++] = n;
  return 0;
}

/* Merge sequences into an orc_job: duplicate k merged, n lists sorted/unique. */
static int finish_job(kseq *seqs, size_t ns, uint32_t base, int32_t sign, orc_job *out) {
  /* merge duplicates of k (keep first-appearance order) */
  uint32_t nk = 0;
  for (size_t i = 0; i < ns; i++) {
    size_t j;
    for (j = 0; j < nk; j++)
      if (seqs[j].k == seqs[i].k) break;
    if (j == nk) {
      if (j != i) { seqs[j] = seqs[i]; seqs[i].n = NULL; seqs[i].cnt = seqs[i].cap = 0; }
      nk++;
    } else {
      for (size_t t = 0; t < seqs[i].cnt; t++)
        if (push_n(&seqs[j], seqs[i].n[t])) return -1;
      free(seqs[i].n);
      seqs[i].n = NULL;
      seqs[i].cnt = 0;
    }
  }
  size_t total = 0;
  for (uint32_t i = 0; i < nk; i++) {
    qsort(seqs[i].n, seqs[i].cnt, sizeof(uint32_t), cmp_u32);
    size_t w = 0;
    for (size_t t = 0; t < seqs[i].cnt; t++)
      if (w == 0 || seqs[i].n[w - 1] != seqs[i].n[t]) seqs[i].n[w++] = seqs[i].n[t];
    seqs[i].cnt = w;
    total += w;
  }
  out->base = base;
  out->sign = sign;
  out->nk = nk;
  out->k = (uint32_t *)malloc((nk ? nk : 1) * sizeof(uint32_t));
  out->noff = (uint32_t *)malloc((nk + 1) * sizeof(uint32_t));
  out->n = (uint32_t *)malloc((total ? total : 1) * sizeof(uint32_t));
  if (!out->k || !out->noff || !out->n) return -1;
  size_t pos = 0;
  for (uint32_t i = 0; i < nk; i++) {
    out->k[i] = seqs[i].k;
    out->noff[i] = (uint32_t)pos;
    memcpy(out->n + pos, seqs[i].n, seqs[i].cnt * sizeof(uint32_t));
    pos += seqs[i].cnt;
  }
  out->noff[nk] = (uint32_t)pos;
  return 0;
}

int orc_parse_abcd(const char *text, size_t len, orc_job *out, char *err, size_t errlen) {
  memset(out, 0, sizeof(*out));
  kseq *seqs = NULL;
  size_t ns = 0, nscap = 0;
  uint32_t base = 0;
  int32_t sign = 0;
  long lineno = 0;
  int64_t total = 0;
  int32_t refmin = 0x7fffffff, refmax = 0;
  size_t i = 0;
  int rc = 0;
  while (i < len) {
    size_t e = i;
    while (e < len && text[e] != '\n') e++;
    lineno++;
    /* strip a trailing '\r' and surrounding blanks */
    size_t a = i, z = e;
    while (z > a && (text[z - 1] == '\r' || text[z - 1] == ' ' || text[z - 1] == '\t')) z--;
    while (a < z && (text[a] == ' ' || text[a] == '\t')) a++;
    i = e + 1;
    if (a == z) continue; /* blank line (the reference's stoi would throw) */
    char buf[512];
    size_t L = z - a < sizeof(buf) - 1 ? z - a : sizeof(buf) - 1;
    memcpy(buf, text + a, L);
    buf[L] = 0;
    if (!strncmp(buf, "ABCD", 4) && (buf[4] == ' ' || buf[4] == '\t')) {
      /* ABCD k*b^$a-1 [n0] ... */
      char *s = buf + 5;
      while (*s == ' ' || *s == '\t') s++;
      char *endp;
      unsigned long long kv = strtoull(s, &endp, 10);
      if (endp == s || *endp != '*' || kv == 0 || kv > 0xffffffffull) {
        seterr(err, errlen, "bad k in header", lineno); rc = 1; break;
      }
      s = endp + 1;
      unsigned long long bv = strtoull(s, &endp, 10);
      if (endp == s || *endp != '^' || bv < 2 || bv > 0xffffffffull) {
        seterr(err, errlen, "bad base in header", lineno); rc = 1; break;
      }
      s = endp + 1;
      char *dol = strstr(s, "$a");
      if (!dol) { seterr(err, errlen, "expected $a exponent", lineno); rc = 1; break; }
      s = dol + 2;
      int32_t sg;
      if (s[0] == '-' && s[1] == '1') sg = -1;
      else if (s[0] == '+' && s[1] == '1') sg = +1;
      else { seterr(err, errlen, "expected -1 or +1", lineno); rc = 1; break; }
      char *lb = strchr(s, '[');
      if (!lb) { seterr(err, errlen, "missing [n0]", lineno); rc = 1; break; }
      s = lb + 1;
      long long n0 = strtoll(s, &endp, 10);
      if (endp == s || *endp != ']' || n0 < 0 || n0 > 0x7fffffffll) {
        seterr(err, errlen, "bad [n0]", lineno); rc = 1; break;
      }
      if (base == 0) { base = (uint32_t)bv; sign = sg; }
      else if (bv != base) { seterr(err, errlen, "all sequences must share one base", lineno); rc = 1; break; }
      else if (sg != sign) { seterr(err, errlen, "all sequences must share one sign", lineno); rc = 1; break; }
      if (ns == nscap) {
        nscap = nscap ? nscap * 2 : 16;
        kseq *nsq = (kseq *)realloc(seqs, nscap * sizeof(kseq));
        if (!nsq) { rc = 2; break; }
        seqs = nsq;
      }
      memset(&seqs[ns], 0, sizeof(kseq));
      seqs[ns].k = (uint32_t)kv;
      total = n0;
      if ((int32_t)n0 < refmin) refmin = (int32_t)n0;
      if (push_n(&seqs[ns], (uint32_t)n0)) { rc = 2; break; }
      ns++;
    } else {
      if (ns == 0) { seterr(err, errlen, "data before the first ABCD header", lineno); rc = 1; break; }
      char *endp;
      long long d = strtoll(buf, &endp, 10);
      if (endp == buf || d <= 0) { seterr(err, errlen, "bad n delta", lineno); rc = 1; break; }
      total += d;
      if (total > 0x7fffffffll) { seterr(err, errlen, "n exceeds 2^31-1", lineno); rc = 1; break; }
      if ((int32_t)total > refmax) refmax = (int32_t)total;
      if (push_n(&seqs[ns - 1], (uint32_t)total)) { rc = 2; break; }
    }
  }
  if (!rc && ns == 0) { seterr(err, errlen, "no ABCD header found", lineno); rc = 1; }
  if (!rc) rc = finish_job(seqs, ns, base, sign, out) ? 2 : 0;
  for (size_t t = 0; t < ns; t++) free(seqs[t].n);
  free(seqs);
  out->ref_minN = refmin;
  out->ref_maxN = refmax;
  out->nlines = (uint32_t)lineno;
  if (rc) orc_job_free(out);
  return rc;
}

int orc_job_from_arrays(uint32_t base, int32_t sign, uint32_t nk, const uint32_t *k,
                        const uint32_t *noff, const uint32_t *n, orc_job *out) {
  memset(out, 0, sizeof(*out));
  kseq *seqs = (kseq *)calloc(nk ? nk : 1, sizeof(kseq));
  if (!seqs) return 2;
  int32_t refmin = 0x7fffffff, refmax = 0;
  for (uint32_t i = 0; i < nk; i++) {
    seqs[i].k = k[i];
    for (uint32_t t = noff[i]; t < noff[i + 1]; t++) {
      if (push_n(&seqs[i], n[t])) return 2;
      if ((int32_t)n[t] < refmin) refmin = (int32_t)n[t];
      if ((int32_t)n[t] > refmax) refmax = (int32_t)n[t];
    }
  }
  int rc = finish_job(seqs, nk, base, sign, out) ? 2 : 0;
  for (uint32_t i = 0; i < nk; i++) free(seqs[i].n);
  free(seqs);
  out->ref_minN = refmin;
  out->ref_maxN = refmax;
  return rc;
}

void orc_job_free(orc_job *job) {
  free(job->k);
  free(job->noff);
  free(job->n);
  job->k = job->noff = job->n = NULL;
  job->nk = 0;
}

/* ------------------------------------------------------------------------ */
/* The reference's planner: Q choice (kernel_v0.24.6.cu:1086-1146), tMin/tMax */
/* (1148-1158), row build (1160-1209) and its selection sort (1220-1254).    */

int orc_ref_plan(const orc_job *job, int32_t Qin, int32_t hash_elems, orc_refplan *out) {
  memset(out, 0, sizeof(*out));
  int32_t count1 = (int32_t)job->nk;
  int32_t minN = job->ref_minN, maxN = job->ref_maxN;
  int32_t range = maxN - minN;
  int32_t minWork = count1 * range, minSubs = count1, minRange = range, minQ = 1;
  int32_t Qlow = 2, Qhigh = 24;
  if (Qin != 0) { Qlow = Qin; Qhigh = Qin + 1; }
  for (int32_t Q = Qlow; Q < Qhigh; Q += 2) {
    char *seen = (char *)calloc((size_t)count1 * Q, 1);
    if (!seen) return 2;
    int32_t subs = 0;
    for (uint32_t i = 0; i < job->nk; i++)
      for (uint32_t t = job->noff[i]; t < job->noff[i + 1]; t++) {
        size_t idx = (size_t)i * Q + job->n[t] % Q;
        if (!seen[idx]) { seen[idx] = 1; subs++; }
      }
    free(seen);
    int32_t r = maxN / Q - minN / Q + 1;
    if (subs * r < minWork) { minQ = Q; minWork = subs * r; minSubs = subs; minRange = r; }
  }
  int32_t shift = -1, temp = hash_elems;
  while (temp) { temp >>= 1; shift++; }
  out->minQ = minQ;
  out->minSubs = minSubs;
  out->minRange = minRange;
  out->minWork = minWork;
  out->shift = shift;
  out->tMin = (minN / minQ) >> shift;
  out->tMax = (((maxN / minQ) + 1) >> shift) + 1;
  out->minimum = minN / minQ;
  out->rowoffset = minRange / 32 + 1 + 2;
  /* rows in order of first appearance (k in file order, n ascending) */
  int32_t *rk = (int32_t *)calloc(minSubs ? minSubs : 1, sizeof(int32_t));
  int32_t *rr = (int32_t *)calloc(minSubs ? minSubs : 1, sizeof(int32_t));
  if (!rk || !rr) return 2;
  int32_t used = 0;
  for (uint32_t i = 0; i < job->nk; i++)
    for (uint32_t t = job->noff[i]; t < job->noff[i + 1]; t++) {
      int32_t mod = (int32_t)(job->n[t] % (uint32_t)minQ);
      int found = 0;
      for (int32_t q = 0; q < used; q++)
        if (rk[q] == (int32_t)job->k[i] && rr[q] == mod) { found = 1; break; }
      if (!found && used < minSubs) { rk[used] = (int32_t)job->k[i]; rr[used] = mod; used++; }
    }
  /* the reference's selection "sort": pick a row when k <= kmin AND r < rmin */
  out->row_k = (int32_t *)malloc((minSubs ? minSubs : 1) * sizeof(int32_t));
  out->row_r = (int32_t *)malloc((minSubs ? minSubs : 1) * sizeof(int32_t));
  if (!out->row_k || !out->row_r) return 2;
  for (int32_t a = 0; a < minSubs; a++) {
    int32_t kmin = 0x7fffffff, rmin = 0x7fffffff, idx = 0;
    for (int32_t q = 0; q < minSubs; q++) {
      if (rk[q] <= kmin && rk[q] != 0x7fffffff) {
        if (rr[q] < rmin) { kmin = rk[q]; rmin = rr[q]; idx = q; }
      }
    }
    out->row_k[a] = rk[idx];
    out->row_r[a] = rr[idx];
    rk[idx] = 0x7fffffff;
  }
  free(rk);
  free(rr);
  return 0;
}

void orc_refplan_free(orc_refplan *pl) {
  free(pl->row_k);
  free(pl->row_r);
  pl->row_k = pl->row_r = NULL;
}

/* ------------------------------------------------------------------------ */
/* Odd primes in [lo, hi] by a segmented sieve of Eratosthenes.              */

static uint32_t *small_primes(uint64_t limit, size_t *cnt) {
  /* odd primes <= limit */
  size_t L = (size_t)limit;
  char *comp = (char *)calloc(L / 2 + 2, 1);
  size_t cap = 1024, c = 0;
  uint32_t *ps = (uint32_t *)malloc(cap * sizeof(uint32_t));
  for (size_t i = 3; i <= L; i += 2) {
    if (comp[i / 2]) continue;
    if (c == cap) { cap *= 2; ps = (uint32_t *)realloc(ps, cap * sizeof(uint32_t)); }
    ps[c++] = (uint32_t)i;
    for (size_t j = i * i; j <= L; j += 2 * i) comp[j / 2] = 1;
  }
  free(comp);
  *cnt = c;
  return ps;
}

size_t orc_primes(uint64_t lo, uint64_t hi, uint64_t *out, size_t cap) {
  if (hi < 3 || hi < lo) return 0;
  if (lo < 3) lo = 3;
  if (!(lo & 1)) lo++;
  uint64_t root = (uint64_t)sqrtl((long double)hi);
  while (root * root > hi) root--;
  while ((root + 1) * (root + 1) <= hi) root++;
  size_t nsp;
  uint32_t *sp = small_primes(root, &nsp);
  const uint64_t SEG = 1u << 20; /* odd numbers per segment */
  char *seg = (char *)malloc(SEG);
  size_t found = 0;
  for (uint64_t s = lo; s <= hi; s += 2 * SEG) {
    uint64_t cnt = (hi - s) / 2 + 1;
    if (cnt > SEG) cnt = SEG;
    memset(seg, 0, cnt);
    uint64_t last = s + 2 * (cnt - 1);
    for (size_t t = 0; t < nsp; t++) {
      uint64_t q = sp[t];
      if (q * q > last) break;
      uint64_t f = q * q;
      if (f < s) {
        uint64_t r = s % q;
        f = r ? s + (q - r) : s;
        if (!(f & 1)) f += q;
      }
      for (uint64_t x = (f - s) / 2; x < cnt; x += q) seg[x] = 1;
    }
    for (uint64_t x = 0; x < cnt; x++)
      if (!seg[x]) {
        if (found < cap) out[found] = s + 2 * x;
        found++;
      }
    if (last >= hi) break;
  }
  free(seg);
  free(sp);
  return found;
}

/* ------------------------------------------------------------------------ */
/* Complete-mode BSGS per prime.                                             */

typedef struct {
  orc_factor *v;
  size_t cnt, cap;
} fvec;

static void fpush(fvec *f, uint64_t p, uint32_t k, uint32_t n) {
  if (f->cnt == f->cap) {
    f->cap = f->cap ? f->cap * 2 : 256;
    f->v = (orc_factor *)realloc(f->v, f->cap * sizeof(orc_factor));
  }
  f->v[f->cnt].p = p;
  f->v[f->cnt].k = k;
  f->v[f->cnt].n = n;
  f->cnt++;
}

typedef struct {
  const orc_job *job;
  int32_t datless;
  uint32_t nmin, nmax;
  uint64_t m;   /* baby steps */
  uint64_t T;   /* giant steps */
  uint32_t hbits;
} sctx;

typedef struct {
  uint64_t *key;
  uint32_t *val;
  uint32_t *stamp;
  uint32_t cur;
  uint64_t *c, *pre; /* batched inversion scratch [nk] */
} scratch;

static int has_candidate(const orc_job *job, uint32_t ki, uint32_t n) {
  const uint32_t *a = job->n + job->noff[ki];
  size_t lo = 0, hi = job->noff[ki + 1] - job->noff[ki];
  while (lo < hi) {
    size_t mid = (lo + hi) / 2;
    if (a[mid] < n) lo = mid + 1;
    else hi = mid;
  }
  return lo < job->noff[ki + 1] - job->noff[ki] && a[lo] == n;
}

static void sieve_prime(const sctx *sc, scratch *s, uint64_t p, fvec *out) {
  const orc_job *job = sc->job;
  uint64_t b = job->base % p;
  if (b == 0 || p >= ((uint64_t)1 << 63)) return;
  mctx c;
  mctx_init(&c, p);
  const uint64_t hmask = ((uint64_t)1 << sc->hbits) - 1;
  s->cur++;
  if (s->cur == 0) { /* stamp wrap: clear */
    memset(s->stamp, 0, ((size_t)1 << sc->hbits) * sizeof(uint32_t));
    s->cur = 1;
  }
  /* baby steps: b^j for j in [0, m), keyed by the Montgomery residue */
  uint64_t bm = to_m(&c, b);
  uint64_t v = c.r1;
  for (uint64_t j = 0; j < sc->m; j++) {
    uint64_t h = (v * 0x9E3779B97F4A7C15ull) >> (64 - sc->hbits);
    while (s->stamp[h] == s->cur) h = (h + 1) & hmask;
    s->stamp[h] = s->cur;
    s->key[h] = v;
    s->val[h] = (uint32_t)j;
    v = mmul(&c, v, bm);
  }
  /* v = b^m; giant step multiplies by (b^m)^-1 */
  uint64_t bmn = mmul(&c, v, 1); /* out of Montgomery form */
  uint64_t ginv = to_m(&c, invmod(bmn, p));
  /* targets y_k = (k * b^nmin)^-1 (Riesel) or its negative (Sierpinski),
   * all inverted with one invmod (Montgomery's batch trick) */
  uint64_t bn = powmod(b, sc->nmin, p);
  uint32_t nk = job->nk, live = 0;
  for (uint32_t i = 0; i < nk; i++) {
    uint64_t kk = job->k[i] % p;
    s->c[i] = kk ? mulmod(kk, bn, p) : 0;
  }
  /* prefix products over nonzero c */
  uint64_t acc = 1;
  for (uint32_t i = 0; i < nk; i++) {
    s->pre[i] = acc;
    if (s->c[i]) { acc = mulmod(acc, s->c[i], p); live++; }
  }
  if (!live) return;
  uint64_t inv = invmod(acc, p);
  for (uint32_t ii = nk; ii-- > 0;) {
    if (!s->c[ii]) continue;
    uint64_t yi = mulmod(inv, s->pre[ii], p); /* = c[ii]^-1 */
    inv = mulmod(inv, s->c[ii], p);
    if (job->sign > 0) yi = (p - yi) % p;
    uint64_t y = to_m(&c, yi);
    for (uint64_t t = 0; t < sc->T; t++) {
      uint64_t h = (y * 0x9E3779B97F4A7C15ull) >> (64 - sc->hbits);
      while (s->stamp[h] == s->cur) {
        if (s->key[h] == y) {
          uint64_t n = (uint64_t)sc->nmin + t * sc->m + s->val[h];
          if (n <= sc->nmax && (sc->datless || has_candidate(job, ii, (uint32_t)n)))
            fpush(out, p, job->k[ii], (uint32_t)n);
        }
        h = (h + 1) & hmask;
      }
      y = mmul(&c, y, ginv);
    }
  }
}

typedef struct {
  const sctx *sc;
  const uint64_t *primes;
  size_t lo, hi;
  fvec out;
} tjob;

static void *worker(void *arg) {
  tjob *tj = (tjob *)arg;
  const sctx *sc = tj->sc;
  scratch s;
  size_t H = (size_t)1 << sc->hbits;
  s.key = (uint64_t *)malloc(H * sizeof(uint64_t));
  s.val = (uint32_t *)malloc(H * sizeof(uint32_t));
  s.stamp = (uint32_t *)calloc(H, sizeof(uint32_t));
  s.cur = 0;
  s.c = (uint64_t *)malloc((sc->job->nk + 1) * sizeof(uint64_t));
  s.pre = (uint64_t *)malloc((sc->job->nk + 1) * sizeof(uint64_t));
  for (size_t i = tj->lo; i < tj->hi; i++) sieve_prime(sc, &s, tj->primes[i], &tj->out);
  free(s.key);
  free(s.val);
  free(s.stamp);
  free(s.c);
  free(s.pre);
  return NULL;
}

static int cmp_factor(const void *a, const void *b) {
  const orc_factor *x = (const orc_factor *)a, *y = (const orc_factor *)b;
  if (x->p != y->p) return x->p < y->p ? -1 : 1;
  if (x->k != y->k) return x->k < y->k ? -1 : 1;
  if (x->n != y->n) return x->n < y->n ? -1 : 1;
  return 0;
}

int orc_default_threads(void) {
  long n = sysconf(_SC_NPROCESSORS_ONLN);
  return n > 0 ? (int)n : 1;
}

int orc_sieve(const orc_job *job, uint64_t p0, uint64_t p1, int32_t datless, int32_t nthreads,
              orc_factor *out, size_t cap, size_t *count, uint64_t *nprimes) {
  *count = 0;
  if (nprimes) *nprimes = 0;
  if (job->nk == 0 || p1 < 3 || p1 < p0) return 0;
  if (p1 >= ((uint64_t)1 << 63)) return 3;
  uint32_t nmin = 0xffffffffu, nmax = 0;
  for (uint32_t i = 0; i < job->noff[job->nk]; i++) {
    if (job->n[i] < nmin) nmin = job->n[i];
    if (job->n[i] > nmax) nmax = job->n[i];
  }
  if (job->noff[job->nk] == 0) return 0;
  /* primes */
  uint64_t lo = p0 < 3 ? 3 : p0;
  size_t est = (size_t)((p1 - lo) / 2 + 2);
  size_t bound = est;
  if (lo > 100) {
    double w = (double)(p1 - lo) + 1.0, l = log((double)lo);
    double b2 = 1.3 * w / (l - 1.1) + 1000.0;
    if (b2 < (double)bound) bound = (size_t)b2;
  }
  uint64_t *primes = (uint64_t *)malloc(bound * sizeof(uint64_t));
  if (!primes) return 2;
  size_t np = orc_primes(lo, p1, primes, bound);
  if (np > bound) {
    free(primes);
    primes = (uint64_t *)malloc(np * sizeof(uint64_t));
    if (!primes) return 2;
    np = orc_primes(lo, p1, primes, np);
  }
  if (nprimes) *nprimes = np;
  sctx sc;
  sc.job = job;
  sc.datless = datless;
  sc.nmin = nmin;
  sc.nmax = nmax;
  uint64_t X = (uint64_t)nmax - nmin + 1;
  double mm = ceil(sqrt((double)job->nk * (double)X));
  sc.m = mm < 1 ? 1 : (uint64_t)mm;
  if (sc.m > X) sc.m = X;
  sc.T = (X + sc.m - 1) / sc.m;
  sc.hbits = 1;
  while (((uint64_t)1 << sc.hbits) < 2 * sc.m) sc.hbits++;
  int nt = nthreads > 0 ? nthreads : orc_default_threads();
  if ((size_t)nt > np) nt = np ? (int)np : 1;
  tjob *tj = (tjob *)calloc(nt, sizeof(tjob));
  pthread_t *th = (pthread_t *)calloc(nt, sizeof(pthread_t));
  for (int t = 0; t < nt; t++) {
    tj[t].sc = &sc;
    tj[t].primes = primes;
    tj[t].lo = np * (size_t)t / nt;
    tj[t].hi = np * (size_t)(t + 1) / nt;
    pthread_create(&th[t], NULL, worker, &tj[t]);
  }
  size_t total = 0;
  for (int t = 0; t < nt; t++) {
    pthread_join(th[t], NULL);
    total += tj[t].out.cnt;
  }
  orc_factor *all = (orc_factor *)malloc((total ? total : 1) * sizeof(orc_factor));
  size_t pos = 0;
  int bad = 0;
  for (int t = 0; t < nt; t++) {
    for (size_t i = 0; i < tj[t].out.cnt; i++) {
      orc_factor f = tj[t].out.v[i];
      if (!orc_verify(f.p, f.k, job->base, f.n, job->sign)) bad = 1;
      all[pos++] = f;
    }
    free(tj[t].out.v);
  }
  qsort(all, total, sizeof(orc_factor), cmp_factor);
  for (size_t i = 0; i < total && i < cap; i++) out[i] = all[i];
  *count = total;
  free(all);
  free(tj);
  free(th);
  free(primes);
  return bad ? 4 : 0;
}

/* ------------------------------------------------------------------------ */
/* Reference projection: what the reference executable would write.          */
/*                                                                           */
/* Restates, on the CPU, the observable behaviour of one reference run:      */
/*  - its prime source (kernel_v0.24.6.cu:1271-1303, 1838-1987): every odd q  */
/*    in range with no factor among the first 4096*s odd primes, so that     */
/*    composites appear above smallP_max^2;                                  */
/*  - its per-prime search (kernel_v0.24.6.cu:288-620) with its plan (Q,     */
/*    rows in its sorted order, tMin/tMax for m = hash_elems): B = b^Q,      */
/*    c1 = B^m, beta = c1^tMin; per row the character filter on (k/q) and    */
/*    (kb/q), the catch-up by b from the previous row of the same k, giant   */
/*    steps t in [tMin, tMax) compared with the baby steps B^j, j < m (the   */
/*    smallest j when several match); a hit of the last t with a match in a */
/*    row is kept, and the last row with a hit is the prime's one report;    */
/*  - its host filter (kernel_v0.24.6.cu:1605-1732): n in [minN, maxN]      */
/*    (its parse quirks), then with verify the candidate bit of the first    */
/*    row at or after k's first row whose residue is n mod Q (which can be   */
/*    another k's row) and k*b^n == 1 mod q; without verify every in-range   */
/*    report is written.                                                     */
/* The reference's hash-chain edge cases (an all-zero chain word, pointer    */
/* 0x7FFF) are not emulated.  Riesel only, q > b and q > every k (so that    */
/* the reference's Legendre routine is the Jacobi symbol).                   */

typedef struct {
  const orc_job *job;
  const orc_refplan *pl;
  uint32_t m;              /* baby steps = hash_elems */
  int32_t verify;
  const uint32_t *row_ki;  /* job index of each row's k */
  const uint64_t *cand;
  size_t lo, hi;
  fvec out;
} rjob;

/* smallest j < m with B^j == y, from a table of (value, j) with linear probing */
typedef struct {
  uint64_t *key;
  uint32_t *val;
  uint8_t *used;
  uint32_t bits;
} btab;

static void ref_prime(rjob *rj, btab *tb, uint64_t q) {
  const orc_job *job = rj->job;
  const orc_refplan *pl = rj->pl;
  const uint32_t m = rj->m, Q = (uint32_t)pl->minQ;
  mctx c;
  mctx_init(&c, q);
  const uint64_t H = (uint64_t)1 << tb->bits, hmask = H - 1;
  memset(tb->used, 0, H);
  const uint64_t bm = to_m(&c, job->base);
  uint64_t B = c.r1;
  for (uint32_t i = 0; i < Q; i++) B = mmul(&c, B, bm);
  uint64_t v = c.r1;
  for (uint32_t j = 0; j < m; j++) {
    uint64_t h = (v * 0x9E3779B97F4A7C15ull) >> (64 - tb->bits);
    int dup = 0;
    while (tb->used[h]) {
      if (tb->key[h] == v) { dup = 1; break; }
      h = (h + 1) & hmask;
    }
    if (!dup) { tb->used[h] = 1; tb->key[h] = v; tb->val[h] = j; }
    v = mmul(&c, v, B);
  }
  uint64_t c1 = c.r1;
  for (uint32_t j = 0; j < m; j++) c1 = mmul(&c, c1, B);
  uint64_t beta = c.r1;
  for (int32_t t = 0; t < pl->tMin; t++) beta = mmul(&c, beta, c1);
  const int legb = orc_jacobi(job->base, q) == 1;
  int32_t rep_k = -1, rep_n = 0;
  uint32_t lastk = 0;
  int leg1 = 0, leg2 = 0;
  uint64_t fb = 0;
  int32_t prev = 0;
  for (int32_t row = 0; row < pl->minSubs; row++) {
    const uint32_t k = (uint32_t)pl->row_k[row];
    const int32_t r = pl->row_r[row];
    if (row == 0 || k != lastk) {
      leg1 = orc_jacobi(k, q) == 1;
      leg2 = leg1 == legb;
      fb = mmul(&c, to_m(&c, k), beta);
      prev = 0;
    }
    lastk = k;
    if (!(leg1 || leg2)) continue;
    if (!((r % 2 == 0 && leg1) || (r % 2 == 1 && leg2))) continue;
    for (int32_t t = prev; t < r; t++) fb = mmul(&c, fb, bm);
    prev = r;
    uint64_t sB = fb;
    int32_t output = -1;
    for (int32_t t = pl->tMin; t < pl->tMax; t++) {
      sB = mmul(&c, sB, c1);
      uint64_t h = (sB * 0x9E3779B97F4A7C15ull) >> (64 - tb->bits);
      while (tb->used[h]) {
        if (tb->key[h] == sB) { output = (t + 1) * (int32_t)m - (int32_t)tb->val[h]; break; }
        h = (h + 1) & hmask;
      }
    }
    if (output > 0) { rep_k = (int32_t)k; rep_n = output * (int32_t)Q + r; }
  }
  if (rep_k < 0) return;
  const int32_t n = rep_n;
  if (!(n > job->ref_minN - 1 && n < job->ref_maxN + 1)) return;
  if (rj->verify) {
    const int32_t mod = n % (int32_t)Q;
    const int32_t idx = (n - mod) / (int32_t)Q - pl->minimum;
    int32_t row = -1;
    for (int32_t a = 0; a < pl->minSubs; a++)
      if (pl->row_k[a] == rep_k) { row = a; break; }
    if (row < 0) return;
    while (row < pl->minSubs && pl->row_r[row] != mod) row++;
    if (row >= pl->minSubs) return; /* past the reference's matrix: not emulated */
    /* candidate bit idx of that row: n' = (idx + minimum)*Q + r of the row's own k */
    const int64_t n2 = ((int64_t)idx + pl->minimum) * Q + pl->row_r[row];
    if (n2 < 0 || n2 > 0x7fffffff || !has_candidate(job, rj->row_ki[row], (uint32_t)n2)) return;
    if (!orc_verify(q, (uint32_t)rep_k, job->base, (uint32_t)n, -1)) return;
  }
  fpush(&rj->out, q, (uint32_t)rep_k, (uint32_t)n);
}

static void *ref_worker(void *arg) {
  rjob *rj = (rjob *)arg;
  btab tb;
  tb.bits = 1;
  while (((uint64_t)1 << tb.bits) < 2ull * rj->m) tb.bits++;
  const size_t H = (size_t)1 << tb.bits;
  tb.key = (uint64_t *)malloc(H * sizeof(uint64_t));
  tb.val = (uint32_t *)malloc(H * sizeof(uint32_t));
  tb.used = (uint8_t *)malloc(H);
  for (size_t i = rj->lo; i < rj->hi; i++) ref_prime(rj, &tb, rj->cand[i]);
  free(tb.key);
  free(tb.val);
  free(tb.used);
  return NULL;
}

/* Odd q in [lo, hi] with no factor among the first nsmall odd primes. */
static size_t ref_candidates(uint64_t lo, uint64_t hi, const uint32_t *sp, size_t nsp, uint64_t **out) {
  const uint64_t cnt = (hi - lo) / 2 + 1;
  char *mark = (char *)calloc(cnt, 1);
  if (!mark) return 0;
  for (size_t t = 0; t < nsp; t++) {
    const uint64_t q = sp[t];
    uint64_t r = lo % q, f = r ? lo + (q - r) : lo;
    if (!(f & 1)) f += q;
    for (uint64_t x = (f - lo) / 2; x < cnt; x += q) mark[x] = 1;
  }
  size_t n = 0;
  for (uint64_t x = 0; x < cnt; x++) n += !mark[x];
  *out = (uint64_t *)malloc((n ? n : 1) * sizeof(uint64_t));
  size_t w = 0;
  for (uint64_t x = 0; x < cnt; x++)
    if (!mark[x]) (*out)[w++] = lo + 2 * x;
  free(mark);
  return n;
}

int orc_sieve_ref(const orc_job *job, const orc_refplan *pl, int32_t hash_elems, int32_t small_prime_scale,
                  uint64_t p0, uint64_t p1, int32_t verify, int32_t nthreads, orc_factor *out, size_t cap,
                  size_t *count, uint64_t *ncand) {
  *count = 0;
  if (ncand) *ncand = 0;
  if (job->sign != -1 || hash_elems < 1 || small_prime_scale < 1 || pl->minSubs < 1) return 1;
  uint32_t kmax = 0;
  for (uint32_t i = 0; i < job->nk; i++)
    if (job->k[i] > kmax) kmax = job->k[i];
  uint64_t lo = p0 % 2 ? p0 : p0 - 1; /* the reference moves an even low down by one */
  if (lo <= job->base || lo <= kmax || p1 >= ((uint64_t)1 << 63) || p1 < lo) return 1;
  /* the first 4096*s odd primes */
  const size_t want = (size_t)4096 * (size_t)small_prime_scale;
  const double lw = log((double)want + 10.0);
  size_t nsp = 0;
  uint32_t *sp = small_primes((uint64_t)((double)want * (lw + log(lw)) + 1000.0), &nsp);
  if (nsp > want) nsp = want;
  uint64_t *cand = NULL;
  const size_t nc = ref_candidates(lo, p1, sp, nsp, &cand);
  free(sp);
  if (ncand) *ncand = nc;
  uint32_t *row_ki = (uint32_t *)malloc((size_t)pl->minSubs * sizeof(uint32_t));
  for (int32_t a = 0; a < pl->minSubs; a++) {
    row_ki[a] = 0;
    for (uint32_t i = 0; i < job->nk; i++)
      if ((int32_t)job->k[i] == pl->row_k[a]) { row_ki[a] = i; break; }
  }
  int nt = nthreads > 0 ? nthreads : orc_default_threads();
  if ((size_t)nt > nc) nt = nc ? (int)nc : 1;
  rjob *rj = (rjob *)calloc(nt, sizeof(rjob));
  pthread_t *th = (pthread_t *)calloc(nt, sizeof(pthread_t));
  for (int t = 0; t < nt; t++) {
    rj[t].job = job;
    rj[t].pl = pl;
    rj[t].m = (uint32_t)hash_elems;
    rj[t].verify = verify;
    rj[t].row_ki = row_ki;
    rj[t].cand = cand;
    rj[t].lo = nc * (size_t)t / nt;
    rj[t].hi = nc * (size_t)(t + 1) / nt;
    pthread_create(&th[t], NULL, ref_worker, &rj[t]);
  }
  size_t total = 0;
  for (int t = 0; t < nt; t++) {
    pthread_join(th[t], NULL);
    total += rj[t].out.cnt;
  }
  orc_factor *all = (orc_factor *)malloc((total ? total : 1) * sizeof(orc_factor));
  size_t pos = 0;
  for (int t = 0; t < nt; t++) {
    for (size_t i = 0; i < rj[t].out.cnt; i++) all[pos++] = rj[t].out.v[i];
    free(rj[t].out.v);
  }
  qsort(all, total, sizeof(orc_factor), cmp_factor);
  for (size_t i = 0; i < total && i < cap; i++) out[i] = all[i];
  *count = total;
  free(all);
  free(rj);
  free(th);
  free(cand);
  free(row_ki);
  return 0;
}
