// rsieve -- command-line drop-in for the reference sieve executable.
//
// Same flags as rob147147/CUDA-Riesel-Sieve kernel_v0.24.6.cu:705-786
// (-i -p -P -b -t -m -Q -s -O -v -h), same factor-file format
// ("%llu | %d*%d^%d-1", kernel_v0.24.6.cu:1833), progress every 20 launches
// (kernel_v0.24.6.cu:1757-1761) and the final "Progress = W at X p/sec" line
// (kernel_v0.24.6.cu:1783).  All the work goes through the C ABI in
// include/rsieve.h; this file only parses flags and prints.
#include <getopt.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "rsieve.h"

static void usage() {
  printf("\nrsieve (GB300) -- a sieve for sequences k*b^n-1 (and k*b^n+1)\n\n");
  printf("-i FILE  : Read in abcd sieve file called FILE (default sr_745.abcd).\n");
  printf("-m M     : Use at most 2<<M baby steps per prime (default: chosen per job).\n");
  printf("-p P0    : Start sieving from P0. Must have a corresponding P1.\n");
  printf("-P P1    : Finish sieving at P1 (inclusive).\n");
  printf("           With neither -p nor -P the range starts at 102297149770000.\n");
  printf("-Q Q     : Use subsequence modulus Q (even). Default: chosen per job.\n");
  printf("-O FILE  : Append factors to FILE (default factors.txt).\n");
  printf("-b SCALE : Primes per launch = 128*2^(b-1) * 128*2^(t-1).\n");
  printf("-t SCALE : (see -b).\n");
  printf("-s SCALE : Accepted for compatibility; the device sieve is always complete.\n");
  printf("-v [X]   : Don't verify: report every n in [nmin,nmax] (datless).\n");
  printf("-w FILE  : After sieving, write FILE: the input ABCD without the candidates whose\n");
  printf("           factors are in the factor file, headers marked \"// Sieved to P1\".\n");
  printf("-A       : Autotune: time the cheapest plans of the cost model on the first part of the\n");
  printf("           range and keep the fastest (replaces hand-tuning -Q/-m/-b/-t).\n");
  printf("-C FILE  : Checkpoint: resume from the p recorded in FILE (if it is for the same\n");
  printf("           input file contents, P0 and P1) and record progress there after every\n");
  printf("           block of launches.\n");
  printf("-h [X]   : Prints this help\n");
}

// FNV-1a hash of the input text: a checkpoint is only resumed for the same contents.
static unsigned long long text_hash(const std::string &t) {
  unsigned long long h = 1469598103934665603ull;
  for (unsigned char c : t) {
    h ^= c;
    h *= 1099511628211ull;
  }
  return h;
}

int main(int argc, char **argv) {
  const char *abcd = "sr_745.abcd";
  const char *factor_file = "factors.txt";
  unsigned long long low = 0, high = 0;
  rs_options opt;
  rs_options_default(&opt);
  int block_scale = 1, thread_scale = 1;
  bool scale_given = false;
  int inp;
  const char *abcd_out = nullptr, *ckpt = nullptr;
  bool autotune = false;
  // -h and -v take an argument in the reference's getopt string ("h:", "v:",
  // kernel_v0.24.6.cu:705) whose value is not used; here it is optional, attached
  // (-v1) or as the next word when that is not an option (-v 1).
  auto skip_optional_arg = [&]() {
    if (!optarg && optind < argc && argv[optind][0] != '-') optind++;
  };
  while ((inp = getopt(argc, argv, "Ab:h::i:m:p:P:Q:O:s:t:v::w:C:")) != -1) {
    switch (inp) {
      case 'b': block_scale = (int)strtol(optarg, nullptr, 0); scale_given = true; break;
      case 't': thread_scale = (int)strtol(optarg, nullptr, 0); scale_given = true; break;
      case 'h': usage(); return 0;
      case 'i': abcd = optarg; break;
      case 'm': opt.hash_m = (int)strtol(optarg, nullptr, 0); break;
      case 'p': low = strtoull(optarg, nullptr, 0); break;
      case 'P': high = strtoull(optarg, nullptr, 0); break;
      case 'Q': {
        int q = (int)strtol(optarg, nullptr, 0);
        if (q < 1 || q % 2 == 1) {
          printf("Bad input parameter : Q must be an even integer greater than 0.\n");
          return 1;
        }
        opt.Q = q;
        break;
      }
      case 'O': factor_file = optarg; break;
      case 's': opt.small_prime_scale = (int)strtol(optarg, nullptr, 0); break;
      case 'v':
        skip_optional_arg();
        opt.datless = 1;
        opt.host_verify = 1;
        break;
      case 'w': abcd_out = optarg; break;
      case 'C': ckpt = optarg; break;
      case 'A': autotune = true; break;
      default: return 0;
    }
  }
  if (block_scale < 1 || block_scale > 31) {
    printf("Bad input parameter : 1 < BlockScale < 32.\n");
    return 1;
  }
  if (thread_scale < 1 || thread_scale > 31) {
    printf("Bad input parameter : 1 < ThreadScale < 32.\n");
    return 1;
  }
  if (scale_given) {
    opt.block_scale = block_scale;
    opt.thread_scale = thread_scale;
  }
  if (low == 0 && high == 0) {
    low = 102297149770000ull;
    high = low + 2500000ull * (1ull << (block_scale - 1)) * (1ull << (thread_scale - 1));
  }
  if (high < low) {
    printf("Bad input parameters : P1 < P0. We want to sieve primes p in the range P0 <= p <= P1.\n");
    return 1;
  }
  printf("Low = %llu\nHigh = %llu\nQ_In = %d\nABCD = %s\nFactorFile = %s\n%s\n\n", low, high, opt.Q, abcd,
         factor_file, rs_version());

  FILE *fp = fopen(abcd, "rb");
  if (!fp) {
    printf("Unable to open file %s\n", abcd);
    return 1;
  }
  std::string text;
  {
    char buf[1 << 16];
    size_t r;
    while ((r = fread(buf, 1, sizeof(buf), fp)) > 0) text.append(buf, r);
    fclose(fp);
  }
  rs_job *job = nullptr;
  int rc = rs_job_create_abcd(text.data(), text.size(), &opt, &job);
  if (rc) {
    fprintf(stderr, "error: %s\n", rs_last_error());
    return 1;
  }
  rs_job_info info;
  rs_job_info_get(job, &info);
  if (info.parts > 1)
    printf("%u (base, sign) groups; the first: base %u; %u k-values and %u candidates in all\n", info.parts,
           info.base, info.num_k, info.num_candidates);
  else
    printf("The base is %u; %u k-values, %u candidates, n in [%u, %u]\n", info.base, info.num_k,
           info.num_candidates, info.nmin, info.nmax);
  printf("Q=%u. Rows=%u. Range=%u. Baby steps=%u. Giant steps=%u. Table slots=%u. Primes per launch=%u\n\n",
         info.Q, info.rows, info.x_range, info.baby_steps, info.giant_steps, info.table_slots,
         info.primes_per_launch);

  if (autotune) {
    // a sample of about four launches' worth of primes at the start of the range
    const double lp = std::log((double)std::max(low, 16ull));
    const unsigned long long w = (unsigned long long)(4.0 * info.primes_per_launch * lp);
    const unsigned long long hi = (high - low < w) ? high : low + w - 1;
    rc = rs_job_autotune(job, low, hi, 3, &info);
    if (rc) {
      fprintf(stderr, "error: %s\n", rs_last_error());
      rs_job_destroy(job);
      return 1;
    }
    printf("Autotuned on [%llu, %llu]: Q=%u. Baby steps=%u. Giant steps=%u. Warps per prime=%u\n\n", low, hi,
           info.Q, info.baby_steps, info.giant_steps, info.warps_per_prime);
  }

  // Resume from a checkpoint of the same input (path and contents), P0 and P1.
  unsigned long long p = low;
  const unsigned long long in_hash = text_hash(text);
  if (ckpt) {
    if (FILE *cf = fopen(ckpt, "r")) {
      char line[4096];
      unsigned long long next = 0, chigh = 0, clow = 0, chash = 0;
      std::string cin;
      while (fgets(line, sizeof(line), cf)) {
        if (!strncmp(line, "next_p=", 7)) next = strtoull(line + 7, nullptr, 10);
        else if (!strncmp(line, "high=", 5)) chigh = strtoull(line + 5, nullptr, 10);
        else if (!strncmp(line, "low=", 4)) clow = strtoull(line + 4, nullptr, 10);
        else if (!strncmp(line, "abcd_hash=", 10)) chash = strtoull(line + 10, nullptr, 16);
        else if (!strncmp(line, "abcd=", 5)) {
          cin = line + 5;
          while (!cin.empty() && (cin.back() == '\n' || cin.back() == '\r')) cin.pop_back();
        }
      }
      fclose(cf);
      if (chigh == high && clow == low && cin == abcd && chash == in_hash && next > p) {
        printf("Resuming from checkpoint %s at p=%llu\n", ckpt, next);
        p = next;
      } else {
        printf("Checkpoint %s is for another input, range or file contents: starting at P0\n", ckpt);
      }
    }
  }
  auto save_ckpt = [&](unsigned long long next) {
    if (!ckpt) return;
    std::string tmp = std::string(ckpt) + ".tmp";
    FILE *cf = fopen(tmp.c_str(), "w");
    if (!cf) return;
    fprintf(cf, "next_p=%llu\nlow=%llu\nhigh=%llu\nabcd_hash=%016llx\nabcd=%s\n", next, low, high, in_hash, abcd);
    fclose(cf);
    rename(tmp.c_str(), ckpt);
  };

  // Progress granularity: ~20 launches' worth of primes per call.
  const auto t_start = std::chrono::high_resolution_clock::now();
  unsigned long long total_factors = 0;
  std::vector<rs_factor> out(1 << 16);
  while (p <= high) {
    const double lp = std::log((double)std::max(p, 16ull));
    unsigned long long width = (unsigned long long)(20.0 * info.primes_per_launch * lp * 0.8);
    if (width < 1000) width = 1000;
    const unsigned long long q = (high - p < width) ? high : p + width - 1;
    const auto t0 = std::chrono::high_resolution_clock::now();
    size_t cnt = 0;
    rs_stats st;
    rc = rs_sieve_range(job, p, q, out.data(), out.size(), &cnt, &st);
    if (rc == RS_ERR_CAPACITY) {
      out.resize(cnt);
      rc = rs_sieve_range(job, p, q, out.data(), out.size(), &cnt, &st);
    }
    if (rc) {
      fprintf(stderr, "error: %s\n", rs_last_error());
      rs_job_destroy(job);
      return 1;
    }
    for (size_t i = 0; i < cnt; i++)
      printf("%llu | %u*%u^%u%s\n", (unsigned long long)out[i].p, out[i].k, out[i].b, out[i].n,
             out[i].c < 0 ? "-1" : "+1");
    if (cnt && rs_write_factors(job, factor_file, out.data(), cnt)) {
      fprintf(stderr, "error: %s\n", rs_last_error());
      rs_job_destroy(job);
      return 1;
    }
    total_factors += cnt;
    save_ckpt(q + 1);
    const auto t1 = std::chrono::high_resolution_clock::now();
    const double dt = std::chrono::duration<double>(t1 - t0).count();
    const double so_far = std::chrono::duration<double>(t1 - t_start).count();
    const double pct = 100.0 * (double)(q - low + 1) / (double)(high - low + 1);
    const double left = pct > 0 ? so_far * (100.0 / pct) - so_far : 0;
    time_t eta = time(nullptr) + (time_t)left;
    char etas[64];
    strftime(etas, sizeof(etas), "%a %b %d %H:%M:%S %Y", localtime(&eta));
    printf("p=%llu, %.0f p/sec,  %.2f%% done, %llu factors found, ETA %s \n", q + 1,
           (double)(q - p + 1) / dt, pct, total_factors, etas);
    fflush(stdout);
    if (q == high) break;
    p = q + 1;
  }
  if (p > high) save_ckpt(high + 1);
  const double total = std::chrono::duration<double>(std::chrono::high_resolution_clock::now() - t_start).count();
  printf("\nTime taken: %gs\n", total);
  printf("Factors found: %llu\n", total_factors);
  printf("Progress = %llu at %.0f p/sec\n\n", high - low + 1, (double)(high - low + 1) / total);
  rs_job_destroy(job);

  if (abcd_out) {
    // every factor line of the factor file (each names its sequence's base and sign)
    std::vector<rs_factor> rm;
    if (FILE *ff = fopen(factor_file, "r")) {
      unsigned long long fp;
      unsigned fk, fb, fn;
      char sg;
      char line[256];
      while (fgets(line, sizeof(line), ff))
        if (sscanf(line, "%llu | %u*%u^%u%c1", &fp, &fk, &fb, &fn, &sg) == 5 && (sg == '-' || sg == '+'))
          rm.push_back(rs_factor{fp, fk, fn, fb, sg == '-' ? -1 : 1});
      fclose(ff);
    }
    size_t need = 0;
    std::string out(text.size() + 4096 + 64 * (size_t)info.num_k, '\0');
    rc = rs_abcd_remove(text.data(), text.size(), rm.data(), rm.size(), high, &out[0], out.size(), &need);
    if (rc == RS_ERR_CAPACITY) {
      out.resize(need);
      rc = rs_abcd_remove(text.data(), text.size(), rm.data(), rm.size(), high, &out[0], out.size(), &need);
    }
    FILE *wf = rc ? nullptr : fopen(abcd_out, "w");
    if (!wf || fwrite(out.data(), 1, need, wf) != need) {
      fprintf(stderr, "error writing %s: %s\n", abcd_out, rc ? rs_last_error() : "I/O error");
      if (wf) fclose(wf);
      return 1;
    }
    fclose(wf);
    printf("Wrote %s: %zu candidates removed\n", abcd_out, rm.size());
  }
  return 0;
}
