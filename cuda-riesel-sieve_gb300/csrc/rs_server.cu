// rs_server.cu -- the served form: jobs submitted while others run are admitted
// as device memory and slots free up, and their work overlaps on the GPU.
//
// The reference runs one job per process: parse, plan, then the
// H2D -> addKernel1 -> D2H loop (kernel_v0.24.6.cu:688-1835).  Here a server
// owns one device and `slots` worker threads.
//
// Admission is by device memory.  At submit the job's footprint is computed
// on the host (parse and plan, no device work): its arrays (rows, per-k data,
// candidate bitmaps, character tables) plus its per-launch buffers, whose
// chunk size follows the job's own p-window (a narrow window gets small
// chunks).  A free worker admits the oldest waiting job when its footprint
// fits the budget next to the running jobs; a job larger than the whole
// budget runs when nothing else does.  Waiting behind the oldest job keeps
// admission first-come first-served.
//
// Job state stays resident.  A finished job releases its per-launch buffers
// but keeps its arrays on the device, keyed by its ABCD text and options; a
// later request for the same job (another p-window) takes it over and skips
// parsing, planning and upload.  Idle resident jobs count against the budget
// and are evicted, least recently used first, when an admission needs room or
// more than `cache_jobs` are idle.
//
// Each job runs exactly the kernels it would run alone on the same inputs, so
// its factors equal those of a standalone rs_sieve_range call.
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "rs_internal.h"
#include "rsieve.h"

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

// FNV-1a over the ABCD text and the options that shape the job on the device.
uint64_t job_key(const char *text, size_t len, const rs_options &o) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](const void *p, size_t n) {
    const unsigned char *c = static_cast<const unsigned char *>(p);
    for (size_t i = 0; i < n; i++) {
      h ^= c[i];
      h *= 1099511628211ull;
    }
  };
  mix(text, len);
  const int32_t f[6] = {o.Q, o.hash_m, o.datless, o.baby_step, o.block_scale, o.thread_scale};
  mix(f, sizeof(f));
  return h;
}

struct ServedJob {
  uint64_t ticket = 0;
  uint64_t key = 0;
  std::string abcd;
  rs_options opt{};
  uint64_t p0 = 0, p1 = 0;
  uint64_t mem_limit = 0;  // chunk-buffer budget of this request
  uint64_t need = 0;       // device bytes charged while it runs
  uint64_t mem_in_use = 0; // charged bytes of all running jobs just after its admission
  bool resident = false;   // its arrays were taken over from an earlier request
  double create_ms = 0;
  Clock::time_point t_submit, t_start, t_end;
  bool done = false;
  int status = RS_OK;
  std::string err;
  std::vector<rs_factor> factors;
  rs_stats st{};
};

struct Resident {
  uint64_t key;
  rs_job *job;
  uint64_t bytes;  // device bytes of its arrays
};

}  // namespace

struct rs_server {
  rs_server_options opt{};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<ServedJob>> waiting;
  std::unordered_map<uint64_t, std::shared_ptr<ServedJob>> jobs;  // submitted and not yet collected
  std::unordered_map<uint64_t, rs::JobFootprint> seen;           // footprints by job key
  std::list<Resident> idle;  // resident jobs not running, least recently used first
  uint64_t idle_bytes = 0;
  uint64_t in_use = 0;       // bytes charged to running jobs
  uint32_t running = 0;
  uint64_t next_ticket = 1;
  bool stop = false;
  std::vector<std::thread> workers;
};

namespace {

// The oldest waiting job if it can start now; evicted resident jobs are
// appended to `evict` (destroyed by the caller outside the lock) and a
// resident copy of the job, if any, is moved to `take`.
std::shared_ptr<ServedJob> try_admit(rs_server &S, std::vector<rs_job *> &evict, rs_job *&take) {
  if (S.waiting.empty()) return nullptr;
  std::shared_ptr<ServedJob> J = S.waiting.front();
  auto res = S.idle.end();
  for (auto it = S.idle.begin(); it != S.idle.end(); ++it)
    if (it->key == J->key) res = it;  // the most recently used copy
  const uint64_t have = res != S.idle.end() ? res->bytes : 0;
  const uint64_t need_new = J->need > have ? J->need - have : 0;
  const uint64_t others = S.idle_bytes - have;
  const uint64_t budget = S.opt.mem_budget;
  const uint64_t room = budget > S.in_use + S.idle_bytes ? budget - S.in_use - S.idle_bytes : 0;
  if (S.running > 0 && need_new > room + others) return nullptr;
  // admit: take the resident copy, then evict the least recently used others
  // until the charged bytes fit the budget (or nothing is left to evict)
  if (res != S.idle.end()) {
    take = res->job;
    S.idle_bytes -= res->bytes;
    S.idle.erase(res);
  }
  S.waiting.pop_front();
  S.in_use += J->need;
  while (!S.idle.empty() && S.in_use + S.idle_bytes > budget) {
    evict.push_back(S.idle.front().job);
    S.idle_bytes -= S.idle.front().bytes;
    S.idle.pop_front();
  }
  S.running++;
  J->mem_in_use = S.in_use;
  return J;
}

rs_job *run_job(const rs_server &S, ServedJob &J, rs_job *job) {
  if (job) {
    J.resident = true;
    rs::job_set_mem_limit(job, J.mem_limit);
  } else {
    rs_options o = J.opt;
    o.device = S.opt.device;
    o.mem_limit = J.mem_limit;
    o.block_scale = o.thread_scale = 0;
    const auto t0 = Clock::now();
    const int rc = rs_job_create_abcd(J.abcd.data(), J.abcd.size(), &o, &job);
    J.create_ms = ms_between(t0, Clock::now());
    if (rc) {
      J.status = rc;
      J.err = rs_last_error();
      return nullptr;
    }
  }
  std::vector<rs_factor> out(1 << 16);
  size_t cnt = 0;
  int rc = rs_sieve_range(job, J.p0, J.p1, out.data(), out.size(), &cnt, &J.st);
  if (rc == RS_ERR_CAPACITY) {  // rare: more than 65536 factors; run again into a large enough buffer
    out.resize(cnt);
    rc = rs_sieve_range(job, J.p0, J.p1, out.data(), out.size(), &cnt, &J.st);
  }
  if (rc) {
    J.status = rc;
    J.err = rs_last_error();
  } else {
    J.factors.assign(out.begin(), out.begin() + cnt);
  }
  rs::job_release_buffers(job);
  return job;
}

void worker_main(rs_server *S) {
  cudaSetDevice(S->opt.device);
  for (;;) {
    std::shared_ptr<ServedJob> J;
    std::vector<rs_job *> evict;
    rs_job *job = nullptr;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_work.wait(lk, [&] { return S->stop || (J = try_admit(*S, evict, job)) != nullptr; });
      if (S->stop && !J) return;
    }
    for (rs_job *e : evict) rs_job_destroy(e);
    J->t_start = Clock::now();
    job = run_job(*S, *J, job);
    J->t_end = Clock::now();
    const uint64_t bytes = job ? rs::job_resident_bytes(job) : 0;
    std::vector<rs_job *> drop;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->in_use -= J->need;
      S->running--;
      if (job) {
        if (S->stop) {
          drop.push_back(job);
        } else {
          S->idle.push_back(Resident{J->key, job, bytes});
          S->idle_bytes += bytes;
          while (S->idle.size() > S->opt.cache_jobs ||
                 (!S->idle.empty() && S->in_use + S->idle_bytes > S->opt.mem_budget)) {
            drop.push_back(S->idle.front().job);
            S->idle_bytes -= S->idle.front().bytes;
            S->idle.pop_front();
          }
        }
      }
      J->done = true;
    }
    for (rs_job *e : drop) rs_job_destroy(e);
    S->cv_done.notify_all();
    S->cv_work.notify_all();  // memory came free
  }
}

}  // namespace

extern "C" void rs_server_options_default(rs_server_options *opt) {
  if (!opt) return;
  *opt = rs_server_options{};
  opt->slots = 4;
  opt->queue_cap = 1024;
  opt->cache_jobs = 64;
  opt->mem_budget = 64ull << 30;
}

extern "C" int rs_server_create(const rs_server_options *optp, rs_server **out) {
  if (!out) return rs::set_error(RS_ERR_INVALID, "rs_server_create: server pointer is NULL");
  *out = nullptr;
  rs_server_options opt;
  rs_server_options_default(&opt);
  if (optp) {
    opt.device = optp->device;
    if (optp->slots) opt.slots = optp->slots;
    if (optp->queue_cap) opt.queue_cap = optp->queue_cap;
    if (optp->cache_jobs) opt.cache_jobs = optp->cache_jobs;
    if (optp->mem_budget) opt.mem_budget = optp->mem_budget;
  }
  if (opt.slots > 64) return rs::set_error(RS_ERR_INVALID, "rs_server_create: at most 64 slots");
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n <= 0)
    return rs::set_error(RS_ERR_NODEVICE, "no CUDA device available; this library has no CPU path");
  if (opt.device < 0 || opt.device >= n) return rs::set_error(RS_ERR_INVALID, "device %d out of range", opt.device);
  e = cudaSetDevice(opt.device);
  if (e == cudaSuccess) {
    // Keep freed job buffers in the device's stream-ordered pool (up to the
    // budget) so that the next job's allocations are served from it.  This is
    // a property of this process's pool, not a device setting.
    cudaMemPool_t pool;
    e = cudaDeviceGetDefaultMemPool(&pool, opt.device);
    uint64_t thr = opt.mem_budget;
    if (e == cudaSuccess) e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  if (e != cudaSuccess) return rs::set_error(RS_ERR_CUDA, "rs_server_create: %s", cudaGetErrorString(e));
  rs_server *S = new rs_server();
  S->opt = opt;
  for (uint32_t i = 0; i < opt.slots; i++) S->workers.emplace_back(worker_main, S);
  *out = S;
  return RS_OK;
}

extern "C" int rs_server_submit(rs_server *S, const char *abcd, size_t len, const rs_options *opt, uint64_t p0,
                                uint64_t p1, uint64_t *ticket) {
  if (!S || !abcd || !ticket) return rs::set_error(RS_ERR_INVALID, "rs_server_submit: NULL argument");
  auto J = std::make_shared<ServedJob>();
  J->abcd.assign(abcd, len);
  if (opt) J->opt = *opt;
  else rs_options_default(&J->opt);
  J->p0 = p0;
  J->p1 = p1;
  J->t_submit = Clock::now();
  J->key = job_key(abcd, len, J->opt);
  // the job's footprint: from an earlier request of the same job, else a
  // host-only parse and plan (a malformed job is refused here)
  rs::JobFootprint fp;
  bool known = false;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->seen.find(J->key);
    if (it != S->seen.end()) {
      fp = it->second;
      known = true;
    }
  }
  if (!known) {
    const int rc = rs::job_footprint(abcd, len, J->opt, &fp);
    if (rc) return rc;
  }
  // per-launch buffers sized for this window's primes (at most the per-slot
  // share of the budget and 2 GiB), then the hit buffers and window bitmap
  const double lp = std::log((double)(p0 > 16 ? p0 : 16));
  const double width = p1 >= p0 ? (double)(p1 - p0) + 1.0 : 1.0;
  const double primes = width / std::max(1.0, lp - 1.2) + 4096.0;
  const uint64_t share = std::min<uint64_t>(S->opt.mem_budget / S->opt.slots, 2ull << 30);
  uint64_t cap = (uint64_t)std::min<double>(1.25 * primes, (double)(share / fp.per_prime));
  cap = std::max<uint64_t>(cap, 4096);
  J->mem_limit = cap * fp.per_prime;
  const uint64_t hits = (uint64_t)fp.parts * ((fp.parts == 1 ? 1u << 20 : 1u << 16) * 2 * 16 + 4096);
  const uint64_t gbits = (uint64_t)(0.8 * (double)cap * (lp > 3 ? lp : 3) / 16.0) + (1u << 20);
  J->need = fp.arrays + J->mem_limit + hits + gbits;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return rs::set_error(RS_ERR_INVALID, "rs_server_submit: server is shutting down");
    if (S->waiting.size() >= S->opt.queue_cap)
      return rs::set_error(RS_ERR_BUSY, "rs_server_submit: %u jobs already waiting", S->opt.queue_cap);
    S->seen[J->key] = fp;
    J->ticket = S->next_ticket++;
    S->waiting.push_back(J);
    S->jobs[J->ticket] = J;
    *ticket = J->ticket;
  }
  S->cv_work.notify_all();
  return RS_OK;
}

extern "C" int rs_server_wait(rs_server *S, uint64_t ticket, int32_t timeout_ms, rs_factor *out, size_t cap,
                              size_t *count, rs_job_report *report) {
  if (!S || !count || (!out && cap)) return rs::set_error(RS_ERR_INVALID, "rs_server_wait: NULL argument");
  std::shared_ptr<ServedJob> J;
  {
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->jobs.find(ticket);
    if (it == S->jobs.end()) return rs::set_error(RS_ERR_INVALID, "rs_server_wait: unknown ticket %llu",
                                                  (unsigned long long)ticket);
    J = it->second;
    auto ready = [&] { return J->done; };
    if (timeout_ms < 0) {
      S->cv_done.wait(lk, ready);
    } else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
      return rs::set_error(RS_ERR_TIMEOUT, "rs_server_wait: job %llu still running", (unsigned long long)ticket);
    }
    *count = J->factors.size();
    if (J->status == RS_OK && J->factors.size() > cap)
      return rs::set_error(RS_ERR_CAPACITY, "rs_server_wait: %zu factors, buffer holds %zu", J->factors.size(), cap);
    S->jobs.erase(it);
  }
  if (J->status == RS_OK && !J->factors.empty()) memcpy(out, J->factors.data(), J->factors.size() * sizeof(rs_factor));
  if (report) {
    *report = rs_job_report{};
    report->status = J->status;
    report->resident = J->resident ? 1u : 0u;
    report->primes = J->st.primes;
    report->factors = J->factors.size();
    report->p_covered = J->st.p_covered;
    report->queue_ms = ms_between(J->t_submit, J->t_start);
    report->run_ms = ms_between(J->t_start, J->t_end);
    report->latency_ms = ms_between(J->t_submit, J->t_end);
    report->gpu_ms = J->st.gpu_ms;
    report->create_ms = J->create_ms;
    report->mem_bytes = J->need;
    report->mem_in_use = J->mem_in_use;
  }
  if (J->status != RS_OK) return rs::set_error(J->status, "%s", J->err.c_str());
  return RS_OK;
}

extern "C" int rs_server_destroy(rs_server *S) {
  if (!S) return RS_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    S->waiting.clear();
  }
  S->cv_work.notify_all();
  for (auto &t : S->workers) t.join();
  for (auto &r : S->idle) rs_job_destroy(r.job);
  S->idle.clear();
  delete S;
  return RS_OK;
}
