// rs_server.cu -- the served form: jobs submitted while others run are admitted
// to free slots and overlap on the GPU.
//
// The reference runs one job per process: parse, plan, then the
// H2D -> addKernel1 -> D2H loop (kernel_v0.24.6.cu:688-1835).  Here a server
// owns one device and `slots` worker threads.  A worker takes the oldest
// waiting job, creates it (parse, plan, upload: rs_job_create_abcd), sieves its
// range on the job's own stream (rs_sieve_range) and releases it, so kernels
// of up to `slots` jobs are in flight together.  Device memory is partitioned:
// a running job's per-launch buffers are limited to mem_budget / slots (and
// the 2 GiB default), job buffers come from the stream-ordered pool, and the
// sieving primes are shared by all jobs on the device.  Each job runs exactly
// the kernels it would run alone, on the same inputs, so its factors are the
// same as in a standalone rs_sieve_range call.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
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

struct ServedJob {
  uint64_t ticket = 0;
  std::string abcd;
  rs_options opt{};
  uint64_t p0 = 0, p1 = 0;
  Clock::time_point t_submit, t_start, t_end;
  bool done = false;
  int status = RS_OK;
  std::string err;
  std::vector<rs_factor> factors;
  rs_stats st{};
};

}  // namespace

struct rs_server {
  rs_server_options opt{};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<ServedJob>> waiting;
  std::unordered_map<uint64_t, std::shared_ptr<ServedJob>> jobs;  // submitted and not yet collected
  uint64_t next_ticket = 1;
  bool stop = false;
  std::vector<std::thread> workers;
};

namespace {

void run_job(const rs_server &S, ServedJob &J) {
  rs_options o = J.opt;
  o.device = S.opt.device;
  const uint64_t share = S.opt.mem_budget / S.opt.slots;
  o.mem_limit = share < (2ull << 30) ? share : (2ull << 30);
  rs_job *job = nullptr;
  int rc = rs_job_create_abcd(J.abcd.data(), J.abcd.size(), &o, &job);
  if (rc) {
    J.status = rc;
    J.err = rs_last_error();
    return;
  }
  std::vector<rs_factor> out(1 << 16);
  size_t cnt = 0;
  rc = rs_sieve_range(job, J.p0, J.p1, out.data(), out.size(), &cnt, &J.st);
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
  rs_job_destroy(job);
}

void worker_main(rs_server *S) {
  cudaSetDevice(S->opt.device);
  for (;;) {
    std::shared_ptr<ServedJob> J;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_work.wait(lk, [&] { return S->stop || !S->waiting.empty(); });
      if (S->stop) return;
      J = S->waiting.front();
      S->waiting.pop_front();
    }
    J->t_start = Clock::now();
    run_job(*S, *J);
    J->t_end = Clock::now();
    {
      std::lock_guard<std::mutex> lk(S->mu);
      J->done = true;
    }
    S->cv_done.notify_all();
  }
}

}  // namespace

extern "C" void rs_server_options_default(rs_server_options *opt) {
  if (!opt) return;
  *opt = rs_server_options{};
  opt->slots = 4;
  opt->queue_cap = 1024;
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
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return rs::set_error(RS_ERR_INVALID, "rs_server_submit: server is shutting down");
    if (S->waiting.size() >= S->opt.queue_cap)
      return rs::set_error(RS_ERR_BUSY, "rs_server_submit: %u jobs already waiting", S->opt.queue_cap);
    J->ticket = S->next_ticket++;
    S->waiting.push_back(J);
    S->jobs[J->ticket] = J;
    *ticket = J->ticket;
  }
  S->cv_work.notify_one();
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
    report->primes = J->st.primes;
    report->factors = J->factors.size();
    report->p_covered = J->st.p_covered;
    report->queue_ms = ms_between(J->t_submit, J->t_start);
    report->run_ms = ms_between(J->t_start, J->t_end);
    report->latency_ms = ms_between(J->t_submit, J->t_end);
    report->gpu_ms = J->st.gpu_ms;
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
  delete S;
  return RS_OK;
}
