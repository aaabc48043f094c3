// serve.cu -- request loop with continuous batching for TSMTTSM / TSMM / SVQB (no counterpart in
// the reference, whose drivers call one launcher at a time on the legacy stream, test.cu:114-143,
// perf.cu:64-96).
//
// One worker thread owns the schedule:
//   * requests wait in arrival order; the head is admitted when its device bytes fit the budget
//     (bytes in use + need <= budget) and an in-flight slot is free;
//   * an admitted request gets stream-ordered device buffers (cudaMallocAsync from the device's
//     pool, kept warm by a high release threshold), its inputs are uploaded, the product runs and
//     the result is downloaded, all on one of the server's streams (round-robin), followed by a
//     completion event -- requests in flight on different streams overlap on the device;
//   * completions are retired by polling their events; retiring frees the buffers (stream-ordered)
//     and returns their bytes to the budget, which admits the next requests while others run;
//   * requests on operands resident in HBM (device flag) skip the buffers and copies: their
//     operand bytes count against the budget while they run, and the product runs in place.
// Dry mode (no handle) replaces the device work by a delay proportional to the request's bytes so
// the admission, ticket and accounting logic can be exercised without a GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "api_internal.h"

namespace skinny {
namespace serve {

using clk = std::chrono::steady_clock;

struct Job {
  uint64_t ticket = 0;
  skinny_request r{};
  size_t bA = 0, bB = 0, bC = 0;  // device bytes per operand (0 = shared with another)
  size_t need = 0;
  double alg_bytes = 0;
  clk::time_point t_submit, t_dry_end;
  void *dA = nullptr, *dB = nullptr, *dC = nullptr;
  cudaEvent_t done = nullptr;
  cudaStream_t stream = nullptr;
  skinny_status status = SKINNY_OK;
};

struct Result {
  skinny_status status;
  double latency_us;
};

static size_t esize(skinny_dtype dt) { return dtype_size(dt); }
static size_t r256(size_t b) { return (b + 255) & ~(size_t)255; }

// device bytes and algorithmic bytes (perf.cu:208-232) of a request
static bool plan_job(Job& j) {
  const skinny_request& r = j.r;
  const size_t s = esize(r.dtype);
  if (s == 0 || r.M < 1 || r.K < 0 || (r.op != SKINNY_OP_SVQB && r.N < 1)) return false;
  if (r.op == SKINNY_OP_TSMTTSM) {
    const bool gram = r.A == r.B && r.lda == r.ldb && r.M == r.N;
    j.bA = r256((size_t)r.K * r.lda * s);
    j.bB = gram ? 0 : r256((size_t)r.K * r.ldb * s);
    j.bC = r256((size_t)r.N * r.ldc * s);
    j.alg_bytes = (double)(r.M + (gram ? 0 : r.N)) * r.K * s;
  } else if (r.op == SKINNY_OP_TSMM) {
    const bool inplace = r.A == (const void*)r.C && r.lda == r.ldc;
    j.bA = r256((size_t)r.K * r.lda * s);
    j.bB = r256((size_t)r.N * r.ldb * s);
    j.bC = inplace ? 0 : r256((size_t)r.K * r.ldc * s);
    const bool bz = r.beta[0] == 0.0 && r.beta[1] == 0.0;
    j.alg_bytes = (double)(r.M * r.K + (bz || inplace ? 1 : 2) * r.N * r.K + r.M * r.N) * s;
  } else if (r.op == SKINNY_OP_SVQB) {
    if (r.dtype != SKINNY_R64) return false;
    j.bA = r256((size_t)r.K * r.lda * 8);
    j.alg_bytes = 3.0 * r.K * r.M * 8;
  } else {
    return false;
  }
  j.need = j.bA + j.bB + j.bC;
  return true;
}

}  // namespace serve
}  // namespace skinny

using namespace skinny;
using namespace skinny::serve;

struct skinny_server_st {
  skinny_handle h = nullptr;
  bool dry = false;
  uint64_t budget = 0;
  int max_inflight = 1;
  std::vector<cudaStream_t> streams;
  int rr = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job*> queue;
  std::vector<Job*> inflight;
  std::unordered_map<uint64_t, Result> results;
  uint64_t next_ticket = 1, in_use = 0;
  bool stop = false;
  std::thread worker;
  // stats
  uint64_t submitted = 0, completed = 0, failed = 0, rejected = 0, peak = 0, max_seen = 0;
  double bytes_done = 0;
  std::vector<double> lat;
  bool started = false;
  clk::time_point t_first, t_last;

  void start_job(Job* j);
  void finish_job(Job* j);
  void run();
};

void skinny_server_st::start_job(Job* j) {
  const skinny_request& r = j->r;
  if (dry) {
    // ~50 GB/s of algorithmic bytes plus 20 us per request
    j->t_dry_end = clk::now() + std::chrono::microseconds(20 + (long long)(j->alg_bytes / 50e3));
    return;
  }
  DevGuard g(h->dev.id);
  j->stream = streams[rr++ % streams.size()];
  cudaStream_t st = j->stream;
  const size_t s = esize(r.dtype);
  // scalars in the request are doubles; single-precision dtypes take floats
  const bool single = r.dtype == SKINNY_R32 || r.dtype == SKINNY_C32;
  const float af[2] = {(float)r.alpha[0], (float)r.alpha[1]}, bf[2] = {(float)r.beta[0], (float)r.beta[1]};
  const void* al = single ? (const void*)af : (const void*)r.alpha;
  const void* be = single ? (const void*)bf : (const void*)r.beta;
  if (r.device) {  // operands resident in HBM: run in place
    if (r.op == SKINNY_OP_TSMTTSM)
      j->status = product(h, false, r.dtype, r.acc, r.M, r.N, r.K, r.A, r.lda, al, r.B, r.ldb, be, r.C, r.ldc, st,
                          nullptr);
    else if (r.op == SKINNY_OP_TSMM)
      j->status = product(h, true, r.dtype, r.acc, r.M, r.N, r.K, r.A, r.lda, al, r.B, r.ldb, be, r.C, r.ldc, st,
                          nullptr);
    else
      j->status = skinny_svqb(h, r.acc, r.K, r.M, (double*)(r.C ? r.C : const_cast<void*>(r.A)), r.lda, nullptr, st);
    if (cudaGetLastError() != cudaSuccess && j->status == SKINNY_OK) j->status = SKINNY_DEVICE_ERROR;
    cudaEventCreateWithFlags(&j->done, cudaEventDisableTiming);
    cudaEventRecord(j->done, st);
    return;
  }
  auto fail = [&](skinny_status why, const char* msg) {
    if (j->status == SKINNY_OK) j->status = why;
    set_error(msg);
  };
  if (j->bA && cudaMallocAsync(&j->dA, j->bA, st) != cudaSuccess) fail(SKINNY_NO_MEM, "serve: allocation");
  if (j->bB && cudaMallocAsync(&j->dB, j->bB, st) != cudaSuccess) fail(SKINNY_NO_MEM, "serve: allocation");
  if (j->bC && cudaMallocAsync(&j->dC, j->bC, st) != cudaSuccess) fail(SKINNY_NO_MEM, "serve: allocation");
  cudaGetLastError();
  if (j->status == SKINNY_OK) {
    void* dB = j->bB ? j->dB : j->dA;
    void* dC = j->bC ? j->dC : j->dA;
    const bool bz = r.beta[0] == 0.0 && r.beta[1] == 0.0;
    if (r.op == SKINNY_OP_TSMTTSM) {
      cudaMemcpyAsync(j->dA, r.A, (size_t)r.K * r.lda * s, cudaMemcpyHostToDevice, st);
      if (j->bB) cudaMemcpyAsync(dB, r.B, (size_t)r.K * r.ldb * s, cudaMemcpyHostToDevice, st);
      if (!bz) cudaMemcpyAsync(dC, r.C, (size_t)r.N * r.ldc * s, cudaMemcpyHostToDevice, st);
      j->status = product(h, false, r.dtype, r.acc, r.M, r.N, r.K, j->dA, r.lda, al, dB, r.ldb, be, dC, r.ldc,
                          st, nullptr);
      if (j->status == SKINNY_OK) cudaMemcpyAsync(r.C, dC, (size_t)r.N * r.ldc * s, cudaMemcpyDeviceToHost, st);
    } else if (r.op == SKINNY_OP_TSMM) {
      cudaMemcpyAsync(j->dA, r.A, (size_t)r.K * r.lda * s, cudaMemcpyHostToDevice, st);
      cudaMemcpyAsync(j->dB, r.B, (size_t)r.N * r.ldb * s, cudaMemcpyHostToDevice, st);
      if (!bz && j->bC) cudaMemcpyAsync(dC, r.C, (size_t)r.K * r.ldc * s, cudaMemcpyHostToDevice, st);
      j->status = product(h, true, r.dtype, r.acc, r.M, r.N, r.K, j->dA, r.lda, al, j->dB, r.ldb, be, dC, r.ldc,
                          st, nullptr);
      if (j->status == SKINNY_OK) cudaMemcpyAsync(r.C, dC, (size_t)r.K * r.ldc * s, cudaMemcpyDeviceToHost, st);
    } else {
      cudaMemcpyAsync(j->dA, r.A, (size_t)r.K * r.lda * 8, cudaMemcpyHostToDevice, st);
      j->status = skinny_svqb(h, r.acc, r.K, r.M, (double*)j->dA, r.lda, nullptr, st);
      if (j->status == SKINNY_OK) cudaMemcpyAsync(r.C, j->dA, (size_t)r.K * r.lda * 8, cudaMemcpyDeviceToHost, st);
    }
    if (cudaGetLastError() != cudaSuccess && j->status == SKINNY_OK) j->status = SKINNY_DEVICE_ERROR;
  }
  cudaEventCreateWithFlags(&j->done, cudaEventDisableTiming);
  cudaEventRecord(j->done, st);
}

void skinny_server_st::finish_job(Job* j) {
  if (!dry) {
    DevGuard g(h->dev.id);
    if (j->dA) cudaFreeAsync(j->dA, j->stream);
    if (j->dB) cudaFreeAsync(j->dB, j->stream);
    if (j->dC) cudaFreeAsync(j->dC, j->stream);
    if (j->done) cudaEventDestroy(j->done);
  }
  in_use -= j->need;
  const clk::time_point now = clk::now();
  const double us = std::chrono::duration<double, std::micro>(now - j->t_submit).count();
  results[j->ticket] = Result{j->status, us};
  t_last = now;
  if (j->status == SKINNY_OK) {
    completed++;
    bytes_done += j->alg_bytes;
    lat.push_back(us);
  } else {
    failed++;
  }
  delete j;
}

void skinny_server_st::run() {
  std::unique_lock<std::mutex> lk(mu);
  for (;;) {
    bool progressed = false;
    // retire finished requests
    for (size_t i = 0; i < inflight.size();) {
      Job* j = inflight[i];
      bool fin;
      if (dry) {
        fin = clk::now() >= j->t_dry_end;
      } else {
        cudaError_t e = cudaEventQuery(j->done);
        fin = e != cudaErrorNotReady;
        if (fin && e != cudaSuccess && j->status == SKINNY_OK) j->status = SKINNY_DEVICE_ERROR;
      }
      if (fin) {
        finish_job(j);
        inflight[i] = inflight.back();
        inflight.pop_back();
        progressed = true;
      } else {
        i++;
      }
    }
    if (progressed) cv_done.notify_all();
    // admit in arrival order while memory and slots allow
    std::vector<Job*> start;
    while (!queue.empty() && (int)(inflight.size() + start.size()) < max_inflight) {
      Job* j = queue.front();
      if (in_use + j->need > budget) break;
      queue.pop_front();
      in_use += j->need;
      peak = std::max<uint64_t>(peak, in_use);
      start.push_back(j);
    }
    if (!start.empty()) {
      if (!started) {
        started = true;
        t_first = clk::now();
      }
      lk.unlock();
      for (Job* j : start) start_job(j);
      lk.lock();
      for (Job* j : start) inflight.push_back(j);
      max_seen = std::max<uint64_t>(max_seen, inflight.size());
      progressed = true;
    }
    if (stop && queue.empty() && inflight.empty()) break;
    if (!progressed) cv_work.wait_for(lk, std::chrono::microseconds(inflight.empty() ? 2000 : 20));
  }
  cv_done.notify_all();
}

extern "C" skinny_status skinny_server_create(skinny_server* out, skinny_handle h, uint64_t budget, int num_streams,
                                              int max_inflight) {
  if (!out || budget == 0 || num_streams < 1 || max_inflight < 1) {
    set_error("server_create: bad arguments");
    return SKINNY_BAD_ARG;
  }
  skinny_server s = new skinny_server_st();
  s->h = h;
  s->dry = h == nullptr;
  s->budget = budget;
  s->max_inflight = max_inflight;
  if (!s->dry) {
    DevGuard g(h->dev.id);
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, h->dev.id) == cudaSuccess) {
      uint64_t thr = ~0ull;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    for (int i = 0; i < num_streams; i++) {
      cudaStream_t st;
      if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        for (cudaStream_t x : s->streams) cudaStreamDestroy(x);
        delete s;
        set_error("server_create: stream creation failed");
        return SKINNY_DEVICE_ERROR;
      }
      s->streams.push_back(st);
    }
  }
  s->worker = std::thread([s] { s->run(); });
  *out = s;
  return SKINNY_OK;
}

extern "C" skinny_status skinny_server_submit(skinny_server s, const skinny_request* r, uint64_t* ticket) {
  if (!s || !r || !ticket) return SKINNY_BAD_ARG;
  Job* j = new Job();
  j->r = *r;
  j->t_submit = clk::now();
  std::lock_guard<std::mutex> lk(s->mu);
  s->submitted++;
  j->ticket = s->next_ticket++;
  *ticket = j->ticket;
  if (!plan_job(*j)) {
    s->rejected++;
    s->results[j->ticket] = Result{SKINNY_BAD_ARG, 0.0};
    delete j;
    set_error("server_submit: malformed request");
    return SKINNY_BAD_ARG;
  }
  if (j->need > s->budget) {
    s->rejected++;
    s->results[j->ticket] = Result{SKINNY_NO_MEM, 0.0};
    delete j;
    set_error("server_submit: request larger than the memory budget");
    return SKINNY_NO_MEM;
  }
  s->queue.push_back(j);
  s->cv_work.notify_one();
  return SKINNY_OK;
}

extern "C" skinny_status skinny_server_poll(skinny_server s, uint64_t ticket, skinny_status* result) {
  if (!s) return SKINNY_BAD_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->results.find(ticket);
  if (it == s->results.end()) return SKINNY_NOT_READY;
  if (result) *result = it->second.status;
  return SKINNY_OK;
}

extern "C" skinny_status skinny_server_wait(skinny_server s, uint64_t ticket, skinny_status* result, double timeout_s) {
  if (!s) return SKINNY_BAD_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  const auto deadline = clk::now() + std::chrono::duration_cast<clk::duration>(std::chrono::duration<double>(timeout_s));
  while (s->results.find(ticket) == s->results.end()) {
    if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout &&
        s->results.find(ticket) == s->results.end())
      return SKINNY_TIMEOUT;
  }
  if (result) *result = s->results[ticket].status;
  return SKINNY_OK;
}

extern "C" skinny_status skinny_server_drain(skinny_server s, double timeout_s) {
  if (!s) return SKINNY_BAD_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  const auto deadline = clk::now() + std::chrono::duration_cast<clk::duration>(std::chrono::duration<double>(timeout_s));
  while (!s->queue.empty() || !s->inflight.empty()) {
    s->cv_work.notify_one();
    if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && (!s->queue.empty() || !s->inflight.empty()))
      return SKINNY_TIMEOUT;
  }
  return SKINNY_OK;
}

extern "C" skinny_status skinny_server_stats_get(skinny_server s, skinny_server_stats* out) {
  if (!s || !out) return SKINNY_BAD_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof *out);
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->failed = s->failed;
  out->rejected = s->rejected;
  out->bytes = s->bytes_done;
  out->peak_bytes_in_use = s->peak;
  out->max_inflight_seen = s->max_seen;
  if (s->started) out->busy_seconds = std::chrono::duration<double>(s->t_last - s->t_first).count();
  if (!s->lat.empty()) {
    std::vector<double> v = s->lat;
    std::sort(v.begin(), v.end());
    out->p50_latency_us = v[(v.size() - 1) / 2];
    out->p99_latency_us = v[std::min(v.size() - 1, (size_t)((v.size() - 1) * 0.99 + 0.5))];
    double sum = 0;
    for (double x : v) sum += x;
    out->mean_latency_us = sum / v.size();
  }
  return SKINNY_OK;
}

extern "C" skinny_status skinny_server_destroy(skinny_server s) {
  if (!s) return SKINNY_BAD_ARG;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  if (!s->dry) {
    DevGuard g(s->h->dev.id);
    for (cudaStream_t st : s->streams) {
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
    }
  }
  delete s;
  return SKINNY_OK;
}
