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
//   * small requests (TSMTTSM / TSMM, native or auto method, M, N <= 64, a cost of at most 32 MiB
//     by default -- bytes, or FMAs priced at the HBM-to-FMA rate ratio where that is larger)
//     take no in-flight slot: admitted requests collect in a pending
//     list and are packed into grouped launches (group.cu, one persistent kernel per dtype present)
//     on a high-priority lane stream.  Each of the lane's two slots owns an instantiated CUDA graph
//     -- a descriptor copy from pinned memory followed by one kernel node per dtype -- that is
//     updated (copy size, kernel nodes switched on or off) and replayed per batch, so a batch of
//     hundreds of requests costs one graph launch; while one slot's batch runs, the next batch
//     collects and goes to the other slot.  A small request may pass a large one that waits for
//     a slot, never one that waits for memory.
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
#include "group.h"

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
  bool small = false;  // eligible for the grouped lane
};

// One slot of the grouped lane: pinned + device batch buffers, unit partials, tickets, and the
// instantiated graph (descriptor copy -> one kernel node per dtype class).
struct LaneSlot {
  unsigned char* hbuf = nullptr;
  unsigned char* dbuf = nullptr;
  size_t cap = 0;
  unsigned char* part = nullptr;
  size_t part_cap = 0;
  unsigned* counters = nullptr;
  size_t ncounters = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphNode_t copy = nullptr;
  cudaGraphNode_t kern[GROUP_CLASSES] = {};
  cudaEvent_t ev = nullptr;
  bool busy = false;
  std::vector<Job*> jobs;
  clk::time_point dry_end;
};
constexpr int LANE_SLOTS = 2;

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

static bool group_eligible(const skinny_request& r) {
  return (r.op == SKINNY_OP_TSMTTSM || r.op == SKINNY_OP_TSMM) &&
         (r.acc == SKINNY_ACC_NATIVE || r.acc == SKINNY_ACC_AUTO) && r.M <= GROUP_MAX_W && r.N <= GROUP_MAX_W;
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
  std::deque<Job*> queue;        // large requests, arrival order
  std::deque<Job*> queue_small;  // grouped-lane requests, arrival order
  std::vector<Job*> inflight;
  std::vector<Job*> pending;     // admitted to the grouped lane, not launched yet
  uint64_t group_max_bytes = 32ull << 20;
  int group_max = 512;
  cudaStream_t lane_st = nullptr;
  LaneSlot slots[LANE_SLOTS];
  uint64_t grouped = 0, group_launches = 0;
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
  void start_batch(LaneSlot& sl);
  bool slot_prepare(LaneSlot& sl, size_t batch_bytes, size_t part_bytes, size_t n);
  void slot_release(LaneSlot& sl);
  size_t starting = 0;  // admitted requests being started by the worker outside the lock
  bool idle() const {
    if (starting || !queue.empty() || !queue_small.empty() || !inflight.empty() || !pending.empty()) return false;
    for (const LaneSlot& sl : slots)
      if (sl.busy) return false;
    return true;
  }
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

void skinny_server_st::slot_release(LaneSlot& sl) {
  if (sl.exec) cudaGraphExecDestroy(sl.exec);
  if (sl.graph) cudaGraphDestroy(sl.graph);
  sl.exec = nullptr;
  sl.graph = nullptr;
  if (sl.hbuf) cudaFreeHost(sl.hbuf);
  if (sl.dbuf) cudaFree(sl.dbuf);
  if (sl.part) cudaFree(sl.part);
  if (sl.counters) cudaFree(sl.counters);
  if (sl.ev) cudaEventDestroy(sl.ev);
  sl = LaneSlot{};
}

// Buffers of at least the sizes asked for (the slot is idle: its last batch completed); the graph
// is (re)built whenever a buffer it names changed.
bool skinny_server_st::slot_prepare(LaneSlot& sl, size_t batch_bytes, size_t part_bytes, size_t n) {
  bool rebuild = sl.exec == nullptr;
  if (!sl.ev && cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming) != cudaSuccess) return false;
  if (batch_bytes > sl.cap) {
    if (sl.hbuf) cudaFreeHost(sl.hbuf);
    if (sl.dbuf) cudaFree(sl.dbuf);
    sl.hbuf = sl.dbuf = nullptr;
    sl.cap = 0;
    const size_t nb = std::max(batch_bytes, sizeof(GroupHeader) + (size_t)group_max * sizeof(GroupDesc));
    if (cudaHostAlloc((void**)&sl.hbuf, nb, cudaHostAllocDefault) != cudaSuccess ||
        cudaMalloc((void**)&sl.dbuf, nb) != cudaSuccess)
      return false;
    sl.cap = nb;
    rebuild = true;
  }
  if (part_bytes > sl.part_cap || !sl.part) {
    if (sl.part) cudaFree(sl.part);
    sl.part = nullptr;
    const size_t nb = std::max<size_t>(part_bytes + part_bytes / 2, 1 << 20);
    if (cudaMalloc((void**)&sl.part, nb) != cudaSuccess) return false;
    sl.part_cap = nb;
    rebuild = true;
  }
  if (n > sl.ncounters) {
    if (sl.counters) cudaFree(sl.counters);
    sl.counters = nullptr;
    const size_t nc = std::max<size_t>(n, (size_t)group_max);
    if (cudaMalloc((void**)&sl.counters, nc * sizeof(unsigned)) != cudaSuccess) return false;
    if (cudaMemsetAsync(sl.counters, 0, nc * sizeof(unsigned), lane_st) != cudaSuccess) return false;
    sl.ncounters = nc;
    rebuild = true;
  }
  if (!rebuild) return true;
  if (sl.exec) cudaGraphExecDestroy(sl.exec);
  if (sl.graph) cudaGraphDestroy(sl.graph);
  sl.exec = nullptr;
  sl.graph = nullptr;
  if (cudaGraphCreate(&sl.graph, 0) != cudaSuccess) return false;
  if (cudaGraphAddMemcpyNode1D(&sl.copy, sl.graph, nullptr, 0, sl.dbuf, sl.hbuf, sizeof(GroupHeader),
                               cudaMemcpyHostToDevice) != cudaSuccess)
    return false;
  for (int c = 0; c < GROUP_CLASSES; c++) {
    int cls = c;
    const unsigned char* batch = sl.dbuf;
    void* args[] = {(void*)&batch, (void*)&cls, (void*)&sl.part, (void*)&sl.counters};
    cudaKernelNodeParams kp;
    std::memset(&kp, 0, sizeof kp);
    kp.func = group_kernel_fn(c);
    if (!kp.func) return false;
    kp.gridDim = dim3(group_grid(h->dev.sms));
    kp.blockDim = dim3(GROUP_THREADS);
    kp.sharedMemBytes = GROUP_SMEM;
    kp.kernelParams = args;
    if (cudaGraphAddKernelNode(&sl.kern[c], sl.graph, &sl.copy, 1, &kp) != cudaSuccess) return false;
  }
  return cudaGraphInstantiate(&sl.exec, sl.graph, 0) == cudaSuccess;
}

// Launch one grouped batch (the slot's jobs): stage host operands, plan, update and replay the
// slot's graph, download host results, record the slot's event.  Called without the lock.
void skinny_server_st::start_batch(LaneSlot& sl) {
  if (dry) {
    double bytes = 0;
    for (Job* j : sl.jobs) bytes += j->alg_bytes;
    sl.dry_end = clk::now() + std::chrono::microseconds(20 + (long long)(bytes / 50e3));
    return;
  }
  DevGuard g(h->dev.id);
  std::vector<skinny_group_item> items;
  std::vector<skinny_dtype> dts;
  std::vector<Job*> members;
  for (Job* j : sl.jobs) {
    const skinny_request& r = j->r;
    j->stream = lane_st;
    skinny_group_item it;
    std::memset(&it, 0, sizeof it);
    it.op = r.op;
    it.M = r.M;
    it.N = r.N;
    it.K = r.K;
    it.A = r.A;
    it.lda = r.lda;
    it.B = r.B;
    it.ldb = r.ldb;
    it.C = r.C;
    it.ldc = r.ldc;
    std::memcpy(it.alpha, r.alpha, sizeof it.alpha);
    std::memcpy(it.beta, r.beta, sizeof it.beta);
    if (!r.device) {  // stage host operands in stream-ordered pool memory
      const size_t es = esize(r.dtype);
      const bool bz = r.beta[0] == 0.0 && r.beta[1] == 0.0;
      if ((j->bA && cudaMallocAsync(&j->dA, j->bA, lane_st) != cudaSuccess) ||
          (j->bB && cudaMallocAsync(&j->dB, j->bB, lane_st) != cudaSuccess) ||
          (j->bC && cudaMallocAsync(&j->dC, j->bC, lane_st) != cudaSuccess)) {
        cudaGetLastError();
        j->status = SKINNY_NO_MEM;
        continue;
      }
      void* dB = j->bB ? j->dB : j->dA;
      void* dC = j->bC ? j->dC : j->dA;
      if (r.op == SKINNY_OP_TSMTTSM) {
        cudaMemcpyAsync(j->dA, r.A, (size_t)r.K * r.lda * es, cudaMemcpyHostToDevice, lane_st);
        if (j->bB) cudaMemcpyAsync(dB, r.B, (size_t)r.K * r.ldb * es, cudaMemcpyHostToDevice, lane_st);
        if (!bz) cudaMemcpyAsync(dC, r.C, (size_t)r.N * r.ldc * es, cudaMemcpyHostToDevice, lane_st);
      } else {
        cudaMemcpyAsync(j->dA, r.A, (size_t)r.K * r.lda * es, cudaMemcpyHostToDevice, lane_st);
        cudaMemcpyAsync(j->dB, r.B, (size_t)r.N * r.ldb * es, cudaMemcpyHostToDevice, lane_st);
        if (!bz && j->bC) cudaMemcpyAsync(dC, r.C, (size_t)r.K * r.ldc * es, cudaMemcpyHostToDevice, lane_st);
      }
      it.A = j->dA;
      it.B = dB;
      it.C = dC;
    }
    {  // the item alone must plan: a malformed request fails alone, not its batch
      std::vector<unsigned char> tmp;
      size_t pb = 0;
      skinny_dtype dt = r.dtype;
      skinny_status st = group_plan(&it, &dt, 1, tmp, &pb, nullptr);
      if (st != SKINNY_OK) {
        j->status = st;
        continue;
      }
    }
    items.push_back(it);
    dts.push_back(r.dtype);
    members.push_back(j);
  }
  if (!items.empty()) {
    std::vector<unsigned char> host;
    size_t part_bytes = 0;
    skinny_status st = group_plan(items.data(), dts.data(), (int)items.size(), host, &part_bytes, nullptr);
    bool ok = st == SKINNY_OK && slot_prepare(sl, host.size(), part_bytes, items.size());
    if (ok) {
      std::memcpy(sl.hbuf, host.data(), host.size());
      const GroupHeader* hd = reinterpret_cast<const GroupHeader*>(host.data());
      ok = cudaGraphExecMemcpyNodeSetParams1D(sl.exec, sl.copy, sl.dbuf, sl.hbuf, host.size(),
                                              cudaMemcpyHostToDevice) == cudaSuccess;
      int nk = 0;
      for (int c = 0; ok && c < GROUP_CLASSES; c++) {
        ok = cudaGraphNodeSetEnabled(sl.exec, sl.kern[c], hd->count[c] > 0 ? 1u : 0u) == cudaSuccess;
        nk += hd->count[c] > 0;
      }
      ok = ok && cudaGraphLaunch(sl.exec, lane_st) == cudaSuccess;
      if (ok)
        for (int k = 0; k < nk; k++) count_launch();
    }
    if (!ok) {
      cudaGetLastError();
      set_error("serve: grouped launch failed");
      for (Job* j : members)
        if (j->status == SKINNY_OK) j->status = SKINNY_DEVICE_ERROR;
    } else {
      for (Job* j : members) {  // results of host requests back to the host
        const skinny_request& r = j->r;
        if (r.device) continue;
        const size_t es = esize(r.dtype);
        void* dC = j->bC ? j->dC : j->dA;
        const size_t cb = r.op == SKINNY_OP_TSMTTSM ? (size_t)r.N * r.ldc * es : (size_t)r.K * r.ldc * es;
        cudaMemcpyAsync(r.C, dC, cb, cudaMemcpyDeviceToHost, lane_st);
      }
    }
  }
  if (!sl.ev && cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming) != cudaSuccess) sl.ev = nullptr;
  if (sl.ev)
    cudaEventRecord(sl.ev, lane_st);
  else
    cudaStreamSynchronize(lane_st);  // no event to poll: the batch is complete when this returns
  if (cudaGetLastError() != cudaSuccess)
    for (Job* j : sl.jobs)
      if (j->status == SKINNY_OK) j->status = SKINNY_DEVICE_ERROR;
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
    // retire finished grouped batches
    bool lane_busy = false;
    for (LaneSlot& sl : slots) {
      if (!sl.busy) continue;
      bool fin;
      cudaError_t e = cudaSuccess;
      if (dry) {
        fin = clk::now() >= sl.dry_end;
      } else {
        e = sl.ev ? cudaEventQuery(sl.ev) : cudaSuccess;
        fin = e != cudaErrorNotReady;
      }
      if (!fin) {
        lane_busy = true;
        continue;
      }
      for (Job* j : sl.jobs) {
        if (e != cudaSuccess && j->status == SKINNY_OK) j->status = SKINNY_DEVICE_ERROR;
        if (j->status == SKINNY_OK) grouped++;
        finish_job(j);
      }
      sl.jobs.clear();
      sl.busy = false;
      progressed = true;
    }
    if (progressed) cv_done.notify_all();
    // admit in arrival order while memory allows: large requests also need an in-flight slot;
    // small ones go to the grouped lane and may pass a large one that waits for a slot (never
    // one that waits for memory)
    std::vector<Job*> start;
    for (;;) {
      Job* sj = queue_small.empty() ? nullptr : queue_small.front();
      Job* bj = queue.empty() ? nullptr : queue.front();
      if (!sj && !bj) break;
      const bool slots_full = (int)(inflight.size() + start.size()) >= max_inflight;
      const bool take_small = sj && (!bj || sj->ticket < bj->ticket || slots_full);
      Job* j = take_small ? sj : bj;
      if (in_use + j->need > budget) break;
      if (!take_small && slots_full) break;
      (take_small ? queue_small : queue).pop_front();
      in_use += j->need;
      peak = std::max<uint64_t>(peak, in_use);
      (take_small ? pending : start).push_back(j);
    }
    // pack pending small requests into the free lane slots
    std::vector<LaneSlot*> batches;
    for (LaneSlot& sl : slots) {
      if (sl.busy || pending.empty()) continue;
      const size_t take = std::min(pending.size(), (size_t)group_max);
      sl.jobs.assign(pending.begin(), pending.begin() + take);
      pending.erase(pending.begin(), pending.begin() + take);
      sl.busy = true;
      batches.push_back(&sl);
      group_launches++;
    }
    if (!start.empty() || !batches.empty()) {
      if (!started) {
        started = true;
        t_first = clk::now();
      }
      starting = start.size();
      lk.unlock();
      if (!batches.empty() && !dry && !lane_st) {
        DevGuard g(h->dev.id);
        int lo = 0, hi = 0;
        cudaDeviceGetStreamPriorityRange(&lo, &hi);
        if (cudaStreamCreateWithPriority(&lane_st, cudaStreamNonBlocking, hi) != cudaSuccess) {
          cudaGetLastError();
          lane_st = streams.empty() ? nullptr : streams[0];
        }
      }
      for (LaneSlot* sl : batches) start_batch(*sl);
      for (Job* j : start) start_job(j);
      lk.lock();
      starting = 0;
      for (Job* j : start) inflight.push_back(j);
      max_seen = std::max<uint64_t>(max_seen, inflight.size());
      progressed = true;
      lane_busy = lane_busy || !batches.empty();
    }
    if (stop && idle()) break;
    if (!progressed)
      cv_work.wait_for(lk, std::chrono::microseconds(inflight.empty() && !lane_busy ? 2000 : 20));
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
  if (s->group_max_bytes > 0 && group_eligible(j->r)) {  // small: its cost, not only its bytes
    skinny_group_item it;
    std::memset(&it, 0, sizeof it);
    it.op = r->op;
    it.M = r->M;
    it.N = r->N;
    it.K = r->K;
    it.A = r->A;
    it.lda = r->lda;
    it.B = r->B;
    it.ldb = r->ldb;
    it.C = r->C;
    it.ldc = r->ldc;
    std::memcpy(it.beta, r->beta, sizeof it.beta);
    j->small = group_item_cost(it, r->dtype) <= (double)s->group_max_bytes;
  }
  (j->small ? s->queue_small : s->queue).push_back(j);
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
  while (!s->idle()) {
    s->cv_work.notify_one();
    if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !s->idle()) return SKINNY_TIMEOUT;
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
  out->grouped = s->grouped;
  out->group_launches = s->group_launches;
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
    if (s->lane_st) cudaStreamSynchronize(s->lane_st);
    for (LaneSlot& sl : s->slots) s->slot_release(sl);
    bool own_lane = s->lane_st != nullptr;
    for (cudaStream_t st : s->streams) {
      own_lane = own_lane && st != s->lane_st;
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
    }
    if (own_lane) cudaStreamDestroy(s->lane_st);
  }
  delete s;
  return SKINNY_OK;
}

extern "C" skinny_status skinny_server_set_grouping(skinny_server s, uint64_t max_request_bytes, int32_t max_group) {
  if (!s || max_group < 1 || max_group > 65536) {
    set_error("server_set_grouping: bad arguments");
    return SKINNY_BAD_ARG;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  s->group_max_bytes = max_request_bytes;
  s->group_max = max_group;
  return SKINNY_OK;
}
