// Serving engine: requests (one subject each: BOLD -> CSR -> centrality) are
// admitted continuously onto a fixed set of worker slots of one GPU.
//
// No reference counterpart: the reference builds one subject per process run
// (CUCorMat, then CUEC on the written .csr).  Here a long-lived server keeps
// every slot's working memory on the device and runs several subjects at
// once:
//   - admission: a queued request is taken by the first free slot as soon as
//     its device-memory estimate (bna_request_bytes) fits the budget beside
//     what the other slots hold; requests are considered in arrival order,
//     and one that does not fit yet does not block smaller ones behind it
//     (backfill).  Idle slots give their memory back when a waiting request
//     needs it;
//   - overlap: each slot has its own context and streams, so the kernels and
//     copies of different requests interleave on the device; requests with
//     less work use a higher-priority stream, and correlation passes are cut
//     into launches of a bounded number of tiles, so the block scheduler can
//     serve a small request between the launches of a large one;
//   - launch gate (shortest job first): below the top priority level a
//     request keeps at most two of its launches queued, and while a request
//     with less correlation work (N^2 T; ties: the one started first) runs on
//     another slot it drains its stream and waits (at most kGateWaitMs per
//     gate) before queueing more; so a small request meets at most one
//     launch of a large one on the device, not its whole queue.  A centrality
//     that has run kLongEc iterations no longer makes others wait, so a slowly
//     converging small graph does not hold up larger requests, and such
//     centralities run one at a time (first started, first served);
//   - results are independent of the mix: each slot's kernels see only their
//     own request's buffers, and every reduction has a fixed order.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "bna.h"

namespace bna {
cudaMemPool_t lib_pool(int device);
cudaError_t copy_from_host(const void* src, void* dst, size_t bytes, int sms, cudaStream_t stream,
                           unsigned long long* blocks, int* grid_out);
int upload_max_blocks();
}
int32_t bna_ctx_trim_idle(bna_ctx* ctx);

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
  int64_t id = 0;
  bna_request req{};
  bna_reply reply{};
  int64_t est = 0;
  double work = 0;  // N^2 T: selects the stream priority
  bool done = false;
};

constexpr int kLevels = 6;  // stream priority levels used (fewer if the device has fewer)

struct Slot {
  bna_server* srv = nullptr;
  int index = 0;
  int level = 0;                  // priority level of the running request
  double work = 0;                // its N^2 T (launch gate order)
  int64_t seq = 0;                // its start order (ties of work)
  int64_t job_id = 0;             // the running request (trace)
  int phase = 0;                  // its pass and progress at its last gate call
  int64_t progress = 0;
  cudaEvent_t fence[2] = {};      // launch gate: queue-depth events
  cudaEvent_t tev[2] = {};        // trace: around the series upload
  unsigned long long* upblk = nullptr;  // trace: the upload's block times and SMs (device)
  int upgrid = 0;
  int nfence = 0;
  bna_ctx* ctx = nullptr;
  cudaStream_t stream[kLevels] = {};  // stream[0]: highest priority
  float* bold = nullptr;
  size_t bold_cap = 0;
  double* ec = nullptr;
  size_t ec_cap = 0;
  int64_t held = 0;        // device bytes this slot holds (accounting)
  bool busy = false;
  bool trim = false;       // asked to give its memory back while idle
  std::thread th;
};

// Priority level of a request: one level per decade of correlation work
// N^2 T above 1e10 (N = 4,096, T = 600 is level 0; N = 180,000, T = 1200 the
// lowest), so smaller requests are served first wherever their kernels and
// a larger request's wait for the same SMs.
int level_of(double work, int levels) {
  int l = 0;
  for (double w = 1.0e10; work >= w && l < levels - 1; w *= 10.0) ++l;
  return l;
}
// Tiles per correlation launch: about 0.16 ms of tensor work (1,536 tiles at
// T = 1200, proportionally more for shorter series).
int tiles_per_launch(int T) { return std::max(512, (int)(1536LL * 1200 / std::max(T, 1))); }
// Longest wait of one gate call for higher-priority requests to finish.
constexpr int kGateWaitMs = 200;
// Series uploads go in chunks of this size, with the launch gate before each.
constexpr size_t kUploadChunk = 32u << 20;
// A centrality past this many iterations (a graph that converges slowly or
// never: the reference stops at 10,000) no longer holds up other requests,
// other such centralities included: they share the device (how many
// iterations one still needs is not known, and run one at a time a request
// whose centrality converged soon after this mark waited 0.35 s behind a
// never-converging one).
constexpr int64_t kLongEc = 1000;

}  // namespace

struct bna_server {
  // optional host-side trace (environment variable BNA_SERVER_TRACE = a file
  // path, written when the server is destroyed): one line per event with the
  // time, slot, request id, event name and a value
  struct TraceEv {
    double t;
    int slot;
    int64_t id;
    const char* what;
    int64_t v;
  };
  bool tracing = false;
  bool upload_ce = false;  // BNA_SERVER_UPLOAD=copy_engine: uploads by cudaMemcpyAsync
  std::string trace_path;
  std::mutex trace_mu;
  std::vector<TraceEv> trace;
  int device = 0;
  int sms = 1;
  int64_t budget = 0;
  Clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv;  // queue, slot and completion changes
  std::deque<Job*> queue;
  std::map<int64_t, Job*> jobs;
  int64_t next_id = 1;
  int64_t next_seq = 0;  // start order of requests on slots
  int levels = 1;
  bool stop = false;
  std::vector<Slot*> slots;

  double now() const {
    return std::chrono::duration<double>(Clock::now() - t0).count();
  }
  int64_t held_by_others(const Slot* s) const {
    int64_t h = 0;
    for (const Slot* o : slots)
      if (o != s) h += o->held;
    return h;
  }
};

namespace {

void trace(bna_server* srv, const Slot* s, int64_t id, const char* what, int64_t v = 0) {
  if (!srv->tracing) return;
  const double t = srv->now();
  std::lock_guard<std::mutex> lk(srv->trace_mu);
  srv->trace.push_back({t, s ? s->index : -1, id, what, v});
}

// Grow-only slot buffer, stream-ordered (no wait for other slots' work), from
// the library's pool.
int32_t grow(int device, void** p, size_t* cap, size_t bytes, cudaStream_t st) {
  if (*cap >= bytes) return BNA_OK;
  if (*p) cudaFreeAsync(*p, st);
  *p = nullptr;
  *cap = 0;
  cudaMemPool_t pool = bna::lib_pool(device);
  if (!pool || cudaMallocFromPoolAsync(p, bytes, pool, st) != cudaSuccess) {
    cudaGetLastError();
    return BNA_OOM;
  }
  *cap = bytes;
  return BNA_OK;
}

int64_t slot_bytes(const Slot* s) {
  return bna_ctx_arena_bytes(s->ctx) + (int64_t)s->bold_cap + (int64_t)s->ec_cap;
}

// The slot is idle: every stream it used was synchronised at the end of its
// last request.
void release_slot_memory(Slot* s) {
  if (s->bold) cudaFreeAsync(s->bold, s->stream[0]);
  if (s->ec) cudaFreeAsync(s->ec, s->stream[0]);
  cudaStreamSynchronize(s->stream[0]);
  bna_ctx_trim_idle(s->ctx);
  s->bold = nullptr;
  s->ec = nullptr;
  s->bold_cap = s->ec_cap = 0;
}

bool long_ec(const Slot* s) { return s->phase == BNA_PHASE_EC && s->progress >= kLongEc; }


// Launch gate of a slot's context (bna_ctx_set_gate).
void slot_gate(void* user, void* stream, int32_t phase, int64_t done) {
  Slot* s = static_cast<Slot*>(user);
  bna_server* srv = s->srv;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  std::unique_lock<std::mutex> lk(srv->mu);
  s->phase = phase;
  s->progress = done;
  lk.unlock();
  if (s->level > 0) {
    // queue depth: the launch before the previous one has finished
    cudaEventRecord(s->fence[s->nfence & 1], st);
    const double t0 = srv->tracing ? srv->now() : 0.0;
    if (s->nfence > 0) cudaEventSynchronize(s->fence[(s->nfence + 1) & 1]);
    if (srv->tracing && srv->now() - t0 > 5e-4)
      trace(srv, s, s->job_id, "fence_wait_us", (int64_t)((srv->now() - t0) * 1e6));
    ++s->nfence;
  }
  lk.lock();
  auto higher = [&]() {
    for (const Slot* o : srv->slots) {
      if (o == s || !o->busy || long_ec(o)) continue;
      if (o->work < s->work || (o->work == s->work && o->seq < s->seq)) return true;
    }
    return false;
  };
  if (!higher()) return;
  lk.unlock();
  const double t0 = srv->now();
  cudaStreamSynchronize(st);  // nothing of this request stays queued
  lk.lock();
  const auto until = Clock::now() + std::chrono::milliseconds(kGateWaitMs);
  while (higher() && srv->cv.wait_until(lk, until) != std::cv_status::timeout) {
  }
  if (srv->tracing) {
    lk.unlock();
    trace(srv, s, s->job_id, "gate_wait_us", (int64_t)((srv->now() - t0) * 1e6));
  }
}

// Trace: how the SM-driven upload's blocks ran (whether they started
// together, how long each took, on how many SMs).
void trace_upload_blocks(bna_server* srv, Slot* s, int64_t id) {
  const int g = s->upgrid;
  if (!s->upblk || g <= 0) return;
  std::vector<unsigned long long> b(3 * (size_t)g);
  if (cudaMemcpy(b.data(), s->upblk, b.size() * sizeof(unsigned long long),
                 cudaMemcpyDeviceToHost) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  unsigned long long s0 = ~0ull, s1 = 0, e1 = 0;
  std::vector<double> dur;
  std::vector<unsigned long long> sm;
  for (int k = 0; k < g; ++k) {
    s0 = std::min(s0, b[3 * k]);
    s1 = std::max(s1, b[3 * k]);
    e1 = std::max(e1, b[3 * k + 1]);
    dur.push_back((double)(b[3 * k + 1] - b[3 * k]));
    sm.push_back(b[3 * k + 2]);
  }
  std::sort(dur.begin(), dur.end());
  std::sort(sm.begin(), sm.end());
  trace(srv, s, id, "upload_grid", g);
  trace(srv, s, id, "upload_start_spread_us", (int64_t)((s1 - s0) / 1000));
  trace(srv, s, id, "upload_span_us", (int64_t)((e1 - s0) / 1000));
  trace(srv, s, id, "upload_block_p50_us", (int64_t)(dur[dur.size() / 2] / 1000));
  trace(srv, s, id, "upload_block_max_us", (int64_t)(dur.back() / 1000));
  trace(srv, s, id, "upload_sms",
        (int64_t)(std::unique(sm.begin(), sm.end()) - sm.begin()));
}

// One request on one slot.
void run_job(bna_server* srv, Slot* s, Job* j) {
  const bna_request& r = j->req;
  bna_reply& out = j->reply;
  cudaStream_t st = s->stream[level_of(j->work, srv->levels)];
  const size_t bytes = (size_t)r.N * r.T * sizeof(float);
  const size_t cap0 = s->bold_cap;
  int32_t rc = grow(srv->device, reinterpret_cast<void**>(&s->bold), &s->bold_cap, bytes, st);
  trace(srv, s, j->id, "bold_grown_bytes", (int64_t)(s->bold_cap - cap0));
  if (srv->tracing) cudaEventRecord(s->tev[0], st);
  // the series by an SM-driven copy from the caller's page-locked buffer
  // (copy-engine uploads slowed to a few GB/s while other requests shared
  // the device); a pageable buffer takes the copy engine.  In chunks with the
  // launch gate before each, the first included: a large request's upload
  // waits while a smaller request runs (an upload whose host reads had turned
  // slow, beside a small request, stretched that request's every kernel
  // several-fold).
  const double tu0 = srv->tracing ? srv->now() : 0.0;
  s->upgrid = 0;
  for (size_t off = 0; rc == BNA_OK && off < bytes; off += kUploadChunk) {
    slot_gate(s, st, BNA_PHASE_UPLOAD, (int64_t)off);
    const size_t n = std::min(kUploadChunk, bytes - off);
    const char* src = reinterpret_cast<const char*>(r.bold_host) + off;
    char* dst = reinterpret_cast<char*>(s->bold) + off;
    if ((srv->upload_ce ||
         bna::copy_from_host(src, dst, n, srv->sms, st, s->upblk, &s->upgrid) != cudaSuccess) &&
        cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, st) != cudaSuccess)
      rc = BNA_CUDA_ERROR;
  }
  if (srv->tracing) {
    trace(srv, s, j->id, "upload_call_us", (int64_t)((srv->now() - tu0) * 1e6));
    cudaEventRecord(s->tev[1], st);
  }
  bna_csr csr{};
  if (rc == BNA_OK) {
    // no CSR larger than the caller's buffers is built (a cap of 0 admits
    // only the empty graph)
    bna_ctx_set_option(s->ctx, BNA_OPT_MAX_NNZ, r.cap > 0 ? r.cap : 1);
    bna_ctx_set_option(s->ctx, BNA_OPT_TILES_PER_LAUNCH, tiles_per_launch(r.T));
    const int64_t arena0 = bna_ctx_arena_bytes(s->ctx);
    rc = bna_corr_csr(s->ctx, s->bold, r.N, r.T, &r.opts, &csr, &out.stats, st);
    out.t_corr = srv->now();
    trace(srv, s, j->id, "corr_arena_grown_bytes", bna_ctx_arena_bytes(s->ctx) - arena0);
    out.nnz = rc == BNA_OK || rc == BNA_CAPACITY ? out.stats.nnz : 0;
    if (rc == BNA_OK && csr.nnz > r.cap) rc = BNA_CAPACITY;
  }
  if (rc == BNA_OK && r.row_ptr_host) {  // without host buffers the CSR stays on the device
    bool ok = cudaMemcpyAsync(r.row_ptr_host, csr.row_ptr, (size_t)(r.N + 1) * 4,
                              cudaMemcpyDeviceToHost, st) == cudaSuccess;
    if (csr.nnz > 0 && r.col_idx_host) {
      ok = ok && cudaMemcpyAsync(r.col_idx_host, csr.col_idx, (size_t)csr.nnz * 4,
                                 cudaMemcpyDeviceToHost, st) == cudaSuccess;
      if (r.val_host && csr.val)
        ok = ok && cudaMemcpyAsync(r.val_host, csr.val, (size_t)csr.nnz * 4,
                                   cudaMemcpyDeviceToHost, st) == cudaSuccess;
    }
    if (!ok) rc = BNA_CUDA_ERROR;
  }
  if (rc == BNA_OK && r.ec_max_iter > 0) {
    rc = grow(srv->device, reinterpret_cast<void**>(&s->ec), &s->ec_cap, (size_t)r.N * sizeof(double),
              st);
    if (rc == BNA_OK) {
      double lam = 0;
      int32_t it = 0;
      const int32_t e = bna_ec(s->ctx, &csr, r.ec_max_iter, r.ec_eps, s->ec, &lam, &it, st);
      if (e == BNA_OK || e == BNA_NOT_CONVERGED) {
        out.lambda = lam;
        out.ec_iters = it;
        out.ec_converged = e == BNA_OK;
        if (r.ec_host && cudaMemcpyAsync(r.ec_host, s->ec, (size_t)r.N * sizeof(double),
                                         cudaMemcpyDeviceToHost, st) != cudaSuccess)
          rc = BNA_CUDA_ERROR;
      } else {
        rc = e;
      }
    }
  }
  trace(srv, s, j->id, "ec_issued", out.ec_iters);
  if (cudaStreamSynchronize(st) != cudaSuccess && rc == BNA_OK) rc = BNA_CUDA_ERROR;
  if (srv->tracing) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, s->tev[0], s->tev[1]) == cudaSuccess)
      trace(srv, s, j->id, "upload_device_us", (int64_t)(ms * 1000));
    cudaGetLastError();
    trace_upload_blocks(srv, s, j->id);
  }
  trace(srv, s, j->id, "done");
  out.status = rc;
}

// First queued job that fits beside the other slots' memory (arrival order,
// with backfill; once the oldest request has waited kMaxBypass seconds, later
// ones no longer pass it).  Caller holds the lock.
constexpr double kMaxBypass = 0.5;
Job* pick(bna_server* srv, Slot* s) {
  const int64_t others = srv->held_by_others(s);
  const double now = srv->now();
  for (auto it = srv->queue.begin(); it != srv->queue.end(); ++it) {
    Job* j = *it;
    if (others + std::max(s->held, j->est) <= srv->budget) {
      srv->queue.erase(it);
      return j;
    }
    if (now - j->reply.t_submit > kMaxBypass) break;
  }
  return nullptr;
}

void worker(bna_server* srv, Slot* s) {
  cudaSetDevice(srv->device);
  std::unique_lock<std::mutex> lk(srv->mu);
  for (;;) {
    if (s->trim) {
      s->trim = false;
      lk.unlock();
      trace(srv, s, 0, "trim_bytes", slot_bytes(s));
      release_slot_memory(s);
      trace(srv, s, 0, "trimmed");
      lk.lock();
      s->held = 0;
      srv->cv.notify_all();
      continue;
    }
    Job* j = pick(srv, s);
    if (!j) {
      if (srv->stop && srv->queue.empty()) break;
      // a waiting request that does not fit: idle slots (this one included)
      // give their memory back
      if (!srv->queue.empty())
        for (Slot* o : srv->slots)
          if (!o->busy && o->held > 0) o->trim = true;
      if (s->trim) continue;
      srv->cv.notify_all();
      // bounded wait: the bypass limit above changes with time alone
      srv->cv.wait_for(lk, std::chrono::milliseconds(50));
      continue;
    }
    s->busy = true;
    s->level = level_of(j->work, srv->levels);
    s->work = j->work;
    s->seq = srv->next_seq++;
    s->job_id = j->id;
    s->phase = BNA_PHASE_CORR;
    s->progress = 0;
    s->nfence = 0;
    s->held = std::max(s->held, j->est);
    j->reply.t_start = srv->now();
    j->reply.slot = s->index;
    lk.unlock();
    trace(srv, s, j->id, "start", (int64_t)j->work);
    if (srv->tracing) {
      size_t fr = 0, tot = 0;
      if (cudaMemGetInfo(&fr, &tot) == cudaSuccess) trace(srv, s, j->id, "device_free_mb", (int64_t)(fr >> 20));
      cudaGetLastError();
    }
    run_job(srv, s, j);
    lk.lock();
    j->reply.t_done = srv->now();
    s->held = slot_bytes(s);
    s->busy = false;
    j->done = true;
    srv->cv.notify_all();
  }
}

}  // namespace

extern "C" {

int32_t bna_server_create(int32_t device, int32_t slots, int64_t hbm_budget_bytes,
                          bna_server** out) {
  if (!out || slots < 1 || slots > 64 || hbm_budget_bytes <= 0) return BNA_BAD_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return BNA_NO_DEVICE;
  }
  if (device < 0 || device >= n) return BNA_BAD_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return BNA_CUDA_ERROR;
  int least = 0, greatest = 0;
  if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) return BNA_CUDA_ERROR;
  bna_server* srv = new bna_server();
  srv->device = device;
  if (cudaDeviceGetAttribute(&srv->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      srv->sms < 1)
    srv->sms = 1;
  srv->budget = hbm_budget_bytes;
  srv->t0 = Clock::now();
  if (const char* up = std::getenv("BNA_SERVER_UPLOAD"))
    srv->upload_ce = std::strcmp(up, "copy_engine") == 0;
  if (const char* tp = std::getenv("BNA_SERVER_TRACE")) {
    if (*tp) {
      srv->tracing = true;
      srv->trace_path = tp;
      // the steady clock's reading at t = 0 (CLOCK_MONOTONIC on Linux), to
      // line the trace up with other processes' records
      trace(srv, nullptr, 0, "clock_origin_ns",
            (int64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
                srv->t0.time_since_epoch())
                .count());
    }
  }
  // numerically lower = higher priority; greatest <= least
  srv->levels = std::min(kLevels, least - greatest + 1);
  int32_t rc = BNA_OK;
  for (int i = 0; i < slots && rc == BNA_OK; ++i) {
    Slot* s = new Slot();
    s->srv = srv;
    s->index = i;
    srv->slots.push_back(s);
    rc = bna_ctx_create(device, &s->ctx);
    for (auto& e : s->fence)
      if (rc == BNA_OK && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
        rc = BNA_CUDA_ERROR;
    for (auto& e : s->tev)
      if (rc == BNA_OK && cudaEventCreate(&e) != cudaSuccess) rc = BNA_CUDA_ERROR;
    if (rc == BNA_OK && srv->tracing &&
        cudaMalloc(&s->upblk, 3 * sizeof(unsigned long long) * bna::upload_max_blocks()) !=
            cudaSuccess)
      rc = BNA_CUDA_ERROR;
    if (rc == BNA_OK) rc = bna_ctx_set_gate(s->ctx, slot_gate, s);
    for (int l = 0; l < srv->levels && rc == BNA_OK; ++l)
      if (cudaStreamCreateWithPriority(&s->stream[l], cudaStreamNonBlocking, greatest + l) !=
          cudaSuccess)
        rc = BNA_CUDA_ERROR;

  }
  if (rc != BNA_OK) {
    for (Slot* s : srv->slots) {
      for (cudaStream_t& q : s->stream)
        if (q) cudaStreamDestroy(q);
      for (cudaEvent_t e : s->fence)
        if (e) cudaEventDestroy(e);
      for (cudaEvent_t e : s->tev)
        if (e) cudaEventDestroy(e);
      if (s->ctx) bna_ctx_destroy(s->ctx);
      delete s;
    }
    delete srv;
    return rc;
  }
  for (Slot* s : srv->slots) s->th = std::thread(worker, srv, s);
  *out = srv;
  return BNA_OK;
}

int32_t bna_server_submit(bna_server* srv, const bna_request* req, int64_t* ticket) {
  if (!srv || !req || !ticket || !req->bold_host || req->N < 2 || req->T < 1 || req->cap < 0 ||
      (req->row_ptr_host && req->cap > 0 && !req->col_idx_host))
    return BNA_BAD_ARG;
  const int64_t est = bna_request_bytes(req->N, req->T, &req->opts, req->cap,
                                        req->ec_max_iter > 0 ? 1 : 0);
  if (est < 0) return BNA_BAD_ARG;
  if (est > srv->budget) return BNA_OVER_BUDGET;
  Job* j = new Job();
  j->req = *req;
  j->est = est;
  j->work = (double)req->N * req->N * req->T;
  std::lock_guard<std::mutex> lk(srv->mu);
  if (srv->stop) {
    delete j;
    return BNA_BAD_ARG;
  }
  j->id = srv->next_id++;
  j->reply.tag = req->tag;
  j->reply.t_submit = srv->now();
  srv->jobs[j->id] = j;
  srv->queue.push_back(j);
  *ticket = j->id;
  trace(srv, nullptr, j->id, "submit_N_T", (int64_t)req->N * 100000 + req->T);
  srv->cv.notify_all();
  return BNA_OK;
}

int32_t bna_server_wait(bna_server* srv, int64_t ticket, double timeout_s, bna_reply* reply) {
  if (!srv || !reply) return BNA_BAD_ARG;
  std::unique_lock<std::mutex> lk(srv->mu);
  auto it = srv->jobs.find(ticket);
  if (it == srv->jobs.end()) return BNA_BAD_ARG;
  Job* j = it->second;
  auto done = [&] { return j->done; };
  if (timeout_s < 0) {
    srv->cv.wait(lk, done);
  } else if (!srv->cv.wait_for(lk, std::chrono::duration<double>(timeout_s), done)) {
    return BNA_TIMEOUT;
  }
  *reply = j->reply;
  srv->jobs.erase(it);
  delete j;
  return BNA_OK;
}

int64_t bna_server_device_bytes(const bna_server* srv) {
  if (!srv) return -1;
  bna_server* s = const_cast<bna_server*>(srv);
  std::lock_guard<std::mutex> lk(s->mu);
  int64_t h = 0;
  for (const Slot* o : s->slots) h += o->held;
  return h;
}

int32_t bna_server_destroy(bna_server* srv) {
  if (!srv) return BNA_BAD_ARG;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stop = true;
    srv->cv.notify_all();
  }
  for (Slot* s : srv->slots)
    if (s->th.joinable()) s->th.join();
  cudaSetDevice(srv->device);
  for (Slot* s : srv->slots) {
    release_slot_memory(s);
    for (cudaStream_t& q : s->stream)
      if (q) cudaStreamDestroy(q);
    for (cudaEvent_t e : s->fence)
      if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : s->tev)
      if (e) cudaEventDestroy(e);
    if (s->upblk) cudaFree(s->upblk);
    bna_ctx_destroy(s->ctx);
    delete s;
  }
  for (auto& kv : srv->jobs) delete kv.second;
  if (srv->tracing) {
    if (FILE* f = std::fopen(srv->trace_path.c_str(), "w")) {
      std::fprintf(f, "t,slot,id,event,value\n");
      for (const auto& e : srv->trace)
        std::fprintf(f, "%.6f,%d,%lld,%s,%lld\n", e.t, e.slot, (long long)e.id, e.what,
                     (long long)e.v);
      std::fclose(f);
    }
  }
  delete srv;
  return BNA_OK;
}

}  // extern "C"
