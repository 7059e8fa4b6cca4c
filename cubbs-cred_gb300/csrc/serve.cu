// Serving queue for the four BBS operations: continuous batching on top of
// the batch entry points.
//
// Requests are submitted one at a time into per-operation queues and complete
// one at a time.  A fixed number of dispatch slots (at most the number of
// device workspaces) each take the next batch as soon as they are free: the
// queue whose oldest ready request has waited longest, as many of its queued
// requests as fit in the queue's batch size and in the device-memory budget
// still unclaimed by the other running batches.  Batches of different slots
// run concurrently on their own streams, so requests that arrive while others
// are on the device are admitted as soon as a slot and memory free up.
//
// Each queue also takes the settings of the reference service's per-operation
// batcher (crates/cubbs-w3c-service/src/batcher.rs:21-60,223-320): a
// coalescing window (a free slot that finds a partial batch waits up to that
// long for it to fill, a full batch leaves at once), a bound on queued
// requests (submit waits for room, like the batcher's bounded channel), and a
// per-queue limit on running batches under the global slot count (the
// service's per-operation pipelines under its shared CUBBS_W3C_PIPELINES).
// Requests complete through a wait on their ticket or through a callback, and
// a snapshot reports the batcher's metrics.  With a caller-supplied processor
// the queue batches opaque items for the caller instead of the device (the
// batcher's generic processor, batcher.rs:130-167).
//
// The "plain" mode is the fixed-size batcher it replaces (one batch at a time,
// a batch leaves when it is full or its oldest request reaches the timeout).
//
// Every request's result is the result of the same request in a batch of its
// own: batching only changes which requests share a launch.
#include <sys/random.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "runtime.cuh"

namespace cubbs {
namespace {

using clk = std::chrono::steady_clock;

// Device queues: operation (queue & 3: 0 sign, 1 verify, 2 proof_gen,
// 3 proof_verify) under ciphersuite queue >> 2 (CUBBS_BBS_CIPHERSUITE_*).
constexpr int QUEUES = CUBBS_BBS_GPU_SERVE_MAX_QUEUES;
static_assert(QUEUES == 8, "two ciphersuites x four operations");
constexpr uint32_t MAX_PROCESSOR_SLOTS = 256;

struct Request {
  int op = 0;
  void *item = nullptr;
  bool seeded = false;
  uint8_t seed[32] = {};
  uint64_t ticket = 0;
  size_t est_bytes = 0;
  clk::time_point t_submit;
  clk::time_point t_done;
  CuBbsBbsGpuResult result = {CUBBS_BBS_GPU_ERR_INTERNAL, 0, 0};
  bool done = false;
  CuBbsBbsGpuServeDone notify = nullptr;
  void *notify_ctx = nullptr;
};

// Device bytes a request occupies while its batch runs (inputs, scalar rows,
// points, MSM partials, outputs), from the arena sizing of the batch planner.
size_t estimate_bytes(int op, const void *item) {
  switch (op & 3) {
    case 0: {
      const auto *it = static_cast<const CuBbsBbsGpuSignItem *>(item);
      return 4096 + 160 * it->message_count + it->header.len;
    }
    case 1: {
      const auto *it = static_cast<const CuBbsBbsGpuVerifyItem *>(item);
      return 6144 + 160 * it->message_count + it->header.len;
    }
    case 2: {
      const auto *it = static_cast<const CuBbsBbsGpuProofGenItem *>(item);
      return 8192 + 320 * it->message_count + it->header.len + it->presentation_header.len;
    }
    default: {
      const auto *it = static_cast<const CuBbsBbsGpuProofVerifyItem *>(item);
      return 8192 + 200 * it->total_message_count + it->header.len + it->presentation_header.len +
             it->proof.len;
    }
  }
}

// One operation's queue: pending requests, its batcher settings, the
// coalescing window a free slot has opened on it, and its dispatch metrics
// (batcher.rs:63-73).
struct Queue {
  std::deque<Request *> q;
  CuBbsBbsGpuServeQueueConfig qc{};
  uint32_t inflight = 0;
  bool collecting = false;
  clk::time_point window_end;
  uint64_t dispatches = 0, dispatched_items = 0, max_batch = 0, last_batch = 0, wait_us = 0;
  std::vector<uint64_t> size_counts;
};

struct Server {
  CuBbsBbsGpuServeConfig cfg{};
  CuBbsBbsGpuServeProcessor proc = nullptr;
  void *proc_ctx = nullptr;
  bool plain = false;
  uint32_t plain_batch = 0, plain_timeout_us = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_space;
  Queue qs[QUEUES];
  std::unordered_map<uint64_t, Request *> tickets;
  uint64_t next_ticket = 1;
  uint64_t last_batch_any = 0;
  size_t inflight_bytes = 0;
  bool stop = false;
  std::vector<std::thread> workers;

  void set_defaults() {
    for (int i = 0; i < QUEUES; i++) qs[i].qc = CuBbsBbsGpuServeQueueConfig{cfg.max_batch_items, 0, 0, 0};
  }

  // Whether queue `op` may dispatch now (mu held).  A queue at its running-
  // batch limit waits; without a window it is ready whenever it holds a
  // request; with one it is ready when a full batch is queued or the window a
  // free slot opened on it has closed.  While shutting down every queued
  // request is served.
  bool ready(int op, clk::time_point now) const {
    const Queue &s = qs[op];
    if (s.q.empty()) return false;
    if (plain) {
      const bool full = s.q.size() >= plain_batch;
      const bool old = now - s.q.front()->t_submit >= std::chrono::microseconds(plain_timeout_us);
      return full || old || stop;
    }
    if (s.qc.max_inflight && s.inflight >= s.qc.max_inflight) return false;
    if (stop || s.qc.coalesce_us == 0 || s.q.size() >= s.qc.max_batch_items) return true;
    return s.collecting && now >= s.window_end;
  }

  // The ready queue whose oldest request has waited longest (mu held); -1 if none.
  int pick(clk::time_point now) const {
    int best = -1;
    for (int op = 0; op < QUEUES; op++)
      if (ready(op, now) && (best < 0 || qs[op].q.front()->t_submit < qs[best].q.front()->t_submit)) best = op;
    return best;
  }

  // A free slot found nothing ready: it opens a coalescing window on every
  // queue that holds a partial batch, may dispatch and has none open yet
  // (batcher.rs:254-268: the window starts once a slot is held) (mu held).
  void open_windows(clk::time_point now) {
    if (plain) return;
    for (int op = 0; op < QUEUES; op++) {
      Queue &s = qs[op];
      if (s.q.empty() || s.collecting || s.qc.coalesce_us == 0) continue;
      if (s.qc.max_inflight && s.inflight >= s.qc.max_inflight) continue;
      s.collecting = true;
      s.window_end = now + std::chrono::microseconds(s.qc.coalesce_us);
    }
  }

  // Earliest time a waiting queue becomes ready by the clock alone (mu held).
  clk::time_point next_deadline() const {
    clk::time_point d = clk::time_point::max();
    for (int op = 0; op < QUEUES; op++) {
      const Queue &s = qs[op];
      if (s.q.empty()) continue;
      if (plain) d = std::min(d, s.q.front()->t_submit + std::chrono::microseconds(plain_timeout_us));
      else if (s.collecting) d = std::min(d, s.window_end);
    }
    return d;
  }

  bool all_empty() const {
    for (int op = 0; op < QUEUES; op++)
      if (!qs[op].q.empty()) return false;
    return true;
  }

  // Dispatch metrics of one batch (batcher.rs:271-294) (mu held).
  void record_dispatch(Queue &s, const std::vector<Request *> &batch, clk::time_point at) {
    const size_t n = batch.size();
    s.dispatches++;
    s.dispatched_items += n;
    s.last_batch = n;
    last_batch_any = n;
    s.max_batch = std::max<uint64_t>(s.max_batch, n);
    if (s.size_counts.size() <= n) s.size_counts.resize(n + 1, 0);
    s.size_counts[n]++;
    for (const Request *r : batch)
      if (at > r->t_submit)
        s.wait_us += (uint64_t)std::chrono::duration_cast<std::chrono::microseconds>(at - r->t_submit).count();
  }

  int32_t run_device(int op, std::vector<Request *> &batch, std::vector<CuBbsBbsGpuResult> &res) {
    const size_t n = batch.size();
    const uint32_t suite = (uint32_t)op >> 2;
    switch (op & 3) {
      case 0: {
        std::vector<CuBbsBbsGpuSignItem> items(n);
        for (size_t i = 0; i < n; i++) items[i] = *static_cast<CuBbsBbsGpuSignItem *>(batch[i]->item);
        const int32_t rc =
            cubbs_bbs_gpu_sign_batch_cs_v2(CUBBS_BBS_GPU_ABI_VERSION, suite, items.data(), n, res.data());
        for (size_t i = 0; i < n; i++)
          static_cast<CuBbsBbsGpuSignItem *>(batch[i]->item)->signature_out.len = items[i].signature_out.len;
        return rc;
      }
      case 1: {
        std::vector<CuBbsBbsGpuVerifyItem> items(n);
        for (size_t i = 0; i < n; i++) items[i] = *static_cast<CuBbsBbsGpuVerifyItem *>(batch[i]->item);
        return cubbs_bbs_gpu_verify_batch_cs_v2(CUBBS_BBS_GPU_ABI_VERSION, suite, items.data(), n, res.data());
      }
      case 2: {
        std::vector<CuBbsBbsGpuProofGenItem> items(n);
        std::vector<uint8_t> seeds(32 * n);
        for (size_t i = 0; i < n; i++) {
          items[i] = *static_cast<CuBbsBbsGpuProofGenItem *>(batch[i]->item);
          if (batch[i]->seeded) {
            std::memcpy(&seeds[32 * i], batch[i]->seed, 32);
          } else {
            size_t got = 0;
            while (got < 32) {
              ssize_t r = getrandom(&seeds[32 * i + got], 32 - got, 0);
              if (r > 0) got += (size_t)r;
            }
          }
        }
        const int32_t rc = cubbs_bbs_gpu_proof_gen_seeded_batch_cs_v2(
            CUBBS_BBS_GPU_ABI_VERSION, suite, items.data(), n, reinterpret_cast<const uint8_t(*)[32]>(seeds.data()),
            res.data());
        for (size_t i = 0; i < n; i++)
          static_cast<CuBbsBbsGpuProofGenItem *>(batch[i]->item)->proof_out.len = items[i].proof_out.len;
        return rc;
      }
      default: {
        std::vector<CuBbsBbsGpuProofVerifyItem> items(n);
        for (size_t i = 0; i < n; i++) items[i] = *static_cast<CuBbsBbsGpuProofVerifyItem *>(batch[i]->item);
        return cubbs_bbs_gpu_proof_verify_batch_cs_v2(CUBBS_BBS_GPU_ABI_VERSION, suite, items.data(), n,
                                                      res.data());
      }
    }
  }

  void run_batch(int op, std::vector<Request *> &batch) {
    const size_t n = batch.size();
    std::vector<CuBbsBbsGpuResult> res(n, CuBbsBbsGpuResult{CUBBS_BBS_GPU_ERR_INTERNAL, 0, 0});
    int32_t rc;
    if (proc) {
      std::vector<void *> items(n);
      for (size_t i = 0; i < n; i++) items[i] = batch[i]->item;
      rc = proc(proc_ctx, op, items.data(), n, res.data());
    } else {
      rc = run_device(op, batch, res);
    }
    const clk::time_point done = clk::now();
    std::vector<Request *> notify;
    {
      std::lock_guard<std::mutex> lk(mu);
      for (size_t i = 0; i < n; i++) {
        Request *r = batch[i];
        r->result = rc == CUBBS_BBS_GPU_SUCCESS ? res[i] : CuBbsBbsGpuResult{rc, 0, 0};
        r->t_done = done;
        inflight_bytes -= r->est_bytes;
        if (r->notify) notify.push_back(r);
        else r->done = true;
      }
      qs[op].inflight--;
    }
    cv_done.notify_all();
    cv_work.notify_all();
    // callbacks run outside the lock, so a callback may submit again
    for (Request *r : notify) {
      r->notify(r->notify_ctx, r->ticket, &r->result);
      delete r;
    }
  }

  void worker() {
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      const clk::time_point now = clk::now();
      const int op = pick(now);
      if (op < 0) {
        if (stop && all_empty()) return;
        open_windows(now);
        const clk::time_point d = next_deadline();
        if (d == clk::time_point::max()) cv_work.wait(lk);
        else cv_work.wait_until(lk, d);
        continue;
      }
      Queue &s = qs[op];
      const size_t cap = plain ? plain_batch : s.qc.max_batch_items;
      std::vector<Request *> batch;
      while (!s.q.empty() && batch.size() < cap) {
        Request *r = s.q.front();
        // admit by device-memory budget; an idle device always takes one request
        if (inflight_bytes + r->est_bytes > cfg.hbm_budget_bytes && (inflight_bytes > 0 || !batch.empty())) break;
        s.q.pop_front();
        inflight_bytes += r->est_bytes;
        batch.push_back(r);
      }
      if (batch.empty()) {  // over budget: wait for a running batch to finish
        cv_work.wait(lk);
        continue;
      }
      s.collecting = false;
      s.inflight++;
      record_dispatch(s, batch, clk::now());
      cv_space.notify_all();
      if (!all_empty()) cv_work.notify_one();
      lk.unlock();
      run_batch(op, batch);
      lk.lock();
    }
  }

  void start() {
    const int slots = plain ? 1 : (int)cfg.max_inflight;
    for (int i = 0; i < slots; i++) workers.emplace_back([this] { worker(); });
  }

  // Queues one request; waits while the queue holds queue_capacity requests.
  // Returns 0 once shut down.
  uint64_t submit(int op, void *item, const uint8_t *seed, CuBbsBbsGpuServeDone done = nullptr,
                  void *done_ctx = nullptr) {
    Request *r = new Request;
    r->op = op;
    r->item = item;
    if (seed) {
      r->seeded = true;
      std::memcpy(r->seed, seed, 32);
    }
    r->notify = done;
    r->notify_ctx = done_ctx;
    r->est_bytes = proc ? 0 : estimate_bytes(op, item);
    r->t_submit = clk::now();  // enqueued_at is taken before waiting for room (batcher.rs:171-180)
    std::unique_lock<std::mutex> lk(mu);
    Queue &s = qs[op];
    cv_space.wait(lk, [&] { return stop || !s.qc.queue_capacity || s.q.size() < s.qc.queue_capacity; });
    if (stop) {
      delete r;
      return 0;
    }
    r->ticket = next_ticket++;
    if (!done) tickets[r->ticket] = r;
    s.q.push_back(r);
    cv_work.notify_one();
    return r->ticket;
  }

  bool wait(uint64_t ticket, CuBbsBbsGpuResult *out, clk::time_point *t_submit, clk::time_point *t_done) {
    std::unique_lock<std::mutex> lk(mu);
    auto it = tickets.find(ticket);
    if (it == tickets.end()) return false;
    Request *r = it->second;
    cv_done.wait(lk, [r] { return r->done; });
    *out = r->result;
    if (t_submit) *t_submit = r->t_submit;
    if (t_done) *t_done = r->t_done;
    tickets.erase(it);
    delete r;
    return true;
  }

  void snapshot(int op, CuBbsBbsGpuServeSnapshot *out, uint64_t *counts, size_t counts_len) {
    std::lock_guard<std::mutex> lk(mu);
    CuBbsBbsGpuServeSnapshot o{};
    uint64_t wait_us = 0;
    if (counts) std::fill(counts, counts + counts_len, 0);
    for (int i = 0; i < QUEUES; i++) {
      if (op >= 0 && i != op) continue;
      const Queue &s = qs[i];
      o.queued += s.q.size();
      o.dispatches += s.dispatches;
      o.dispatched_items += s.dispatched_items;
      o.max_observed_batch = std::max(o.max_observed_batch, s.max_batch);
      o.inflight_batches += s.inflight;
      wait_us += s.wait_us;
      if (counts)
        for (size_t k = 0; k < std::min(counts_len, s.size_counts.size()); k++) counts[k] += s.size_counts[k];
    }
    o.last_batch_size = op >= 0 ? qs[op].last_batch : last_batch_any;
    o.total_queue_wait_ms = (double)wait_us / 1000.0;
    o.average_queue_wait_ms = o.dispatched_items ? (double)wait_us / (double)o.dispatched_items / 1000.0 : 0.0;
    *out = o;
  }

  // Stops taking requests, serves every queued one, then joins the slots.
  void shutdown() {
    {
      std::lock_guard<std::mutex> lk(mu);
      stop = true;
    }
    cv_work.notify_all();
    cv_space.notify_all();
    for (auto &t : workers) t.join();
    workers.clear();
  }
  ~Server() {
    shutdown();
    for (auto &kv : tickets) delete kv.second;
  }
};

CuBbsBbsGpuServeConfig normalise(const CuBbsBbsGpuServeConfig *in, bool device) {
  CuBbsBbsGpuServeConfig c = in ? *in : CuBbsBbsGpuServeConfig{};
  if (device) {
    SharedState &sh = SharedState::get();
    sh.init();
    if (c.max_inflight == 0 || c.max_inflight > (uint32_t)sh.workspaces) c.max_inflight = (uint32_t)sh.workspaces;
  } else {
    if (c.max_inflight == 0) c.max_inflight = 1;
    c.max_inflight = std::min(c.max_inflight, MAX_PROCESSOR_SLOTS);
  }
  if (c.max_batch_items == 0) c.max_batch_items = 1024;
  if (c.hbm_budget_bytes == 0) c.hbm_budget_bytes = (uint64_t)1 << 30;
  return c;
}

int32_t create_server(const CuBbsBbsGpuServeConfig *cfg, CuBbsBbsGpuServeProcessor proc, void *ctx,
                      void **server) {
  try {
    Server *s = new Server;
    s->proc = proc;
    s->proc_ctx = ctx;
    s->cfg = normalise(cfg, proc == nullptr);
    s->set_defaults();
    s->start();
    *server = s;
    return CUBBS_BBS_GPU_SUCCESS;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}

bool valid_queue(int32_t op) { return op >= 0 && op < QUEUES; }

}  // namespace
}  // namespace cubbs

using namespace cubbs;

extern "C" int32_t cubbs_bbs_gpu_serve_create(uint32_t abi, const CuBbsBbsGpuServeConfig *cfg, void **server) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || !server) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  return create_server(cfg, nullptr, nullptr, server);
}

extern "C" int32_t cubbs_bbs_gpu_serve_create_with_processor(uint32_t abi, const CuBbsBbsGpuServeConfig *cfg,
                                                             CuBbsBbsGpuServeProcessor processor, void *ctx,
                                                             void **server) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || !server || !processor) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  return create_server(cfg, processor, ctx, server);
}

extern "C" int32_t cubbs_bbs_gpu_serve_configure_queue(void *server, int32_t queue,
                                                       const CuBbsBbsGpuServeQueueConfig *config,
                                                       CuBbsBbsGpuServeQueueConfig *effective) {
  Server *s = static_cast<Server *>(server);
  if (!s || !valid_queue(queue)) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    Queue &q = s->qs[queue];
    if (config) {
      q.qc = *config;
      if (q.qc.max_batch_items == 0) q.qc.max_batch_items = s->cfg.max_batch_items;
      if (!q.qc.coalesce_us) q.collecting = false;
    }
    if (effective) *effective = q.qc;
  }
  s->cv_work.notify_all();
  s->cv_space.notify_all();
  return CUBBS_BBS_GPU_SUCCESS;
}

extern "C" int32_t cubbs_bbs_gpu_serve_submit(void *server, int32_t op, void *item, const uint8_t *seed32,
                                              uint64_t *ticket) {
  Server *s = static_cast<Server *>(server);
  if (!s || !item || !ticket || !valid_queue(op)) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  *ticket = s->submit(op, item, ((op & 3) == 2 && !s->proc) ? seed32 : nullptr);
  return *ticket ? CUBBS_BBS_GPU_SUCCESS : CUBBS_BBS_GPU_ERR_INVALID_INPUT;
}

extern "C" int32_t cubbs_bbs_gpu_serve_submit_notify(void *server, int32_t op, void *item, const uint8_t *seed32,
                                                     CuBbsBbsGpuServeDone done, void *ctx, uint64_t *ticket) {
  Server *s = static_cast<Server *>(server);
  if (!s || !item || !done || !valid_queue(op)) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  const uint64_t t = s->submit(op, item, ((op & 3) == 2 && !s->proc) ? seed32 : nullptr, done, ctx);
  if (ticket) *ticket = t;
  return t ? CUBBS_BBS_GPU_SUCCESS : CUBBS_BBS_GPU_ERR_INVALID_INPUT;
}

extern "C" int32_t cubbs_bbs_gpu_serve_wait(void *server, uint64_t ticket, CuBbsBbsGpuResult *result) {
  if (!server || !result) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  return static_cast<Server *>(server)->wait(ticket, result, nullptr, nullptr) ? CUBBS_BBS_GPU_SUCCESS
                                                                               : CUBBS_BBS_GPU_ERR_INVALID_INPUT;
}

extern "C" int32_t cubbs_bbs_gpu_serve_snapshot(void *server, int32_t queue, CuBbsBbsGpuServeSnapshot *out,
                                                uint64_t *batch_size_counts, size_t counts_len) {
  Server *s = static_cast<Server *>(server);
  if (!s || !out || (queue != -1 && !valid_queue(queue)) || (!batch_size_counts && counts_len))
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  s->snapshot(queue, out, batch_size_counts, counts_len);
  return CUBBS_BBS_GPU_SUCCESS;
}

extern "C" int32_t cubbs_bbs_gpu_serve_destroy(void *server) {
  if (!server) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  delete static_cast<Server *>(server);
  return CUBBS_BBS_GPU_SUCCESS;
}

// Load replay: request i (operation ops[i], ABI item items[i], optional seed)
// arrives arrival_ns[i] after the start and is submitted then by a generator
// thread; latency_ns[i] = completion - scheduled arrival.  mode 0: serving
// queue with `cfg`; mode 1: plain batches of plain_batch requests, flushed
// after plain_timeout_us.  wall_s = first arrival to last completion.
extern "C" int32_t cubbs_bbs_gpu_serve_replay(uint32_t abi, int32_t mode, const CuBbsBbsGpuServeConfig *cfg,
                                              const int32_t *ops, void *const *items, const uint8_t (*seeds)[32],
                                              const uint64_t *arrival_ns, size_t n, uint32_t plain_batch,
                                              uint32_t plain_timeout_us, uint64_t *latency_ns,
                                              CuBbsBbsGpuResult *results, double *wall_s) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || (mode != 0 && mode != 1) || !ops || !items || !arrival_ns ||
      !latency_ns || !results || !wall_s || (mode == 1 && plain_batch == 0))
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  for (size_t i = 0; i < n; i++)
    if (!valid_queue(ops[i]) || !items[i] || (i && arrival_ns[i] < arrival_ns[i - 1]))
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  try {
    Server s;
    s.cfg = normalise(cfg, true);
    s.set_defaults();
    s.plain = mode == 1;
    s.plain_batch = plain_batch;
    s.plain_timeout_us = plain_timeout_us;
    s.start();
    std::vector<uint64_t> tickets(n);
    const clk::time_point t0 = clk::now();
    std::thread gen([&] {
      for (size_t i = 0; i < n; i++) {
        const clk::time_point at = t0 + std::chrono::nanoseconds(arrival_ns[i]);
        while (clk::now() < at) {
          auto left = at - clk::now();
          if (left > std::chrono::microseconds(200)) std::this_thread::sleep_for(left - std::chrono::microseconds(100));
        }
        tickets[i] = s.submit(ops[i], items[i], ((ops[i] & 3) == 2 && seeds) ? seeds[i] : nullptr);
      }
    });
    gen.join();
    clk::time_point last = t0;
    for (size_t i = 0; i < n; i++) {
      clk::time_point ts, td;
      s.wait(tickets[i], &results[i], &ts, &td);
      const clk::time_point at = t0 + std::chrono::nanoseconds(arrival_ns[i]);
      latency_ns[i] = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(td - at).count();
      last = std::max(last, td);
    }
    *wall_s = std::chrono::duration<double>(last - t0).count();
    return CUBBS_BBS_GPU_SUCCESS;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}
