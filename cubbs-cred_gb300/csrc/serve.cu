// Serving queue for the four BBS operations: continuous batching on top of
// the batch entry points.
//
// Requests of any of the four operations are submitted one at a time and
// complete one at a time.  A fixed number of dispatch slots (at most the
// number of device workspaces) each take the next batch as soon as they are
// free: the operation whose oldest request has waited longest, as many of its
// queued requests as fit in the batch size and in the device-memory budget
// still unclaimed by the other running batches.  Batches of different slots
// run concurrently on their own streams, so requests that arrive while others
// are on the device are admitted as soon as a slot and memory free up.
//
// The "plain" mode is the fixed-size batcher it replaces (one batch at a time,
// a batch leaves when it is full or its oldest request reaches the timeout),
// the shape of the reference service's interval batcher
// (crates/cubbs-w3c-service/src/batcher.rs:21-60,223-320).
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

enum { OPS = 4 };  // 0 sign, 1 verify, 2 proof_gen, 3 proof_verify

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
};

// Device bytes a request occupies while its batch runs (inputs, scalar rows,
// points, MSM partials, outputs), from the arena sizing of the batch planner.
size_t estimate_bytes(int op, const void *item) {
  switch (op) {
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

struct Server {
  CuBbsBbsGpuServeConfig cfg{};
  bool plain = false;
  uint32_t plain_batch = 0, plain_timeout_us = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request *> q[OPS];
  std::unordered_map<uint64_t, Request *> tickets;
  uint64_t next_ticket = 1;
  size_t inflight_bytes = 0;
  bool stop = false;
  std::vector<std::thread> workers;

  // Picks the operation to serve next (mu held); -1 if nothing is ready.
  int pick(clk::time_point now) {
    int best = -1;
    for (int op = 0; op < OPS; op++) {
      if (q[op].empty()) continue;
      if (plain) {
        bool full = q[op].size() >= plain_batch;
        bool old = now - q[op].front()->t_submit >= std::chrono::microseconds(plain_timeout_us);
        if (!full && !old) continue;
      }
      if (best < 0 || q[op].front()->t_submit < q[best].front()->t_submit) best = op;
    }
    return best;
  }

  // Earliest time a plain-mode queue times out (mu held).
  clk::time_point next_deadline() {
    clk::time_point d = clk::time_point::max();
    for (int op = 0; op < OPS; op++)
      if (!q[op].empty()) d = std::min(d, q[op].front()->t_submit + std::chrono::microseconds(plain_timeout_us));
    return d;
  }

  void run_batch(int op, std::vector<Request *> &batch) {
    const size_t n = batch.size();
    std::vector<CuBbsBbsGpuResult> res(n);
    int32_t rc = CUBBS_BBS_GPU_ERR_INTERNAL;
    switch (op) {
      case 0: {
        std::vector<CuBbsBbsGpuSignItem> items(n);
        for (size_t i = 0; i < n; i++) items[i] = *static_cast<CuBbsBbsGpuSignItem *>(batch[i]->item);
        rc = cubbs_bbs_gpu_sign_batch_v2(CUBBS_BBS_GPU_ABI_VERSION, items.data(), n, res.data());
        for (size_t i = 0; i < n; i++)
          static_cast<CuBbsBbsGpuSignItem *>(batch[i]->item)->signature_out.len = items[i].signature_out.len;
        break;
      }
      case 1: {
        std::vector<CuBbsBbsGpuVerifyItem> items(n);
        for (size_t i = 0; i < n; i++) items[i] = *static_cast<CuBbsBbsGpuVerifyItem *>(batch[i]->item);
        rc = cubbs_bbs_gpu_verify_batch_v2(CUBBS_BBS_GPU_ABI_VERSION, items.data(), n, res.data());
        break;
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
        rc = cubbs_bbs_gpu_proof_gen_seeded_batch_v2(CUBBS_BBS_GPU_ABI_VERSION, items.data(), n,
                                                     reinterpret_cast<const uint8_t(*)[32]>(seeds.data()),
                                                     res.data());
        for (size_t i = 0; i < n; i++)
          static_cast<CuBbsBbsGpuProofGenItem *>(batch[i]->item)->proof_out.len = items[i].proof_out.len;
        break;
      }
      default: {
        std::vector<CuBbsBbsGpuProofVerifyItem> items(n);
        for (size_t i = 0; i < n; i++) items[i] = *static_cast<CuBbsBbsGpuProofVerifyItem *>(batch[i]->item);
        rc = cubbs_bbs_gpu_proof_verify_batch_v2(CUBBS_BBS_GPU_ABI_VERSION, items.data(), n, res.data());
        break;
      }
    }
    const clk::time_point done = clk::now();
    std::lock_guard<std::mutex> lk(mu);
    for (size_t i = 0; i < n; i++) {
      Request *r = batch[i];
      r->result = rc == CUBBS_BBS_GPU_SUCCESS ? res[i] : CuBbsBbsGpuResult{rc, 0, 0};
      r->t_done = done;
      r->done = true;
      inflight_bytes -= r->est_bytes;
    }
    cv_done.notify_all();
    cv_work.notify_all();
  }

  void worker() {
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      int op = -1;
      while (!stop) {
        op = pick(clk::now());
        if (op >= 0) break;
        if (plain) {
          clk::time_point d = next_deadline();
          if (d == clk::time_point::max()) cv_work.wait(lk);
          else cv_work.wait_until(lk, d);
        } else {
          cv_work.wait(lk);
        }
      }
      if (stop && op < 0) return;
      const size_t cap = plain ? plain_batch : cfg.max_batch_items;
      std::vector<Request *> batch;
      while (!q[op].empty() && batch.size() < cap) {
        Request *r = q[op].front();
        // admit by device-memory budget; an idle device always takes one request
        if (inflight_bytes + r->est_bytes > cfg.hbm_budget_bytes && (inflight_bytes > 0 || !batch.empty())) break;
        q[op].pop_front();
        inflight_bytes += r->est_bytes;
        batch.push_back(r);
      }
      if (batch.empty()) {  // over budget: wait for a running batch to finish
        cv_work.wait(lk);
        continue;
      }
      lk.unlock();
      run_batch(op, batch);
      lk.lock();
    }
  }

  void start() {
    const int slots = plain ? 1 : (int)cfg.max_inflight;
    for (int i = 0; i < slots; i++) workers.emplace_back([this] { worker(); });
  }

  uint64_t submit(int op, void *item, const uint8_t *seed) {
    Request *r = new Request;
    r->op = op;
    r->item = item;
    if (seed) {
      r->seeded = true;
      std::memcpy(r->seed, seed, 32);
    }
    r->est_bytes = estimate_bytes(op, item);
    r->t_submit = clk::now();
    std::lock_guard<std::mutex> lk(mu);
    r->ticket = next_ticket++;
    tickets[r->ticket] = r;
    q[op].push_back(r);
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

  void shutdown() {
    {
      std::lock_guard<std::mutex> lk(mu);
      stop = true;
    }
    cv_work.notify_all();
    for (auto &t : workers) t.join();
    workers.clear();
  }
  ~Server() {
    shutdown();
    for (auto &kv : tickets) delete kv.second;
    for (int op = 0; op < OPS; op++) q[op].clear();
  }
};

bool valid_op(int32_t op) { return op >= 0 && op < OPS; }

CuBbsBbsGpuServeConfig normalise(const CuBbsBbsGpuServeConfig *in) {
  CuBbsBbsGpuServeConfig c = in ? *in : CuBbsBbsGpuServeConfig{};
  SharedState &sh = SharedState::get();
  sh.init();
  if (c.max_inflight == 0 || c.max_inflight > (uint32_t)sh.workspaces) c.max_inflight = (uint32_t)sh.workspaces;
  if (c.max_batch_items == 0) c.max_batch_items = 1024;
  if (c.hbm_budget_bytes == 0) c.hbm_budget_bytes = (uint64_t)1 << 30;
  return c;
}

}  // namespace
}  // namespace cubbs

using namespace cubbs;

extern "C" int32_t cubbs_bbs_gpu_serve_create(uint32_t abi, const CuBbsBbsGpuServeConfig *cfg, void **server) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || !server) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  try {
    Server *s = new Server;
    s->cfg = normalise(cfg);
    s->start();
    *server = s;
    return CUBBS_BBS_GPU_SUCCESS;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}

extern "C" int32_t cubbs_bbs_gpu_serve_submit(void *server, int32_t op, void *item, const uint8_t *seed32,
                                              uint64_t *ticket) {
  if (!server || !item || !ticket || !valid_op(op)) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  *ticket = static_cast<Server *>(server)->submit(op, item, op == 2 ? seed32 : nullptr);
  return CUBBS_BBS_GPU_SUCCESS;
}

extern "C" int32_t cubbs_bbs_gpu_serve_wait(void *server, uint64_t ticket, CuBbsBbsGpuResult *result) {
  if (!server || !result) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  return static_cast<Server *>(server)->wait(ticket, result, nullptr, nullptr) ? CUBBS_BBS_GPU_SUCCESS
                                                                               : CUBBS_BBS_GPU_ERR_INVALID_INPUT;
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
    if (!valid_op(ops[i]) || !items[i] || (i && arrival_ns[i] < arrival_ns[i - 1]))
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  try {
    Server s;
    s.cfg = normalise(cfg);
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
        tickets[i] = s.submit(ops[i], items[i], (ops[i] == 2 && seeds) ? seeds[i] : nullptr);
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
