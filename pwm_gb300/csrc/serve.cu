// Serving: a continuous-batching request loop over device-resident wavelet
// structures.
//
// A server owns `slots` worker threads, each with its own context (its own
// CUDA stream and scratch, stream-ordered allocations).  Requests wait in one
// FIFO queue; the head is admitted as soon as a slot is idle and its device
// bytes fit the HBM budget next to the resident structures and the requests
// in flight.  Admitted requests run concurrently, one per slot, so their
// kernels overlap on the device: a build request copies its text, builds the
// structure(s) with rank/select support, answers its first batch of
// access/rank/select queries and leaves the structure resident; a query
// request answers a batch against a resident structure.  A structure's bytes
// return to the budget when the client releases it (after its queries).
//
// Everything goes through the library's C ABI, so a request's answers are
// exactly those of the same calls made alone.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <stdexcept>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/pwmgpu.h"
#include "common.cuh"

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
  uint64_t id = 0;
  bool build = true;  // false: queries against structure `target`
  pwmgpu_request req{};
  uint64_t target = 0;
  uint64_t transient = 0;  // device bytes while running (text, queries, scratch growth)
  uint64_t resident = 0;   // device bytes of the structure(s) it leaves behind
  int state = 0;           // 0 queued, 1 running, 2 done
  pwmgpu_status status = PWMGPU_OK;
  std::string error;
  double t_submit = 0, t_start = 0, t_done = 0;
  pwmgpu_wx* wx = nullptr;  // build requests: the resident structure
  int users = 0;            // query requests in flight against it
  bool released = false;
  uint32_t slot = 0;
};

// Device bytes of a structure pair with rank/select support (an upper bound).
uint64_t structure_bytes(uint64_t n, uint32_t levels, uint32_t flags) {
  const uint64_t words = pwmgpu::padded_words(n);
  const uint64_t per_level = words * 8 + (words / 32 + 2) * 8 + 2 * (n / 8192 + 2) * 4 + 3 * 256;
  const uint64_t structs = ((flags & PWMGPU_MATRIX) ? 1 : 0) + ((flags & PWMGPU_TREE) ? 1 : 0) +
                           ((flags & PWMGPU_MATRIX) ? 0 : 1);  // a tree alone keeps its matrix source
  return structs * (levels * per_level + 4096);
}

// Transient device bytes of a build: the text, the key sequences of the split
// passes, histograms and tables (per symbol value 8 bytes of leaf histogram,
// 16 of prefix counts of every level and up to 16 of a tree's regroup
// segments, rounded up to 48), queries and answers.
uint64_t build_scratch_bytes(uint64_t n, uint32_t width, uint32_t levels, uint64_t nq) {
  return 3 * n * width + (uint64_t(8) << std::min<uint32_t>(levels, 24)) * 6 + (n / 1024 + 64) * 256 +
         nq * 25 + (uint64_t(16) << 20);
}

}  // namespace

struct pwmgpu_server {
  int device = 0;
  uint64_t budget = 0;
  uint64_t in_use = 0;  // resident + in-flight estimates
  uint64_t peak = 0;
  uint64_t next_id = 1;
  uint64_t completed = 0, running = 0;
  bool stop = false;
  double t0 = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> queue;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> all;
  std::vector<pwmgpu_ctx*> slots;
  std::vector<std::thread> workers;

  bool admissible(const Request* r) const { return in_use + r->transient + r->resident <= budget; }
  void worker(uint32_t slot);
  void run(Request* r, pwmgpu_ctx* ctx);
  void free_structure(Request* r);
};

namespace {

// Answers a batch of queries against a resident structure on one context:
// the mixed batch in one launch, answers in request order.
void answer(pwmgpu_ctx* ctx, pwmgpu_wx* wx, uint32_t which, uint64_t count, const uint8_t* ops, const uint64_t* qa,
            const uint64_t* qb, uint64_t* results) {
  if (count == 0) return;
  for (uint64_t i = 0; i < count; ++i) {
    if (ops[i] > PWMGPU_Q_SELECT) throw std::runtime_error("unknown query kind");
    if (ops[i] != PWMGPU_Q_ACCESS && !qb) throw std::runtime_error("rank and select queries need query_b");
  }
  if (pwmgpu_wx_query_batch_host(ctx, wx, int(which), ops, qa, qb, count, results) != PWMGPU_OK)
    throw std::runtime_error(pwmgpu_ctx_last_error(ctx));
}

}  // namespace

void pwmgpu_server::free_structure(Request* r) {
  if (r->wx) pwmgpu_wx_free(r->wx);
  r->wx = nullptr;
  in_use -= r->resident;
  r->resident = 0;
}

void pwmgpu_server::run(Request* r, pwmgpu_ctx* ctx) {
  const pwmgpu_request& q = r->req;
  if (r->build) {
    pwmgpu_wx* wx = nullptr;
    pwmgpu_status st = pwmgpu_wx_create(ctx, q.size, q.word_width, q.levels, q.shape_flags | PWMGPU_RANK_SELECT, &wx);
    if (st == PWMGPU_OK) st = pwmgpu_wx_build_host(ctx, wx, q.text);
    if (st == PWMGPU_OK) st = pwmgpu_wx_check(ctx, wx);
    if (st != PWMGPU_OK) {
      r->status = st;
      r->error = pwmgpu_ctx_last_error(ctx);
      pwmgpu_wx_free(wx);
      return;
    }
    r->wx = wx;
    try {
      answer(ctx, wx, q.query_structure, q.nqueries, q.query_ops, q.query_a, q.query_b, q.results);
    } catch (const std::exception& e) {
      r->status = PWMGPU_ERR_ARG;
      r->error = e.what();
    }
  } else {
    Request* t = nullptr;
    {
      std::lock_guard<std::mutex> g(mu);
      auto it = all.find(r->target);
      if (it != all.end() && it->second->wx && !it->second->released) t = it->second.get();
    }
    if (!t) {
      r->status = PWMGPU_ERR_ARG;
      r->error = "no resident structure with that id";
      return;
    }
    try {
      answer(ctx, t->wx, q.query_structure, q.nqueries, q.query_ops, q.query_a, q.query_b, q.results);
    } catch (const std::exception& e) {
      r->status = PWMGPU_ERR_ARG;
      r->error = e.what();
    }
  }
}

void pwmgpu_server::worker(uint32_t slot) {
  cudaSetDevice(device);
  pwmgpu_ctx* ctx = slots[slot];
  for (;;) {
    Request* r = nullptr;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_work.wait(lk, [&]() { return stop || (!queue.empty() && admissible(queue.front())); });
      if (stop && queue.empty()) return;
      if (queue.empty() || !admissible(queue.front())) continue;
      r = queue.front();
      queue.pop_front();
      in_use += r->transient + r->resident;
      peak = std::max(peak, in_use);
      ++running;
      r->state = 1;
      r->slot = slot;
      r->t_start = now_s() - t0;
      if (!r->build) {
        auto it = all.find(r->target);
        if (it != all.end()) ++it->second->users;
      }
    }
    run(r, ctx);
    {
      std::lock_guard<std::mutex> g(mu);
      in_use -= r->transient;
      if (r->status != PWMGPU_OK && r->build) free_structure(r);  // a failed build keeps nothing
      if (!r->build) {
        auto it = all.find(r->target);
        if (it != all.end()) {
          Request* t = it->second.get();
          if (--t->users == 0 && t->released) free_structure(t);
        }
      }
      --running;
      ++completed;
      r->t_done = now_s() - t0;
      r->state = 2;
    }
    cv_done.notify_all();
    cv_work.notify_all();
  }
}

extern "C" {

pwmgpu_status pwmgpu_server_create(int device, uint64_t hbm_budget_bytes, uint32_t slots, pwmgpu_server** out) {
  if (!out || slots == 0 || slots > 64 || hbm_budget_bytes == 0) return PWMGPU_ERR_ARG;
  *out = nullptr;
  auto s = std::make_unique<pwmgpu_server>();
  s->device = device;
  s->budget = hbm_budget_bytes;
  s->t0 = now_s();
  for (uint32_t i = 0; i < slots; ++i) {
    pwmgpu_ctx* ctx = nullptr;
    pwmgpu_status st = pwmgpu_ctx_create(device, nullptr, &ctx);
    if (st == PWMGPU_OK) st = pwmgpu_ctx_set_stream_ordered_alloc(ctx, 1);
    if (st != PWMGPU_OK) {
      if (ctx) pwmgpu_ctx_destroy(ctx);
      for (auto* c : s->slots) pwmgpu_ctx_destroy(c);
      return st;
    }
    s->slots.push_back(ctx);
  }
  for (uint32_t i = 0; i < slots; ++i) s->workers.emplace_back([p = s.get(), i]() { p->worker(i); });
  *out = s.release();
  return PWMGPU_OK;
}

pwmgpu_status pwmgpu_server_submit(pwmgpu_server* s, const pwmgpu_request* req, uint64_t* id) {
  if (!s || !req || !id) return PWMGPU_ERR_ARG;
  if (req->size && !req->text) return PWMGPU_ERR_ARG;
  if (req->nqueries && (!req->query_ops || !req->query_a || !req->results)) return PWMGPU_ERR_ARG;
  if (req->word_width != 1 && req->word_width != 2 && req->word_width != 4) return PWMGPU_ERR_ARG;
  if (req->levels == 0 || req->levels > 24 || req->size == 0) return PWMGPU_ERR_ARG;
  if (!(req->shape_flags & (PWMGPU_MATRIX | PWMGPU_TREE)) || req->query_structure > 1) return PWMGPU_ERR_ARG;
  if (req->query_structure == 1 && !(req->shape_flags & PWMGPU_TREE)) return PWMGPU_ERR_ARG;
  if (req->query_structure == 0 && !(req->shape_flags & PWMGPU_MATRIX)) return PWMGPU_ERR_ARG;
  auto r = std::make_unique<Request>();
  r->req = *req;
  r->build = true;
  r->resident = structure_bytes(req->size, req->levels, req->shape_flags);
  r->transient = build_scratch_bytes(req->size, req->word_width, req->levels, req->nqueries);
  if (r->resident + r->transient > s->budget) return PWMGPU_ERR_OOM;  // can never be admitted
  {
    std::lock_guard<std::mutex> g(s->mu);
    r->id = s->next_id++;
    r->t_submit = now_s() - s->t0;
    *id = r->id;
    s->queue.push_back(r.get());
    s->all.emplace(r->id, std::move(r));
  }
  s->cv_work.notify_all();
  return PWMGPU_OK;
}

pwmgpu_status pwmgpu_server_submit_queries(pwmgpu_server* s, uint64_t structure_id, uint32_t query_structure,
                                           uint64_t nqueries, const uint8_t* ops, const uint64_t* a,
                                           const uint64_t* b, uint64_t* results, uint64_t* id) {
  if (!s || !id || (nqueries && (!ops || !a || !results)) || query_structure > 1) return PWMGPU_ERR_ARG;
  auto r = std::make_unique<Request>();
  r->build = false;
  r->target = structure_id;
  r->req.nqueries = nqueries;
  r->req.query_ops = ops;
  r->req.query_a = a;
  r->req.query_b = b;
  r->req.results = results;
  r->req.query_structure = query_structure;
  r->transient = nqueries * 24 + (uint64_t(1) << 20);
  {
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->all.find(structure_id);
    if (it == s->all.end() || !it->second->build || it->second->released || it->second->state != 2 ||
        !it->second->wx)
      return PWMGPU_ERR_ARG;  // needs a finished, unreleased build
    const uint32_t f = it->second->req.shape_flags;
    if ((query_structure == 1 && !(f & PWMGPU_TREE)) || (query_structure == 0 && !(f & PWMGPU_MATRIX)))
      return PWMGPU_ERR_ARG;
    r->id = s->next_id++;
    r->t_submit = now_s() - s->t0;
    *id = r->id;
    s->queue.push_back(r.get());
    s->all.emplace(r->id, std::move(r));
  }
  s->cv_work.notify_all();
  return PWMGPU_OK;
}

static void fill_info(const Request* r, pwmgpu_request_info* info) {
  if (!info) return;
  info->id = r->id;
  info->status = int(r->status);
  info->submit_s = r->t_submit;
  info->start_s = r->t_start;
  info->done_s = r->t_done;
  info->device_bytes = r->resident;
  info->slot = r->slot;
}

pwmgpu_status pwmgpu_server_wait(pwmgpu_server* s, uint64_t id, pwmgpu_request_info* info) {
  if (!s) return PWMGPU_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return PWMGPU_ERR_ARG;
  Request* r = it->second.get();
  s->cv_done.wait(lk, [&]() { return r->state == 2; });
  fill_info(r, info);
  return r->status;
}

pwmgpu_status pwmgpu_server_poll(pwmgpu_server* s, uint64_t id, pwmgpu_request_info* info) {
  if (!s) return PWMGPU_ERR_ARG;
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return PWMGPU_ERR_ARG;
  const Request* r = it->second.get();
  if (r->state != 2) return PWMGPU_ERR_BUSY;
  fill_info(r, info);
  return r->status;
}

const char* pwmgpu_server_error(pwmgpu_server* s, uint64_t id) {
  if (!s) return "";
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->all.find(id);
  return it == s->all.end() ? "" : it->second->error.c_str();
}

pwmgpu_status pwmgpu_server_release(pwmgpu_server* s, uint64_t id) {
  if (!s) return PWMGPU_ERR_ARG;
  {
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end() || it->second->state != 2) return PWMGPU_ERR_ARG;
    Request* r = it->second.get();
    if (r->build && !r->released) {
      r->released = true;
      if (r->users == 0) s->free_structure(r);
    }
    if (!r->build) s->all.erase(it);  // a finished query request has nothing left
  }
  s->cv_work.notify_all();
  return PWMGPU_OK;
}

pwmgpu_status pwmgpu_server_stats(pwmgpu_server* s, pwmgpu_server_stats_t* st) {
  if (!s || !st) return PWMGPU_ERR_ARG;
  std::lock_guard<std::mutex> g(s->mu);
  st->budget_bytes = s->budget;
  st->in_use_bytes = s->in_use;
  st->peak_bytes = s->peak;
  st->queued = s->queue.size();
  st->running = s->running;
  st->completed = s->completed;
  return PWMGPU_OK;
}

void pwmgpu_server_destroy(pwmgpu_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
    for (auto* r : s->queue) {  // never started
      r->status = PWMGPU_ERR_ARG;
      r->error = "server destroyed";
      r->state = 2;
    }
    s->queue.clear();
  }
  s->cv_work.notify_all();
  s->cv_done.notify_all();
  for (auto& t : s->workers) t.join();
  for (auto& kv : s->all)
    if (kv.second->wx) pwmgpu_wx_free(kv.second->wx);
  for (auto* c : s->slots) pwmgpu_ctx_destroy(c);
  delete s;
}

}  // extern "C"
