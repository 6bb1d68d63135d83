// server.cpp -- h2h_server_*: a query server over resident graphs with
// continuous batching.  No counterpart in the reference, whose Query_noHub
// flow (main.cu:218-240) runs one prepared batch of one graph at a time.
//
// Requests (pairs of one graph in one mode) are queued by any thread and
// answered asynchronously.  One worker thread owns all CUDA work.  It keeps
// up to `slots` device batches in flight, each on its own stream: copy the
// pairs in, run the query kernel, copy the answers out, record an event.
// Whenever a batch retires, its answers are scattered to the requests and
// the slot is refilled at once from the pending queue: the oldest request
// picks the (graph, mode) and later requests with the same key join the
// batch in arrival order up to the slot's capacity (a larger request is
// split over several batches).  So requests that arrive while others run are
// admitted as soon as a slot frees, and the transfers and kernels of
// different slots overlap on the device.  Graphs are admitted against a
// device-memory budget.  Pairs with a vertex id out of range answer -1.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "gpuh2h.h"
#include "handle.h"

namespace {

double now_us() {
  using namespace std::chrono;
  return duration<double, std::micro>(steady_clock::now().time_since_epoch()).count();
}

// cudaMemoryTypeHost for page-locked memory, Unregistered for pageable
// memory, Device / Managed for memory the server does not take.
cudaMemoryType memory_type(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return cudaMemoryTypeUnregistered;
  }
  return a.type;
}

struct Request {
  uint64_t id = 0;
  int graph = 0, mode = 0;
  const int *x = nullptr, *y = nullptr;
  int *out = nullptr;
  int64_t n = 0;
  int64_t next = 0;      // first pair not yet placed in a batch
  int64_t remaining = 0; // pairs not yet answered
  bool pinned = false;
  double t_submit = 0, t_done = 0;
  bool done = false;
};

struct Piece {
  Request *r;
  int64_t req_off, slot_off, count;
};

struct Slot {
  int64_t cap = 0;
  int *dx = nullptr, *dy = nullptr, *dout = nullptr;
  int *dbad = nullptr;  // this slot's out-of-range flag (answers carry -1 instead)
  int *hx = nullptr, *hy = nullptr, *hout = nullptr;  // pinned staging
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr, k0 = nullptr, k1 = nullptr;
  std::vector<Piece> pieces;
  bool busy = false;
  int64_t pairs = 0;
};

}  // namespace

struct h2h_server {
  h2h_server_config cfg{};
  int device = 0;
  std::vector<h2h_graph *> graphs;      // by graph id (nullptr = removed)
  std::vector<int64_t> graph_bytes;
  int64_t admitted_bytes = 0;
  std::vector<Slot> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request *> pending;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> requests;
  uint64_t next_id = 1;
  bool stop = false;
  std::string worker_error;
  std::thread worker;
  // statistics (worker writes, readers take mu)
  int64_t st_requests = 0, st_pairs = 0, st_batches = 0, st_max_inflight = 0;
  double st_kernel_us = 0, st_first_submit = 0, st_last_done = 0;

  ~h2h_server() {
    {
      std::lock_guard<std::mutex> l(mu);
      stop = true;
    }
    cv_work.notify_all();
    if (worker.joinable()) worker.join();
    for (Slot &s : slots) {
      if (s.stream) cudaStreamSynchronize(s.stream);
      cudaFree(s.dx); cudaFree(s.dy); cudaFree(s.dout); cudaFree(s.dbad);
      cudaFreeHost(s.hx); cudaFreeHost(s.hy); cudaFreeHost(s.hout);
      if (s.done) cudaEventDestroy(s.done);
      if (s.k0) cudaEventDestroy(s.k0);
      if (s.k1) cudaEventDestroy(s.k1);
      if (s.stream) cudaStreamDestroy(s.stream);
    }
  }

  // Fills slot s from the pending queue (called with mu held).  Returns
  // false when nothing is pending.
  bool take(Slot &s, const gh::Graph *&gp, int &mode) {
    if (pending.empty()) return false;
    Request *head = pending.front();
    const int graph = head->graph;
    gp = &graphs[graph]->g;
    mode = head->mode;
    s.pieces.clear();
    s.pairs = 0;
    for (auto it = pending.begin(); it != pending.end() && s.pairs < s.cap;) {
      Request *r = *it;
      if (r->graph != graph || r->mode != mode) { ++it; continue; }
      const int64_t c = std::min(r->n - r->next, s.cap - s.pairs);
      s.pieces.push_back({r, r->next, s.pairs, c});
      r->next += c;
      s.pairs += c;
      if (r->next == r->n) it = pending.erase(it);
      else ++it;
    }
    return true;
  }

  void launch(Slot &s, const gh::Graph &g, int mode) {
    for (const Piece &p : s.pieces) {
      if (p.r->pinned) {
        GH_CUDA(cudaMemcpyAsync(s.dx + p.slot_off, p.r->x + p.req_off, sizeof(int) * p.count,
                                cudaMemcpyHostToDevice, s.stream));
        GH_CUDA(cudaMemcpyAsync(s.dy + p.slot_off, p.r->y + p.req_off, sizeof(int) * p.count,
                                cudaMemcpyHostToDevice, s.stream));
      } else {
        std::memcpy(s.hx + p.slot_off, p.r->x + p.req_off, sizeof(int) * p.count);
        std::memcpy(s.hy + p.slot_off, p.r->y + p.req_off, sizeof(int) * p.count);
      }
    }
    bool staged = false;
    for (const Piece &p : s.pieces) staged |= !p.r->pinned;
    if (staged) {  // one copy of the staged range (pinned pieces land on top in stream order first)
      // copy only the staged pieces, merged where contiguous
      int64_t a = -1, b = -1;
      auto flush = [&]() {
        if (a < 0) return;
        GH_CUDA(cudaMemcpyAsync(s.dx + a, s.hx + a, sizeof(int) * (b - a), cudaMemcpyHostToDevice, s.stream));
        GH_CUDA(cudaMemcpyAsync(s.dy + a, s.hy + a, sizeof(int) * (b - a), cudaMemcpyHostToDevice, s.stream));
        a = b = -1;
      };
      for (const Piece &p : s.pieces) {
        if (p.r->pinned) { flush(); continue; }
        if (a >= 0 && b == p.slot_off) b += p.count;
        else { flush(); a = p.slot_off; b = p.slot_off + p.count; }
      }
      flush();
    }
    GH_CUDA(cudaEventRecord(s.k0, s.stream));
    gh::run_query_batch(g, s.dx, s.dy, s.dout, s.pairs, mode, s.stream, s.dbad);
    GH_CUDA(cudaEventRecord(s.k1, s.stream));
    for (const Piece &p : s.pieces) {
      if (p.r->pinned)
        GH_CUDA(cudaMemcpyAsync(p.r->out + p.req_off, s.dout + p.slot_off, sizeof(int) * p.count,
                                cudaMemcpyDeviceToHost, s.stream));
    }
    if (staged)
      GH_CUDA(cudaMemcpyAsync(s.hout, s.dout, sizeof(int) * s.pairs, cudaMemcpyDeviceToHost, s.stream));
    GH_CUDA(cudaEventRecord(s.done, s.stream));
    s.busy = true;
  }

  void retire(Slot &s) {
    float kms = 0;
    cudaEventElapsedTime(&kms, s.k0, s.k1);
    for (const Piece &p : s.pieces)
      if (!p.r->pinned) std::memcpy(p.r->out + p.req_off, s.hout + p.slot_off, sizeof(int) * p.count);
    const double t = now_us();
    {
      std::lock_guard<std::mutex> l(mu);
      for (const Piece &p : s.pieces) {
        p.r->remaining -= p.count;
        if (p.r->remaining == 0) {
          p.r->done = true;
          p.r->t_done = t;
          st_requests++;
          st_pairs += p.r->n;
        }
      }
      st_batches++;
      st_kernel_us += kms * 1000.0;
      st_last_done = t;
    }
    s.pieces.clear();
    s.busy = false;
    cv_done.notify_all();
  }

  void run() {
    cudaSetDevice(device);
    try {
      for (;;) {
        bool progressed = false;
        int inflight = 0;
        for (Slot &s : slots) {
          if (!s.busy) continue;
          const cudaError_t q = cudaEventQuery(s.done);
          if (q == cudaSuccess) {
            retire(s);
            progressed = true;
          } else if (q != cudaErrorNotReady) {
            GH_CUDA(q);
          } else {
            inflight++;
          }
        }
        for (Slot &s : slots) {
          if (s.busy) continue;
          const gh::Graph *gp = nullptr;
          int mode = 0;
          {
            std::lock_guard<std::mutex> l(mu);
            if (!take(s, gp, mode)) break;
          }
          launch(s, *gp, mode);
          progressed = true;
          inflight++;
        }
        {
          std::lock_guard<std::mutex> l(mu);
          st_max_inflight = std::max<int64_t>(st_max_inflight, inflight);
        }
        if (progressed) continue;
        std::unique_lock<std::mutex> l(mu);
        if (stop && pending.empty() && inflight == 0) return;
        if (inflight == 0) {
          cv_work.wait(l, [&] { return stop || !pending.empty(); });
        } else {
          // batches in flight: poll their events, waking early for new work
          cv_work.wait_for(l, std::chrono::microseconds(std::max(1, cfg.poll_us)),
                           [&] { return stop || !pending.empty(); });
        }
      }
    } catch (const std::exception &e) {
      std::lock_guard<std::mutex> l(mu);
      worker_error = e.what();
      for (auto &kv : requests)
        if (!kv.second->done) {
          kv.second->done = true;
          kv.second->t_done = now_us();
        }
      cv_done.notify_all();
    }
  }
};

extern "C" {

void h2h_server_default_config(h2h_server_config *c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->slots = 4;
  c->slot_pairs = 1 << 20;
  c->poll_us = 5;
  c->memory_budget = 0;
}

int h2h_server_create(const h2h_server_config *cfg, h2h_server **out) {
  if (out) *out = nullptr;
  if (!out) { gh::set_last_error("null output"); return H2H_ERR_ARG; }
  return gh::guarded([&] {
    h2h_server_config c;
    h2h_server_default_config(&c);
    if (cfg) c = *cfg;
    GH_CHECK(c.slots >= 1 && c.slots <= 64, H2H_ERR_ARG, "slots must be 1..64");
    GH_CHECK(c.slot_pairs >= 1 && c.slot_pairs <= (int64_t(1) << 30), H2H_ERR_ARG, "slot_pairs must be 1..2^30");
    GH_CHECK(c.poll_us >= 0, H2H_ERR_ARG, "poll_us must be >= 0");
    auto s = std::make_unique<h2h_server>();
    s->cfg = c;
    GH_CUDA(cudaGetDevice(&s->device));
    if (c.memory_budget <= 0) {
      size_t fr = 0, tot = 0;
      GH_CUDA(cudaMemGetInfo(&fr, &tot));
      s->cfg.memory_budget = (int64_t)fr;
    }
    s->slots.resize(c.slots);
    for (Slot &sl : s->slots) {
      sl.cap = c.slot_pairs;
      GH_CUDA(cudaMalloc(&sl.dx, sizeof(int) * sl.cap));
      GH_CUDA(cudaMalloc(&sl.dy, sizeof(int) * sl.cap));
      GH_CUDA(cudaMalloc(&sl.dout, sizeof(int) * sl.cap));
      GH_CUDA(cudaMalloc(&sl.dbad, sizeof(int)));
      GH_CUDA(cudaMallocHost(&sl.hx, sizeof(int) * sl.cap));
      GH_CUDA(cudaMallocHost(&sl.hy, sizeof(int) * sl.cap));
      GH_CUDA(cudaMallocHost(&sl.hout, sizeof(int) * sl.cap));
      GH_CUDA(cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking));
      GH_CUDA(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming));
      GH_CUDA(cudaEventCreate(&sl.k0));
      GH_CUDA(cudaEventCreate(&sl.k1));
    }
    h2h_server *raw = s.get();
    s->worker = std::thread([raw] { raw->run(); });
    *out = s.release();
  });
}

int h2h_server_add_graph(h2h_server *s, h2h_graph *g, int *graph_id) {
  if (!s || !g || !graph_id) { gh::set_last_error("null argument"); return H2H_ERR_ARG; }
  return gh::guarded([&] {
    GH_CHECK(g->g.labelled, H2H_ERR_STATE, "graph has no labels");
    const int64_t b = g->g.dev.bytes;
    std::lock_guard<std::mutex> l(s->mu);
    GH_CHECK(s->admitted_bytes + b <= s->cfg.memory_budget, H2H_ERR_NOMEM,
             "graph's resident index exceeds the server's remaining memory budget");
    s->admitted_bytes += b;
    s->graphs.push_back(g);
    s->graph_bytes.push_back(b);
    *graph_id = (int)s->graphs.size() - 1;
  });
}

int h2h_server_remove_graph(h2h_server *s, int graph_id) {
  if (!s) { gh::set_last_error("null server"); return H2H_ERR_ARG; }
  return gh::guarded([&] {
    std::unique_lock<std::mutex> l(s->mu);
    GH_CHECK(graph_id >= 0 && graph_id < (int)s->graphs.size() && s->graphs[graph_id], H2H_ERR_ARG,
             "unknown graph id");
    // wait until no request of this graph is unanswered
    s->cv_done.wait(l, [&] {
      for (auto &kv : s->requests)
        if (kv.second->graph == graph_id && !kv.second->done) return false;
      return true;
    });
    s->admitted_bytes -= s->graph_bytes[graph_id];
    s->graphs[graph_id] = nullptr;
  });
}

int h2h_server_submit(h2h_server *s, int graph_id, const int *x, const int *y, int *out, int64_t n, int mode,
                      uint64_t *request) {
  if (!s || !request) { gh::set_last_error("null argument"); return H2H_ERR_ARG; }
  return gh::guarded([&] {
    GH_CHECK(mode == H2H_QUERY_LCA || mode == H2H_QUERY_NOLCA, H2H_ERR_ARG, "mode must be 0 (LCA) or 1 (noLCA)");
    GH_CHECK(n >= 1, H2H_ERR_ARG, "a request holds at least one pair");
    GH_CHECK(x && y && out, H2H_ERR_ARG, "null buffer");
    const cudaMemoryType tx = memory_type(x), ty = memory_type(y), to = memory_type(out);
    for (cudaMemoryType t : {tx, ty, to})
      GH_CHECK(t == cudaMemoryTypeHost || t == cudaMemoryTypeUnregistered, H2H_ERR_ARG,
               "the server takes host buffers (pageable or page-locked)");
    const bool pinned = tx == cudaMemoryTypeHost && ty == cudaMemoryTypeHost && to == cudaMemoryTypeHost;
    auto r = std::make_unique<Request>();
    r->graph = graph_id;
    r->mode = mode;
    r->x = x;
    r->y = y;
    r->out = out;
    r->n = n;
    r->remaining = n;
    r->pinned = pinned;
    {
      std::lock_guard<std::mutex> l(s->mu);
      GH_CHECK(s->worker_error.empty(), H2H_ERR_CUDA, "server worker stopped: " + s->worker_error);
      GH_CHECK(graph_id >= 0 && graph_id < (int)s->graphs.size() && s->graphs[graph_id], H2H_ERR_ARG,
               "unknown graph id");
      r->id = s->next_id++;
      r->t_submit = now_us();
      if (s->st_first_submit == 0) s->st_first_submit = r->t_submit;
      *request = r->id;
      s->pending.push_back(r.get());
      s->requests.emplace(r->id, std::move(r));
    }
    s->cv_work.notify_one();
  });
}

int h2h_server_wait(h2h_server *s, uint64_t request, int64_t timeout_us) {
  if (!s) { gh::set_last_error("null server"); return H2H_ERR_ARG; }
  return gh::guarded([&] {
    std::unique_lock<std::mutex> l(s->mu);
    auto it = s->requests.find(request);
    GH_CHECK(it != s->requests.end(), H2H_ERR_ARG, "unknown request");
    Request *r = it->second.get();
    auto ready = [&] { return r->done; };
    if (timeout_us < 0) s->cv_done.wait(l, ready);
    else if (!s->cv_done.wait_for(l, std::chrono::microseconds(timeout_us), ready))
      throw gh::Error(H2H_ERR_STATE, "request not finished within the timeout");
    GH_CHECK(s->worker_error.empty(), H2H_ERR_CUDA, "server worker stopped: " + s->worker_error);
  });
}

int h2h_server_test(h2h_server *s, uint64_t request) {
  if (!s) return H2H_ERR_ARG;
  std::lock_guard<std::mutex> l(s->mu);
  auto it = s->requests.find(request);
  if (it == s->requests.end()) return H2H_ERR_ARG;
  return it->second->done ? 1 : 0;
}

int h2h_server_release(h2h_server *s, uint64_t request, double *latency_us) {
  if (!s) { gh::set_last_error("null server"); return H2H_ERR_ARG; }
  return gh::guarded([&] {
    std::lock_guard<std::mutex> l(s->mu);
    auto it = s->requests.find(request);
    GH_CHECK(it != s->requests.end(), H2H_ERR_ARG, "unknown request");
    GH_CHECK(it->second->done, H2H_ERR_STATE, "request still running");
    if (latency_us) *latency_us = it->second->t_done - it->second->t_submit;
    s->requests.erase(it);
  });
}

int h2h_server_get_stats(h2h_server *s, h2h_server_stats *st) {
  if (!s || !st) { gh::set_last_error("null argument"); return H2H_ERR_ARG; }
  std::lock_guard<std::mutex> l(s->mu);
  std::memset(st, 0, sizeof(*st));
  st->requests = s->st_requests;
  st->pairs = s->st_pairs;
  st->batches = s->st_batches;
  st->max_inflight = s->st_max_inflight;
  st->pending = (int64_t)s->pending.size();
  st->kernel_us = s->st_kernel_us;
  st->span_us = s->st_last_done > s->st_first_submit ? s->st_last_done - s->st_first_submit : 0;
  st->admitted_bytes = s->admitted_bytes;
  st->memory_budget = s->cfg.memory_budget;
  return H2H_OK;
}

int h2h_server_reset_stats(h2h_server *s) {
  if (!s) return H2H_ERR_ARG;
  std::lock_guard<std::mutex> l(s->mu);
  s->st_requests = s->st_pairs = s->st_batches = s->st_max_inflight = 0;
  s->st_kernel_us = 0;
  s->st_first_submit = s->st_last_done = 0;
  return H2H_OK;
}

void h2h_server_free(h2h_server *s) { delete s; }

}  // extern "C"
