// loadgen.cpp -- h2h_server_load: open- and closed-loop request streams for
// measuring the query server (a measurement tool, not a product path).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>

#include "gpuh2h.h"
#include "gpuh2h_tools.h"
#include "handle.h"

namespace {

struct SplitMix {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0, 1)
};

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Pinned {
  int *p = nullptr;
  ~Pinned() {
    if (p) cudaFreeHost(p);
  }
  void alloc(int64_t n) { GH_CUDA(cudaMallocHost(&p, sizeof(int) * std::max<int64_t>(n, 1))); }
};

struct Outstanding {
  uint64_t id;
  int64_t ring_off, n, waste;  // waste: ring tail skipped to place this request
  int graph;
  double lag_us;  // submission behind its scheduled arrival
};

}  // namespace

extern "C" int h2h_server_load(h2h_server *s, const int *graph_ids, const int *graph_n, int ngraphs,
                               const h2h_load_params *p, double *latency_us, int64_t *sizes, int *graph_of,
                               int64_t max_requests, h2h_load_result *res) {
  if (!s || !graph_ids || !graph_n || ngraphs <= 0 || !p || !res) {
    gh::set_last_error("null or empty argument");
    return H2H_ERR_ARG;
  }
  return gh::guarded([&] {
    GH_CHECK(p->size_lo >= 1 && p->size_hi >= p->size_lo, H2H_ERR_ARG, "need 1 <= size_lo <= size_hi");
    GH_CHECK(p->rate > 0 || (p->inflight >= 1 && p->requests >= 1), H2H_ERR_ARG,
             "closed loop needs inflight >= 1 and requests >= 1");
    std::memset(res, 0, sizeof(*res));
    SplitMix rng{p->seed ? p->seed : 1};
    // pair pools: per graph 4 x size_hi uniform pairs (requests take random windows)
    const int64_t pool = std::max<int64_t>(4 * p->size_hi, 1 << 16);
    std::vector<Pinned> px(ngraphs), py(ngraphs);
    for (int g = 0; g < ngraphs; g++) {
      px[g].alloc(pool);
      py[g].alloc(pool);
      for (int64_t i = 0; i < pool; i++) {
        px[g].p[i] = (int)(rng.next() % (uint64_t)graph_n[g]);
        py[g].p[i] = (int)(rng.next() % (uint64_t)graph_n[g]);
      }
    }
    // answer ring: regions are taken in submission order and freed in
    // release order (also submission order)
    const int64_t ring_cap = std::max<int64_t>(64 * p->size_hi, 1 << 22);
    Pinned ring;
    ring.alloc(ring_cap);
    std::mutex mu;
    std::deque<Outstanding> outq;
    int64_t ring_head = 0, ring_used = 0;
    std::atomic<bool> submit_done{false};
    std::atomic<int64_t> finished{0}, inflight_now{0};
    std::string err;
    // collector: waits for requests in submission order and records latency
    std::thread collector([&] {
      for (;;) {
        Outstanding o{};
        {
          std::unique_lock<std::mutex> l(mu);
          if (outq.empty()) {
            if (submit_done.load()) return;
            l.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(20));
            continue;
          }
          o = outq.front();
        }
        double lat = 0;
        int rc = h2h_server_wait(s, o.id, -1);
        if (rc == H2H_OK) rc = h2h_server_release(s, o.id, &lat);
        std::lock_guard<std::mutex> l(mu);
        if (rc != H2H_OK && err.empty()) err = h2h_last_error();
        const int64_t k = finished.load();
        if (k < max_requests) {
          if (latency_us) latency_us[k] = lat + o.lag_us;
          if (sizes) sizes[k] = o.n;
          if (graph_of) graph_of[k] = o.graph;
        }
        res->pairs += o.n;
        finished.fetch_add(1);
        inflight_now.fetch_sub(1);
        outq.pop_front();
        ring_used -= o.n + o.waste;
      }
    });
    const double lo = std::log((double)p->size_lo), hi = std::log((double)p->size_hi + 1.0);
    const double t0 = now_s();
    double next_arrival = t0;
    int64_t submitted = 0;
    try {
      for (;;) {
        if (p->rate > 0) {
          if (next_arrival - t0 >= p->duration_s) break;
        } else {
          if (submitted >= p->requests) break;
          while (inflight_now.load() >= p->inflight) std::this_thread::yield();
        }
        const int g = (int)(rng.next() % (uint64_t)ngraphs);
        const int64_t n = std::min<int64_t>(p->size_hi, (int64_t)std::exp(lo + (hi - lo) * rng.uniform()));
        const int64_t off = (int64_t)(rng.next() % (uint64_t)(pool - n + 1));
        double lag = 0;
        if (p->rate > 0) {
          next_arrival += -std::log(1.0 - rng.uniform()) / p->rate;
          while (now_s() < next_arrival) {
          }
          lag = (now_s() - next_arrival) * 1e6;
          if (lag > 100) res->late++;
        }
        // an answer region in the ring (wait for older requests to drain)
        int64_t roff = 0, rwaste = 0;
        for (;;) {
          std::lock_guard<std::mutex> l(mu);
          if (!err.empty()) throw gh::Error(H2H_ERR_CUDA, err);
          int64_t start = ring_head;
          int64_t waste = 0;
          if (start + n > ring_cap) { waste = ring_cap - start; start = 0; }
          if (ring_used + waste + n <= ring_cap) {
            ring_used += waste + n;
            ring_head = start + n;
            roff = start;
            rwaste = waste;
            break;
          }
        }
        uint64_t id = 0;
        const int rc = h2h_server_submit(s, graph_ids[g], px[g].p + off, py[g].p + off, ring.p + roff, n, p->mode, &id);
        if (rc != H2H_OK) throw gh::Error(rc, h2h_last_error());
        {
          std::lock_guard<std::mutex> l(mu);
          outq.push_back({id, roff, n, rwaste, g, lag});
        }
        inflight_now.fetch_add(1);
        submitted++;
      }
    } catch (...) {
      submit_done = true;
      collector.join();
      throw;
    }
    submit_done = true;
    collector.join();
    GH_CHECK(err.empty(), H2H_ERR_CUDA, err);
    res->wall_s = now_s() - t0;
    res->requests = finished.load();
  });
}
