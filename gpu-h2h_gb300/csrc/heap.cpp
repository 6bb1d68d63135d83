// heap.cpp -- elimination of the vertices of partition levels <= C in global
// minimum-degree order: Graph::uploadCHset + CHUsingHeap_2
// (Traditional_H2H.cu:28-118, :216-351).
//
// Order: the reference keeps a std::set<HostRank> keyed by
// (CHInfo.first + CHInfo.second, CHInfo.first, id) and erases/reinserts a
// vertex whenever its key changes; a lazy-deletion binary heap over the same
// key pops the same vertex at every step.  Initial keys are (number of valid
// list entries, counting parallel duplicates, height from the partition
// levels); after an elimination a neighbour's key becomes (|adjacency|,
// max(height(v) + 1, height(u))).  Adjacency maps keep the first-seen entry
// of a duplicated neighbour, like unordered_map::emplace.
//
// Fill-in: the reference inserts/updates pair by pair in hash maps; here each
// neighbour's sorted adjacency is merged with the eliminated vertex's list in
// one linear pass (min on equal ids), in parallel across neighbours.
#include <algorithm>
#include <queue>
#include <tuple>

#include "graph.h"
#include "pool.h"

namespace gh {

namespace {
struct Entry {
  int id, w;
};
}  // namespace

void contract_global_heap(Graph &g, const std::vector<int64_t> &lst_off, const std::vector<int> &lst_nbr,
                          const std::vector<int> &lst_w) {
  Clock clk;
  const int n = g.n;
  if ((int)g.height.size() != n) g.height.assign(n, 0);
  std::vector<std::vector<Entry>> adj(n);
  std::vector<int> key_deg(n, -1), key_h(n, -1);
  std::vector<char> in_heap(n, 0);
  // map built from a list: keep the first occurrence of every id, sort by id
  auto build_map = [&](int v, int &count) {
    std::vector<Entry> e;
    count = 0;
    for (int64_t k = lst_off[v]; k < lst_off[v + 1]; k++) {
      if (lst_nbr[k] == INT32_MAX) continue;
      count++;
      e.push_back({lst_nbr[k], lst_w[k]});
    }
    std::stable_sort(e.begin(), e.end(), [](const Entry &a, const Entry &b) { return a.id < b.id; });
    e.erase(std::unique(e.begin(), e.end(), [](const Entry &a, const Entry &b) { return a.id == b.id; }), e.end());
    adj[v].swap(e);
  };
  int64_t tmp_index = INT32_MAX;
  for (int h = g.C; h > 0; h--) {                                 // :43-75
    const int64_t lo = (int64_t(1) << (h - 1)) - 1, hi = (int64_t(1) << h) - 2;
    for (int64_t c = hi; c >= lo; c--) {
      tmp_index = std::min<int64_t>(tmp_index, g.cell_start[c]);
      for (int i = 0; i < g.cell_count[c]; i++) {
        int v = g.elim[g.cell_start[c] + i];
        int cnt = 0;
        build_map(v, cnt);
        key_deg[v] = cnt;
        key_h[v] = g.height[v];
        in_heap[v] = 1;
      }
    }
  }
  for (int h = g.H; h > g.C; h--) {                               // :76-104
    const int64_t lo = (int64_t(1) << (h - 1)) - 1, hi = (int64_t(1) << h) - 2;
    for (int64_t c = hi; c >= lo; c--)
      for (int i = 0; i < g.cell_count[c]; i++) {
        int v = g.elim[g.cell_start[c] + i], cnt;
        build_map(v, cnt);
      }
  }
  g.gpu_vertices = (int)tmp_index;
  using K = std::tuple<int, int, int>;  // (deg + height, deg, id)
  std::priority_queue<K, std::vector<K>, std::greater<K>> pq;
  for (int v = 0; v < n; v++)
    if (in_heap[v]) pq.push(K(key_deg[v] + key_h[v], key_deg[v], v));
  Pool pool(g.threads);
  int64_t idx = tmp_index;
  std::vector<Entry> nei;
  while (!pq.empty()) {                                           // :222-323
    K top = pq.top();
    pq.pop();
    const int v = std::get<2>(top);
    if (!in_heap[v] || std::get<1>(top) != key_deg[v] || std::get<0>(top) != key_deg[v] + key_h[v]) continue;
    in_heap[v] = 0;
    g.elim[idx++] = v;
    nei = adj[v];
    const int d = (int)nei.size();
    const int hv = key_h[v];
    auto merge_one = [&](int i) {
      const int u = nei[i].id, wu = nei[i].w;
      std::vector<Entry> &au = adj[u];
      std::vector<Entry> out;
      out.reserve(au.size() + d);
      size_t a = 0;
      int b = 0;
      while (a < au.size() || b < d) {
        if (b < d && nei[b].id == u) { b++; continue; }
        if (a < au.size() && au[a].id == v) { a++; continue; }
        if (b >= d || (a < au.size() && au[a].id < nei[b].id)) {
          out.push_back(au[a++]);
        } else if (a >= au.size() || nei[b].id < au[a].id) {
          out.push_back({nei[b].id, wu + nei[b].w});
          b++;
        } else {
          int w = std::min(au[a].w, wu + nei[b].w);
          out.push_back({au[a].id, w});
          a++;
          b++;
        }
      }
      au.swap(out);
    };
    if (d >= 48 && pool.size() > 1) {
      pool.parallel_for(d, 4, [&](int64_t b, int64_t e, int) {
        for (int64_t i = b; i < e; i++) merge_one((int)i);
      });
    } else {
      for (int i = 0; i < d; i++) merge_one(i);
    }
    for (int i = 0; i < d; i++) {
      const int u = nei[i].id;
      key_deg[u] = (int)adj[u].size();
      key_h[u] = std::max(hv + 1, key_h[u]);
      pq.push(K(key_deg[u] + key_h[u], key_deg[u], u));
    }
  }
  GH_CHECK(idx == n, H2H_ERR_STATE, "global elimination did not reach every vertex");
  // X(v)\{v} for every vertex: adjacency at elimination time, sorted by id
  g.x_off.assign(n + 1, 0);
  for (int v = 0; v < n; v++) g.x_off[v + 1] = g.x_off[v] + (int64_t)adj[v].size();
  g.x_id.resize(g.x_off[n]);
  g.x_w.resize(g.x_off[n]);
  for (int v = 0; v < n; v++) {
    int64_t o = g.x_off[v];
    for (size_t k = 0; k < adj[v].size(); k++) { g.x_id[o + k] = adj[v][k].id; g.x_w[o + k] = adj[v][k].w; }
  }
  g.decomposition_size = g.x_off[n] + n;
  g.t.td_cpu = clk.us();
}

}  // namespace gh
