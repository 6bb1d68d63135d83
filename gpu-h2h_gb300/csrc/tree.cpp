// tree.cpp -- tree decomposition structure and label layout on the host:
//   getTreeStructure / OULADFS (TreeStructure.cu:102-262): children, Euler
//     tour, depths, from the fathers the contraction picked on the GPU
//   mallocH2HLabel_noHub (H2HConsturction.cu:618-722): row and position
//     offsets (the position lists themselves are built on the GPU for L4)
//   constructBFSTree     (H2HConsturction.cu:324-377)
//
// The Euler tour is walked with an explicit stack (the reference recurses),
// children in increasing id order as Childs lists them.  The sparse table is
// built on the GPU (query.cu).
#include <algorithm>
#include <atomic>

#include "graph.h"
#include "pool.h"

namespace gh {

void build_tree(Graph &g) {
  Clock clk;
  const int n = g.n;
  GH_CHECK((int)g.father.size() == n, H2H_ERR_STATE, "fathers missing");
  g.head = g.elim[n - 1];
  for (int v = 0; v < n; v++)
    GH_CHECK((g.father[v] < 0) == (v == g.head), H2H_ERR_STATE, "decomposition is not a single tree");
  std::vector<int> cnt(n, 0);
  for (int v = 0; v < n; v++) if (g.father[v] >= 0) cnt[g.father[v]]++;
  g.child_off.assign(n + 1, 0);
  for (int v = 0; v < n; v++) g.child_off[v + 1] = g.child_off[v] + cnt[v];
  g.childs.assign(std::max(0, n - 1), -1);
  std::vector<int> fill(g.child_off.begin(), g.child_off.end() - 1);
  for (int v = 0; v < n; v++) if (g.father[v] >= 0) g.childs[fill[g.father[v]]++] = v;
  GH_CHECK(g.child_off[n] == n - 1, H2H_ERR_STATE, "decomposition is not a single tree");
  // Euler tour
  const int64_t L = 2 * (int64_t)n - 1;
  std::vector<int> eid(L);
  g.first.assign(n, -1);
  g.depth.assign(n, -1);
  std::vector<int> stk, cur;
  stk.reserve(1024);
  cur.reserve(1024);
  int64_t e = 0;
  g.h2h_size = 0;
  g.tree_height = 0;
  stk.push_back(g.head);
  cur.push_back(0);
  eid[e] = g.head; g.first[g.head] = 0; e++;
  g.depth[g.head] = 1;
  g.h2h_size = 1;
  g.tree_height = 1;
  while (!stk.empty()) {
    int v = stk.back();
    int &c = cur.back();
    if (g.child_off[v] + c < g.child_off[v + 1]) {
      int ch = g.childs[g.child_off[v] + c];
      c++;
      int d = (int)stk.size() + 1;
      eid[e] = ch; g.first[ch] = (int)e; e++;
      g.depth[ch] = d;
      g.h2h_size += d;
      g.tree_height = std::max(g.tree_height, d);
      stk.push_back(ch);
      cur.push_back(0);
    } else {
      stk.pop_back();
      cur.pop_back();
      if (!stk.empty()) { eid[e] = stk.back(); e++; }
    }
  }
  GH_CHECK(e == L, H2H_ERR_STATE, "Euler tour does not cover the tree");
  g.euler_n = L;
  g.euler_id.swap(eid);
  g.t.tree = clk.us();
}

// Prefix sums and the per-node heavy-child choice run on the host's threads
// (ranges of up to kGrain nodes inline); the level order, subtree sizes and
// path layout stay single passes -- level-by-level parallel versions were
// measured slower on a 4,180-level tree.
namespace {
constexpr int64_t kGrain = 32768;

// out[0] = 0, out[i + 1] = out[i] + val(i) for i < n, in chunks on the pool.
template <typename F>
void prefix_sums(Pool &pool, int64_t n, std::vector<int64_t> &out, F val) {
  out.assign(n + 1, 0);
  const int64_t nch = (n + kGrain - 1) / kGrain;
  std::vector<int64_t> part(nch + 1, 0);
  pool.parallel_for(nch, 1, [&](int64_t lo, int64_t hi, int) {
    for (int64_t c = lo; c < hi; c++) {
      int64_t t = 0;
      for (int64_t i = c * kGrain; i < std::min(n, (c + 1) * kGrain); i++) t += val(i);
      part[c + 1] = t;
    }
  });
  for (int64_t c = 0; c < nch; c++) part[c + 1] += part[c];
  pool.parallel_for(nch, 1, [&](int64_t lo, int64_t hi, int) {
    for (int64_t c = lo; c < hi; c++) {
      int64_t t = part[c];
      for (int64_t i = c * kGrain; i < std::min(n, (c + 1) * kGrain); i++) {
        t += val(i);
        out[i + 1] = t;
      }
    }
  });
}
}  // namespace

void allocate_labels_and_bfs(Graph &g) {
  Clock clk;
  const int n = g.n;
  Pool pool(g.threads);
  if (!g.tree_layout) prefix_sums(pool, n, g.dis_hash, [&](int64_t v) { return (int64_t)g.depth[v]; });
  prefix_sums(pool, n, g.pos_hash, [&](int64_t v) { return (int64_t)(g.x_off[v + 1] - g.x_off[v]) + 1; });
  // host position lists only for the level-synchronous fill; the dataflow
  // fill builds them on the GPU from the device lists
  if (uses_level_fill(g)) {
    if ((int64_t)g.x_id.size() != g.x_off[n]) download_lists(g);
    g.pos_id.resize(g.pos_hash[n]);
    g.pos_pos.resize(g.pos_hash[n]);
    g.pos_w.resize(g.pos_hash[n]);
    std::atomic<int> bad{-1};
    pool.parallel_for(n, 1024, [&](int64_t b, int64_t e, int) {
      std::vector<std::pair<int64_t, int>> tmp;
      for (int64_t vv = b; vv < e; vv++) {
        const int v = (int)vv;
        const int d = g.depth[v];
        tmp.clear();
        for (int64_t k = g.x_off[v]; k < g.x_off[v + 1]; k++) {
          int a = g.x_id[k], p = g.depth[a] - 1;
          if (p < 0 || p >= d - 1) { bad = v; continue; }
          tmp.push_back({(int64_t)p << 32 | (uint32_t)a, g.x_w[k]});
        }
        tmp.push_back({(int64_t)(d - 1) << 32 | (uint32_t)v, 0});
        std::sort(tmp.begin(), tmp.end());  // positions are distinct
        int64_t o = g.pos_hash[v];
        for (size_t k = 0; k < tmp.size(); k++) {
          g.pos_pos[o + k] = (int)(tmp[k].first >> 32);
          g.pos_id[o + k] = (int)(tmp[k].first & 0xffffffff);
          g.pos_w[o + k] = tmp[k].second;
        }
      }
    });
    GH_CHECK(bad.load() < 0, H2H_ERR_STATE, "an upper neighbour is not an ancestor in the tree");
  } else {
    std::vector<int>().swap(g.pos_id);
    std::vector<int>().swap(g.pos_pos);
    std::vector<int>().swap(g.pos_w);
  }
  g.t.malloc_labels = clk.us();
  clk.reset();
  if (g.tree_layout) {  // built with the tree on the GPU (tree_gpu.cu)
    g.t.bfs = clk.us();
    return;
  }
  // level order from the head, children in Childs order
  g.tree_bfs.clear();
  g.tree_bfs.reserve(n);
  g.tree_hash.assign(1, 0);
  g.tree_bfs.push_back(g.head);
  g.tree_hash.push_back(1);
  size_t qh = 0;
  while (qh < g.tree_bfs.size()) {
    size_t end = g.tree_bfs.size();
    for (; qh < end; qh++) {
      int v = g.tree_bfs[qh];
      for (int k = g.child_off[v]; k < g.child_off[v + 1]; k++) g.tree_bfs.push_back(g.childs[k]);
    }
    if (g.tree_bfs.size() > end) g.tree_hash.push_back((int)g.tree_bfs.size());
  }
  // heavy paths: subtree sizes bottom-up over the level order, heavy child
  // = largest subtree (first in Childs order on ties), paths laid out by a
  // depth-first walk that continues along the heavy child
  std::vector<int> size(n, 1), heavy(n, -1), top(n, -1), hpos(n, -1);
  for (int i = n - 1; i > 0; i--) size[g.father[g.tree_bfs[i]]] += size[g.tree_bfs[i]];
  pool.parallel_for(n, kGrain, [&](int64_t lo, int64_t hi, int) {
    for (int64_t v = lo; v < hi; v++) {
      int best = 0;
      for (int k = g.child_off[v]; k < g.child_off[v + 1]; k++)
        if (size[g.childs[k]] > best) { best = size[g.childs[k]]; heavy[v] = g.childs[k]; }
    }
  });
  g.hld.assign(n, -1);
  int next = 0;
  std::vector<int> starts{g.head};
  while (!starts.empty()) {
    const int t = starts.back();
    starts.pop_back();
    for (int v = t; v >= 0; v = heavy[v]) {
      top[v] = t;
      hpos[v] = next;
      g.hld[next++] = v;
      for (int k = g.child_off[v + 1] - 1; k >= g.child_off[v]; k--)
        if (g.childs[k] != heavy[v]) starts.push_back(g.childs[k]);
    }
  }
  GH_CHECK(next == n, H2H_ERR_STATE, "heavy-path layout does not cover the tree");
  // root-path segments per node: one more than the father's when the node
  // starts a heavy path (counted top-down over the level order); the
  // segment lists themselves are written on the GPU
  std::vector<int> segs(n, 0);
  for (int i = 0; i < n; i++) {
    const int v = g.tree_bfs[i], f = g.father[v];
    segs[v] = (f < 0 ? 0 : segs[f]) + (top[v] == v ? 1 : 0);
  }
  prefix_sums(pool, n, g.seg_off, [&](int64_t v) { return (int64_t)segs[v]; });
  g.max_segs = *std::max_element(segs.begin(), segs.end());
  g.htop.swap(top);
  g.hpos.swap(hpos);
  g.t.bfs = clk.us();
}

}  // namespace gh
