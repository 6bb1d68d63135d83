// elim_sets.cpp -- the per-cell elimination sets and the LUB capacities,
// Graph::makeAdjcentNode(0) (GraphPartition.cu:178-308).
//
// Bottom-up over partition levels h = H..1, cells of a level from the highest
// index down: a vertex of a cell that has no alive neighbour outside the cell
// is interior and joins the cell's candidate range of `elim`; vertices stay
// alive for the parent level otherwise.  The capacity of a vertex's adjacency
// slot range is the largest (alive cell size + alive out-of-cell arcs) over
// the levels it takes part in, at least its input degree.  Capacities bound
// every list the partition-level contraction can build, so the device lists
// never move.
#include <algorithm>

#include "graph.h"

namespace gh {

void build_elimination_sets(Graph &g) {
  Clock clk;
  const int n = g.n;
  const int64_t cells = (int64_t(1) << g.H) - 1;
  std::vector<char> alive(n, 1), alive_next(n, 1);
  std::vector<int> stamp(n, -1);
  g.cap.resize(n);
  for (int v = 0; v < n; v++) g.cap[v] = g.adj_off[v + 1] - g.adj_off[v];
  g.cell_start.assign(cells, 0);
  g.cell_count.assign(cells, 0);
  g.elim.clear();
  g.elim.reserve(n);
  g.layer_rate.assign(g.H + 1, 0.0);
  std::vector<int> members;
  for (int h = g.H; h > 0; h--) {
    const int64_t lo = (int64_t(1) << (h - 1)) - 1, hi = (int64_t(1) << h) - 2;
    alive_next = alive;
    for (int64_t c = hi; c >= lo; c--) {
      g.cell_start[c] = (int)g.elim.size();
      members.clear();
      for (int j = g.cut_l[c]; j < g.cut_r[c]; j++) {
        int v = g.part_ids[j];
        if (!alive[v] || stamp[v] == (int)c) continue;
        stamp[v] = (int)c;
        members.push_back(v);
      }
      std::sort(members.begin(), members.end());  // std::map iteration order of the reference
      const int sz = (int)members.size();
      for (int v : members) {
        int out = sz;
        for (int e = g.adj_off[v]; e < g.adj_off[v + 1]; e++) {
          int u = g.adj_v[e];
          if (alive[u] && stamp[u] != (int)c) out++;
        }
        if (out == sz) {
          alive_next[v] = 0;
          g.elim.push_back(v);
          g.cell_count[c]++;
        }
        g.cap[v] = std::max(g.cap[v], out);
      }
      for (int v : members) stamp[v] = -1;
    }
    alive.swap(alive_next);
    g.layer_rate[h] = (double)g.elim.size() / n;
  }
  g.t.rank_tree = clk.us();
  clk.reset();
  GH_CHECK((int)g.elim.size() == n, H2H_ERR_FORMAT,
           "partition does not cover every vertex (root cut row must span all vertices)");
  // LUB layout: slot ranges in partition-array order (GraphPartition.cu:270-292)
  g.slot_off.assign(n, 0);
  int64_t off = 0;
  for (int i = 0; i < n; i++) {
    int v = g.part_ids[i];
    g.slot_off[v] = off;
    off += g.cap[v];
  }
  g.lub = off;
  g.t.lub = clk.us();
}

}  // namespace gh
