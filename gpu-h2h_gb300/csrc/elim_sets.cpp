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
#include "pool.h"

namespace gh {

void build_elimination_sets(Graph &g) {
  Clock clk;
  const int n = g.n;
  const int64_t cells = (int64_t(1) << g.H) - 1;
  std::vector<char> alive(n, 1), alive_next(n, 1);
  g.cap.resize(n);
  for (int v = 0; v < n; v++) g.cap[v] = g.adj_off[v + 1] - g.adj_off[v];
  g.cell_start.assign(cells, 0);
  g.cell_count.assign(cells, 0);
  g.elim.clear();
  g.elim.reserve(n);
  g.layer_rate.assign(g.H + 1, 0.0);
  Pool pool(g.threads);
  for (int h = g.H; h > 0; h--) {
    const int64_t lo = (int64_t(1) << (h - 1)) - 1, hi = (int64_t(1) << h) - 2;
    alive_next = alive;
    {
      std::vector<std::pair<int, int>> rs;
      for (int64_t c = lo; c <= hi; c++)
        if (g.cut_r[c] > g.cut_l[c]) rs.push_back({g.cut_l[c], g.cut_r[c]});
      std::sort(rs.begin(), rs.end());
      for (size_t i = 1; i < rs.size(); i++)
        GH_CHECK(rs[i].first >= rs[i - 1].second, H2H_ERR_FORMAT, "partition cells of one level overlap");
    }
    // cells of one level cover disjoint ranges of the partition array, so
    // they are independent: "u is in cell c" is a range test on id_hash[u]
    std::vector<std::vector<int>> interior(hi - lo + 1);
    pool.parallel_for(hi - lo + 1, 1, [&](int64_t b, int64_t e, int) {
      std::vector<int> members;
      for (int64_t k = b; k < e; k++) {
        const int64_t c = hi - k;  // the reference walks the cells from the highest index down
        const int cl = g.cut_l[c], cr = g.cut_r[c];
        members.clear();
        for (int j = cl; j < cr; j++)
          if (alive[g.part_ids[j]]) members.push_back(g.part_ids[j]);
        std::sort(members.begin(), members.end());  // std::map iteration order of the reference
        const int sz = (int)members.size();
        for (int v : members) {
          int out = sz;
          for (int e2 = g.adj_off[v]; e2 < g.adj_off[v + 1]; e2++) {
            const int u = g.adj_v[e2], iu = g.id_hash[u];
            if (alive[u] && (iu < cl || iu >= cr)) out++;
          }
          if (out == sz) {
            alive_next[v] = 0;
            interior[k].push_back(v);
          }
          g.cap[v] = std::max(g.cap[v], out);
        }
      }
    });
    for (int64_t k = 0; k <= hi - lo; k++) {
      const int64_t c = hi - k;
      g.cell_start[c] = (int)g.elim.size();
      g.cell_count[c] = (int)interior[k].size();
      g.elim.insert(g.elim.end(), interior[k].begin(), interior[k].end());
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
