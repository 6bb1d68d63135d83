// ref_harness.cpp -- driver for the CPU-only build of the reference's own
// translation units (test infrastructure; built by oracle/build_ref.sh into
// oracle/_ref/).  It runs the Graph members in the order main.cu:84-124 and
// main.cu:167-171 run them for `G2H <G> H C T M 1 1 0` (GPU-hybrid
// contraction, multithread PF label fill on the CPU), then answers query
// pairs with H2HDistancQuery_UsingLCA_noHub / _noLCA_noHub (Query.cu:108-151)
// and dumps every array as raw little-endian files for the parity tests.
//
// usage: ref_harness EDGE ID CUT H C THREADS OUTDIR [PAIRS.i32]
#include "Graph_D.cuh"

#include <cstdio>
#include <string>
#include <vector>

template <typename T>
static void dump(const std::string &dir, const char *name, const T *p, size_t n) {
  std::string path = dir + "/" + name;
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) { std::perror(path.c_str()); std::exit(2); }
  if (n) std::fwrite(p, sizeof(T), n, f);
  std::fclose(f);
}

int main(int argc, char **argv) {
  if (argc < 8) {
    std::fprintf(stderr, "usage: %s EDGE ID CUT H C THREADS OUTDIR [PAIRS]\n", argv[0]);
    return 2;
  }
  const std::string edge = argv[1], id = argv[2], cut = argv[3], out = argv[7];
  const int H = std::atoi(argv[4]), C = std::atoi(argv[5]), T = std::atoi(argv[6]);
  auto *g = new Graph_D_H::Graph("harness", H, "unused-node-file", edge, T, C, cut, id);
  g->PartitionMethod = 1;
  g->contractDevice = 1;
  g->parallelFine = 1;
  g->parallelFine_Construct = 1;
  g->constructDevice = 0;
  g->checklink();

  // TDAndH2HConstruct_Tradition_plus_G_2_noHub (main.cu:84-124), goalHeight = H.
  g->ConstructMethod = 2;
  g->startGPU();
  g->makeAdjcentNode(0);
  if (H != C) {
    g->translateBeforeCH();
    g->partition_TD_Parallel_D_2(C);
    g->translateInTD();
  }
  g->TDInCPU(C);
  {
    std::vector<int> order(g->nonAdjcentNode.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = g->nonAdjcentNode[i].second;
    dump(out, "order.i32", order.data(), order.size());
    int gv = g->vertexesConstructedInGPU;
    dump(out, "gpu_vertices.i32", &gv, 1);
  }
  g->beforeH2H_noHub();
  const int n = g->NodeNumber;
  dump(out, "father.i32", g->father.data(), (size_t)n);
  dump(out, "depth.i32", g->H2H_TreeHeight_Hash.data(), (size_t)n);
  dump(out, "first.i32", g->firstAppeare.data(), (size_t)n);
  dump(out, "rmq_hash.i64", g->RMQHash.data(), g->RMQHash.size());
  dump(out, "rmq_id.i32", g->RMQ_ID.data(), g->RMQ_ID.size());
  {
    std::vector<int64_t> ah(n + 1);
    std::vector<int> aid, aw;
    for (int v = 0; v < n; v++) {
      ah[v] = (int64_t)aid.size();
      std::vector<std::pair<int, int>> row;
      for (auto &kv : g->CHAdjlist[v]) row.push_back({kv.first, kv.second.first});
      std::sort(row.begin(), row.end());
      for (auto &p : row) { aid.push_back(p.first); aw.push_back(p.second); }
    }
    ah[n] = (int64_t)aid.size();
    dump(out, "adj_hash.i64", ah.data(), ah.size());
    dump(out, "adj_id.i32", aid.data(), aid.size());
    dump(out, "adj_w.i32", aw.data(), aw.size());
  }

  // constructLabel_noHub(parallelFine=1, constructDevice=0) (main.cu:167-171).
  g->inConstructH2H_noHub_multiThread();
  dump(out, "dis_hash.i64", g->H2H_dis_hash.data(), g->H2H_dis_hash.size());
  dump(out, "dis.i32", g->H2H_dis.data(), g->H2H_dis.size());
  dump(out, "pos_hash.i64", g->H2H_pos_hash.data(), g->H2H_pos_hash.size());
  dump(out, "pos_id.i32", g->H2H_pos_ID.data(), g->H2H_pos_ID.size());
  dump(out, "pos_pos.i32", g->H2H_pos_POS.data(), g->H2H_pos_POS.size());
  dump(out, "tree_bfs.i32", g->TreeBFS.data(), g->TreeBFS.size());
  dump(out, "tree_hash.i32", g->TreeHash.data(), g->TreeHash.size());

  if (argc > 8) {
    FILE *f = std::fopen(argv[8], "rb");
    if (!f) { std::perror(argv[8]); return 2; }
    std::vector<int> xy;
    int buf[2];
    while (std::fread(buf, sizeof(int), 2, f) == 2) { xy.push_back(buf[0]); xy.push_back(buf[1]); }
    std::fclose(f);
    const size_t q = xy.size() / 2;
    std::vector<int> lca(q), nolca(q);
    for (size_t i = 0; i < q; i++) {
      lca[i] = g->H2HDistancQuery_UsingLCA_noHub(xy[2 * i], xy[2 * i + 1]);
      nolca[i] = g->H2HDistancQuery_noLCA_noHub(xy[2 * i], xy[2 * i + 1]);
    }
    dump(out, "q_lca.i32", lca.data(), q);
    dump(out, "q_nolca.i32", nolca.data(), q);
  }
  return 0;
}
