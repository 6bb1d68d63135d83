// ref_harness.cpp -- driver for builds of the reference's own translation
// units (test infrastructure).  Two builds:
//
//  * CPU-only (oracle/build_ref.sh, g++ with Thrust's CPP backend): runs the
//    Graph members in the order main.cu:84-124 and main.cu:167-171 run them
//    for `G2H <G> H C T M 1 1 0` (GPU-hybrid contraction, multithread PF
//    label fill on the CPU), then answers query pairs with
//    H2HDistancQuery_UsingLCA_noHub / _noLCA_noHub (Query.cu:108-151).
//  * GPU (REF_GPU_BUILD, oracle/build_ref_gpu.sh, nvcc for sm_103a on the
//    reference's real kernels): the same contraction with the reference's
//    makeCHPerHeight_D_2 kernel on the GPU, the GPU LL label fill of
//    `G2H <G> H C T M 1 2 1` (main.cu:182-186, inConstructH2H_noHub_D) and the
//    reference's batched GPU query wrappers (H2Hquery_bunch_*_D_noHub,
//    tanslate.cu:310-330) on the pairs; it also writes the reference's own
//    phase timers to times.txt.
//
// Both dump every array as raw little-endian files for the parity tests.
//
// usage: ref_harness EDGE ID CUT H C THREADS OUTDIR [PAIRS.i32]
#include "Graph_D.cuh"

#include <algorithm>
#include <climits>
#include <cstdio>
#include <sstream>
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

#ifdef REF_GPU_BUILD
#include <chrono>
static const auto g_t0 = std::chrono::steady_clock::now();
static long long wall_us() {
  return std::chrono::duration_cast<std::chrono::microseconds>(std::chrono::steady_clock::now() - g_t0).count();
}
#endif

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
#ifdef REF_GPU_BUILD
  g->parallelFine = 2;
  g->parallelFine_Construct = 2;
  g->constructDevice = 1;
#else
  g->parallelFine = 1;
  g->parallelFine_Construct = 1;
  g->constructDevice = 0;
#endif
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

#ifdef REF_GPU_BUILD
  // constructLabel_noHub(parallelFine=2, constructDevice=1) (main.cu:182-186);
  // it copies the device labels back into H2H_dis (H2HConsturction.cu:549).
  g->inConstructH2H_noHub_D();
#else
  // constructLabel_noHub(parallelFine=1, constructDevice=0) (main.cu:167-171).
  g->inConstructH2H_noHub_multiThread();
#endif
  dump(out, "dis_hash.i64", g->H2H_dis_hash.data(), g->H2H_dis_hash.size());
  dump(out, "dis.i32", g->H2H_dis.data(), g->H2H_dis.size());
  dump(out, "pos_hash.i64", g->H2H_pos_hash.data(), g->H2H_pos_hash.size());
  dump(out, "pos_id.i32", g->H2H_pos_ID.data(), g->H2H_pos_ID.size());
  dump(out, "pos_pos.i32", g->H2H_pos_POS.data(), g->H2H_pos_POS.size());
  dump(out, "tree_bfs.i32", g->TreeBFS.data(), g->TreeBFS.size());
  dump(out, "tree_hash.i32", g->TreeHash.data(), g->TreeHash.size());
#ifdef REF_GPU_BUILD
  std::ostringstream times;
  times << "translateLUBToGPUTime " << g->translateLUBToGPUTime << "\nTDInGPUTime " << g->TDInGPUTime
        << "\nTDInCPUTime " << g->TDInCPUTime << "\nH2HmallocTime " << g->H2HmallocTime
        << "\nH2HConstructBFSTreeTime " << g->H2HConstructBFSTreeTime << "\nH2HUsingTime_CPU "
        << g->H2HUsingTime_CPU << "\nH2HTranslateTime " << g->H2HTranslateTime << "\nH2HUsingTime_GPU "
        << g->H2HUsingTime_GPU << "\nwall_build_us " << wall_us() << "\n";
#endif

  if (argc > 8) {
    FILE *f = std::fopen(argv[8], "rb");
    if (!f) { std::perror(argv[8]); return 2; }
    std::vector<int> xy;
    int buf[2];
    while (std::fread(buf, sizeof(int), 2, f) == 2) { xy.push_back(buf[0]); xy.push_back(buf[1]); }
    std::fclose(f);
    const size_t q = xy.size() / 2;
    std::vector<int> lca(q), nolca(q);
#ifdef REF_GPU_BUILD
    // Query_noHub's device path (main.cu:222-240): RMQ and pairs to the
    // device, then the reference's batched kernels at 256 threads per block.
    g->x.assign(q, 0);
    g->y.assign(q, 0);
    for (size_t i = 0; i < q; i++) { g->x[i] = xy[2 * i]; g->y[i] = xy[2 * i + 1]; }
    g->result.assign(q, INT_MAX);
    g->queryMaxSize = (int)q;
    g->cleanBeforeQuery();
    g->translateRMQ_noHub();
    g->translateQuery();
    g->cudaThreadNum = 256;
    long long t_lca = g->H2Hquery_bunch_UsingLCA_D_noHub((int)q);
    g->translateQueryResultBack();
    for (size_t i = 0; i < q; i++) lca[i] = g->result[i];
    long long t_nolca = g->H2Hquery_bunch_noLCA_D_noHub((int)q);
    g->translateQueryResultBack();
    for (size_t i = 0; i < q; i++) nolca[i] = g->result[i];
    // repeated batches: the reference's per-batch microseconds, best of 5
    long long best_lca = t_lca, best_nolca = t_nolca;
    for (int r = 0; r < 5; r++) {
      best_lca = std::min(best_lca, g->H2Hquery_bunch_UsingLCA_D_noHub((int)q));
      best_nolca = std::min(best_nolca, g->H2Hquery_bunch_noLCA_D_noHub((int)q));
    }
    times << "queries " << q << "\nquery_lca_us " << best_lca << "\nquery_nolca_us " << best_nolca << "\n";
#else
    for (size_t i = 0; i < q; i++) {
      lca[i] = g->H2HDistancQuery_UsingLCA_noHub(xy[2 * i], xy[2 * i + 1]);
      nolca[i] = g->H2HDistancQuery_noLCA_noHub(xy[2 * i], xy[2 * i + 1]);
    }
#endif
    dump(out, "q_lca.i32", lca.data(), q);
    dump(out, "q_nolca.i32", nolca.data(), q);
  }
#ifdef REF_GPU_BUILD
  {
    std::string path = out + "/times.txt";
    FILE *f = std::fopen(path.c_str(), "w");
    if (f) {
      std::fputs(times.str().c_str(), f);
      std::fclose(f);
    }
  }
#endif
  return 0;
}
