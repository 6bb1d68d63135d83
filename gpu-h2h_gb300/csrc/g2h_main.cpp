// g2h_main.cpp -- the G2H command line (main.cu:244-307) over the C ABI:
//
//   G2H GraphName PartitionHeight ChangeToGlobalHeight threadNum partitionMethod
//       useGPUContract parallelFine useGPUConstruct
//
// Same argument count rule (anything but 8 arguments exits 0 silently), same
// input paths relative to the working directory, same CSV outputs
// (<Method>PartitionRate.csv, ConstructInfo/<G>/contract.csv and
// constructInfo.csv, QueryResult/<G>/random.csv).  Options that the
// reference hard-codes are environment variables so the argument count stays
// the reference's: H2H_LABEL=L3|L4 (default L4), H2H_QUERIES (default
// 1000000, queryMaxSize in Graph_D.cuh:500), H2H_SEED (default time(0) as in
// Query.cu:12).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "gpuh2h.h"
#include "gpuh2h_tools.h"

static const char *prefix(int m) { return m == 2 ? "Minimum" : m == 3 ? "metis" : m == 4 ? "scotch" : "Latitude"; }

int main(int argc, char **argv) {
  if (argc != 9) return 0;
  const std::string name = argv[1];
  const int H = (int)std::strtol(argv[2], nullptr, 10);
  const int C = (int)std::strtol(argv[3], nullptr, 10);
  const int threads = (int)std::strtol(argv[4], nullptr, 10);
  const int method = (int)std::strtol(argv[5], nullptr, 10);
  const int contract_device = (int)std::strtol(argv[6], nullptr, 10);
  const int parallel_fine = (int)std::strtol(argv[7], nullptr, 10);
  const int construct_device = (int)std::strtol(argv[8], nullptr, 10);
  const char *lab = std::getenv("H2H_LABEL");
  const int label_mode = (lab && std::strcmp(lab, "L3") == 0) ? H2H_LABEL_L3 : H2H_LABEL_L4;
  const char *qs = std::getenv("H2H_QUERIES");
  const int64_t nq = qs ? std::strtoll(qs, nullptr, 10) : 1000000;
  const char *sd = std::getenv("H2H_SEED");
  const uint64_t seed = sd ? std::strtoull(sd, nullptr, 10) : (uint64_t)std::time(nullptr);

  std::printf("./Graph/USA/%sNode.txt\n./Graph/USA/%sEdge.txt\n", name.c_str(), name.c_str());
  std::printf("./Partition/%s/%sCut.txt\n./Partition/%s/%sID.txt\n", name.c_str(), prefix(method), name.c_str(),
              prefix(method));
  h2h_graph *g = nullptr;
  if (h2h_load(".", name.c_str(), H, C, threads, method, &g) != H2H_OK) {
    std::fprintf(stderr, "G2H: load failed: %s\n", h2h_last_error());
    return 1;
  }
  std::printf("connect!\n");
  if (h2h_contract(g, contract_device) != H2H_OK) {
    std::fprintf(stderr, "G2H: contraction failed: %s\n", h2h_last_error());
    h2h_free(g);
    return 1;
  }
  if (h2h_write_partition_rate(g, ".") != H2H_OK) std::fprintf(stderr, "Unable to open file for writing.\n");
  if (h2h_write_contract_csv(g, ".") != H2H_OK) std::fprintf(stderr, "Unable to open file for writing.\n");
  if (h2h_build_labels(g, parallel_fine, construct_device, label_mode) != H2H_OK) {
    std::fprintf(stderr, "G2H: label construction failed: %s\n", h2h_last_error());
    h2h_free(g);
    return 1;
  }
  if (h2h_write_construct_info(g, ".") != H2H_OK) std::fprintf(stderr, "Unable to open file for writing.\n");
  h2h_info info;
  h2h_get_info(g, &info);
  std::printf("n=%d m=%lld tree_height=%d levels=%d label_ints=%lld gpu_vertices=%d\n", info.n, (long long)info.m,
              info.tree_height, info.n_levels, (long long)info.label_size, info.gpu_vertices);
  std::printf("TDInGPUTime=%lld TDInCPUTime=%lld tree=%lld malloc=%lld bfs=%lld H2HUsingTime_GPU=%lld (us)\n",
              (long long)info.t_td_gpu_us, (long long)info.t_td_cpu_us, (long long)info.t_tree_us,
              (long long)info.t_malloc_us, (long long)info.t_bfs_us, (long long)info.t_fill_gpu_us);

  // Query_noHub (main.cu:218-240): uniform pairs, device batches, QueryResult CSV.
  std::vector<int> x(nq), y(nq);
  h2h_gen_uniform_pairs(info.n, nq, seed, x.data(), y.data());
  int *dx = nullptr, *dy = nullptr, *dout = nullptr;
  int64_t times[18] = {0};
  if (cudaMalloc(&dx, sizeof(int) * nq) == cudaSuccess && cudaMalloc(&dy, sizeof(int) * nq) == cudaSuccess &&
      cudaMalloc(&dout, sizeof(int) * nq) == cudaSuccess) {
    cudaMemcpy(dx, x.data(), sizeof(int) * nq, cudaMemcpyHostToDevice);
    cudaMemcpy(dy, y.data(), sizeof(int) * nq, cudaMemcpyHostToDevice);
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    for (int mode = 0; mode < 2; mode++) {
      h2h_query_batch(g, dx, dy, dout, nq, mode, nullptr);  // warm-up
      cudaEventRecord(a);
      int rc = h2h_query_batch(g, dx, dy, dout, nq, mode, nullptr);
      cudaEventRecord(b);
      cudaEventSynchronize(b);
      float ms = 0;
      cudaEventElapsedTime(&ms, a, b);
      if (rc != H2H_OK) std::fprintf(stderr, "G2H: query failed: %s\n", h2h_last_error());
      // columns GPUnoLCA-* (mode 1) and GPUwithLCA-* (mode 0): one kernel configuration, same time in each
      for (int k = 0; k < 5; k++) times[8 + 2 * k + (mode == 0 ? 1 : 0)] = (int64_t)(ms * 1000.0f);
      std::printf("%s query: %lld pairs in %.3f ms\n", mode == 0 ? "UsingLCA" : "noLCA", (long long)nq, ms);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
  cudaFree(dx);
  cudaFree(dy);
  cudaFree(dout);
  if (h2h_write_query_result(g, ".", nq, times) != H2H_OK) std::fprintf(stderr, "Unable to open file for writing.\n");
  h2h_free(g);
  return 0;
}
