// graph.h -- the handle behind h2h_graph: host arrays of one road graph, its
// tree decomposition and its no-hub labels, plus the device-resident index.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "common.h"

namespace gh {

// Device-resident index used by the label fill and the query kernels.
// Label rows are padded so every row starts on a 16-byte boundary
// (drow[v] is a multiple of 4 ints); the reference layout is restored on
// export.  All pointers are cudaMalloc'd and owned by the handle.
struct DeviceIndex {
  int n = 0;
  int64_t euler = 0, rmq = 0, pos = 0, dis_padded = 0;
  int *first = nullptr;       // firstAppeare           [n]
  int *depth = nullptr;       // H2H_TreeHeight_Hash    [n]
  int64_t *rmq_hash = nullptr;// RMQHash                [euler]
  int *rmq_id = nullptr;      // RMQ_ID                 [rmq]
  int64_t *pos_hash = nullptr;// H2H_pos_hash           [n+1]
  int *pos_pos = nullptr;     // H2H_pos_POS            [pos]
  int *pos_id = nullptr;      // H2H_pos_ID             [pos]
  int64_t *drow = nullptr;    // padded row offsets     [n+1]
  int *dis = nullptr;         // padded labels          [dis_padded]
  int *father = nullptr;      // father                 [n]
  int *err = nullptr;         // kernel error word      [1]
  int64_t bytes = 0;
  void release();
};

struct Timings {
  long long load = 0, rank_tree = 0, lub = 0, translate_lub = 0, td_gpu = 0, translate_back = 0, td_cpu = 0,
            tree = 0, malloc_labels = 0, bfs = 0, translate_labels = 0, fill_gpu = 0;
};

struct Graph {
  // configuration (the G2H command line, main.cu:252-260)
  std::string name;
  int H_cli = 0, H = 0, C = 0, threads = 1, method = 1;
  int contract_device = 1, parallel_fine = 2, construct_device = 1, label_mode = H2H_LABEL_L4;
  // input (Graph_Fundamental.cu:4-95)
  int n = 0;
  int64_t m = 0;
  std::vector<int> adj_off;        // CSR offsets of adjList in file order [n+1]
  std::vector<int> adj_v, adj_w;   // arcs, self loops dropped, parallel arcs kept
  std::vector<int> part_ids;       // NE_P[idx].NodeID (partition array)
  std::vector<int> id_hash;        // ID_hash[vertex] = idx
  std::vector<int> cut_l, cut_r;   // partition_Tree rows [2^H-1]
  // elimination sets (GraphPartition.cu:178-308)
  std::vector<int> cell_start, cell_count;  // NANHash first / NodeID per cell
  std::vector<int> elim;                    // nonAdjcentNode ids; rewritten to elimination order
  std::vector<int> cap;                     // placeOccupy (LUB capacity) per vertex
  std::vector<int64_t> slot_off;            // LUB offset per vertex (partition-array layout)
  int64_t lub = 0;
  std::vector<double> layer_rate;           // afs[h] / n for the PartitionRate CSV
  // contraction results
  std::vector<int> height;                  // CHInfo.second after the partition levels
  std::vector<int64_t> x_off;               // X(v)\{v}: upper neighbours, CSR by vertex [n+1]
  std::vector<int> x_id, x_w;               //   sorted by id, shortcut weights
  int gpu_vertices = 0;                     // vertexesConstructedInGPU
  int64_t decomposition_size = 0;           // size1 = sum(|X(v)|+1)
  bool contracted = false;
  // tree (TreeStructure.cu)
  int head = -1, tree_height = 0;
  std::vector<int> father, depth, first, child_off, childs;
  std::vector<int64_t> rmq_hash;
  std::vector<int> rmq_id;
  int64_t euler_n = 0, h2h_size = 0;
  // labels (H2HConsturction.cu), reference layout on the host
  std::vector<int64_t> dis_hash, pos_hash;
  std::vector<int> pos_id, pos_pos, pos_w;  // pos_w: shortcut weight per pos entry (0 for v itself)
  std::vector<int64_t> drow_host;           // padded device row offsets
  std::vector<int> tree_bfs, tree_hash;     // TreeBFS / TreeHash
  bool labelled = false;
  int64_t max_label = 0;
  // device
  DeviceIndex dev;
  Timings t;

  ~Graph() { dev.release(); }
};

// Phases (one translation unit each).
void load_graph(Graph &g, const std::string &edge, const std::string &idf, const std::string &cut);
void build_elimination_sets(Graph &g);                 // elim_sets.cpp
// contract.cu: partition levels H..C+1 and the global heap over levels <= C;
// fills g.elim (elimination order) and g.x_off / x_id / x_w
void contract_gpu(Graph &g);
void build_tree_and_rmq(Graph &g);                     // tree.cpp
void allocate_labels_and_bfs(Graph &g);                // tree.cpp
void fill_labels_gpu(Graph &g);                        // labels.cu
void download_labels(const Graph &g, int *dis_out);    // labels.cu, reference layout
void upload_query_index(Graph &g);                     // query.cu
void run_query_batch(const Graph &g, const int *x, const int *y, int *out, int64_t n, int mode,
                     cudaStream_t s);                  // query.cu
void run_query_batch_plain(const Graph &g, const int *x, const int *y, int *out, int64_t n, int mode,
                           cudaStream_t s);                  // query.cu, one thread per query

}  // namespace gh
