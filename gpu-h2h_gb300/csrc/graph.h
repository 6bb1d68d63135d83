// graph.h -- the handle behind h2h_graph: host arrays of one road graph, its
// tree decomposition and its no-hub labels, plus the device-resident index.
#pragma once

#include <cstdint>
#include <cstdlib>
#include <memory>
#include <string>
#include <vector>

#include "common.h"

namespace gh {

// X(v)\{v} lists after contraction, on the device, in the numbering of the
// contraction that produced them (a batch's forest, or one graph): list of
// vertex v is id[off[v] .. off[v+1]) (neighbour ids, sorted) with shortcut
// weights w.  `keep` owns the arrays.
struct ListStore {
  int64_t *off = nullptr;
  int *id = nullptr, *w = nullptr;
  int64_t total = 0;
  std::shared_ptr<void> keep;
};

// Device-resident index used by the label fill and the query kernels.
// Label rows are padded so every row starts on a 16-byte boundary
// (drow[v] is a multiple of 4 ints); the reference layout is restored on
// export.  Pointers in `owned` belong to the handle.  A graph labelled in a
// batch points into the batch's forest arrays instead (`keep` holds them):
// depth, pos_hash, drow and father are then offset to the graph's first
// vertex, while drow and pos_hash values stay absolute offsets into the
// shared dis and pos_pos / pos_id arrays.
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
  // views into the contraction's device lists and the fill's position
  // arrays: the graph's entries start at x_base / pos_base, its vertex ids
  // at id_base (non-zero in a batch)
  ListStore lists;
  int64_t x_base = 0, pos_base = 0;
  int id_base = 0;
  int64_t bytes = 0, rmq_bytes = 0;
  std::vector<void *> owned;      // label-side allocations of this handle
  std::vector<void *> owned_rmq;  // first, rmq_hash, rmq_id (built with the tree)
  std::shared_ptr<void> keep;
  void release();
  void release_labels();  // everything but the sparse table
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
  std::vector<int> cell_bound;              // per partition cell: bound on a list while its level runs
  std::vector<int> dup;                     // parallel arcs per vertex (repeated neighbour ids)
  std::vector<int64_t> slot_off;            // LUB offset per vertex (partition-array layout)
  int64_t lub = 0;
  std::vector<double> layer_rate;           // afs[h] / n for the PartitionRate CSV
  // contraction results
  std::vector<int> height;                  // CHInfo.second after the partition levels
  std::vector<int64_t> x_off;               // X(v)\{v}: upper neighbours, CSR by vertex [n+1]
  std::vector<int> x_id, x_w;               //   sorted by id, shortcut weights (host copies on demand)
  int gpu_vertices = 0;                     // vertexesConstructedInGPU
  int64_t decomposition_size = 0;           // size1 = sum(|X(v)|+1)
  bool contracted = false;
  // tree (TreeStructure.cu)
  int head = -1, tree_height = 0;
  std::vector<int> father, depth, first, child_off, childs;
  std::vector<int> euler_id;                // Euler tour (vertex per position), until the table is built
  int64_t euler_n = 0, h2h_size = 0, rmq_total = 0;  // rmq_total: RMQ_ID entries (the table is on the GPU)
  // labels (H2HConsturction.cu), reference layout on the host
  std::vector<int64_t> dis_hash, pos_hash;
  // host position lists: built for L3 labels only (L4 builds them on the GPU;
  // accessors download them)
  std::vector<int> pos_id, pos_pos, pos_w;  // pos_w: shortcut weight per pos entry (0 for v itself)
  std::vector<int64_t> drow_host;           // padded device row offsets (absolute in a batch's forest)
  std::vector<int> tree_bfs, tree_hash;     // TreeBFS / TreeHash
  // heavy-path decomposition of the tree for ancestor lookups in the fill:
  // hld lists the heavy paths one after another, top to bottom (hpos[v] =
  // v's index, htop[v] = the top of v's path); node v's root path is the
  // segments seg_off[v] .. seg_off[v+1]-1, shallowest first, one per heavy
  // path it crosses (written on the GPU by FillPlan)
  std::vector<int> hld, htop, hpos;
  std::vector<int64_t> seg_off;
  int max_segs = 0;
  bool tree_layout = false;  // depth, first, level order, heavy paths, segments and dis_hash built on the GPU
  bool labelled = false;
  int64_t max_label = 0;  // -1: not computed yet (label_max computes it)
  // device
  DeviceIndex dev;
  Timings t;

  ~Graph() { dev.release(); }
};

// Vertex elimination over one or more graphs in one set of launches
// (contract.cu).  The graphs' vertices are numbered consecutively (graph i
// starts at vbase[i]); launch s eliminates the cells of level H_i - s of
// every graph i with H_i - s > C_i, and one last launch runs every graph's
// global order (levels <= C_i) as one cell per graph.  The list structure
// and the elimination order depend only on the topology, so enqueue() can be
// replayed (or captured in a CUDA graph) after set_weights().
struct ElimPlan {
  struct Launch {
    int step, level, ncell, kmax, lmax, cs, nw, slots;
    int arena = 0;               // cooperative launches: ints of shared-memory arena per block
    bool arena_merges = false;   // ... that merges take their buffers from
    int64_t lo, smem, pstage_off;
    bool heap, global_stage;
    // cell_grid_kernel: the step's cells in one cooperative launch, `slots`
    // blocks (block -> cell map at grid_map + map_off, cell -> first block
    // after it), one barrier counter per cell at grid_bar + bar_off, at most
    // slice_max candidates owned by one block
    bool grid;
    int slice_max;
    int64_t map_off, bar_off;
  };
  std::vector<Graph *> gs;
  std::vector<int> vbase;
  std::vector<int64_t> mbase;
  int N = 0, heap_total = 0;
  int64_t M = 0, lub = 0, pool_size = 0;
  std::vector<Launch> launches;  // in step order; launches of one step are independent
  int nsm = 0, max_group = 1;
  bool elim_balance = true;  // cooperative steps: merges split over a cell's blocks by work
  int64_t partial_cap = 0;   // blocks the per-block arrays of cooperative launches hold
  std::vector<cudaStream_t> side;  // streams for the second and later launches of a step
  std::vector<cudaEvent_t> ev_join;
  cudaEvent_t ev_fork = nullptr;
  // device state (global vertex ids)
  int *slot_nbr = nullptr, *slot_w = nullptr, *lsize = nullptr, *cap = nullptr, *cap_init = nullptr;
  int *height = nullptr, *elim = nullptr;
  int *deg0 = nullptr, *h0 = nullptr, *cpos = nullptr, *err = nullptr, *ljunk = nullptr, *cell_start = nullptr;
  int *cell_count = nullptr, *adj_off = nullptr, *adj_v = nullptr, *adj_w = nullptr, *pstage = nullptr;
  int *deg_init = nullptr, *elim_init = nullptr, *heap_verts = nullptr;
  int64_t *slot_off = nullptr, *slot_off_init = nullptr;
  unsigned long long *pool_next = nullptr, *pool_first = nullptr;
  ListStore lists;       // compact final lists (forest numbering), after build_lists()
  int *rank = nullptr, *father_dev = nullptr;
  // cell_grid_kernel state: per-block argmins, block maps, barrier counters
  int *grid_map = nullptr;
  void *hg_partial = nullptr;
  unsigned *grid_bar = nullptr;
  int64_t grid_bar_words = 0;
  int64_t bytes = 0;
  explicit ElimPlan(const std::vector<Graph *> &graphs);
  ~ElimPlan();
  void release();
  ElimPlan(const ElimPlan &) = delete;
  ElimPlan &operator=(const ElimPlan &) = delete;
  // Resets the lists from the input arcs and runs every launch on s.  With
  // heap_ev non-null, records heap_ev[0] before the global-order launch and
  // heap_ev[1] after it.
  void enqueue(cudaStream_t s, cudaEvent_t *heap_ev = nullptr, bool trace = false);
  void launch_one(const Launch &Lc, cudaStream_t s, bool trace);
  void check_error();  // synchronises; throws on a kernel error code
  // After the first enqueue: compact the final lists on the device, pick each
  // vertex's father (min elimination rank over its list) there, and hand each
  // graph its elimination order, list offsets and fathers; the lists stay on
  // the device (each graph's DeviceIndex gets a view).
  void build_lists();
  // Refreshes the compact lists' entries from the slot arrays (replays).
  void enqueue_gather(cudaStream_t s);
  void set_weights(int gi, const int *w, cudaStream_t s);  // arc weights in the graph's file order
};

// Tile shapes of the L4 dataflow fill, keyed on the node's tree level --
// class 0: fewer nodes than SMs (the chain-like top, on the critical path);
// class 1: wider; class 2: wider and heavy (its nodes average at least 2^18
// min-plus updates m*d) -- and on its separator size m (buckets m <= 16, <= 64,
// <= 256, > 256).  A node whose m * d is at most small_work is one tile; a
// larger one is cut into col_block columns x sep_chunk separator members.
struct TilePolicy {
  static constexpr int kWidth = 3, kSep = 4;
  int small_work[kWidth][kSep], col_block[kWidth][kSep], sep_chunk[kWidth][kSep];
  TilePolicy();  // the shallow preset
  // the default for a forest whose deepest tree has `height` levels: the
  // shallow preset up to 2048 levels, the deep one beyond
  static TilePolicy for_height(int height);
  static int sep_bucket(int m) { return m <= 16 ? 0 : m <= 64 ? 1 : m <= 256 ? 2 : 3; }
  std::string str() const;
  bool parse(const std::string &s);
};

// The L4 label fill over one or more graphs as one forest (labels.cu): the
// graphs' trees are laid side by side (graph i's vertex v is forest vertex
// vbase[i] + v) and filled by one dataflow launch.  Each graph's DeviceIndex
// becomes a view into the forest arrays.
struct FillPlan {
  std::vector<Graph *> gs;
  std::vector<int> vbase;
  int N = 0;
  int64_t pos_total = 0, dis_total = 0;
  TilePolicy policy;
  std::shared_ptr<void> storage;  // forest arrays shared with the graphs' views
  int64_t *drow = nullptr, *pos_hash = nullptr;
  int *pos_pos = nullptr, *pos_id = nullptr, *pos_w = nullptr, *pos_src = nullptr, *father = nullptr;
  ListStore lists;
  int *depth = nullptr, *dis = nullptr;
  // workspace
  int *hld = nullptr, *htop = nullptr, *hpos = nullptr, *seg_top = nullptr, *seg_pos = nullptr;
  int64_t *hld_row = nullptr;
  int64_t *seg_off = nullptr;
  int *done = nullptr, *next = nullptr, *err = nullptr, *tiles = nullptr;
  unsigned long long *trace_t = nullptr;  // publish time per node (GPUH2H_TRACE)
  int64_t ntiles = 0, tiles_cap = 0, nchunks = 0;
  int max_u = 1, max_c = 1, max_segs = 1, blocks = 1, threads = 128;
  int scalar_cols = 32;  // tiles this narrow sweep one column per lane (labels.cu)
  size_t smem = 0;
  int nsm = 0;
  int64_t work_bytes = 0;
  // lists: the graphs' X lists in the same forest numbering.
  FillPlan(const std::vector<Graph *> &graphs, const TilePolicy &pol, const ListStore &lists);
  ~FillPlan();
  void release_work();
  FillPlan(const FillPlan &) = delete;
  FillPlan &operator=(const FillPlan &) = delete;
  void build_tiles(const TilePolicy &pol);
  std::vector<int> level_classes() const;  // TilePolicy class per forest level
  // Gathers the shortcut weights of the pos entries from the lists, resets
  // rows and flags and runs the fill on s.
  void enqueue(cudaStream_t s, cudaEvent_t *fill_ev = nullptr);
  void check_error();            // synchronises; throws if a dependency wait ran out
  void trace_report();           // GPUH2H_TRACE: the last fill's time per level class
  void attach(bool first);       // per-graph views, max_label; first: also drow_host
};

// Phases (one translation unit each).
void load_graph(Graph &g, const std::string &edge, const std::string &idf, const std::string &cut);
// elim_sets.cu: elimination sets, LUB capacities and layout, cell list
// bounds and parallel-arc counts of one or more graphs, on the GPU
void build_elimination_sets(const std::vector<Graph *> &gs);
// contract.cu: partition levels H..C+1 and the global heap over levels <= C;
// fills g.elim (elimination order) and g.x_off / x_id / x_w
void contract_gpu(Graph &g);
void build_tree(Graph &g);                             // tree.cpp: father, children, Euler tour
// tree_gpu.cu: the same on the GPU, plus the level order, heavy paths and
// root-path segment offsets (sets g.tree_layout)
void build_tree_gpu(Graph &g);
// query.cu: the compacted sparse tables of the graphs' Euler tours on the
// GPU (first, rmq_hash, rmq_id in each graph's DeviceIndex)
void build_rmq_gpu(const std::vector<Graph *> &gs);
void download_rmq(const Graph &g, int64_t *rmq_hash, int *rmq_id);  // query.cu
inline void build_tree_and_rmq(Graph &g) {
  build_tree_gpu(g);
  build_rmq_gpu({&g});
}
void allocate_labels_and_bfs(Graph &g);                // tree.cpp
void fill_labels_gpu(Graph &g);                        // labels.cu
// The level-synchronous fill (L3 labels, or L4 with GPUH2H_LEVEL_FILL set)
// runs from host position lists; the L4 dataflow fill builds them on the GPU.
inline bool uses_level_fill(const Graph &g) {
  return g.label_mode == H2H_LABEL_L3 || std::getenv("GPUH2H_LEVEL_FILL") != nullptr;
}
void download_labels(const Graph &g, int *dis_out);    // labels.cu, reference layout
int64_t label_max(const Graph &g);                     // labels.cu: largest finite label, computed once
// labels.cu: the reference's level-by-level GPU fill mapping on a built L4
// graph (measurement baseline): device ms and mismatches against the labels
void fill_labels_plain(const Graph &g, int mapping, double *ms, int64_t *mismatches);
// labels.cu: the graph's position lists (reference layout, graph-local ids)
void download_positions(const Graph &g, int *pos_id, int *pos_pos);
// contract.cu: host copies of the X lists (graph-local ids) from the device
void download_lists(Graph &g);
// Device copies of a saved index (index_io.cpp loads the file):
ListStore upload_lists(const std::vector<int64_t> &off, const std::vector<int> &id,
                       const std::vector<int> &w);                         // contract.cu
void upload_rmq(Graph &g, const std::vector<int64_t> &rmq_hash, const std::vector<int> &rmq_id);  // query.cu
// labels.cu: rows (reference layout, dis_hash offsets) into padded device
// rows plus the position arrays; sets drow_host and the DeviceIndex
void upload_labels(Graph &g, const std::vector<int> &dis, const std::vector<int> &pos_id,
                   const std::vector<int> &pos_pos);
void upload_query_index(Graph &g);                     // query.cu
// query.cu; bad: the flag word set when a pair holds an id out of range
// (nullptr: the graph's own)
void run_query_batch(const Graph &g, const int *x, const int *y, int *out, int64_t n, int mode, cudaStream_t s,
                     int *bad = nullptr);
void run_query_batch_plain(const Graph &g, const int *x, const int *y, int *out, int64_t n, int mode,
                           cudaStream_t s);                  // query.cu, one thread per query

}  // namespace gh
