/*
 * gpuh2h.h -- C ABI of the GB300-native GPU-H2H hot path.
 *
 * The reference (sauccjy/GPU-H2H) has no library interface: its operator
 * API is the G2H command line plus the Graph_D_H::Graph members that
 * main.cu calls and the wrappers of kernel_functions.cuh.  Each entry point
 * below names the reference member or wrapper it stands in for (paths are
 * relative to the reference project root).  Plain pointers and sizes only.
 *
 * Conventions kept from the reference:
 *   - vertex ids are 0-based here and 1-based in Edge files;
 *   - distances are int32, x == y gives 0, INT_MAX means "no label path";
 *   - labels are the no-hub layout: dis_hash/pos_hash are int64 prefix
 *     offsets, dis holds depth(v) entries per vertex (ancestor distances by
 *     depth), pos_pos/pos_id list X(v) sorted by position.
 * Differences, by design:
 *   - every call returns a status (H2H_OK = 0 or a negative H2H_ERR_*) and
 *     keeps a per-thread message for h2h_last_error(); nothing exits;
 *   - the handle owns its host and device memory; h2h_free releases it;
 *   - batched queries take caller-owned buffers and a caller stream.
 */
#ifndef GPUH2H_H
#define GPUH2H_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define H2H_OK 0
#define H2H_ERR_ARG (-1)         /* bad argument or out-of-range vertex          */
#define H2H_ERR_IO (-2)          /* file missing / unreadable                    */
#define H2H_ERR_FORMAT (-3)      /* malformed Edge / ID / Cut file               */
#define H2H_ERR_STATE (-4)       /* call out of order (e.g. query before build)  */
#define H2H_ERR_CUDA (-5)        /* CUDA runtime error                           */
#define H2H_ERR_NOMEM (-6)       /* host or device allocation failed             */
#define H2H_ERR_UNSUPPORTED (-7) /* option outside the GPU hot path              */
#define H2H_ERR_DEVICE (-8)      /* a kernel reported an error (overflow, ...)   */

#define H2H_LABEL_L3 3           /* labels as the reference ships them           */
#define H2H_LABEL_L4 4           /* L4 father-walk enabled (exact distances)     */
#define H2H_QUERY_LCA 0          /* H2HDistancQuery_UsingLCA_noHub semantics     */
#define H2H_QUERY_NOLCA 1        /* H2HDistancQuery_noLCA_noHub semantics        */

typedef struct h2h_graph h2h_graph;

/* Graph_D_H::Graph::Graph (Graph_Fundamental.cu:4-95) with the path rules of
 * main.cu:262-292: <root>/Graph/USA/<name>Edge.txt and
 * <root>/Partition/<name>/{Latitude|Minimum|metis|scotch}{ID,Cut}.txt for
 * partition_method 1/2/3/4.  root NULL means ".". */
int h2h_load(const char *root, const char *graph_name, int partition_height, int change_height,
             int thread_num, int partition_method, h2h_graph **out);

/* The same loader with explicit file paths (Graph_Fundamental.cu:4-95). */
int h2h_load_files(const char *edge_file, const char *id_file, const char *cut_file, const char *graph_name,
                   int partition_height, int change_height, int thread_num, int partition_method,
                   h2h_graph **out);

/* Releases host and device memory of the handle (the reference's Graph
 * destructor, Graph_Fundamental.cu:98-100, releases nothing). */
void h2h_free(h2h_graph *g);

/* Message of the last failing call on this thread. */
const char *h2h_last_error(void);

/* contraction_noHub (main.cu:149-158) with useGPUContract = 1:
 * makeAdjcentNode (GraphPartition.cu:178-308), the partition levels
 * H..C+1 on the GPU (makeCHPerHeight_2, kernel_functions.cu:520-553), the
 * global min-degree heap for levels <= C (TDInCPU, Traditional_H2H.cu:6-25)
 * and beforeH2H_noHub (TreeStructure.cu:41-100: ranks, tree, Euler tour,
 * sparse table).  use_gpu_contract = 0 (the CPU partition contraction
 * partition_TD_T) is outside the GPU hot path: H2H_ERR_UNSUPPORTED. */
int h2h_contract(h2h_graph *g, int use_gpu_contract);

/* constructLabel_noHub (main.cu:160-188): mallocH2HLabel_noHub
 * (H2HConsturction.cu:618-722), constructBFSTree (:324-377) and the
 * level-synchronous label fill on the GPU (makeH2HLabel_noHub_noComm_3,
 * tanslate.cu:511-617, for parallel_fine = 2; the PF form for 0 and 1
 * computes the same values).  label_mode is H2H_LABEL_L4 or H2H_LABEL_L3.
 * use_gpu_construct = 0 (CPU label fill) is H2H_ERR_UNSUPPORTED. */
int h2h_build_labels(h2h_graph *g, int parallel_fine, int use_gpu_construct, int label_mode);

/* Graph::H2HDistancQuery_UsingLCA_noHub (Query.cu:108-122), one pair, on the
 * device-resident index.  Returns the distance, or -1 on error. */
int h2h_query_lca_nohub(const h2h_graph *g, int x, int y);

/* Graph::H2HDistancQuery_noLCA_noHub (Query.cu:124-151), one pair. */
int h2h_query_nolca_nohub(const h2h_graph *g, int x, int y);

/* H2HQuery_UsingLCA_noHub / H2HQuery_noLCA_noHub (kernel_functions.cuh:94-127):
 * n pairs from device buffers x, y into device buffer out, enqueued on the
 * caller's cudaStream_t (NULL = legacy default stream); does not synchronize.
 * A pair with an id outside [0, n) answers -1 (the reference reads out of
 * bounds there); this call does not report it otherwise, so a caller that
 * cannot trust its ids checks the answers for -1.  Host batches and single
 * pairs keep their own flag, so such a batch never fails a later call.
 * The reference wrappers return elapsed microseconds; time with events on
 * the same stream instead. */
int h2h_query_batch(const h2h_graph *g, const int *x_dev, const int *y_dev, int *out_dev, int64_t n,
                    int mode, void *stream);

/* The same from host buffers: copies x, y to the device, runs the batch and
 * copies the answers back before returning (the Query_noHub flow,
 * main.cu:218-240: translateQuery, kernel, translateQueryResultBack).
 * Returns H2H_ERR_ARG when a pair holds an id outside [0, n) (those pairs
 * answer -1); the flag it reads belongs to this call path alone. */
int h2h_query_batch_host(const h2h_graph *g, const int *x, const int *y, int *out, int64_t n, int mode);

/* Sizes and per-phase times of a built index (the printConstructInfo columns,
 * Graph_Fundamental.cu:132-170, plus device sizes). Times in microseconds. */
typedef struct {
  int32_t n, partition_height, change_height, head, tree_height, n_levels, gpu_vertices, label_mode;
  int64_t m, label_size, pos_size, rmq_size, euler_size, lub_size, adj_size;
  int64_t device_bytes;               /* resident index bytes on the GPU           */
  double lub_mb, decomposition_tree_mb, rmq_mb, label_mb;
  int64_t t_load_us, t_rank_tree_us, t_lub_us, t_translate_lub_us, t_td_gpu_us, t_translate_back_us,
      t_td_cpu_us, t_tree_us, t_malloc_us, t_bfs_us, t_translate_labels_us, t_fill_gpu_us;
  int64_t max_label;                  /* largest finite label value (computed on the
                                         first request after a build: one pass over
                                         the labels)                               */
  int64_t label_updates;              /* sum over v of m(v)*(d(v)-2): min-plus updates of the L4 fill */
} h2h_info;
int h2h_get_info(const h2h_graph *g, h2h_info *info);

/* Parity accessors (copies into caller buffers sized from h2h_info). */
int h2h_copy_order(const h2h_graph *g, int *order);                 /* nonAdjcentNode[i].second      */
int h2h_copy_tree(const h2h_graph *g, int *father, int *depth, int *first); /* father, H2H_TreeHeight_Hash, firstAppeare */
int h2h_copy_rmq(const h2h_graph *g, int64_t *rmq_hash, int *rmq_id);      /* RMQHash, RMQ_ID       */
int h2h_copy_adj(const h2h_graph *g, int64_t *adj_hash, int *adj_id, int *adj_w); /* X(v)\{v} by id  */
int h2h_copy_labels(const h2h_graph *g, int64_t *dis_hash, int *dis, int64_t *pos_hash, int *pos_id,
                    int *pos_pos);                                     /* H2H_* no-hub arrays          */
int h2h_copy_bfs(const h2h_graph *g, int *tree_bfs, int *tree_hash);  /* TreeBFS, TreeHash             */

/* CSV outputs with the reference's headers and columns:
 *   <dir>/<Method>PartitionRate.csv          GraphPartition.cu:252-265
 *   <root>/ConstructInfo/<name>/contract.csv TreeStructure.cu:54-99
 *   <root>/ConstructInfo/<name>/constructInfo.csv Graph_Fundamental.cu:132-170
 *   <root>/QueryResult/<name>/random.csv     Query.cu:597-622 (times in us,
 *   19 timing columns in the reference order; unmeasured columns are 0). */
int h2h_write_partition_rate(const h2h_graph *g, const char *dir);
int h2h_write_contract_csv(const h2h_graph *g, const char *root);
int h2h_write_construct_info(const h2h_graph *g, const char *root);
int h2h_write_query_result(const h2h_graph *g, const char *root, int64_t query_number, const int64_t *times_us19);

/* L4 label fill that allocates nothing.  No counterpart in the reference: it
 * is for callers that cannot call cudaMalloc -- code running inside another
 * framework's device-memory budget, services whose device memory is
 * partitioned up front, or plugins that may only use the buffers their host
 * hands them.  Every input and the output `dis` are caller-owned device
 * buffers laid out as h2h_copy_tree / h2h_copy_bfs / h2h_copy_labels return
 * them (order = TreeBFS, any order that lists each father before its
 * children works; pos_w = shortcut weight of each pos entry, 0 for the node
 * itself; pos_id / pos_pos / pos_w hold pos_hash[n] entries, dis holds
 * total_label).  A first pass checks every offset, id and depth (dis_hash
 * and pos_hash non-decreasing within [0, total_label] / from 0, ids in
 * [0, n), depth[father[v]] == depth[v] - 1, each position list sorted by
 * position, ending with the node itself and naming ancestors at their own
 * depths) and returns H2H_ERR_DEVICE with nothing written when one fails.
 * The fill's scratch lives in a fixed 32 MiB __device__ array that every
 * GPU loading the library holds until exit, so the call takes at most
 * n + total_label + 2 <= 8,388,608 (larger trees: H2H_ERR_ARG), and
 * max_depth / max_sep (largest depth, largest |X(v)|-1) must fit the
 * shared-memory staging (16*max_sep + 8*max_depth bytes).  The first call on
 * a device looks up the array's device address (make it before any stream
 * capture).  All calls share the array: calls that overlap on the GPU race.
 * Runs on `stream` and synchronizes it before returning (the status is read
 * back from the device). */
int h2h_fill_labels_l4_noalloc(int n, const int *order, const int *father, const int *depth,
                               const int64_t *pos_hash, const int *pos_id, const int *pos_pos, const int *pos_w,
                               const int64_t *dis_hash, int64_t total_label, int *dis, int max_depth, int max_sep,
                               void *stream);

/* ---- Batched construction.  No counterpart in the reference, which builds
 * one graph per process (main.cu:84-147).  Many loaded graphs are contracted
 * together (one elimination launch per level step across every graph, one
 * launch for every graph's global order over levels <= C) and labelled (L4)
 * by one dataflow launch over the forest of their trees.  Each graph ends in
 * the state h2h_contract(g, 1) + h2h_build_labels(g, 2, 1, H2H_LABEL_L4)
 * leaves, with bit-identical order, tree and labels, and answers queries on
 * its own handle.  The graphs must outlive the batch. */
typedef struct h2h_batch h2h_batch;

typedef struct {
  int32_t graphs, vertices, elim_launches, graph_captured;
  int64_t fill_tiles, device_bytes, label_updates;
  int64_t t_sets_us, t_plan_us, t_contract_us, t_global_us, t_download_us, t_tree_us, t_fill_plan_us, t_fill_us,
      t_attach_us, t_total_us; /* the batched build, by phase (wall time; GPU phases by CUDA events) */
  int64_t t_rebuild_us;       /* device time of the last h2h_batch_rebuild */
  int64_t t_rebuild_fill_us;  /* its label-fill part */
} h2h_batch_info;

/* Builds `count` graphs loaded by h2h_load / h2h_load_files and not yet
 * contracted.  threads: host threads for the per-graph host phases (each
 * graph's own phase runs on one thread). */
int h2h_batch_build(h2h_graph *const *graphs, int count, int threads, h2h_batch **out);
/* Replaces the arc weights of graph `index` for the next h2h_batch_rebuild:
 * w holds one weight per stored arc in h2h_copy_input_arcs order. */
int h2h_batch_set_weights(h2h_batch *b, int index, const int *w);
/* Recomputes contraction and labels of every graph from the current weights
 * on the GPU, replaying one CUDA graph captured on the first call (the tree
 * shape depends only on the arcs, not on their weights, so it is kept).
 * Waits for the result; the graphs' queries see the new labels. */
int h2h_batch_rebuild(h2h_batch *b);
/* Waits for the batch's stream.  Accessors (h2h_copy_adj, h2h_copy_labels)
 * read the device arrays, so they see the last rebuild once it returned. */
int h2h_batch_sync_host(h2h_batch *b);
/* Tile shapes of the forest label fill.  policy is 12 entries
 * "small_work/col_block/sep_chunk" separated by spaces: level class (fewer
 * nodes than SMs / wider / heavy: nodes averaging 2^18+ min-plus updates),
 * times separator size m <= 16, <= 64, <= 256, > 256.
 * h2h_batch_tune times candidate shapes on this batch (coordinate descent,
 * `rounds` passes), keeps the fastest and writes it to policy_out. */
int h2h_batch_set_policy(h2h_batch *b, const char *policy);
int h2h_batch_get_policy(const h2h_batch *b, char *policy_out, int cap);
int h2h_batch_tune(h2h_batch *b, int rounds, char *policy_out, int cap);
int h2h_batch_get_info(const h2h_batch *b, h2h_batch_info *info);
void h2h_batch_free(h2h_batch *b);

/* ---- Query server with continuous batching.  No counterpart in the
 * reference, whose Query_noHub flow (main.cu:218-240) runs one prepared
 * batch of one graph at a time.  Built graphs stay resident; requests
 * (host buffers of pairs for one graph, one mode) are queued from any thread
 * and answered asynchronously by a worker that keeps `slots` device batches
 * in flight on separate streams and refills a slot from the queue as soon as
 * it retires, joining requests of the same graph and mode (a request larger
 * than a slot spans several).  Page-locked request buffers are transferred
 * directly; pageable ones go through the slot's page-locked staging.  Pairs
 * with a vertex id out of range answer -1.  Graphs must outlive the server
 * (or be removed first). */
typedef struct h2h_server h2h_server;

typedef struct {
  int32_t slots;          /* device batches in flight, one stream each      */
  int32_t poll_us;        /* worker's event poll period while batches run   */
  int64_t slot_pairs;     /* capacity of one batch, in pairs                */
  int64_t memory_budget;  /* resident index bytes the server admits (<= 0:
                             the free device memory at creation)            */
} h2h_server_config;

typedef struct {
  int64_t requests, pairs, batches, max_inflight, pending;
  double kernel_us;       /* summed device time of the query kernels        */
  double span_us;         /* first submit to last answer since the last reset */
  int64_t admitted_bytes, memory_budget;
} h2h_server_stats;

void h2h_server_default_config(h2h_server_config *c);
int h2h_server_create(const h2h_server_config *c, h2h_server **out);
/* Admits a labelled graph if its resident index fits the remaining budget
 * (H2H_ERR_NOMEM otherwise). */
int h2h_server_add_graph(h2h_server *s, h2h_graph *g, int *graph_id);
/* Waits for the graph's requests, then frees its share of the budget. */
int h2h_server_remove_graph(h2h_server *s, int graph_id);
/* Queues n pairs; out receives the distances.  The buffers must stay valid
 * until the request finishes. */
int h2h_server_submit(h2h_server *s, int graph_id, const int *x, const int *y, int *out, int64_t n, int mode,
                      uint64_t *request);
/* Waits up to timeout_us (< 0: no limit) for a request (H2H_ERR_STATE on
 * timeout); h2h_server_test returns 1 when finished, 0 when not. */
int h2h_server_wait(h2h_server *s, uint64_t request, int64_t timeout_us);
int h2h_server_test(h2h_server *s, uint64_t request);
/* Forgets a finished request, returning its submit-to-answer latency. */
int h2h_server_release(h2h_server *s, uint64_t request, double *latency_us);
int h2h_server_get_stats(h2h_server *s, h2h_server_stats *st);
int h2h_server_reset_stats(h2h_server *s);
/* Drains the queue, then stops the worker and frees the slots. */
void h2h_server_free(h2h_server *s);

/* The built index on disk, so a process (a server) restarts without a
 * rebuild.  No counterpart in the reference, which rebuilds on every run.
 * h2h_save_index writes the elimination order, tree, Euler tour and sparse
 * table, X(v) lists, label and position arrays in the reference's layouts
 * (a versioned binary format); h2h_load_index validates sizes, offsets and
 * id ranges before it allocates on the GPU (H2H_ERR_FORMAT otherwise) and
 * returns a handle that answers queries and serves every accessor; it has no
 * input arcs (h2h_gen_local_pairs, h2h_batch_build need a loaded graph). */
int h2h_save_index(const h2h_graph *g, const char *path);
int h2h_load_index(const char *path, h2h_graph **out);

/* The stored arcs of a loaded graph in CSR order (self-loops dropped,
 * parallel arcs kept, each vertex's arcs in Edge-file order):
 * adj_off[n+1], adj_v[m], adj_w[m]. */
int h2h_copy_input_arcs(const h2h_graph *g, int *adj_off, int *adj_v, int *adj_w);

/* The partition array of a loaded graph as the ID file gives it
 * (Graph_Fundamental.cu:27-31): part_ids[idx] = NE_P[idx].NodeID (the vertex
 * at partition position idx) and id_hash[vertex] = idx, n entries each. */
int h2h_copy_partition(const h2h_graph *g, int *part_ids, int *id_hash);

#ifdef __cplusplus
}
#endif
#endif /* GPUH2H_H */
