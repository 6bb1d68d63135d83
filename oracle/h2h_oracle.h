/*
 * h2h_oracle.h -- CPU oracle for the GPU-H2H hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (sauccjy/GPU-H2H) used as the parity checker.  Only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm may
 * load it.  The product library never links or calls it.
 *
 * Parity pinning: the restatement is checked against a g++ build of the
 * reference's own CPU translation units (oracle/build_ref.sh) on the
 * 13-vertex sample graph (all four partitions) and on the seeded 64x64
 * road-like graph; the committed fixtures under tests/golden/ carry those
 * outputs to machines without the reference tree.  The per-cell GPU
 * contraction restatement (kernel_functions.cu:309-479) cannot run inside
 * the CPU build of the reference; it is pinned by the L4 label/Dijkstra
 * identity and by tree equality with the CUDA implementation.
 */
#ifndef H2H_ORACLE_H
#define H2H_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Reference data layouts (Graph_D.cuh), kept byte-compatible so the
 * reference harness can hand its thrust vectors to the restated kernel. */
typedef struct { int first, second, third, childSize; } or_tdrank; /* Graph_D.cuh:135-207 */
typedef struct { int NodeID, first, second; } or_mypair;           /* Graph_D.cuh:232-264 */
typedef struct { int first, second; } or_pairs;                    /* Graph_D.cuh:86-133  */

typedef struct or_graph or_graph;

/* Graph_Fundamental.cu:4-95 (loader quirks kept: self loops dropped,
 * parallel arcs kept, 2^min(H_file,H)-1 cut rows). NULL on I/O error. */
or_graph *or_load(const char *edge_file, const char *id_file, const char *cut_file,
                  int partition_height, int change_height, int threads);
void or_free(or_graph *g);
const char *or_error(const or_graph *g);

/* Whole contraction as main.cu:84-124 runs it with useGPUContract=1:
 * makeAdjcentNode(0), the partition levels H..C+1 with the restated
 * per-cell kernel, then uploadCHset + CHUsingHeap_2, then the tree,
 * Euler tour and RMQ table (beforeH2H_noHub).  Returns 0 on success. */
int or_contract(or_graph *g);

/* mallocH2HLabel_noHub + constructBFSTree + makeH2HLabel_noHub_multiThred.
 * l4 != 0 enables the father-walk block that the reference ships commented
 * out (H2HConsturction.cu:850-857). */
int or_build_labels(or_graph *g, int l4, int threads);

/* Query.cu:108-151 (single pair) and a threaded batch loop over them. */
int or_query_lca(const or_graph *g, int x, int y);
int or_query_nolca(const or_graph *g, int x, int y);
void or_query_batch(const or_graph *g, const int *x, const int *y, int *out, int64_t n,
                    int mode /*0 = UsingLCA, 1 = noLCA*/, int threads);

/* Plain Dijkstra on the loaded graph (min over parallel arcs). */
void or_dijkstra(const or_graph *g, int src, int *dist);

/* Sizes and array accessors (copies into caller buffers). */
int or_n(const or_graph *g);
int or_tree_height(const or_graph *g);
int64_t or_label_size(const or_graph *g);   /* sum of depths (H2H_Size)   */
int64_t or_pos_size(const or_graph *g);     /* sum of |X(v)|              */
int64_t or_rmq_size(const or_graph *g);     /* |RMQ_ID|                   */
int64_t or_euler_size(const or_graph *g);   /* 2n-1                       */
int or_n_levels(const or_graph *g);         /* BFS tree levels            */
int or_head(const or_graph *g);
int64_t or_lub_size(const or_graph *g);     /* LUB slots (CHTree length)  */
int or_gpu_vertices(const or_graph *g);     /* vertexesConstructedInGPU   */
void or_get_order(const or_graph *g, int *order);  /* nonAdjcentNode[i].second */
void or_get_father(const or_graph *g, int *father);
void or_get_depth(const or_graph *g, int *depth);
void or_get_first(const or_graph *g, int *first);
void or_get_rmq(const or_graph *g, int64_t *rmq_hash, int *rmq_id);
void or_get_labels(const or_graph *g, int64_t *dis_hash, int *dis, int64_t *pos_hash,
                   int *pos_id, int *pos_pos);
void or_get_bfs(const or_graph *g, int *tree_bfs, int *tree_hash);
/* Upper neighbour list X(v)\{v} with shortcut weights, sorted by id. */
int64_t or_adj_total(const or_graph *g);
void or_get_adj(const or_graph *g, int64_t *adj_hash, int *adj_id, int *adj_w);

/* Input arcs in the loader's adjList order (file order, self loops
 * dropped): off receives n+1 offsets, v the or_input_arcs() targets. */
int64_t or_input_arcs(const or_graph *g);
void or_get_input_arcs(const or_graph *g, int *off, int *v);

/* Workload generators (oracle/gen_shim.cpp over the library's generator
 * source, so a CPU-only run draws the same graph and pairs without the GPU
 * library).  Status 0 = ok; on error msg receives a message. */
void or_gen_default(void *params /* h2h_gen_params: the 64x64 test grid */);
int or_generate_road(const void *params /* h2h_gen_params, include/gpuh2h_tools.h */, const char *root, const char *name, int64_t *n_arcs,
                     char *msg, int msg_len);
int or_gen_uniform_pairs(int n_vertices, int64_t n, uint64_t seed, int *x, int *y);
int or_gen_local_pairs(const or_graph *g, int64_t n, int max_hops, uint64_t seed, int *x, int *y);

/* Restated per-cell body of makeCHPerHeight_D_2 (kernel_functions.cu:319-478)
 * on the reference's AoS arrays.  Exposed for the reference harness, which
 * substitutes it for the GPU launch in the CPU-only build.  Returns 0, or
 * -1 when a list would overflow its LUB capacity or an empty list is read
 * (both undefined in the reference). */
int or_contract_cell(int cell_index, or_tdrank *nonAdj, const int *ID_hash,
                     or_mypair *CHTreeHash, const or_mypair *NANHash, or_mypair *CHTree,
                     unsigned char *visited, or_pairs *CHInfo, int n_vertices);

#ifdef __cplusplus
}
#endif
#endif
