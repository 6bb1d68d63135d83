/*
 * gpuh2h_tools.h -- workload helpers that have no counterpart in the
 * reference: a seeded synthetic road-graph generator that writes the
 * reference's Edge / Node / ID / Cut formats, and seeded query-pair
 * generators.  All arithmetic is integer, so every machine writes the same
 * bytes for the same parameters.
 */
#ifndef GPUH2H_TOOLS_H
#define GPUH2H_TOOLS_H
#include <stdint.h>

#include "gpuh2h.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int64_t n;              /* vertices (grid filled row-major, last row partial)       */
  int32_t cols;           /* grid columns; 0 = derived from n and aspect_milli         */
  int32_t aspect_milli;   /* rows/cols * 1000 (1000 = square, 1300 = 1:1.3)            */
  int32_t jitter_milli;   /* +- jitter of each point in 1/1000 cell (300 = +-0.3)      */
  int32_t drop_permille;  /* grid edges dropped, keeping the graph connected           */
  int64_t target_arcs;    /* if > 0, overrides drop_permille to approach this arc count */
  int32_t diag_permille;  /* grid squares that get one diagonal                        */
  int32_t hw_tiers;       /* highway tiers (0 = none)                                  */
  int32_t hw_permille10;  /* tier-1 highway vertices in 1/10000 of n (50 = 0.5%)       */
  int32_t hw_k;           /* links from each highway vertex to its k nearest peers     */
  int32_t hw_scale_milli; /* tier-1 weight scale in 1/1000 (400 = 0.4x)                */
  int32_t weight_max;     /* clamp weights to [1, weight_max]; 0 = no clamp            */
  int32_t partition_height; /* latitude/longitude median bisection height             */
  uint64_t seed;
} h2h_gen_params;

/* Fills p with the defaults of the 64x64 test grid (4,096 vertices). */
void h2h_gen_default(h2h_gen_params *p);

/* Writes <root>/Graph/USA/<name>{Edge,Node}.txt and
 * <root>/Partition/<name>/Latitude{ID,Cut}.txt.  Returns H2H_OK or an error;
 * *n_arcs receives the arc count written (both directions). */
int h2h_generate_road(const h2h_gen_params *p, const char *root, const char *name, int64_t *n_arcs);

/* n uniform pairs over [0, n_vertices), seeded. */
int h2h_gen_uniform_pairs(int n_vertices, int64_t n, uint64_t seed, int *x, int *y);

/* n "local" pairs: t is the end of a random walk of 1..max_hops steps from a
 * uniform s over the loaded graph's arcs, so t lies within max_hops hops. */
int h2h_gen_local_pairs(const h2h_graph *g, int64_t n, int max_hops, uint64_t seed, int *x, int *y);

/* Measurement baseline, not a product path: the same batch answered with the
 * reference's thread mapping (one thread per query, kernel_functions.cu:
 * 1143-1296) on the same device index, so a bench can report the "plain GPU
 * path" beside the tuned kernel.  Same arguments and results as
 * h2h_query_batch. */
int h2h_query_batch_plain(const h2h_graph *g, const int *x_dev, const int *y_dev, int *out_dev, int64_t n,
                          int mode, void *stream);

/* Measurement baseline, not a product path: the labels of a built L4 graph
 * recomputed with the reference's GPU fill mapping (one thread per (v, u)
 * pair, one launch and one device synchronisation per tree level, father-
 * pointer walks for the L4 columns; kernel_functions.cu:717-744,
 * tanslate.cu:511-617) into scratch rows.  *ms receives the device time,
 * *mismatches the entries that differ from the built labels (0 expected:
 * L4 labels are exact whatever the order). */
int h2h_fill_labels_plain(const h2h_graph *g, double *ms, int64_t *mismatches);

/* The same with the reference's other GPU fill mapping (parallelFine = 1:
 * one thread per node of a tree level walking its position list, one launch
 * and one device synchronisation per level, L4 block enabled;
 * makeH2HLabel_noCommunication_noHub / _D_noHub, kernel_functions.cu:802-888). */
int h2h_fill_labels_plain_node(const h2h_graph *g, double *ms, int64_t *mismatches);

/* Load generator for a query server (measurement tool).  Each request goes
 * to a uniformly drawn graph of graph_ids (vertex counts graph_n) with a
 * size drawn log-uniform in [size_lo, size_hi] pairs of uniform vertices.
 * rate > 0: open loop, Poisson arrivals at `rate` per second for duration_s;
 * a request's latency counts from its scheduled arrival, so a generator
 * that falls behind does not hide queueing.  rate <= 0: closed loop,
 * `inflight` requests outstanding until `requests` have finished.  Pairs are
 * drawn beforehand into page-locked pools; answers land in a page-locked
 * ring, one region per outstanding request. */
typedef struct {
  double rate, duration_s;
  int64_t size_lo, size_hi, requests;
  int32_t inflight, mode;
  uint64_t seed;
} h2h_load_params;

typedef struct {
  int64_t requests, pairs, late;  /* late: submissions more than 100 us behind schedule */
  double wall_s;
} h2h_load_result;

/* latency_us / sizes / graph_of receive one entry per finished request, up
 * to max_requests. */
int h2h_server_load(h2h_server *s, const int *graph_ids, const int *graph_n, int ngraphs, const h2h_load_params *p,
                    double *latency_us, int64_t *sizes, int *graph_of, int64_t max_requests, h2h_load_result *res);

#ifdef __cplusplus
}
#endif
#endif
