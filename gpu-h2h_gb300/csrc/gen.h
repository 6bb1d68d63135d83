// gen.h -- seeded workload generators (gen.cpp).  They throw gh::Error on bad
// parameters or I/O failure; the C ABI wrappers turn that into a status.
#pragma once

#include <cstdint>
#include <string>

#include "gpuh2h_tools.h"
#include "status.h"

namespace gh {

// The defaults of the 64x64 test grid (4,096 vertices, height-6 partition).
void gen_default(h2h_gen_params *p);

// Writes <root>/Graph/USA/<name>{Edge,Node}.txt and
// <root>/Partition/<name>/Latitude{ID,Cut}.txt; *n_arcs = arcs written.
void generate_road(const h2h_gen_params &p, const std::string &root, const std::string &name, int64_t *n_arcs);

// n pairs, both ends uniform over [0, nv).
void gen_uniform_pairs(int nv, int64_t n, uint64_t seed, int *x, int *y);

// n pairs (s, t): s uniform, t the end of a walk of 1..hops random arcs of
// the CSR (off[nv + 1], adj_v), stopping early at a vertex without arcs.
void gen_local_pairs_csr(int nv, const int *off, const int *adj_v, int64_t n, int hops, uint64_t seed, int *x,
                         int *y);

}  // namespace gh
