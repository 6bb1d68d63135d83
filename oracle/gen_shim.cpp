// gen_shim.cpp -- TEST INFRASTRUCTURE (part of liboracle.so).  C entry points
// of the oracle over the library's workload generators
// (gpu-h2h_gb300/csrc/gen.cpp, compiled into the oracle as well), so the
// CPU baseline run draws the same seeded graph and query pairs as the GPU
// path without loading the GPU library.
#include <cstdio>
#include <cstring>
#include <vector>

#include "gen.h"
#include "h2h_oracle.h"

extern "C" {

void or_gen_default(void *params) { gh::gen_default(static_cast<h2h_gen_params *>(params)); }

int or_generate_road(const void *params, const char *root, const char *name, int64_t *n_arcs, char *msg,
                     int msg_len) {
  try {
    gh::generate_road(*static_cast<const h2h_gen_params *>(params), root, name, n_arcs);
    return 0;
  } catch (const gh::Error &e) {
    if (msg && msg_len > 0) std::snprintf(msg, (size_t)msg_len, "%s", e.what());
    return e.code;
  } catch (const std::exception &e) {
    if (msg && msg_len > 0) std::snprintf(msg, (size_t)msg_len, "%s", e.what());
    return H2H_ERR_ARG;
  }
}

int or_gen_uniform_pairs(int n_vertices, int64_t n, uint64_t seed, int *x, int *y) {
  if (n_vertices <= 0 || n < 0) return H2H_ERR_ARG;
  gh::gen_uniform_pairs(n_vertices, n, seed, x, y);
  return 0;
}

int or_gen_local_pairs(const or_graph *g, int64_t n, int max_hops, uint64_t seed, int *x, int *y) {
  if (!g || n < 0) return H2H_ERR_ARG;
  const int nv = or_n(g);
  std::vector<int> off((size_t)nv + 1), v((size_t)or_input_arcs(g));
  or_get_input_arcs(g, off.data(), v.data());
  gh::gen_local_pairs_csr(nv, off.data(), v.data(), n, max_hops, seed, x, y);
  return 0;
}

}  // extern "C"
