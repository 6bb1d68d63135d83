// capi.cpp -- the extern "C" entry points of include/gpuh2h.h and
// include/gpuh2h_tools.h.  Every call converts internal exceptions into a
// status code and a per-thread message; nothing exits the process.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>
#include <string>

#include "gen.h"
#include "gpuh2h_tools.h"
#include "handle.h"
#include "pool.h"

namespace gh {
void write_partition_rate(const Graph &g, const std::string &dir);
void write_contract_csv(const Graph &g, const std::string &root);
void write_construct_info(const Graph &g, const std::string &root);
void write_query_result(const Graph &g, const std::string &root, int64_t qn, const int64_t *t19);
const char *partition_file_prefix(int method);

static thread_local std::string g_last_error;
void set_last_error(const std::string &msg) { g_last_error = msg; }
const std::string &last_error() { return g_last_error; }

}  // namespace gh

namespace {

using gh::guarded;

// Every arc u->v needs a reverse arc v->u: the partition-level kernel applies
// the reference's pairwise fill-in per neighbour, which is the same only when
// "u lists v" is symmetric (true for the both-directions Edge format).  Per
// vertex in parallel: each vertex's neighbours sorted once, then every arc
// u->v looks u up among v's neighbours (parallel arcs count once, as sets).
void check_symmetric(const gh::Graph &g, gh::Pool &pool) {
  std::vector<int> sorted(g.adj_v.begin(), g.adj_v.end());
  pool.parallel_for(g.n, 4096, [&](int64_t lo, int64_t hi, int) {
    for (int64_t v = lo; v < hi; v++) std::sort(sorted.begin() + g.adj_off[v], sorted.begin() + g.adj_off[v + 1]);
  });
  std::atomic<bool> bad{false};
  pool.parallel_for(g.n, 4096, [&](int64_t lo, int64_t hi, int) {
    for (int64_t u = lo; u < hi && !bad.load(std::memory_order_relaxed); u++)
      for (int e = g.adj_off[u]; e < g.adj_off[u + 1]; e++) {
        const int v = g.adj_v[e];
        if (!std::binary_search(sorted.begin() + g.adj_off[v], sorted.begin() + g.adj_off[v + 1], (int)u)) {
          bad = true;
          break;
        }
      }
  });
  GH_CHECK(!bad.load(), H2H_ERR_UNSUPPORTED, "Edge file lists an arc without its reverse arc");
}

// Connectivity by union-find over the arcs in parallel (lock-free: a root
// is linked under the other by compare-and-swap, the larger id under the
// smaller; finds halve their paths).
void check_connected(const gh::Graph &g, gh::Pool &pool) {
  std::vector<std::atomic<int>> parent(g.n);
  for (int v = 0; v < g.n; v++) parent[v].store(v, std::memory_order_relaxed);
  auto find = [&](int x) {
    for (;;) {
      int p = parent[x].load(std::memory_order_relaxed);
      if (p == x) return x;
      const int gp = parent[p].load(std::memory_order_relaxed);
      if (gp != p) parent[x].compare_exchange_weak(p, gp, std::memory_order_relaxed);
      x = gp;
    }
  };
  pool.parallel_for(g.n, 4096, [&](int64_t lo, int64_t hi, int) {
    for (int64_t u = lo; u < hi; u++)
      for (int e = g.adj_off[u]; e < g.adj_off[u + 1]; e++) {
        int a = find((int)u), b = find(g.adj_v[e]);
        while (a != b) {
          if (a > b) std::swap(a, b);
          int expect = b;  // link root b under a
          if (parent[b].compare_exchange_strong(expect, a, std::memory_order_relaxed)) break;
          a = find(a);
          b = find(b);
        }
      }
  });
  std::atomic<bool> split{false};
  const int r0 = find(0);
  pool.parallel_for(g.n, 4096, [&](int64_t lo, int64_t hi, int) {
    for (int64_t v = lo; v < hi; v++)
      if (find((int)v) != r0) { split = true; break; }
  });
  GH_CHECK(!split.load(), H2H_ERR_UNSUPPORTED,
           "graph is disconnected (the reference's elimination reads out of bounds on such input)");
}

int load_common(const std::string &edge, const std::string &idf, const std::string &cut, const char *name, int H,
                int C, int threads, int method, h2h_graph **out) {
  if (!out) { gh::set_last_error("out is NULL"); return H2H_ERR_ARG; }
  *out = nullptr;
  h2h_graph *h = nullptr;
  int rc = guarded([&] {
    GH_CHECK(H >= 1, H2H_ERR_ARG, "PartitionHeight must be >= 1");
    GH_CHECK(C >= 1, H2H_ERR_ARG, "ChangeToGlobalHeight must be >= 1 (0 eliminates the root cell on the GPU, "
                                  "where the reference reads out of bounds)");
    GH_CHECK(method >= 1 && method <= 4, H2H_ERR_ARG, "partitionMethod must be 1..4");
    h = new h2h_graph();
    gh::Graph &g = h->g;
    g.name = name ? name : "graph";
    g.H_cli = H;
    g.C = C;
    g.threads = std::max(1, threads);
    g.method = method;
    gh::load_graph(g, edge, idf, cut);
    GH_CHECK(g.C <= g.H, H2H_ERR_ARG, "ChangeToGlobalHeight exceeds the partition height");
    gh::Clock clk;
    {
      gh::Pool pool(g.threads);
      check_symmetric(g, pool);
      check_connected(g, pool);
    }
    g.t.load += clk.us();  // the load phase includes the input checks
  });
  if (rc != H2H_OK) { delete h; return rc; }
  *out = h;
  return H2H_OK;
}

}  // namespace

extern "C" {

const char *h2h_last_error(void) { return gh::last_error().c_str(); }

int h2h_load_files(const char *edge_file, const char *id_file, const char *cut_file, const char *graph_name,
                   int partition_height, int change_height, int thread_num, int partition_method, h2h_graph **out) {
  if (!edge_file || !id_file || !cut_file) { gh::set_last_error("file path is NULL"); return H2H_ERR_ARG; }
  return load_common(edge_file, id_file, cut_file, graph_name, partition_height, change_height, thread_num,
                     partition_method, out);
}

int h2h_load(const char *root, const char *graph_name, int partition_height, int change_height, int thread_num,
             int partition_method, h2h_graph **out) {
  if (!graph_name) { gh::set_last_error("graph_name is NULL"); return H2H_ERR_ARG; }
  std::string r = root ? root : ".";
  std::string name = graph_name;
  std::string edge = r + "/Graph/USA/" + name + "Edge.txt";      // main.cu:262-270
  std::string pre = r + "/Partition/" + name + "/" + gh::partition_file_prefix(partition_method);
  return load_common(edge, pre + "ID.txt", pre + "Cut.txt", graph_name, partition_height, change_height, thread_num,
                     partition_method, out);
}

void h2h_free(h2h_graph *g) { delete g; }

int h2h_contract(h2h_graph *h, int use_gpu_contract) {
  if (!h) { gh::set_last_error("null handle"); return H2H_ERR_ARG; }
  return guarded([&] {
    gh::Graph &g = h->g;
    GH_CHECK(!g.contracted, H2H_ERR_STATE, "graph already contracted");
    GH_CHECK(use_gpu_contract == 1, H2H_ERR_UNSUPPORTED,
             "useGPUContract=0 selects the CPU partition contraction (partition_TD_T), which is not part of the "
             "GPU hot path");
    g.contract_device = use_gpu_contract;
    gh::build_elimination_sets({&g});
    gh::contract_gpu(g);  // with H == C no partition level runs (main.cu:96): the heap takes every vertex
    gh::build_tree_and_rmq(g);
    g.contracted = true;
  });
}

int h2h_build_labels(h2h_graph *h, int parallel_fine, int use_gpu_construct, int label_mode) {
  if (!h) { gh::set_last_error("null handle"); return H2H_ERR_ARG; }
  return guarded([&] {
    gh::Graph &g = h->g;
    GH_CHECK(g.contracted, H2H_ERR_STATE, "h2h_contract must run before h2h_build_labels");
    GH_CHECK(!g.labelled, H2H_ERR_STATE, "labels already built");
    GH_CHECK(use_gpu_construct == 1, H2H_ERR_UNSUPPORTED,
             "useGPUConstruct=0 selects the CPU label fill, which is not part of the GPU hot path");
    GH_CHECK(parallel_fine >= 0 && parallel_fine <= 2, H2H_ERR_ARG, "parallelFine must be 0, 1 or 2");
    GH_CHECK(label_mode == H2H_LABEL_L3 || label_mode == H2H_LABEL_L4, H2H_ERR_ARG, "label_mode must be 3 or 4");
    g.parallel_fine = parallel_fine;
    g.construct_device = use_gpu_construct;
    g.label_mode = label_mode;
    gh::allocate_labels_and_bfs(g);
    gh::fill_labels_gpu(g);
    gh::upload_query_index(g);
    g.labelled = true;
  });
}

static int single_query(const h2h_graph *h, int x, int y, int mode) {
  if (!h) { gh::set_last_error("null handle"); return -1; }
  int res = -1;
  int rc = guarded([&] {
    const gh::Graph &g = h->g;
    GH_CHECK(g.labelled, H2H_ERR_STATE, "labels not built");
    GH_CHECK(x >= 0 && x < g.n && y >= 0 && y < g.n, H2H_ERR_ARG, "vertex out of range");
    int out = 0;
    GH_CHECK(h2h_query_batch_host(h, &x, &y, &out, 1, mode) == H2H_OK, H2H_ERR_CUDA, gh::last_error());
    res = out;
  });
  return rc == H2H_OK ? res : -1;
}

int h2h_query_lca_nohub(const h2h_graph *h, int x, int y) { return single_query(h, x, y, H2H_QUERY_LCA); }
int h2h_query_nolca_nohub(const h2h_graph *h, int x, int y) { return single_query(h, x, y, H2H_QUERY_NOLCA); }

int h2h_query_batch(const h2h_graph *h, const int *x_dev, const int *y_dev, int *out_dev, int64_t n, int mode,
                    void *stream) {
  if (!h) { gh::set_last_error("null handle"); return H2H_ERR_ARG; }
  return guarded([&] {
    const gh::Graph &g = h->g;
    GH_CHECK(g.labelled, H2H_ERR_STATE, "labels not built");
    GH_CHECK(mode == H2H_QUERY_LCA || mode == H2H_QUERY_NOLCA, H2H_ERR_ARG, "mode must be 0 (LCA) or 1 (noLCA)");
    GH_CHECK(n >= 0, H2H_ERR_ARG, "negative batch size");
    GH_CHECK(n == 0 || (x_dev && y_dev && out_dev), H2H_ERR_ARG, "null buffer");
    gh::run_query_batch(g, x_dev, y_dev, out_dev, n, mode, (cudaStream_t)stream);
  });
}

int h2h_query_batch_plain(const h2h_graph *h, const int *x_dev, const int *y_dev, int *out_dev, int64_t n, int mode,
                          void *stream) {
  if (!h) { gh::set_last_error("null handle"); return H2H_ERR_ARG; }
  return guarded([&] {
    GH_CHECK(h->g.labelled, H2H_ERR_STATE, "labels not built");
    GH_CHECK(mode == H2H_QUERY_LCA || mode == H2H_QUERY_NOLCA, H2H_ERR_ARG, "mode must be 0 (LCA) or 1 (noLCA)");
    GH_CHECK(n == 0 || (x_dev && y_dev && out_dev), H2H_ERR_ARG, "null buffer");
    gh::run_query_batch_plain(h->g, x_dev, y_dev, out_dev, n, mode, (cudaStream_t)stream);
  });
}

int h2h_fill_labels_plain(const h2h_graph *h, double *ms, int64_t *mismatches) {
  if (!h) { gh::set_last_error("null handle"); return H2H_ERR_ARG; }
  return guarded([&] { gh::fill_labels_plain(h->g, 0, ms, mismatches); });
}

int h2h_fill_labels_plain_node(const h2h_graph *h, double *ms, int64_t *mismatches) {
  if (!h) { gh::set_last_error("null handle"); return H2H_ERR_ARG; }
  return guarded([&] { gh::fill_labels_plain(h->g, 1, ms, mismatches); });
}

int h2h_query_batch_host(const h2h_graph *hc, const int *x, const int *y, int *out, int64_t n, int mode) {
  if (!hc) { gh::set_last_error("null handle"); return H2H_ERR_ARG; }
  h2h_graph *h = const_cast<h2h_graph *>(hc);
  return guarded([&] {
    const gh::Graph &g = h->g;
    GH_CHECK(g.labelled, H2H_ERR_STATE, "labels not built");
    GH_CHECK(mode == H2H_QUERY_LCA || mode == H2H_QUERY_NOLCA, H2H_ERR_ARG, "mode must be 0 (LCA) or 1 (noLCA)");
    GH_CHECK(n >= 0, H2H_ERR_ARG, "negative batch size");
    if (n == 0) return;
    GH_CHECK(x && y && out, H2H_ERR_ARG, "null buffer");
    gh::HostQueryStage &s = h->stage;
    std::lock_guard<std::mutex> lock(s.mu);
    if (!s.stream) GH_CUDA(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking));
    if (!s.stream2) GH_CUDA(cudaStreamCreateWithFlags(&s.stream2, cudaStreamNonBlocking));
    if (!s.joined) GH_CUDA(cudaEventCreateWithFlags(&s.joined, cudaEventDisableTiming));
    if (!s.dbad) {
      GH_CUDA(cudaMalloc(&s.dbad, sizeof(int)));
      GH_CUDA(cudaMemsetAsync(s.dbad, 0, sizeof(int), s.stream));
    }
    if (n > s.cap) {
      cudaFree(s.dx); cudaFree(s.dy); cudaFree(s.dout);
      s.dx = s.dy = s.dout = nullptr;
      s.cap = 0;
      GH_CUDA(cudaMalloc(&s.dx, sizeof(int) * n));
      GH_CUDA(cudaMalloc(&s.dy, sizeof(int) * n));
      GH_CUDA(cudaMalloc(&s.dout, sizeof(int) * n));
      s.cap = n;
    }
    // A batch of a million pairs or more goes in up to eight chunks on two
    // alternating streams, so one chunk's copies overlap another's queries;
    // a chunk keeps at least a quarter million pairs.  Smaller batches are
    // one chunk (the latency path).
    const int64_t chunk = n >= (int64_t(1) << 20) ? std::max<int64_t>(int64_t(1) << 18, (n + 7) / 8) : n;
    int k = 0;
    try {
      for (int64_t a = 0; a < n; a += chunk, k++) {
        const int64_t c = std::min(chunk, n - a);
        cudaStream_t st = (k & 1) ? s.stream2 : s.stream;
        GH_CUDA(cudaMemcpyAsync(s.dx + a, x + a, sizeof(int) * c, cudaMemcpyHostToDevice, st));
        GH_CUDA(cudaMemcpyAsync(s.dy + a, y + a, sizeof(int) * c, cudaMemcpyHostToDevice, st));
        gh::run_query_batch(g, s.dx + a, s.dy + a, s.dout + a, c, mode, st, s.dbad);
        GH_CUDA(cudaMemcpyAsync(out + a, s.dout + a, sizeof(int) * c, cudaMemcpyDeviceToHost, st));
      }
    } catch (...) {  // nothing of this call may still run when the next one reuses the buffers
      cudaStreamSynchronize(s.stream);
      cudaStreamSynchronize(s.stream2);
      throw;
    }
    if (k > 1) {  // the flag read waits for both streams
      GH_CUDA(cudaEventRecord(s.joined, s.stream2));
      GH_CUDA(cudaStreamWaitEvent(s.stream, s.joined, 0));
    }
    int bad = 0;
    GH_CUDA(cudaMemcpyAsync(&bad, s.dbad, sizeof(int), cudaMemcpyDeviceToHost, s.stream));
    GH_CUDA(cudaStreamSynchronize(s.stream));
    if (bad) {
      GH_CUDA(cudaMemsetAsync(s.dbad, 0, sizeof(int), s.stream));
      GH_CUDA(cudaStreamSynchronize(s.stream));
      throw gh::Error(H2H_ERR_ARG, "vertex id out of range in batch (those pairs answered -1)");
    }
  });
}

int h2h_get_info(const h2h_graph *h, h2h_info *info) {
  if (!h || !info) { gh::set_last_error("null argument"); return H2H_ERR_ARG; }
  const gh::Graph &g = h->g;
  std::memset(info, 0, sizeof(*info));
  const double MB = 1024.0 * 1024.0;
  info->n = g.n;
  info->partition_height = g.H;
  info->change_height = g.C;
  info->head = g.head;
  info->tree_height = g.tree_height;
  info->n_levels = g.tree_hash.empty() ? 0 : (int)g.tree_hash.size() - 1;
  info->gpu_vertices = g.gpu_vertices;
  info->label_mode = g.label_mode;
  info->m = g.m;
  info->label_size = g.h2h_size;
  info->pos_size = g.pos_hash.empty() ? 0 : g.pos_hash.back();
  info->rmq_size = g.rmq_total;
  info->euler_size = g.euler_n;
  info->lub_size = g.lub;
  info->adj_size = g.x_off.empty() ? 0 : g.x_off.back();
  info->device_bytes = g.dev.bytes;
  info->lub_mb = (double)g.lub * 12.0 / MB;
  info->decomposition_tree_mb = (double)g.decomposition_size * 12.0 / MB;
  info->rmq_mb = ((double)g.euler_n * 8 + (double)g.rmq_total * 4 + (double)g.n * 4) / MB;
  info->label_mb = ((double)(g.n + 1) * 16 + (double)info->pos_size * 4 + (double)g.h2h_size * 4) / MB;
  const gh::Timings &t = g.t;
  info->t_load_us = t.load;
  info->t_rank_tree_us = t.rank_tree;
  info->t_lub_us = t.lub;
  info->t_translate_lub_us = t.translate_lub;
  info->t_td_gpu_us = t.td_gpu;
  info->t_translate_back_us = t.translate_back;
  info->t_td_cpu_us = t.td_cpu;
  info->t_tree_us = t.tree;
  info->t_malloc_us = t.malloc_labels;
  info->t_bfs_us = t.bfs;
  info->t_translate_labels_us = t.translate_labels;
  info->t_fill_gpu_us = t.fill_gpu;
  try {
    info->max_label = g.labelled ? gh::label_max(g) : 0;
  } catch (const gh::Error &e) {
    gh::set_last_error(e.what());
    return e.code;
  }
  info->label_updates = 0;
  if (!g.pos_hash.empty() && (int)g.depth.size() == g.n)
    for (int v = 0; v < g.n; v++)
      info->label_updates += (g.pos_hash[v + 1] - g.pos_hash[v] - 1) * (int64_t)std::max(g.depth[v] - 2, 0);
  return H2H_OK;
}

int h2h_copy_order(const h2h_graph *h, int *order) {
  if (!h || !order) { gh::set_last_error("null argument"); return H2H_ERR_ARG; }
  return guarded([&] {
    GH_CHECK(h->g.contracted, H2H_ERR_STATE, "not contracted");
    std::copy(h->g.elim.begin(), h->g.elim.end(), order);
  });
}

int h2h_copy_tree(const h2h_graph *h, int *father, int *depth, int *first) {
  if (!h) { gh::set_last_error("null handle"); return H2H_ERR_ARG; }
  return guarded([&] {
    const gh::Graph &g = h->g;
    GH_CHECK(g.contracted, H2H_ERR_STATE, "not contracted");
    if (father) std::copy(g.father.begin(), g.father.end(), father);
    if (depth) std::copy(g.depth.begin(), g.depth.end(), depth);
    if (first) std::copy(g.first.begin(), g.first.end(), first);
  });
}

int h2h_copy_rmq(const h2h_graph *h, int64_t *rmq_hash, int *rmq_id) {
  if (!h) { gh::set_last_error("null handle"); return H2H_ERR_ARG; }
  return guarded([&] {
    const gh::Graph &g = h->g;
    GH_CHECK(g.contracted, H2H_ERR_STATE, "not contracted");
    gh::download_rmq(g, rmq_hash, rmq_id);
  });
}

int h2h_copy_adj(const h2h_graph *h, int64_t *adj_hash, int *adj_id, int *adj_w) {
  if (!h) { gh::set_last_error("null handle"); return H2H_ERR_ARG; }
  return guarded([&] {
    const gh::Graph &g = h->g;
    GH_CHECK(g.contracted, H2H_ERR_STATE, "not contracted");
    if (adj_hash) std::copy(g.x_off.begin(), g.x_off.end(), adj_hash);
    if (adj_id || adj_w) {
      gh::Graph &gm = const_cast<gh::Graph &>(g);
      gh::download_lists(gm);  // the lists live on the device
      if (adj_id) std::copy(g.x_id.begin(), g.x_id.end(), adj_id);
      if (adj_w) std::copy(g.x_w.begin(), g.x_w.end(), adj_w);
      if (!gh::uses_level_fill(g)) {
        std::vector<int>().swap(gm.x_id);
        std::vector<int>().swap(gm.x_w);
      }
    }
  });
}

int h2h_copy_labels(const h2h_graph *h, int64_t *dis_hash, int *dis, int64_t *pos_hash, int *pos_id, int *pos_pos) {
  if (!h) { gh::set_last_error("null handle"); return H2H_ERR_ARG; }
  return guarded([&] {
    const gh::Graph &g = h->g;
    GH_CHECK(g.labelled, H2H_ERR_STATE, "labels not built");
    if (dis_hash) std::copy(g.dis_hash.begin(), g.dis_hash.end(), dis_hash);
    if (dis) gh::download_labels(g, dis);
    if (pos_hash) std::copy(g.pos_hash.begin(), g.pos_hash.end(), pos_hash);
    if (pos_id || pos_pos) gh::download_positions(g, pos_id, pos_pos);
  });
}

int h2h_copy_input_arcs(const h2h_graph *h, int *adj_off, int *adj_v, int *adj_w) {
  if (!h) { gh::set_last_error("null handle"); return H2H_ERR_ARG; }
  return guarded([&] {
    const gh::Graph &g = h->g;
    if (adj_off) std::copy(g.adj_off.begin(), g.adj_off.end(), adj_off);
    if (adj_v) std::copy(g.adj_v.begin(), g.adj_v.end(), adj_v);
    if (adj_w) std::copy(g.adj_w.begin(), g.adj_w.end(), adj_w);
  });
}

int h2h_copy_partition(const h2h_graph *h, int *part_ids, int *id_hash) {
  if (!h) { gh::set_last_error("null handle"); return H2H_ERR_ARG; }
  return guarded([&] {
    const gh::Graph &g = h->g;
    GH_CHECK((int)g.part_ids.size() == g.n, H2H_ERR_STATE, "no partition array (a loaded index has none)");
    if (part_ids) std::copy(g.part_ids.begin(), g.part_ids.end(), part_ids);
    if (id_hash) std::copy(g.id_hash.begin(), g.id_hash.end(), id_hash);
  });
}

int h2h_copy_bfs(const h2h_graph *h, int *tree_bfs, int *tree_hash) {
  if (!h) { gh::set_last_error("null handle"); return H2H_ERR_ARG; }
  return guarded([&] {
    const gh::Graph &g = h->g;
    GH_CHECK(g.labelled, H2H_ERR_STATE, "labels not built");
    if (tree_bfs) std::copy(g.tree_bfs.begin(), g.tree_bfs.end(), tree_bfs);
    if (tree_hash) std::copy(g.tree_hash.begin(), g.tree_hash.end(), tree_hash);
  });
}

int h2h_write_partition_rate(const h2h_graph *h, const char *dir) {
  if (!h) { gh::set_last_error("null handle"); return H2H_ERR_ARG; }
  return guarded([&] { gh::write_partition_rate(h->g, dir ? dir : "."); });
}
int h2h_write_contract_csv(const h2h_graph *h, const char *root) {
  if (!h) { gh::set_last_error("null handle"); return H2H_ERR_ARG; }
  return guarded([&] { gh::write_contract_csv(h->g, root ? root : "."); });
}
int h2h_write_construct_info(const h2h_graph *h, const char *root) {
  if (!h) { gh::set_last_error("null handle"); return H2H_ERR_ARG; }
  return guarded([&] { gh::write_construct_info(h->g, root ? root : "."); });
}
int h2h_write_query_result(const h2h_graph *h, const char *root, int64_t query_number, const int64_t *times_us19) {
  if (!h) { gh::set_last_error("null handle"); return H2H_ERR_ARG; }
  return guarded([&] { gh::write_query_result(h->g, root ? root : ".", query_number, times_us19); });
}

// ------------------------------------------------------------ tools

void h2h_gen_default(h2h_gen_params *p) {
  if (p) gh::gen_default(p);
}

int h2h_generate_road(const h2h_gen_params *p, const char *root, const char *name, int64_t *n_arcs) {
  if (!p || !root || !name) { gh::set_last_error("null argument"); return H2H_ERR_ARG; }
  return guarded([&] { gh::generate_road(*p, root, name, n_arcs); });
}

int h2h_gen_uniform_pairs(int n_vertices, int64_t n, uint64_t seed, int *x, int *y) {
  if (n_vertices <= 0 || n < 0 || (n > 0 && (!x || !y))) { gh::set_last_error("bad argument"); return H2H_ERR_ARG; }
  gh::gen_uniform_pairs(n_vertices, n, seed, x, y);
  return H2H_OK;
}

int h2h_gen_local_pairs(const h2h_graph *h, int64_t n, int max_hops, uint64_t seed, int *x, int *y) {
  if (!h || n < 0 || (n > 0 && (!x || !y))) { gh::set_last_error("bad argument"); return H2H_ERR_ARG; }
  if ((int)h->g.adj_off.size() != h->g.n + 1 || h->g.n == 0) {
    gh::set_last_error("the input arcs are not loaded (an index read by h2h_load_index has none)");
    return H2H_ERR_STATE;
  }
  gh::gen_local_pairs_csr(h->g.n, h->g.adj_off.data(), h->g.adj_v.data(), n, max_hops, seed, x, y);
  return H2H_OK;
}

}  // extern "C"
