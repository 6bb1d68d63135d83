// batch.cpp -- h2h_batch_*: many graphs contracted and labelled together.
//
// The reference builds one graph per process: every partition level is a
// launch with one thread per cell and the label fill is a launch per tree
// level (main.cu:84-147, kernel_functions.cu:520-553, tanslate.cu:511-617).
// A batch of small graphs therefore spends its time on launches that fill a
// few SMs.  Here the graphs' vertices share one numbering: ElimPlan runs
// level H_i - s of every graph in launch s and every graph's global order in
// one last launch; FillPlan fills the forest of all trees in one dataflow
// launch.  Host phases between them (elimination sets, tree, Euler tour,
// sparse table, label layout) run per graph on a thread pool.
//
// The list structure, the elimination order, the tree and the label layout
// depend only on the arcs, never on their weights, so a rebuild after new
// weights replays the device work alone: the reset of the lists, every
// elimination launch, the gather of shortcut weights into the pos entries
// and the fill, captured once as a CUDA graph.
#include <algorithm>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <memory>

#include "gpuh2h.h"
#include "handle.h"
#include "pool.h"

namespace gh {
std::string tile_policy_tune(FillPlan &plan, cudaStream_t s, int rounds);
}

struct h2h_batch {
  std::vector<h2h_graph *> handles;
  std::vector<gh::Graph *> gs;
  std::unique_ptr<gh::ElimPlan> elim;
  std::unique_ptr<gh::FillPlan> fill;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  h2h_batch_info info{};
  ~h2h_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
    fill.reset();
    elim.reset();
    if (stream) cudaStreamDestroy(stream);
  }
  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    info.graph_captured = 0;
  }
  void fill_info() {
    info.graphs = (int)gs.size();
    info.vertices = elim->N;
    info.elim_launches = (int)elim->launches.size();
    info.fill_tiles = fill->ntiles;
    int64_t db = elim->bytes + fill->work_bytes;
    int64_t upd = 0;
    for (gh::Graph *g : gs) {
      db += g->dev.bytes;
      for (int v = 0; v < g->n; v++)
        upd += (g->pos_hash[v + 1] - g->pos_hash[v] - 1) * (int64_t)std::max(g->depth[v] - 2, 0);
    }
    info.device_bytes = db;
    info.label_updates = upd;
  }
};

namespace {

long long event_us(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  GH_CUDA(cudaEventElapsedTime(&ms, a, b));
  return (long long)(ms * 1000.0f);
}

void copy_policy(const std::string &p, char *out, int cap) {
  if (!out || cap <= 0) return;
  const size_t n = std::min<size_t>(p.size(), (size_t)cap - 1);
  std::memcpy(out, p.data(), n);
  out[n] = 0;
}

}  // namespace

extern "C" {

int h2h_batch_build(h2h_graph *const *graphs, int count, int threads, h2h_batch **out) {
  if (out) *out = nullptr;
  if (!graphs || count <= 0 || !out) {
    gh::set_last_error("need graphs, count >= 1 and an output pointer");
    return H2H_ERR_ARG;
  }
  return gh::guarded([&] {
    auto b = std::make_unique<h2h_batch>();
    for (int i = 0; i < count; i++) {
      GH_CHECK(graphs[i] != nullptr, H2H_ERR_ARG, "null graph handle in batch");
      gh::Graph &g = graphs[i]->g;
      GH_CHECK(!g.contracted, H2H_ERR_STATE, "graph already contracted");
      for (int j = 0; j < i; j++) GH_CHECK(graphs[j] != graphs[i], H2H_ERR_ARG, "a graph appears twice in the batch");
      b->handles.push_back(graphs[i]);
      b->gs.push_back(&g);
    }
    gh::Clock total, clk;
    gh::Pool pool(std::max(1, threads));
    // per-graph host phases run one graph per thread, largest graph first
    std::vector<int> by_size(count);
    for (int i = 0; i < count; i++) by_size[i] = i;
    std::stable_sort(by_size.begin(), by_size.end(), [&](int x, int y) { return b->gs[x]->m > b->gs[y]->m; });
    auto per_graph = [&](const std::function<void(gh::Graph &)> &fn) {
      std::vector<int> saved(count);
      for (int i = 0; i < count; i++) {
        saved[i] = b->gs[i]->threads;
        b->gs[i]->threads = 1;
      }
      std::vector<std::exception_ptr> errs(count);
      pool.parallel_for(count, 1, [&](int64_t lo, int64_t hi, int) {
        for (int64_t k = lo; k < hi; k++) {
          const int i = by_size[k];
          try {
            fn(*b->gs[i]);
          } catch (...) {
            errs[i] = std::current_exception();
          }
        }
      });
      for (int i = 0; i < count; i++) b->gs[i]->threads = saved[i];
      for (auto &e : errs)
        if (e) std::rethrow_exception(e);
    };
    gh::build_elimination_sets(b->gs);
    b->info.t_sets_us = clk.us();
    clk.reset();
    GH_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    for (auto &e : b->ev) GH_CUDA(cudaEventCreate(&e));
    b->elim = std::make_unique<gh::ElimPlan>(b->gs);
    GH_CUDA(cudaDeviceSynchronize());
    b->info.t_plan_us = clk.us();
    clk.reset();
    GH_CUDA(cudaEventRecord(b->ev[0], b->stream));
    cudaEvent_t hev[2] = {b->ev[1], b->ev[2]};
    b->elim->enqueue(b->stream, hev, std::getenv("GPUH2H_TRACE") != nullptr);
    b->elim->check_error();
    b->info.t_contract_us = event_us(b->ev[0], b->ev[1]);
    b->info.t_global_us = event_us(b->ev[1], b->ev[2]);
    clk.reset();
    b->elim->build_lists();
    for (gh::Graph *g : b->gs) {
      g->contract_device = 1;
      g->t.td_gpu = 0;
      g->t.td_cpu = 0;
    }
    b->info.t_download_us = clk.us();
    clk.reset();
    per_graph([](gh::Graph &g) {
      gh::build_tree(g);
      g.contracted = true;
      g.parallel_fine = 2;
      g.construct_device = 1;
      g.label_mode = H2H_LABEL_L4;
      gh::allocate_labels_and_bfs(g);
    });
    gh::build_rmq_gpu(b->gs);
    b->info.t_tree_us = clk.us();
    if (std::getenv("GPUH2H_TRACE")) {
      long long sum = 0, mx = 0;
      for (gh::Graph *g : b->gs) {
        const long long t = g->t.tree + g->t.malloc_labels + g->t.bfs;
        sum += t;
        mx = std::max(mx, t);
      }
      std::fprintf(stderr, "[gpuh2h] batch tree phase: %lld us wall, per-graph sum %lld us, max %lld us\n",
                   (long long)b->info.t_tree_us, sum, mx);
    }
    clk.reset();
    int height = 0;
    for (const gh::Graph *g : b->gs) height = std::max(height, g->tree_height);
    gh::TilePolicy pol = gh::TilePolicy::for_height(height);
    if (const char *e = std::getenv("GPUH2H_TILE_POLICY"))
      GH_CHECK(pol.parse(e), H2H_ERR_ARG, "GPUH2H_TILE_POLICY: expected 12 entries small_work/col_block/sep_chunk");
    b->fill = std::make_unique<gh::FillPlan>(b->gs, pol, b->elim->lists);
    GH_CUDA(cudaDeviceSynchronize());
    b->info.t_fill_plan_us = clk.us();
    clk.reset();
    cudaEvent_t fev[2] = {b->ev[0], b->ev[3]};
    b->fill->enqueue(b->stream, fev);
    b->fill->check_error();
    b->info.t_fill_us = event_us(b->ev[0], b->ev[3]);
    b->fill->trace_report();
    clk.reset();
    b->fill->attach(true);
    for (gh::Graph *g : b->gs) {
      gh::upload_query_index(*g);
      g->labelled = true;
    }
    b->info.t_attach_us = clk.us();
    b->info.t_total_us = total.us();
    b->fill_info();
    *out = b.release();
  });
}

int h2h_batch_set_weights(h2h_batch *b, int index, const int *w) {
  if (!b || !w) { gh::set_last_error("null batch or weights"); return H2H_ERR_ARG; }
  return gh::guarded([&] {
    GH_CHECK(index >= 0 && index < (int)b->gs.size(), H2H_ERR_ARG, "graph index out of range");
    const gh::Graph &g = *b->gs[index];
    for (int64_t e = 0; e < g.m; e++) GH_CHECK(w[e] >= 0, H2H_ERR_ARG, "negative arc weight");
    b->elim->set_weights(index, w, b->stream);
    GH_CUDA(cudaStreamSynchronize(b->stream));
  });
}

int h2h_batch_rebuild(h2h_batch *b) {
  if (!b) { gh::set_last_error("null batch"); return H2H_ERR_ARG; }
  return gh::guarded([&] {
    if (!b->exec) {
      cudaGraph_t graph = nullptr;
      GH_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      try {
        b->elim->enqueue(b->stream);
        b->elim->enqueue_gather(b->stream);
        cudaEvent_t fev[2] = {b->ev[1], b->ev[2]};  // recorded by the graph around the fill kernel
        b->fill->enqueue(b->stream, fev);
      } catch (...) {
        cudaStreamEndCapture(b->stream, &graph);
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        throw;
      }
      GH_CUDA(cudaStreamEndCapture(b->stream, &graph));
      cudaError_t e = cudaGraphInstantiate(&b->exec, graph, 0);
      cudaGraphDestroy(graph);
      GH_CHECK(e == cudaSuccess, H2H_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
      b->info.graph_captured = 1;
    }
    GH_CUDA(cudaEventRecord(b->ev[0], b->stream));
    GH_CUDA(cudaGraphLaunch(b->exec, b->stream));
    GH_CUDA(cudaEventRecord(b->ev[3], b->stream));
    GH_CUDA(cudaStreamSynchronize(b->stream));
    b->elim->check_error();
    b->fill->check_error();
    b->info.t_rebuild_us = event_us(b->ev[0], b->ev[3]);
    b->info.t_rebuild_fill_us = event_us(b->ev[1], b->ev[2]);
    b->fill->attach(false);
  });
}

int h2h_batch_sync_host(h2h_batch *b) {
  if (!b) { gh::set_last_error("null batch"); return H2H_ERR_ARG; }
  return gh::guarded([&] {
    // the lists and position arrays are read from the device on demand
    GH_CUDA(cudaStreamSynchronize(b->stream));
  });
}

int h2h_batch_set_policy(h2h_batch *b, const char *policy) {
  if (!b || !policy) { gh::set_last_error("null batch or policy"); return H2H_ERR_ARG; }
  return gh::guarded([&] {
    gh::TilePolicy p;
    GH_CHECK(p.parse(policy), H2H_ERR_ARG, "policy: expected 12 entries small_work/col_block/sep_chunk");
    GH_CUDA(cudaStreamSynchronize(b->stream));
    b->drop_graph();
    b->fill->build_tiles(p);
    b->fill_info();
  });
}

int h2h_batch_get_policy(const h2h_batch *b, char *policy_out, int cap) {
  if (!b || !policy_out || cap <= 0) { gh::set_last_error("null batch or buffer"); return H2H_ERR_ARG; }
  const std::string p = b->fill->policy.str();
  if ((int)p.size() >= cap) { gh::set_last_error("buffer too small"); return H2H_ERR_ARG; }
  copy_policy(p, policy_out, cap);
  return H2H_OK;
}

int h2h_batch_tune(h2h_batch *b, int rounds, char *policy_out, int cap) {
  if (!b) { gh::set_last_error("null batch"); return H2H_ERR_ARG; }
  return gh::guarded([&] {
    GH_CHECK(rounds >= 1 && rounds <= 8, H2H_ERR_ARG, "rounds must be 1..8");
    GH_CUDA(cudaStreamSynchronize(b->stream));
    b->drop_graph();
    const std::string p = gh::tile_policy_tune(*b->fill, b->stream, rounds);
    b->fill->attach(false);
    b->fill_info();
    copy_policy(p, policy_out, cap);
  });
}

int h2h_batch_get_info(const h2h_batch *b, h2h_batch_info *info) {
  if (!b || !info) { gh::set_last_error("null batch or info"); return H2H_ERR_ARG; }
  *info = b->info;
  return H2H_OK;
}

void h2h_batch_free(h2h_batch *b) { delete b; }

}  // extern "C"
