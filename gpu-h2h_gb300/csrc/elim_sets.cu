// elim_sets.cu -- the per-cell elimination sets, the LUB capacities and the
// per-cell list bounds, Graph::makeAdjcentNode(0) (GraphPartition.cu:178-308),
// on the GPU for one graph or a batch of graphs.
//
// Bottom-up over partition levels h = H..1: a vertex of a level-h cell that
// has no alive neighbour outside the cell is interior and joins the cell's
// candidate range of `elim`; the others stay alive for the parent level.
// The capacity of a vertex's adjacency slot range is the largest (alive cell
// size + alive out-of-cell arcs) over the levels it takes part in, at least
// its input degree: it bounds every list the partition-level contraction
// builds, so the device lists never move.  The same pass gives every cell its
// list bound -- alive cell size - 1 + alive out-of-cell arcs + parallel arcs,
// maximised over its alive members -- which sizes the elimination kernels'
// staging.
//
// Cell ranges of `elim` are laid out as the reference lays them (levels
// bottom-up, a level's cells from the highest index down).  Inside a range
// the reference keeps std::map order (by id); the elimination kernels pick by
// a strict key over the whole range, so that order reaches no result, and a
// range here holds its vertices in partition-array order.
//
// Work unit: a chunk of at most kChunk partition positions of one cell.  Per
// level: alive members per cell (atomic count); per member the out-of-cell
// arcs, interior flag, capacity and cell bound, interior count per chunk; a
// one-block segmented scan over the level's chunks (per graph, continuing
// from the levels below) gives every chunk and cell its offset; each chunk
// writes its interior vertices in position order and retires them.
#include <algorithm>

#include "graph.h"

namespace gh {

namespace {

constexpr int kChunk = 1024;   // partition positions per work unit
constexpr int kThreads = 256;

struct Chunk {
  int cell;    // global cell id (graph's cell base + cell index)
  int graph;
  int start;   // forest partition positions [start, end)
  int end;
};

struct SetsArgs {
  const Chunk *chunks;     // this level's chunks, graph-major, cells from the highest index down
  int nchunks;
  const int *vbase, *abase, *mbase;  // per graph: vertex / position base, adj_off base, arc base
  const int *adj_off;      // per graph n + 1 offsets (local), at abase
  const int *adj_v;        // local neighbour ids, at mbase
  const int *part;         // local vertex per local position, at vbase
  const int *pos;          // local position per local vertex, at vbase
  int *dup;                // parallel arcs per vertex (forest)
  const int *cut_l, *cut_r;  // per global cell, local positions
  unsigned char *alive;    // per forest vertex
  unsigned char *flag;     // per forest position: interior at this level
  int *cap;                // per forest vertex
  int *cell_sz, *cell_bound, *cell_start, *cell_count;  // per global cell
  int *chunk_cnt, *chunk_out;  // per chunk of the level
  int *gfill;              // per graph: elim entries written so far
  int *elim;               // per graph's vertices, local ids, at vbase
};

__device__ __forceinline__ int block_sum(int v, int *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  int t = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
  return t;  // valid in thread 0
}

// Parallel arcs of every vertex: entries whose neighbour id appeared earlier
// in the same input list.  One warp per vertex.
__global__ void dup_kernel(SetsArgs A, const int *vertex_graph, int N) {
  const int lane = threadIdx.x & 31;
  for (int64_t V = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; V < N;
       V += (gridDim.x * (int64_t)blockDim.x) >> 5) {
    const int gi = vertex_graph[V];
    const int v = (int)V - A.vbase[gi];
    const int *off = A.adj_off + A.abase[gi];
    const int *nb = A.adj_v + A.mbase[gi];
    const int b = off[v], e = off[v + 1];
    int d = 0;
    for (int i = b + lane; i < e; i += 32) {
      const int x = nb[i];
      bool seen = false;
      for (int j = b; j < i && !seen; j++) seen = nb[j] == x;
      d += seen;
    }
    for (int o = 16; o > 0; o >>= 1) d += __shfl_down_sync(0xffffffffu, d, o);
    if (lane == 0) A.dup[V] = d;
  }
}

// Alive members per cell.
__global__ void __launch_bounds__(kThreads) count_alive_kernel(SetsArgs A) {
  __shared__ int red[32];
  for (int k = blockIdx.x; k < A.nchunks; k += gridDim.x) {
    const Chunk c = A.chunks[k];
    const int vb = A.vbase[c.graph];
    int n = 0;
    for (int j = c.start + threadIdx.x; j < c.end; j += blockDim.x) n += A.alive[vb + A.part[j]];
    const int t = block_sum(n, red);
    if (threadIdx.x == 0 && t) atomicAdd(A.cell_sz + c.cell, t);
  }
}

// Per alive member: alive out-of-cell arcs, interior flag, capacity, bound.
__global__ void __launch_bounds__(kThreads) classify_kernel(SetsArgs A) {
  __shared__ int red[32];
  for (int k = blockIdx.x; k < A.nchunks; k += gridDim.x) {
    const Chunk c = A.chunks[k];
    const int gi = c.graph, vb = A.vbase[gi];
    const int *off = A.adj_off + A.abase[gi];
    const int *nb = A.adj_v + A.mbase[gi];
    const int cl = A.cut_l[c.cell], cr = A.cut_r[c.cell];  // local positions
    const int sz = A.cell_sz[c.cell];
    int interior = 0, bound = 0;
    for (int j = c.start + threadIdx.x; j < c.end; j += blockDim.x) {
      const int v = A.part[j];  // local
      unsigned char f = 0;
      if (A.alive[vb + v]) {
        int out = 0;
        for (int e = off[v]; e < off[v + 1]; e++) {
          const int u = nb[e];
          const int pu = A.pos[vb + u];
          out += A.alive[vb + u] && (pu < cl || pu >= cr);
        }
        f = out == 0;
        interior += f;
        A.cap[vb + v] = max(A.cap[vb + v], sz + out);
        bound = max(bound, sz - 1 + out + A.dup[vb + v]);
      }
      A.flag[j] = f;
    }
    const int t = block_sum(interior, red);
    if (threadIdx.x == 0) A.chunk_cnt[k] = t;
    for (int o = 16; o > 0; o >>= 1) bound = max(bound, __shfl_down_sync(0xffffffffu, bound, o));
    if ((threadIdx.x & 31) == 0 && bound > 0) atomicMax(A.cell_bound + c.cell, bound);
  }
}

// One block: offsets of the level's chunks, graph by graph in chunk order,
// continuing each graph's range from its earlier levels; cell starts and
// counts; the graphs' running totals.
__global__ void __launch_bounds__(1024) scan_kernel(SetsArgs A) {
  __shared__ int s_val[1024], s_flag[1024];
  __shared__ int s_carry, s_graph;
  if (threadIdx.x == 0) {
    s_carry = 0;
    s_graph = -1;
  }
  __syncthreads();
  for (int base = 0; base < A.nchunks; base += blockDim.x) {
    const int k = base + threadIdx.x;
    const bool in = k < A.nchunks;
    const Chunk c = in ? A.chunks[k] : Chunk{0, -1, 0, 0};
    const int cnt = in ? A.chunk_cnt[k] : 0;
    // inclusive scan of cnt with a reset at every graph boundary
    const bool head = in && (k == 0 || A.chunks[k - 1].graph != c.graph);
    int v = cnt, hd = head;
    s_val[threadIdx.x] = v;
    __syncthreads();
    // segmented Hillis-Steele: flags travel with the values
    s_flag[threadIdx.x] = hd;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
      int pv = 0, pf = 0;
      if ((int)threadIdx.x >= o) { pv = s_val[threadIdx.x - o]; pf = s_flag[threadIdx.x - o]; }
      __syncthreads();
      if ((int)threadIdx.x >= o && !hd) { v += pv; hd |= pf; }
      s_val[threadIdx.x] = v;
      s_flag[threadIdx.x] = hd;
      __syncthreads();
    }
    // exclusive offset inside the graph's level: the carry applies to the
    // leading segment when it continues the previous tile's graph
    const int carry = (!hd && in && c.graph == s_graph) ? s_carry : 0;
    if (in) {
      const int excl = v - cnt + carry;
      A.chunk_out[k] = A.gfill[c.graph] + excl;
      const bool first_of_cell = k == 0 || A.chunks[k - 1].cell != c.cell;
      if (first_of_cell) A.cell_start[c.cell] = A.gfill[c.graph] + excl;
    }
    __syncthreads();
    // the last chunk of a graph in this level closes the graph's total
    if (in) {
      const bool last_of_graph = k == A.nchunks - 1 || A.chunks[k + 1].graph != c.graph;
      if (last_of_graph) A.gfill[c.graph] += v + carry;
    }
    __syncthreads();
    if (k == min(base + (int)blockDim.x, A.nchunks) - 1) {  // the tile's last chunk carries on
      s_carry = v + carry;
      s_graph = c.graph;
    }
    __syncthreads();
  }
}

// Cell counts from the chunk offsets (the chunks of a cell are consecutive).
__global__ void cell_count_kernel(SetsArgs A) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < A.nchunks; k += gridDim.x * blockDim.x) {
    const Chunk c = A.chunks[k];
    const bool last_of_cell = k == A.nchunks - 1 || A.chunks[k + 1].cell != c.cell;
    if (last_of_cell) A.cell_count[c.cell] = A.chunk_out[k] + A.chunk_cnt[k] - A.cell_start[c.cell];
  }
}

// Each chunk writes its interior vertices in position order and retires them.
__global__ void __launch_bounds__(kThreads) write_kernel(SetsArgs A) {
  __shared__ int s_warp[kThreads / 32];
  __shared__ int s_base;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = blockIdx.x; k < A.nchunks; k += gridDim.x) {
    const Chunk c = A.chunks[k];
    const int vb = A.vbase[c.graph];
    if (threadIdx.x == 0) s_base = A.chunk_out[k];
    __syncthreads();
    for (int j0 = c.start; j0 < c.end; j0 += blockDim.x) {
      const int j = j0 + threadIdx.x;
      const bool f = j < c.end && A.flag[j];
      const unsigned bal = __ballot_sync(0xffffffffu, f);
      if (lane == 0) s_warp[wid] = __popc(bal);
      __syncthreads();
      int before = 0, total = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
        if (w < wid) before += s_warp[w];
        total += s_warp[w];
      }
      if (f) {
        const int v = A.part[j];
        A.elim[vb + s_base + before + __popc(bal & ((1u << lane) - 1u))] = v;
        A.alive[vb + v] = 0;
      }
      __syncthreads();
      if (threadIdx.x == 0) s_base += total;
      __syncthreads();
    }
  }
}

template <typename T>
T *sets_alloc(size_t n, std::vector<void *> &owned) {
  T *p = nullptr;
  GH_CUDA(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
  owned.push_back(p);
  return p;
}

}  // namespace

void build_elimination_sets(const std::vector<Graph *> &gs) {
  Clock clk;
  const int K = (int)gs.size();
  GH_CHECK(K >= 1, H2H_ERR_ARG, "no graph");
  std::vector<int> vbase(K), abase(K), mbase(K), cbase(K);
  int64_t N = 0, A = 0, M = 0, CELLS = 0;
  int Hmax = 0;
  for (int i = 0; i < K; i++) {
    const Graph &g = *gs[i];
    vbase[i] = (int)N;
    abase[i] = (int)A;
    mbase[i] = (int)M;
    cbase[i] = (int)CELLS;
    N += g.n;
    A += g.n + 1;
    M += g.m;
    CELLS += (int64_t(1) << g.H) - 1;
    Hmax = std::max(Hmax, g.H);
    GH_CHECK((int64_t)g.cut_l.size() >= (int64_t(1) << g.H) - 1, H2H_ERR_FORMAT, "cut table shorter than 2^H - 1");
  }
  GH_CHECK(N + K < INT32_MAX && M < INT32_MAX && CELLS < INT32_MAX, H2H_ERR_ARG, "batch too large");
  // ---- chunks per level (graph-major, cells from the highest index down),
  // with the reference's checks on the cut rows
  std::vector<std::vector<Chunk>> lv(Hmax + 1);
  std::vector<int> f_cut_l(CELLS), f_cut_r(CELLS);
  for (int i = 0; i < K; i++) {
    const Graph &g = *gs[i];
    for (int h = g.H; h > 0; h--) {
      const int64_t lo = (int64_t(1) << (h - 1)) - 1, hi = (int64_t(1) << h) - 2;
      std::vector<std::pair<int, int>> rs;
      for (int64_t c = lo; c <= hi; c++) {
        const int cl = std::max(0, g.cut_l[c]), cr = std::min(g.n, g.cut_r[c]);
        f_cut_l[cbase[i] + c] = cl;
        f_cut_r[cbase[i] + c] = std::max(cl, cr);
        if (cr > cl) rs.push_back({cl, cr});
      }
      std::sort(rs.begin(), rs.end());
      for (size_t r = 1; r < rs.size(); r++)
        GH_CHECK(rs[r].first >= rs[r - 1].second, H2H_ERR_FORMAT, "partition cells of one level overlap");
      for (int64_t c = hi; c >= lo; c--) {
        const int cl = f_cut_l[cbase[i] + c], cr = f_cut_r[cbase[i] + c];
        const int cell = cbase[i] + (int)c;
        if (cr <= cl) {
          lv[h].push_back({cell, i, vbase[i] + cl, vbase[i] + cl});  // empty: still gets a start
          continue;
        }
        for (int s = cl; s < cr; s += kChunk)
          lv[h].push_back({cell, i, vbase[i] + s, vbase[i] + std::min(cr, s + kChunk)});
      }
    }
  }
  int64_t nchunk_max = 1, nchunk_total = 0;
  for (int h = 1; h <= Hmax; h++) {
    nchunk_max = std::max<int64_t>(nchunk_max, (int64_t)lv[h].size());
    nchunk_total += (int64_t)lv[h].size();
  }
  // ---- device state
  std::vector<void *> owned;
  auto cleanup = [&]() {
    for (void *p : owned) cudaFree(p);
    owned.clear();
  };
  std::vector<int> f_cell_start(CELLS), f_cell_count(CELLS), f_cell_bound(CELLS), f_cap(N), f_dup(N), f_elim(N),
      f_fill(K);
  try {
    SetsArgs S{};
    int *d_vbase = sets_alloc<int>(K, owned), *d_abase = sets_alloc<int>(K, owned), *d_mbase = sets_alloc<int>(K, owned);
    int *d_adj_off = sets_alloc<int>(A, owned), *d_adj_v = sets_alloc<int>(M, owned);
    int *d_part = sets_alloc<int>(N, owned), *d_pos = sets_alloc<int>(N, owned), *d_dup = sets_alloc<int>(N, owned);
    int *d_vgraph = sets_alloc<int>(N, owned);
    int *d_cut_l = sets_alloc<int>(CELLS, owned), *d_cut_r = sets_alloc<int>(CELLS, owned);
    unsigned char *d_alive = sets_alloc<unsigned char>(N, owned), *d_flag = sets_alloc<unsigned char>(N, owned);
    int *d_cap = sets_alloc<int>(N, owned), *d_elim = sets_alloc<int>(N, owned);
    int *d_cell = sets_alloc<int>(4 * CELLS, owned);  // size, bound, start, count
    int *d_chunk_cnt = sets_alloc<int>(nchunk_max, owned), *d_chunk_out = sets_alloc<int>(nchunk_max, owned);
    Chunk *d_chunks = sets_alloc<Chunk>(std::max<int64_t>(nchunk_total, 1), owned);
    int *d_fill = sets_alloc<int>(K, owned);
    GH_CUDA(cudaMemcpy(d_vbase, vbase.data(), sizeof(int) * K, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_abase, abase.data(), sizeof(int) * K, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_mbase, mbase.data(), sizeof(int) * K, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_cut_l, f_cut_l.data(), sizeof(int) * CELLS, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_cut_r, f_cut_r.data(), sizeof(int) * CELLS, cudaMemcpyHostToDevice));
    {
      std::vector<int> vgraph(N);
      for (int i = 0; i < K; i++) {
        const Graph &g = *gs[i];
        std::fill(vgraph.begin() + vbase[i], vgraph.begin() + vbase[i] + g.n, i);
        GH_CUDA(cudaMemcpy(d_adj_off + abase[i], g.adj_off.data(), sizeof(int) * (g.n + 1), cudaMemcpyHostToDevice));
        if (g.m) GH_CUDA(cudaMemcpy(d_adj_v + mbase[i], g.adj_v.data(), sizeof(int) * g.m, cudaMemcpyHostToDevice));
        if (g.n) {
          GH_CUDA(cudaMemcpy(d_part + vbase[i], g.part_ids.data(), sizeof(int) * g.n, cudaMemcpyHostToDevice));
          GH_CUDA(cudaMemcpy(d_pos + vbase[i], g.id_hash.data(), sizeof(int) * g.n, cudaMemcpyHostToDevice));
        }
        for (int v = 0; v < g.n; v++) f_cap[vbase[i] + v] = g.adj_off[v + 1] - g.adj_off[v];
      }
      GH_CUDA(cudaMemcpy(d_vgraph, vgraph.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
    }
    GH_CUDA(cudaMemcpy(d_cap, f_cap.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
    {
      int64_t at = 0;
      for (int h = Hmax; h >= 1; h--) {
        if (!lv[h].empty())
          GH_CUDA(cudaMemcpy(d_chunks + at, lv[h].data(), sizeof(Chunk) * lv[h].size(), cudaMemcpyHostToDevice));
        at += (int64_t)lv[h].size();
      }
    }
    GH_CUDA(cudaMemset(d_alive, 1, N));
    GH_CUDA(cudaMemset(d_cell, 0, sizeof(int) * 4 * CELLS));
    GH_CUDA(cudaMemset(d_fill, 0, sizeof(int) * K));
    S.vbase = d_vbase;
    S.abase = d_abase;
    S.mbase = d_mbase;
    S.adj_off = d_adj_off;
    S.adj_v = d_adj_v;
    S.part = d_part;
    S.pos = d_pos;
    S.dup = d_dup;
    S.cut_l = d_cut_l;
    S.cut_r = d_cut_r;
    S.alive = d_alive;
    S.flag = d_flag;
    S.cap = d_cap;
    S.cell_sz = d_cell;
    S.cell_bound = d_cell + CELLS;
    S.cell_start = d_cell + 2 * CELLS;
    S.cell_count = d_cell + 3 * CELLS;
    S.chunk_cnt = d_chunk_cnt;
    S.chunk_out = d_chunk_out;
    S.gfill = d_fill;
    S.elim = d_elim;
    int dev = 0, nsm = 0;
    GH_CUDA(cudaGetDevice(&dev));
    GH_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    if (N) {
      dup_kernel<<<std::max(1, std::min<int>(nsm * 16, (int)((N * 32 + 255) / 256))), 256>>>(S, d_vgraph, (int)N);
      GH_CUDA(cudaGetLastError());
    }
    int64_t at = 0;
    for (int h = Hmax; h >= 1; h--) {
      const int nc = (int)lv[h].size();
      if (nc == 0) continue;
      S.chunks = d_chunks + at;
      S.nchunks = nc;
      at += nc;
      const int grid = std::max(1, std::min(nc, nsm * 8));
      count_alive_kernel<<<grid, kThreads>>>(S);
      classify_kernel<<<grid, kThreads>>>(S);
      scan_kernel<<<1, 1024>>>(S);
      cell_count_kernel<<<std::max(1, std::min(nsm * 4, (nc + 255) / 256)), 256>>>(S);
      write_kernel<<<grid, kThreads>>>(S);
      GH_CUDA(cudaGetLastError());
    }
    GH_CUDA(cudaMemcpy(f_fill.data(), d_fill, sizeof(int) * K, cudaMemcpyDeviceToHost));
    GH_CUDA(cudaMemcpy(f_elim.data(), d_elim, sizeof(int) * N, cudaMemcpyDeviceToHost));
    GH_CUDA(cudaMemcpy(f_cap.data(), d_cap, sizeof(int) * N, cudaMemcpyDeviceToHost));
    GH_CUDA(cudaMemcpy(f_dup.data(), d_dup, sizeof(int) * N, cudaMemcpyDeviceToHost));
    GH_CUDA(cudaMemcpy(f_cell_bound.data(), S.cell_bound, sizeof(int) * CELLS, cudaMemcpyDeviceToHost));
    GH_CUDA(cudaMemcpy(f_cell_start.data(), S.cell_start, sizeof(int) * CELLS, cudaMemcpyDeviceToHost));
    GH_CUDA(cudaMemcpy(f_cell_count.data(), S.cell_count, sizeof(int) * CELLS, cudaMemcpyDeviceToHost));
  } catch (...) {
    cleanup();
    throw;
  }
  cleanup();
  const long long t_sets = clk.us();
  // ---- per graph: tables, LUB layout (GraphPartition.cu:270-292), level rates
  for (int i = 0; i < K; i++) {
    Graph &g = *gs[i];
    clk.reset();
    GH_CHECK(f_fill[i] == g.n, H2H_ERR_FORMAT,
             "partition does not cover every vertex (root cut row must span all vertices)");
    const int64_t cells = (int64_t(1) << g.H) - 1;
    g.cell_start.assign(f_cell_start.begin() + cbase[i], f_cell_start.begin() + cbase[i] + cells);
    g.cell_count.assign(f_cell_count.begin() + cbase[i], f_cell_count.begin() + cbase[i] + cells);
    g.cell_bound.resize(cells);
    for (int64_t c = 0; c < cells; c++) g.cell_bound[c] = std::max(1, f_cell_bound[cbase[i] + c]);
    g.elim.assign(f_elim.begin() + vbase[i], f_elim.begin() + vbase[i] + g.n);
    g.cap.assign(f_cap.begin() + vbase[i], f_cap.begin() + vbase[i] + g.n);
    g.dup.assign(f_dup.begin() + vbase[i], f_dup.begin() + vbase[i] + g.n);
    g.layer_rate.assign(g.H + 1, 0.0);
    int64_t done = 0;
    for (int h = g.H; h > 0; h--) {
      const int64_t lo = (int64_t(1) << (h - 1)) - 1, hi = (int64_t(1) << h) - 2;
      for (int64_t c = lo; c <= hi; c++) done += g.cell_count[c];
      g.layer_rate[h] = g.n ? (double)done / g.n : 0.0;
    }
    g.slot_off.assign(g.n, 0);
    int64_t off = 0;
    for (int j = 0; j < g.n; j++) {
      const int v = g.part_ids[j];
      g.slot_off[v] = off;
      off += g.cap[v];
    }
    g.lub = off;
    g.t.rank_tree = t_sets;
    g.t.lub = clk.us();
  }
}

}  // namespace gh
