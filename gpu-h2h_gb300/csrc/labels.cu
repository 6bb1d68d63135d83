// labels.cu -- no-hub H2H label fill on the GPU, the work of
// makeH2HLabel_noHub_noComm_3 / makeH2HLabel_noCommunication_D_noHub_3
// (tanslate.cu:511-617, kernel_functions.cu:717-796), with the L4 block
// (kernel_functions.cu:738-743, H2HConsturction.cu:850-857) enabled.
//
// Row v holds dis[v][j] = distance from v to its ancestor at depth j+1.  For
// every u in X(v)\{v}, in descending position p (H2HConsturction.cu:840):
//   t = dis[v][p]
//   dis[v][j] = min(dis[v][j], t + dis[u][j])            j < p   (ancestors above u)
//   dis[v][j] = min(dis[v][j], t + dis[anc_j(v)][p])     p < j < d-1 (L4: below u)
// Rows of a tree level depend only on rows of shallower levels, so levels run
// in order and the nodes of a level in parallel: one warp owns a node, keeps
// its row in shared memory (lanes own columns, no atomics), reads u's row
// with coalesced loads and the L4 column entries through the ancestor chain.
// The chain (row offsets of the node's ancestors) is staged in shared memory
// from the father's chain, which the previous level wrote to a ping-pong
// buffer.  The update order is the reference's, so L3 rows match its PF CPU
// fill and L4 rows equal exact ancestor distances.
//
// Rows are padded to 16-byte starts (drow[v] is a multiple of 4 ints) so the
// u-row reads are 128-bit vector loads.
#include <algorithm>
#include <climits>

#include "graph.h"

namespace gh {

void DeviceIndex::release() {
  cudaFree(first); cudaFree(depth); cudaFree(rmq_hash); cudaFree(rmq_id); cudaFree(pos_hash);
  cudaFree(pos_pos); cudaFree(pos_id); cudaFree(drow); cudaFree(dis); cudaFree(father); cudaFree(err);
  first = depth = rmq_id = pos_pos = pos_id = dis = father = err = nullptr;
  rmq_hash = pos_hash = drow = nullptr;
  bytes = 0;
}

namespace {

template <typename T>
T *dalloc(size_t n, int64_t &bytes) {
  T *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc(&p, n * sizeof(T));
  if (e != cudaSuccess) throw Error(H2H_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  bytes += (int64_t)(n * sizeof(T));
  return p;
}

// Initial rows (mallocH2HLabel_noHub, H2HConsturction.cu:636-654): INT_MAX,
// shortcut weights at the positions of X(v), 0 at the own position.
__global__ void init_rows_kernel(const int64_t *drow, const int *depth, const int64_t *pos_hash, const int *pos_pos,
                                 const int *pos_w, int *dis, int n) {
  const int lane = threadIdx.x & 31;
  for (int64_t v = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; v < n;
       v += (gridDim.x * (int64_t)blockDim.x) >> 5) {
    const int64_t b = drow[v];
    const int64_t e = drow[v + 1];
    for (int64_t j = b + lane; j < e; j += 32) dis[j] = INT_MAX;
    __syncwarp();
    for (int64_t t = pos_hash[v] + lane; t < pos_hash[v + 1]; t += 32) dis[b + pos_pos[t]] = pos_w[t];
  }
}

struct FillArgs {
  const int *nodes;      // tree_bfs slice of this level
  int count;             // nodes in the level
  int level;             // 0-based; depth d = level + 1
  const int *father;
  const int *lvl_idx;    // position of a node within its level
  const int64_t *drow;
  int *dis;
  const int64_t *pos_hash;
  const int *pos_id;
  const int *pos_pos;
  const int64_t *chain_prev;  // father chains: per node of level-1, (level-1) row offsets
  int64_t *chain_cur;         // chains of this level: per node, level row offsets
  int l4;
};

__global__ void fill_level_kernel(FillArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  const int d = A.level + 1;
  // per-warp staging: row (d ints, rounded to 4) then chain (d-1 int64)
  const int row_cap = (d + 3) & ~3;
  unsigned char *mine = smem + (size_t)wid * ((size_t)row_cap * 4 + (size_t)d * 8);
  int *row = (int *)mine;
  int64_t *anc = (int64_t *)(mine + (size_t)row_cap * 4);
  for (int w = blockIdx.x * wpb + wid; w < A.count; w += gridDim.x * wpb) {
    const int v = A.nodes[w];
    const int f = A.father[v];
    const int64_t base = A.drow[v];
    // ancestor chain: father's chain + father
    if (d >= 2) {
      const int64_t *fc = A.chain_prev + (int64_t)A.lvl_idx[f] * (d - 2);
      for (int j = lane; j < d - 2; j += 32) anc[j] = fc[j];
      if (lane == 0) anc[d - 2] = A.drow[f];
    }
    for (int j = lane; j < d; j += 32) row[j] = A.dis[base + j];
    __syncwarp();
    if (A.chain_cur) {
      int64_t *mc = A.chain_cur + (int64_t)w * (d - 1);
      for (int j = lane; j < d - 1; j += 32) mc[j] = anc[j];
    }
    const int64_t pb = A.pos_hash[v], pe = A.pos_hash[v + 1];
    for (int64_t t = pe - 2; t >= pb; t--) {      // X(v)\{v} in descending position
      const int p = A.pos_pos[t];
      const int u = A.pos_id[t];
      const int tv = row[p];
      const int *urow = A.dis + A.drow[u];
      // j < p: 128-bit loads of u's row (16-byte aligned), 4 columns per lane
      const int p4 = p >> 2;
      for (int q = lane; q < p4; q += 32) {
        int4 x = __ldg(reinterpret_cast<const int4 *>(urow) + q);
        int j = q << 2;
        row[j] = min(row[j], tv + x.x);
        row[j + 1] = min(row[j + 1], tv + x.y);
        row[j + 2] = min(row[j + 2], tv + x.z);
        row[j + 3] = min(row[j + 3], tv + x.w);
      }
      for (int j = (p4 << 2) + lane; j < p; j += 32) row[j] = min(row[j], tv + __ldg(urow + j));
      if (A.l4) {
        for (int j = p + 1 + lane; j < d - 1; j += 32) row[j] = min(row[j], tv + __ldg(A.dis + anc[j] + p));
      }
      __syncwarp();
    }
    for (int j = lane; j < d; j += 32) A.dis[base + j] = row[j];
    __syncwarp();
  }
}

__global__ void max_label_kernel(const int *dis, int64_t n, int *out) {
  int m = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int x = dis[i];
    if (x != INT_MAX && x > m) m = x;
  }
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

}  // namespace

void fill_labels_gpu(Graph &g) {
  Clock clk;
  const int n = g.n;
  DeviceIndex &D = g.dev;
  D.release();
  D.n = n;
  // padded row offsets
  std::vector<int64_t> drow(n + 1, 0);
  for (int v = 0; v < n; v++) drow[v + 1] = drow[v] + ((g.depth[v] + 3) & ~3);
  D.dis_padded = drow[n];
  D.pos = g.pos_hash[n];
  std::vector<int> lvl_idx(n, 0);
  const int nlev = (int)g.tree_hash.size() - 1;
  for (int l = 0; l < nlev; l++)
    for (int i = g.tree_hash[l]; i < g.tree_hash[l + 1]; i++) lvl_idx[g.tree_bfs[i]] = i - g.tree_hash[l];
  int64_t chain_max = 1;
  for (int l = 0; l < nlev; l++) chain_max = std::max<int64_t>(chain_max, (int64_t)(g.tree_hash[l + 1] - g.tree_hash[l]) * l);

  int64_t tmp_bytes = 0;
  D.drow = dalloc<int64_t>(n + 1, D.bytes);
  D.dis = dalloc<int>(D.dis_padded, D.bytes);
  D.pos_hash = dalloc<int64_t>(n + 1, D.bytes);
  D.pos_pos = dalloc<int>(D.pos, D.bytes);
  D.pos_id = dalloc<int>(D.pos, D.bytes);
  D.father = dalloc<int>(n, D.bytes);
  D.depth = dalloc<int>(n, D.bytes);
  D.err = dalloc<int>(1, D.bytes);
  int *d_pos_w = dalloc<int>(D.pos, tmp_bytes);
  int *d_nodes = dalloc<int>(n, tmp_bytes);
  int *d_lvl = dalloc<int>(n, tmp_bytes);
  int64_t *d_chain[2] = {dalloc<int64_t>(chain_max, tmp_bytes), dalloc<int64_t>(chain_max, tmp_bytes)};
  auto cleanup = [&]() {
    cudaFree(d_pos_w); cudaFree(d_nodes); cudaFree(d_lvl); cudaFree(d_chain[0]); cudaFree(d_chain[1]);
  };
  try {
    GH_CUDA(cudaMemcpy(D.drow, drow.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(D.pos_hash, g.pos_hash.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(D.pos_pos, g.pos_pos.data(), sizeof(int) * D.pos, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(D.pos_id, g.pos_id.data(), sizeof(int) * D.pos, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_pos_w, g.pos_w.data(), sizeof(int) * D.pos, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(D.father, g.father.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(D.depth, g.depth.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_nodes, g.tree_bfs.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_lvl, lvl_idx.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    init_rows_kernel<<<std::max(1, std::min(65535, (n * 32 + 255) / 256)), 256>>>(D.drow, D.depth, D.pos_hash,
                                                                                  D.pos_pos, d_pos_w, D.dis, n);
    GH_CUDA(cudaGetLastError());
    GH_CUDA(cudaDeviceSynchronize());
    g.t.translate_labels = clk.us();
    clk.reset();
    int dev = 0, nsm = 0;
    GH_CUDA(cudaGetDevice(&dev));
    GH_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int smem_dyn = enable_max_dynamic_smem(fill_level_kernel);
    cudaEvent_t e0, e1;
    GH_CUDA(cudaEventCreate(&e0));
    GH_CUDA(cudaEventCreate(&e1));
    GH_CUDA(cudaEventRecord(e0));
    for (int l = 1; l < nlev; l++) {
      const int d = l + 1;
      const size_t per_warp = (size_t)((d + 3) & ~3) * 4 + (size_t)d * 8;
      int wpb = (int)std::min<size_t>(8, (size_t)smem_dyn / per_warp);
      GH_CHECK(wpb >= 1, H2H_ERR_DEVICE, "tree too deep for the shared-memory row staging");
      const int count = g.tree_hash[l + 1] - g.tree_hash[l];
      FillArgs A;
      A.nodes = d_nodes + g.tree_hash[l];
      A.count = count;
      A.level = l;
      A.father = D.father;
      A.lvl_idx = d_lvl;
      A.drow = D.drow;
      A.dis = D.dis;
      A.pos_hash = D.pos_hash;
      A.pos_id = D.pos_id;
      A.pos_pos = D.pos_pos;
      A.chain_prev = d_chain[(l + 1) & 1];
      A.chain_cur = (l + 1 < nlev) ? d_chain[l & 1] : nullptr;
      A.l4 = g.label_mode == H2H_LABEL_L4;
      int blocks = std::min<int64_t>((count + wpb - 1) / wpb, (int64_t)nsm * 16);
      fill_level_kernel<<<std::max(1, blocks), wpb * 32, per_warp * wpb>>>(A);
      GH_CUDA(cudaGetLastError());
    }
    GH_CUDA(cudaEventRecord(e1));
    GH_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    GH_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    g.t.fill_gpu = (long long)(ms * 1000.0f);
    GH_CUDA(cudaMemset(D.err, 0, sizeof(int)));
    max_label_kernel<<<nsm * 4, 256>>>(D.dis, D.dis_padded, D.err);
    GH_CUDA(cudaGetLastError());
    int mx = 0;
    GH_CUDA(cudaMemcpy(&mx, D.err, sizeof(int), cudaMemcpyDeviceToHost));
    GH_CUDA(cudaMemset(D.err, 0, sizeof(int)));
    g.max_label = mx;
  } catch (...) {
    cleanup();
    throw;
  }
  cleanup();
  g.drow_host.swap(drow);
}

// Copies the filled labels back into the reference's unpadded layout.
void download_labels(const Graph &g, int *dis_out) {
  const int n = g.n;
  std::vector<int> tmp(g.dev.dis_padded);
  GH_CUDA(cudaMemcpy(tmp.data(), g.dev.dis, sizeof(int) * g.dev.dis_padded, cudaMemcpyDeviceToHost));
  for (int v = 0; v < n; v++)
    std::copy(tmp.begin() + g.drow_host[v], tmp.begin() + g.drow_host[v] + g.depth[v], dis_out + g.dis_hash[v]);
}

}  // namespace gh
