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
#include <cstdlib>

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

// ---------------------------------------------------------------------------
// L4 fill as a dataflow over the tree (the fast path for label_mode L4).
//
// L4 rows are exact: dis[v][j] = D(v, a_j) for the ancestor a_j at depth
// j+1, and D(v, a) = min over u in X(v)\{v} of sc(v,u) + D(u, a), where
// D(u, a) is dis[u][j] when u is below a (p_u > j), 0 when u = a, and
// dis[a][p_u] when u is above a.  The reference reaches the same values with
// its in-place descending-position updates, so every column can be computed
// independently from shortcut weights and finished ancestor rows.
//
// A node needs only its ancestors' rows, and its father finishes after all
// of them, so CTAs take nodes in BFS order from a device counter and wait
// for the father's flag alone: no level barriers, so the thin top of the
// tree pipelines with the wide middle.  A CTA spins on the flag with an
// acquire load, a nanosleep back-off and a clock limit (on expiry it records
// an error and stops); rows and chains produced in this launch are read
// through L2 (ld.global.cg) so no stale L1 line is used.
//
// Each node also publishes its ancestor chain (ids of the ancestors at depth
// 1..d-1, then itself) in a scratch array laid out like the labels, so its
// children can locate the rows a_j without walking father pointers.
// Bound on one dependency wait, in SM clock cycles: 2 s at 2 GHz, or
// GPUH2H_SPIN_LIMIT_MS (profilers replay instrumented kernels much slower).
long long spin_limit_cycles() {
  long long ms = 2000;
  if (const char *e = std::getenv("GPUH2H_SPIN_LIMIT_MS")) ms = std::max(1LL, std::atoll(e));
  return ms * 2000000LL;
}

struct FlowArgs {
  // tiles in BFS node order: tile t covers columns [c0, c1) of node tile_node[t]
  // and separator members [u0, u1) of X(v)\{v}
  const int *tile_node, *tile_c0, *tile_c1, *tile_u0, *tile_u1;
  int ntiles;
  const int *node_ntiles;  // tiles per node
  int *node_cnt;           // finished tiles per node
  const int *father;
  const int *depth;
  const int *nchild;
  const int64_t *drow;
  int *dis;
  const int64_t *pos_hash;
  const int *pos_id;
  const int *pos_pos;
  const int *pos_w;
  int *chain;         // per node row: ancestor ids then the node itself
  int *done;          // per vertex: 1 once its row and chain are visible
  int *next;          // work counter
  int *err;           // 0 = ok, 4 = a wait ran out
  long long spin_limit;
  int max_u;          // max separator members in one tile (staging size)
  int max_c;          // max columns in one tile (staging size)
};

__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int *p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed(const int *p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__global__ void __launch_bounds__(128) fill_flow_kernel(FlowArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_t, s_stop;
  const int tid = threadIdx.x, T = blockDim.x;
  int64_t *xs_row = (int64_t *)smem;                 // [max_u]
  int64_t *anc_row = xs_row + A.max_u;               // [max_c]
  int *xs_p = (int *)(anc_row + A.max_c);            // [max_u]
  int *xs_w = xs_p + A.max_u;                        // [max_u]
  for (;;) {
    if (tid == 0) s_t = atomicAdd(A.next, 1);
    __syncthreads();
    const int t = s_t;
    if (t >= A.ntiles) return;
    const int v = __ldg(A.tile_node + t);
    const int c0 = __ldg(A.tile_c0 + t), c1 = __ldg(A.tile_c1 + t);
    const int u0 = __ldg(A.tile_u0 + t), u1 = __ldg(A.tile_u1 + t);
    const int d = __ldg(A.depth + v);
    const int f = __ldg(A.father + v);
    if (tid == 0) {
      s_stop = 0;
      if (f >= 0) {
        long long t0 = clock64();
        while (ld_acquire(A.done + f) == 0) {
          if (ld_relaxed(A.err) != 0 || clock64() - t0 > A.spin_limit) {
            atomicCAS(A.err, 0, 4);
            s_stop = 1;
            break;
          }
          __nanosleep(64);
        }
      }
    }
    __syncthreads();
    if (s_stop) return;
    const int64_t base = __ldg(A.drow + v);
    const int64_t pb = __ldg(A.pos_hash + v);
    const int m = (int)(__ldg(A.pos_hash + v + 1) - pb) - 1;   // X(v)\{v}
    const bool whole_sep = u0 == 0 && u1 == m;                  // this tile sees every member
    const int nu = u1 - u0;
    for (int i = tid; i < nu; i += T) {
      xs_p[i] = __ldg(A.pos_pos + pb + u0 + i);
      xs_w[i] = __ldg(A.pos_w + pb + u0 + i);
      xs_row[i] = __ldg(A.drow + __ldg(A.pos_id + pb + u0 + i));
    }
    // ancestor chain for this tile's columns, from the father's published chain
    const bool publish = u0 == 0 && __ldg(A.nchild + v) > 0;
    const int cend = min(c1, d - 1);
    if (d >= 2) {
      const int64_t fb = __ldg(A.drow + f);
      for (int j = c0 + tid; j < cend; j += T) {
        const int a = __ldcg(A.chain + fb + j);
        anc_row[j - c0] = __ldg(A.drow + a);
        if (publish) A.chain[base + j] = a;
      }
    }
    if (tid == 0 && c1 == d && u0 == 0) {
      A.dis[base + d - 1] = 0;
      if (publish) A.chain[base + d - 1] = v;
    }
    __syncthreads();
    for (int j = c0 + tid; j < cend; j += T) {
      int r = INT_MAX;
      const int64_t arow = anc_row[j - c0];
#pragma unroll 8
      for (int i = 0; i < nu; i++) {
        const int p = xs_p[i];
        int val;
        if (p > j) val = __ldcg(A.dis + xs_row[i] + j);
        else if (p == j) val = 0;
        else val = __ldcg(A.dis + arow + p);
        r = min(r, xs_w[i] + val);
      }
      if (whole_sep) A.dis[base + j] = r;
      else atomicMin(A.dis + base + j, r);
    }
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      const int nt = __ldg(A.node_ntiles + v);
      if (nt == 1 || atomicAdd(A.node_cnt + v, 1) == nt - 1) {
        __threadfence();
        st_release(A.done + v, 1);
      }
    }
  }
}

__global__ void fill_int_kernel(int *p, int64_t n, int value) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = value;
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
  const int nlev = (int)g.tree_hash.size() - 1;
  // L4 runs as a dataflow over the tree; L3 (order-dependent, as shipped)
  // keeps the level-synchronous kernel that applies the reference's order.
  const bool flow = g.label_mode == H2H_LABEL_L4 && !std::getenv("GPUH2H_LEVEL_FILL");

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
  int *d_aux = dalloc<int>(n, tmp_bytes);          // level index (level path) or child count (flow path)
  int *d_done = nullptr, *d_next = nullptr, *d_chainf = nullptr, *d_tiles = nullptr;
  int64_t *d_chain[2] = {nullptr, nullptr};
  auto cleanup = [&]() {
    cudaFree(d_pos_w); cudaFree(d_nodes); cudaFree(d_aux); cudaFree(d_done); cudaFree(d_next); cudaFree(d_chainf);
    cudaFree(d_tiles);
    cudaFree(d_chain[0]); cudaFree(d_chain[1]);
  };
  try {
    std::vector<int> aux(n, 0);
    int64_t chain_max = 1;
    // tiles of the dataflow fill: a node whose separator work m*d is small is
    // one tile; a larger one is cut into column blocks x separator chunks so
    // the thin, clique-heavy top of the tree spreads over many SMs
    std::vector<int> tn, tc0, tc1, tu0, tu1, nt(n, 0);
    int max_u = 1, max_c = 1;
    if (flow) {
      for (int v = 0; v < n; v++) aux[v] = g.child_off[v + 1] - g.child_off[v];
      const int kSmallWork = 1 << 16, kColBlock = 128, kSepChunk = 32;
      for (int i = 0; i < n; i++) {
        const int v = g.tree_bfs[i], d = g.depth[v];
        const int m = (int)(g.pos_hash[v + 1] - g.pos_hash[v]) - 1;
        if ((int64_t)m * d <= kSmallWork && m <= 256) {
          tn.push_back(v); tc0.push_back(0); tc1.push_back(d); tu0.push_back(0); tu1.push_back(m);
          nt[v] = 1;
          max_u = std::max(max_u, m);
          max_c = std::max(max_c, d);
        } else {
          for (int c = 0; c < d; c += kColBlock)
            for (int u = 0; u < std::max(m, 1); u += kSepChunk) {
              tn.push_back(v); tc0.push_back(c); tc1.push_back(std::min(d, c + kColBlock));
              tu0.push_back(u); tu1.push_back(std::min(m, u + kSepChunk));
              nt[v]++;
            }
          max_u = std::max(max_u, std::min(m, kSepChunk));
          max_c = std::max(max_c, kColBlock);
        }
      }
      const int64_t ntiles = (int64_t)tn.size();
      d_done = dalloc<int>(2 * (int64_t)n, tmp_bytes);     // done flags, then per-node tile counters
      d_next = dalloc<int>(1, tmp_bytes);
      d_chainf = dalloc<int>(D.dis_padded, tmp_bytes);
      d_tiles = dalloc<int>(5 * ntiles + n, tmp_bytes);   // node, c0, c1, u0, u1, then tiles per node
      GH_CUDA(cudaMemset(d_done, 0, sizeof(int) * 2 * (int64_t)n));
      GH_CUDA(cudaMemset(d_next, 0, sizeof(int)));
      const std::vector<int> *parts[5] = {&tn, &tc0, &tc1, &tu0, &tu1};
      for (int k = 0; k < 5; k++)
        GH_CUDA(cudaMemcpy(d_tiles + k * ntiles, parts[k]->data(), sizeof(int) * ntiles, cudaMemcpyHostToDevice));
      GH_CUDA(cudaMemcpy(d_tiles + 5 * ntiles, nt.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    } else {
      for (int l = 0; l < nlev; l++)
        for (int i = g.tree_hash[l]; i < g.tree_hash[l + 1]; i++) aux[g.tree_bfs[i]] = i - g.tree_hash[l];
      for (int l = 0; l < nlev; l++)
        chain_max = std::max<int64_t>(chain_max, (int64_t)(g.tree_hash[l + 1] - g.tree_hash[l]) * l);
      d_chain[0] = dalloc<int64_t>(chain_max, tmp_bytes);
      d_chain[1] = dalloc<int64_t>(chain_max, tmp_bytes);
    }
    GH_CUDA(cudaMemcpy(D.drow, drow.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(D.pos_hash, g.pos_hash.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(D.pos_pos, g.pos_pos.data(), sizeof(int) * D.pos, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(D.pos_id, g.pos_id.data(), sizeof(int) * D.pos, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_pos_w, g.pos_w.data(), sizeof(int) * D.pos, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(D.father, g.father.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(D.depth, g.depth.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_nodes, g.tree_bfs.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_aux, aux.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemset(D.err, 0, sizeof(int)));
    if (flow) {  // rows start at INT_MAX: split tiles combine with atomicMin; padding stays defined
      fill_int_kernel<<<1024, 256>>>(D.dis, D.dis_padded, INT_MAX);
      GH_CUDA(cudaGetLastError());
    }
    if (!flow) {
      init_rows_kernel<<<std::max(1, std::min(65535, (n * 32 + 255) / 256)), 256>>>(D.drow, D.depth, D.pos_hash,
                                                                                    D.pos_pos, d_pos_w, D.dis, n);
      GH_CUDA(cudaGetLastError());
    }
    GH_CUDA(cudaDeviceSynchronize());
    g.t.translate_labels = clk.us();
    clk.reset();
    int dev = 0, nsm = 0;
    GH_CUDA(cudaGetDevice(&dev));
    GH_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    cudaEvent_t e0, e1;
    GH_CUDA(cudaEventCreate(&e0));
    GH_CUDA(cudaEventCreate(&e1));
    GH_CUDA(cudaEventRecord(e0));
    if (flow) {
      const int smem_dyn = enable_max_dynamic_smem(fill_flow_kernel);
      const size_t smem = (size_t)max_u * 16 + (size_t)max_c * 8;
      GH_CHECK(smem <= (size_t)smem_dyn, H2H_ERR_DEVICE, "separator or tree too large for the fill staging");
      const int threads = 128;
      int per_sm = 0;
      GH_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fill_flow_kernel, threads, smem));
      per_sm = std::max(1, per_sm);
      const int64_t ntiles = (int64_t)tn.size();
      FlowArgs A;
      A.tile_node = d_tiles;
      A.tile_c0 = d_tiles + ntiles;
      A.tile_c1 = d_tiles + 2 * ntiles;
      A.tile_u0 = d_tiles + 3 * ntiles;
      A.tile_u1 = d_tiles + 4 * ntiles;
      A.ntiles = (int)ntiles;
      A.node_ntiles = d_tiles + 5 * ntiles;
      A.node_cnt = d_done + n;
      A.father = D.father;
      A.depth = D.depth;
      A.nchild = d_aux;
      A.drow = D.drow;
      A.dis = D.dis;
      A.pos_hash = D.pos_hash;
      A.pos_id = D.pos_id;
      A.pos_pos = D.pos_pos;
      A.pos_w = d_pos_w;
      A.chain = d_chainf;
      A.done = d_done;
      A.next = d_next;
      A.err = D.err;
      A.spin_limit = spin_limit_cycles();
      A.max_u = max_u;
      A.max_c = max_c;
      const int blocks = (int)std::min<int64_t>((int64_t)nsm * per_sm, ntiles);
      fill_flow_kernel<<<std::max(1, blocks), threads, smem>>>(A);
      GH_CUDA(cudaGetLastError());
    } else {
      const int smem_dyn = enable_max_dynamic_smem(fill_level_kernel);
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
        A.lvl_idx = d_aux;
        A.drow = D.drow;
        A.dis = D.dis;
        A.pos_hash = D.pos_hash;
        A.pos_id = D.pos_id;
        A.pos_pos = D.pos_pos;
        A.chain_prev = d_chain[(l + 1) & 1];
        A.chain_cur = (l + 1 < nlev) ? d_chain[l & 1] : nullptr;
        A.l4 = g.label_mode == H2H_LABEL_L4;
        int blocks = (int)std::min<int64_t>((count + wpb - 1) / wpb, (int64_t)nsm * 16);
        fill_level_kernel<<<std::max(1, blocks), wpb * 32, per_warp * wpb>>>(A);
        GH_CUDA(cudaGetLastError());
      }
    }
    GH_CUDA(cudaEventRecord(e1));
    GH_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    GH_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    g.t.fill_gpu = (long long)(ms * 1000.0f);
    int kerr = 0;
    GH_CUDA(cudaMemcpy(&kerr, D.err, sizeof(int), cudaMemcpyDeviceToHost));
    GH_CHECK(kerr == 0, H2H_ERR_DEVICE, "label fill: a dependency wait ran out (error code " + std::to_string(kerr) + ")");
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
