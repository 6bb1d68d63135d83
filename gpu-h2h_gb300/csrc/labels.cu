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
//
// Three fills live here:
//   * fill_flow_kernel, the L4 fill: a dataflow over tiles of the forest of
//     one or more graphs, one warp per tile (FillPlan, further down);
//   * fill_level_kernel, level-synchronous, one warp per node in the
//     reference's update order: L3 rows (order-dependent) and L4 on request;
//     the node's row stays in shared memory, and its ancestors' row offsets
//     are staged from the father's, which the previous level wrote to a
//     ping-pong buffer;
//   * plain_fill_level_kernel and plain_node_fill_kernel, the reference's own
//     two GPU mappings (one thread per (v, u) pair, or one per node; a launch
//     per level), kept as measurement baselines.
//
// Rows are padded to 16-byte starts (drow[v] is a multiple of 4 ints) so the
// u-row reads are 128-bit vector loads.
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <sstream>

#include "graph.h"
#include "pool.h"

namespace gh {

void DeviceIndex::release_labels() {
  for (void *p : owned) cudaFree(p);
  owned.clear();
  keep.reset();
  depth = pos_pos = pos_id = dis = father = err = nullptr;
  pos_hash = drow = nullptr;
  bytes = rmq_bytes;
}

void DeviceIndex::release() {
  release_labels();
  lists = ListStore();
  x_base = pos_base = 0;
  id_base = 0;
  for (void *p : owned_rmq) cudaFree(p);
  owned_rmq.clear();
  first = rmq_id = nullptr;
  rmq_hash = nullptr;
  bytes = rmq_bytes = 0;
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

// An allocation the handle's DeviceIndex owns.
template <typename T>
T *dalloc_owned(size_t n, DeviceIndex &D) {
  T *p = dalloc<T>(n, D.bytes);
  D.owned.push_back(p);
  return p;
}

// Device arrays shared by the graphs of one forest fill.
struct DevArrays {
  std::vector<void *> p;
  int64_t bytes = 0;
  template <typename T>
  T *alloc(size_t n) {
    T *q = dalloc<T>(n, bytes);
    p.push_back(q);
    return q;
  }
  ~DevArrays() {
    for (void *q : p) cudaFree(q);
  }
};

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
// an error and stops); rows produced in this launch are read through L2
// (ld.global.cg) so no stale L1 line is used.
//
// The ancestor a_j of a column comes from the tree's heavy-path layout: the
// node's root path is a handful of heavy-path segments (at most one more
// than the light edges above it, so O(log n)), staged in shared memory; a
// short search finds the segment holding depth j+1 and the path array gives
// the node.  No per-node ancestor list is stored.

struct FlowArgs {
  // tiles in forest BFS order: ticket t belongs to node tile_node[t]; the
  // node's tiles are tickets node_first .. + node_ntiles, its column blocks
  // (node_cb columns) outer and separator chunks (node_sc members) inner
  const int *tile_node;
  int ntiles;
  const int *node_first, *node_ntiles, *node_cb, *node_sc;
  // the counter hands out chunks of consecutive tickets: one tile on the
  // narrow levels, several on the wide ones (fewer atomics)
  const int *chunk_start;  // [nchunks + 1]; nullptr: chunk k is tile k
  int nchunks;
  int *node_cnt;           // finished tiles per node
  const int *father;
  const int *depth;
  const int64_t *drow;
  int *dis;
  const int64_t *pos_hash;
  const int *pos_id;
  const int *pos_pos;
  const int *pos_w;
  const int64_t *hld_row;  // heavy paths, top to bottom: the row offset of the node at each position
  const int64_t *seg_off;  // root-path segments per node
  const int *seg_top, *seg_pos;
  int *done;          // per vertex: 1 once its row is visible
  int *next;          // work counter
  int *err;           // 0 = ok, 4 = a wait ran out
  long long spin_limit;
  int max_u;          // max separator members in one tile (staging size)
  int max_segs;       // max root-path segments of a node (staging size)
  int scalar_cols;    // tiles of at most this many columns sweep one column per lane
  unsigned long long *trace_t;  // non-null (GPUH2H_TRACE): each node's publish time, ns
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

// Every warp is an independent worker: it takes a ticket, stages the tile's
// separator entries and the node's root-path segments in its own slice of
// shared memory while lane 0 waits for the father, sweeps the columns (lane
// per column) and publishes; only warp-level barriers, so a thin tile or a
// dependency wait stalls one warp, not a CTA.
// Ten 4-warp blocks per SM (48 registers, 8 bytes of spill) instead of eight
// at 64 registers: the 6.26M-vertex fill 1,003 -> 928 ms, the 264k-vertex
// fill 28.9 -> 28.2 ms.
__global__ void __launch_bounds__(128, 10) fill_flow_kernel(FlowArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int ual = (A.max_u + 1) & ~1, sal = (A.max_segs + 1) & ~1;
  unsigned char *mine = smem + (size_t)wid * ((size_t)ual * 16 + (size_t)sal * 8);
  int64_t *xs_row = (int64_t *)mine;                 // [max_u]
  int *xs_p = (int *)(xs_row + ual);                 // [max_u]
  int *xs_w = xs_p + ual;                            // [max_u]
  int *s_top = xs_w + ual;                           // [max_segs]
  int *s_pos = s_top + sal;                          // [max_segs]
  for (;;) {
    int k = 0;
    if (lane == 0) k = atomicAdd(A.next, 1);
    k = __shfl_sync(0xffffffffu, k, 0);
    if (k >= A.nchunks) return;
    const int t_beg = A.chunk_start ? max(__ldg(A.chunk_start + k), 0) : k;
    const int t_end = A.chunk_start ? min(__ldg(A.chunk_start + k + 1), A.ntiles) : k + 1;
    for (int t = t_beg; t < t_end; t++) {
    const int v = __ldg(A.tile_node + t);
    const int d = __ldg(A.depth + v);
    const int f = __ldg(A.father + v);
    const int64_t base = __ldg(A.drow + v);
    const int64_t pb = __ldg(A.pos_hash + v);
    const int m = (int)(__ldg(A.pos_hash + v + 1) - pb) - 1;   // X(v)\{v}
    const int sub = t - __ldg(A.node_first + v);
    const int cb = __ldg(A.node_cb + v), sc = __ldg(A.node_sc + v);
    const int nuc = (max(m, 1) + sc - 1) / sc;
    const int ci = sub / nuc, ui = sub - ci * nuc;
    const int c0 = ci * cb, c1 = min(d, c0 + cb);
    const int u0 = ui * sc, u1 = min(m, u0 + sc);
    const bool whole_sep = u0 == 0 && u1 == m;                  // this tile sees every member
    const int nu = u1 - u0;
    // separator entries and root-path segments need no finished row
#pragma unroll 4
    for (int i = lane; i < nu; i += 32) {
      xs_p[i] = __ldg(A.pos_pos + pb + u0 + i);
      xs_w[i] = __ldg(A.pos_w + pb + u0 + i);
      xs_row[i] = __ldg(A.drow + __ldg(A.pos_id + pb + u0 + i));
    }
    const int64_t sb = __ldg(A.seg_off + v);
    const int ns = (int)(__ldg(A.seg_off + v + 1) - sb);
    for (int i = lane; i < ns; i += 32) {
      s_top[i] = __ldg(A.seg_top + sb + i);
      s_pos[i] = __ldg(A.seg_pos + sb + i);
    }
    int stop = 0;
    if (lane == 0) {
      if (f >= 0) {
        long long t0 = clock64();
        while (ld_acquire(A.done + f) == 0) {
          if (ld_relaxed(A.err) != 0 || clock64() - t0 > A.spin_limit) {
            atomicCAS(A.err, 0, 4);
            stop = 1;
            break;
          }
          __nanosleep(64);
        }
      }
      if (c1 == d && u0 == 0) A.dis[base + d - 1] = 0;
    }
    stop = __shfl_sync(0xffffffffu, stop, 0);
    __syncwarp();
    if (stop) return;
    // Column sweep, four consecutive columns [J, J + 4) per lane (rows start
    // on 16-byte boundaries and column blocks are multiples of four, so J is
    // a multiple of four inside every row).  The tile's members are sorted by
    // position, so for a lane's columns they fall into three runs:
    //   i >= hi  (p >= J + 4): every column lies above u_i -- one 128-bit
    //            load of u_i's row gives all four candidates;
    //   i <  lo  (p <  J):     every column lies below u_i -- the candidate
    //            of column j is the ancestor a_j's entry at p (L4);
    //   lo <= i < hi:          at most four members with p inside the quad,
    //            resolved column by column.
    // No per-member branch, and a quarter of the iterations of a
    // column-per-lane sweep.  A tile of 33 to 127 columns spreads its
    // members over 2 or 4 lane groups (every group takes every G-th member)
    // and combines the groups' minima with shuffles, so all 32 lanes work.
    const int cend = min(c1, d - 1);
    if (cend - c0 <= A.scalar_cols) {
      // a tile of at most scalar_cols columns (32 on trees of up to 2,048
      // levels, whose narrow levels are a latency chain): one column per
      // lane, one ancestor lookup each -- the shortest chain of dependent
      // loads per tile
      const int j = c0 + lane;
      if (j < cend) {
        int lo = 0, hi = ns - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (s_top[mid] <= j + 1) lo = mid; else hi = mid - 1;
        }
        const int64_t arow = __ldg(A.hld_row + s_pos[lo] + (j + 1 - s_top[lo]));
        int r = INT_MAX;
#pragma unroll 8
        for (int i = 0; i < nu; i++) {
          const int p = xs_p[i];
          const int val = p > j ? __ldcg(A.dis + xs_row[i] + j) : p == j ? 0 : __ldcg(A.dis + arow + p);
          r = min(r, xs_w[i] + val);
        }
        if (whole_sep) A.dis[base + j] = r;
        else atomicMin(A.dis + base + j, r);
      }
    }
    const int nquad = cend - c0 <= A.scalar_cols ? 0 : (cend - c0 + 3) >> 2;
    const int QW = nquad > 16 ? 32 : nquad > 8 ? 16 : 8;  // lanes along the columns
    const int G = 32 / QW;                                 // member groups
    const int qi = lane & (QW - 1), grp = lane / QW;
    for (int Jb = c0; nquad > 0 && Jb < cend; Jb += 4 * QW) {  // the same trip count in every lane
      const int J = Jb + 4 * qi;
      const bool active = J < cend;
      const int nvalid = active ? min(4, cend - J) : 0;
      int r0 = INT_MAX, r1 = INT_MAX, r2 = INT_MAX, r3 = INT_MAX;
      if (active) {
        int64_t arow[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
          // ancestor at depth j + 1 (a column past cend reuses column J's
          // ancestor: its reads stay inside that row or its padding and its
          // result is discarded)
          const int j = J + (k < nvalid ? k : 0);
          int lo = 0, hi = ns - 1;
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_top[mid] <= j + 1) lo = mid; else hi = mid - 1;
          }
          arow[k] = __ldg(A.hld_row + s_pos[lo] + (j + 1 - s_top[lo]));
        }
        int ilo = 0, ihi = nu;  // first member with p >= J
        while (ilo < ihi) {
          const int mid = (ilo + ihi) >> 1;
          if (xs_p[mid] < J) ilo = mid + 1; else ihi = mid;
        }
        const int mlo = ilo;
        ihi = nu;               // first member with p >= J + 4
        while (ilo < ihi) {
          const int mid = (ilo + ihi) >> 1;
          if (xs_p[mid] < J + 4) ilo = mid + 1; else ihi = mid;
        }
        const int mhi = ilo;
#pragma unroll 4
        for (int i = mhi + grp; i < nu; i += G) {
          const int4 x = __ldcg(reinterpret_cast<const int4 *>(A.dis + xs_row[i] + J));
          const int w = xs_w[i];
          r0 = min(r0, w + x.x);
          r1 = min(r1, w + x.y);
          r2 = min(r2, w + x.z);
          r3 = min(r3, w + x.w);
        }
#pragma unroll 4
        for (int i = grp; i < mlo; i += G) {
          const int p = xs_p[i], w = xs_w[i];
          r0 = min(r0, w + __ldcg(A.dis + arow[0] + p));
          r1 = min(r1, w + __ldcg(A.dis + arow[1] + p));
          r2 = min(r2, w + __ldcg(A.dis + arow[2] + p));
          r3 = min(r3, w + __ldcg(A.dis + arow[3] + p));
        }
        for (int i = mlo + grp; i < mhi; i += G) {
          const int p = xs_p[i], w = xs_w[i];
          const int64_t ur = xs_row[i];
          int c[4];
#pragma unroll
          for (int k = 0; k < 4; k++) {
            const int j = J + k;
            c[k] = p > j ? __ldcg(A.dis + ur + j) : p == j ? 0 : __ldcg(A.dis + arow[k] + p);
          }
          r0 = min(r0, w + c[0]);
          r1 = min(r1, w + c[1]);
          r2 = min(r2, w + c[2]);
          r3 = min(r3, w + c[3]);
        }
      }
      for (int o = QW; o < 32; o <<= 1) {  // combine the member groups (lanes qi, qi + QW, ...)
        r0 = min(r0, __shfl_xor_sync(0xffffffffu, r0, o));
        r1 = min(r1, __shfl_xor_sync(0xffffffffu, r1, o));
        r2 = min(r2, __shfl_xor_sync(0xffffffffu, r2, o));
        r3 = min(r3, __shfl_xor_sync(0xffffffffu, r3, o));
      }
      if (active && grp == 0) {
        int *out = A.dis + base + J;
        if (whole_sep && nvalid == 4) {
          *reinterpret_cast<int4 *>(out) = make_int4(r0, r1, r2, r3);
        } else {
          const int r[4] = {r0, r1, r2, r3};
#pragma unroll
          for (int k = 0; k < 4; k++)
            if (k < nvalid) {
              if (whole_sep) out[k] = r[k];
              else atomicMin(out + k, r[k]);
            }
        }
      }
    }
    __syncwarp();
    if (lane == 0) {
      __threadfence();
      const int nt = __ldg(A.node_ntiles + v);
      if (nt == 1 || atomicAdd(A.node_cnt + v, 1) == nt - 1) {
        __threadfence();
        st_release(A.done + v, 1);
        if (A.trace_t) {
          unsigned long long now;
          asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
          A.trace_t[v] = now;
        }
      }
    }
    __syncwarp();  // the slice is restaged only after every lane left the sweep
    }
  }
}

// The reference's GPU label fill mapping, kept as a measurement baseline
// (makeH2HLabel_noCommunication_D_noHub_3, kernel_functions.cu:717-744, with
// the L4 block :738-743 enabled): one thread per (v, u) pair of one tree
// level; the thread min-updates the columns above u directly and walks
// father pointers for the columns below u.  Launched once per level with a
// device synchronisation in between, as the reference does.
__global__ void plain_fill_level_kernel(const int *pair_v, const int64_t *pair_k, int npairs, const int64_t *drow,
                                        const int *depth, const int *father, const int *pos_pos, const int *pos_id,
                                        const int *pos_w, int *dis) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npairs; i += gridDim.x * blockDim.x) {
    const int v = pair_v[i];
    const int64_t k = pair_k[i];
    const int p = pos_pos[k], u = pos_id[k], t = pos_w[k], d = depth[v];
    const int64_t base = drow[v], ub = drow[u];
    for (int j = 0; j < p; j++) atomicMin(dis + base + j, t + __ldcg(dis + ub + j));
    int a = father[v];
    for (int j = d - 2; j > p && a >= 0; j--) {
      atomicMin(dis + base + j, t + __ldcg(dis + drow[a] + p));
      a = father[a];
    }
  }
}

// The reference's other GPU fill mapping (parallelFine = 1:
// makeH2HLabel_noCommunication_D_noHub, kernel_functions.cu:802-837, with its
// commented L4 block enabled), kept as a measurement baseline: one thread per
// node of one tree level, walking the node's position list from the highest
// position down (its own entry, the last, excluded); each entry u at position
// p min-updates the columns below p from u's row and, for L4, the columns
// above p from the ancestors' column p along the father chain.  The thread
// owns its row: no atomics.
__global__ void plain_node_fill_kernel(const int *nodes, int cnt, const int64_t *drow, const int *depth,
                                       const int *father, const int64_t *pos_hash, const int *pos_pos,
                                       const int *pos_id, const int *pos_w, int *dis) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
    const int v = nodes[i];
    const int64_t base = drow[v];
    const int d = depth[v];
    for (int64_t k = pos_hash[v + 1] - 1; k >= pos_hash[v]; k--) {
      const int u = pos_id[k];
      if (u == v) continue;
      const int p = pos_pos[k];
      const int t = dis[base + p];
      const int64_t ub = drow[u];
      for (int j = p - 1; j >= 0; j--) dis[base + j] = min(dis[base + j], t + __ldcg(dis + ub + j));
      int a = v;
      for (int j = d - 2; j > p; j--) {
        a = father[a];
        if (a < 0) break;
        dis[base + j] = min(dis[base + j], t + __ldcg(dis + drow[a] + p));
      }
    }
  }
}

__global__ void count_mismatch_kernel(const int *a, const int *b, int64_t n, unsigned long long *bad) {
  unsigned long long c = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    c += a[i] != b[i];
  if (c) atomicAdd(bad, c);
}

// Chunk k's first ticket, from per-level rows (first chunk, first ticket,
// step): the level holding k by binary search, then an arithmetic step;
// entry nchunks closes the table.
__global__ void chunk_table_kernel(const int64_t *ltab, int nlev, int64_t nchunks, int64_t ntiles, int *chunks) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k <= nchunks;
       k += (int64_t)gridDim.x * blockDim.x) {
    if (k == nchunks) {
      chunks[k] = (int)ntiles;
      continue;
    }
    int lo = 0, hi = nlev - 1;  // last level whose first chunk is <= k
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (ltab[3 * mid] <= k) lo = mid; else hi = mid - 1;
    }
    chunks[k] = (int)(ltab[3 * lo + 1] + (k - ltab[3 * lo]) * ltab[3 * lo + 2]);
  }
}

// tile_node[t] = v for the tickets of every node v.  One warp per node.
__global__ void expand_tiles_kernel(const int *node_first, const int *node_ntiles, int *tile_node, int n) {
  const int lane = threadIdx.x & 31;
  for (int64_t v = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; v < n;
       v += (gridDim.x * (int64_t)blockDim.x) >> 5) {
    const int f = node_first[v], c = node_ntiles[v];
    for (int k = lane; k < c; k += 32) tile_node[f + k] = (int)v;
  }
}

// Row offset of the node at every heavy-path position (the fill reads an
// ancestor's row offset with one load instead of two dependent ones).
__global__ void hld_row_kernel(const int *hld, const int64_t *drow, int64_t *hld_row, int n) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) hld_row[k] = drow[hld[k]];
}

// Root-path segments of every node, shallowest first: walking up from v,
// each heavy path met contributes (depth of its top, index of its top in
// hld).  One thread per node; the walk crosses O(log n) light edges.
__global__ void root_path_segments_kernel(const int *father, const int *depth, const int *htop, const int *hpos,
                                          const int64_t *seg_off, int *seg_top, int *seg_pos, int n) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const int64_t b = seg_off[v];
    int64_t k = seg_off[v + 1];
    for (int u = v; u >= 0 && k > b;) {
      const int t = htop[u];
      --k;
      seg_top[k] = depth[t];
      seg_pos[k] = hpos[t];
      u = father[t];
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

// Shortcut weights of every pos entry, read from the contraction's lists:
// entry k of v takes list index pos_src[k] of v's list, or 0 for v itself.
// One warp per vertex.
__global__ void gather_pos_weights_kernel(const int64_t *pos_hash, const int *pos_src, const int64_t *list_off,
                                          const int *list_w, int *pos_w, int n) {
  const int lane = threadIdx.x & 31;
  for (int64_t v = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; v < n;
       v += (gridDim.x * (int64_t)blockDim.x) >> 5) {
    const int64_t b = pos_hash[v], e = pos_hash[v + 1], so = list_off[v];
    for (int64_t k = b + lane; k < e; k += 32) {
      const int src = pos_src[k];
      pos_w[k] = src < 0 ? 0 : list_w[so + src];
    }
  }
}

// Position lists (mallocH2HLabel_noHub, H2HConsturction.cu:656-700): X(v)
// and v itself ordered by position (depth - 1 of the member).  Positions of
// one list are distinct, so an entry's slot is the number of smaller
// positions in the list.  One block per vertex, the list's positions staged
// in shared memory.  A member that is not a proper ancestor (position >=
// d - 1) sets *err = 5.
__global__ void build_positions_kernel(const int64_t *list_off, const int *list_id, const int *list_w,
                                       const int *depth, const int64_t *pos_hash, int *pos_pos, int *pos_id,
                                       int *pos_w, int *pos_src, int *err, int n) {
  extern __shared__ int keys[];
  const int tid = threadIdx.x, T = blockDim.x;
  for (int v = blockIdx.x; v < n; v += gridDim.x) {
    const int64_t b = list_off[v];
    const int m = (int)(list_off[v + 1] - b);
    const int d = depth[v];
    const int64_t pb = pos_hash[v];
    for (int i = tid; i <= m; i += T) {
      int key = d - 1;
      if (i < m) {
        key = depth[list_id[b + i]] - 1;
        if (key < 0 || key >= d - 1) atomicCAS(err, 0, 5);
      }
      keys[i] = key;
    }
    __syncthreads();
    for (int i = tid; i <= m; i += T) {
      const int key = keys[i];
      int r = 0;
      for (int j = 0; j <= m; j++) r += keys[j] < key;
      pos_pos[pb + r] = key;
      pos_id[pb + r] = i < m ? list_id[b + i] : v;
      pos_w[pb + r] = i < m ? list_w[b + i] : 0;
      pos_src[pb + r] = i < m ? i : -1;
    }
    __syncthreads();
  }
}

}  // namespace

// Defaults measured on road graphs (one warp per tile): narrow levels cut a
// node into 32-column x 4-member tiles once m*d exceeds 1,024 (the 264k-
// vertex graph's fill is a latency chain through 1,343 such levels); wider
// levels 32 x 16 above 4,096; heavy levels (the 6.26M-vertex graph's middle)
// 128 x 256 above 16,384 -- whole separators, so no atomicMin combining.
// Separators above 256 members always split.
// Two measured presets.  Shallow trees (the 264k-vertex graph, tree height
// 1,343; batches of road graphs) fill as a latency chain through the narrow
// levels and want small tiles.  Deep trees have rows several thousand
// columns long, so the same tiles are too many: the autotuner on the
// 3.6M-vertex graph (height 4,180) moved the wide levels to 64-column x
// 32-member tiles and the narrow levels' widest separators to 16-member
// chunks, fill 1,080 -> 788 ms; on the 264k-vertex graph those shapes cost
// 29 -> 40 ms.
TilePolicy::TilePolicy() {
  static const int sw[kWidth] = {1024, 4096, 16384}, cb[kWidth] = {32, 32, 128}, sc[kWidth] = {4, 16, 256};
  for (int w = 0; w < kWidth; w++)
    for (int b = 0; b < kSep; b++) {
      small_work[w][b] = b == kSep - 1 ? 0 : sw[w];
      col_block[w][b] = cb[w];
      sep_chunk[w][b] = sc[w];
    }
}

TilePolicy TilePolicy::for_height(int height) {
  TilePolicy t;
  if (height <= 2048) return t;
  static const int sw[kWidth][kSep] = {{1024, 1024, 1024, 0}, {16384, 4096, 4096, 0}, {16384, 16384, 16384, 0}};
  static const int cb[kWidth][kSep] = {{32, 32, 32, 32}, {32, 64, 64, 64}, {128, 128, 128, 128}};
  static const int sc[kWidth][kSep] = {{4, 4, 4, 16}, {16, 32, 32, 32}, {256, 256, 256, 256}};
  for (int w = 0; w < kWidth; w++)
    for (int b = 0; b < kSep; b++) {
      t.small_work[w][b] = sw[w][b];
      t.col_block[w][b] = cb[w][b];
      t.sep_chunk[w][b] = sc[w][b];
    }
  return t;
}

std::string TilePolicy::str() const {
  std::ostringstream o;
  for (int w = 0; w < kWidth; w++)
    for (int b = 0; b < kSep; b++)
      o << (w || b ? " " : "") << small_work[w][b] << "/" << col_block[w][b] << "/" << sep_chunk[w][b];
  return o.str();
}

bool TilePolicy::parse(const std::string &text) {
  TilePolicy t;
  std::istringstream in(text);
  for (int w = 0; w < kWidth; w++)
    for (int b = 0; b < kSep; b++) {
      long long sw, cb, sc;
      char s1, s2;
      if (!(in >> sw >> s1 >> cb >> s2 >> sc) || s1 != '/' || s2 != '/') return false;
      if (sw < 0 || sw > (1LL << 30) || cb < 1 || cb > 4096 || sc < 1 || sc > 1024) return false;
      t.small_work[w][b] = (int)sw;
      t.col_block[w][b] = (int)cb;
      t.sep_chunk[w][b] = (int)sc;
    }
  std::string rest;
  if (in >> rest) return false;
  *this = t;
  return true;
}

FillPlan::FillPlan(const std::vector<Graph *> &graphs, const TilePolicy &pol, const ListStore &lst)
    : gs(graphs), policy(pol), lists(lst) {
  const bool trace = std::getenv("GPUH2H_TRACE") != nullptr;
  Clock tclk;
  auto mark = [&](const char *what) {
    if (!trace) return;
    cudaDeviceSynchronize();
    std::fprintf(stderr, "[gpuh2h] fill plan: %s %.3f ms\n", what, tclk.us() / 1e3);
    tclk.reset();
  };
  const int K = (int)gs.size();
  GH_CHECK(K >= 1, H2H_ERR_ARG, "no graph to label");
  int host_threads = 1;
  for (const Graph *g : gs) host_threads = std::max(host_threads, g->threads);
  // vertex ranges of every graph, in parallel: padded row totals and the
  // widest separator
  struct VRange {
    int g, v0, v1;
  };
  std::vector<VRange> vr;
  for (int i = 0; i < K; i++)
    for (int v = 0; v < gs[i]->n; v += 65536) vr.push_back({i, v, std::min(gs[i]->n, v + 65536)});
  const int64_t nvr = (int64_t)vr.size();
  std::vector<int64_t> rdis(nvr, 0), rbase(nvr, 0);
  std::vector<int> rmax_m(nvr, 0);
  Pool pool(host_threads);
  pool.parallel_for(nvr, 1, [&](int64_t lo, int64_t hi, int) {
    for (int64_t r = lo; r < hi; r++) {
      const Graph &g = *gs[vr[r].g];
      int64_t d = 0, mm = 0;
      for (int v = vr[r].v0; v < vr[r].v1; v++) {
        d += (g.depth[v] + 3) & ~3;
        mm = std::max<int64_t>(mm, g.x_off[v + 1] - g.x_off[v]);
      }
      rdis[r] = d;
      rmax_m[r] = (int)mm;
    }
  });
  std::vector<int64_t> gdis(K, 0);
  std::vector<int> gmax_m(K, 0);
  for (int64_t r = 0; r < nvr; r++) {
    rbase[r] = gdis[vr[r].g];  // offset inside the graph's rows
    gdis[vr[r].g] += rdis[r];
    gmax_m[vr[r].g] = std::max(gmax_m[vr[r].g], rmax_m[r]);
  }
  vbase.assign(K, 0);
  std::vector<int64_t> pbase(K, 0), dbase(K, 0);
  int max_m = 0;
  for (int i = 0; i < K; i++) {
    const Graph &g = *gs[i];
    GH_CHECK((int64_t)N + g.n < INT32_MAX, H2H_ERR_ARG, "too many vertices in one batch");
    vbase[i] = N;
    pbase[i] = pos_total;
    dbase[i] = dis_total;
    N += g.n;
    pos_total += g.pos_hash[g.n];
    dis_total += gdis[i];
    max_m = std::max(max_m, gmax_m[i]);
  }
  // forest arrays, every entry written below (so not zero-filled first)
  std::vector<int64_t, NoInit<int64_t>> f_drow(N + 1), f_pos_hash(N + 1);
  std::vector<int, NoInit<int>> f_father(N), f_depth(N), f_hld(N);
  std::vector<int64_t> sbase(K, 0);
  int64_t seg_total = 0;
  for (int i = 0; i < K; i++) {
    sbase[i] = seg_total;
    seg_total += gs[i]->seg_off[gs[i]->n];
    max_segs = std::max(max_segs, gs[i]->max_segs);
  }
  std::vector<int64_t, NoInit<int64_t>> f_seg_off(N + 1);
  std::vector<int, NoInit<int>> f_htop(N), f_hpos(N);
  pool.parallel_for(nvr, 1, [&](int64_t lo, int64_t hi, int) {
    for (int64_t r = lo; r < hi; r++) {
      const int i = vr[r].g;
      const Graph &g = *gs[i];
      const int vb = vbase[i];
      const int64_t pb = pbase[i];
      int64_t d = dbase[i] + rbase[r];
      for (int v = vr[r].v0; v < vr[r].v1; v++) {
        const int V = vb + v;
        f_drow[V] = d;
        d += (g.depth[v] + 3) & ~3;
        f_pos_hash[V] = pb + g.pos_hash[v];
        f_father[V] = g.father[v] < 0 ? -1 : g.father[v] + vb;
        f_depth[V] = g.depth[v];
        f_hld[V] = g.hld[v] + vb;
        f_htop[V] = g.htop[v] + vb;
        f_hpos[V] = g.hpos[v] + vb;
        f_seg_off[V] = sbase[i] + g.seg_off[v];
      }
    }
  });
  f_drow[N] = dis_total;
  f_pos_hash[N] = pos_total;
  // Narrow tiles sweep one column per lane on trees of up to 2,048 levels,
  // whose narrow levels fill as a latency chain (264k-vertex graph: 29 ms
  // against 34 ms with four columns per lane); deeper trees cut their long
  // rows into many more tiles per level and take four columns per lane
  // throughout (6.26M-vertex graph: narrow levels 500 -> 300 ms).
  {
    int height = 0;
    for (const Graph *g : gs) height = std::max(height, g->tree_height);
    scalar_cols = height <= 2048 ? 32 : 0;
    if (const char *e = std::getenv("GPUH2H_FILL_SCALAR_COLS")) scalar_cols = std::max(0, std::atoi(e));
  }
  f_seg_off[N] = seg_total;
  mark("host assembly");
  threads = 128;
  int dev = 0;
  GH_CUDA(cudaGetDevice(&dev));
  GH_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  auto st = std::make_shared<DevArrays>();
  storage = st;
  drow = st->alloc<int64_t>(N + 1);
  pos_hash = st->alloc<int64_t>(N + 1);
  pos_pos = st->alloc<int>(pos_total);
  pos_id = st->alloc<int>(pos_total);
  father = st->alloc<int>(N);
  depth = st->alloc<int>(N);
  dis = st->alloc<int>(dis_total);
  try {
    pos_w = dalloc<int>(pos_total, work_bytes);
    pos_src = dalloc<int>(pos_total, work_bytes);
    hld = dalloc<int>(N, work_bytes);
    htop = dalloc<int>(N, work_bytes);
    hpos = dalloc<int>(N, work_bytes);
    seg_off = dalloc<int64_t>(N + 1, work_bytes);
    seg_top = dalloc<int>(std::max<int64_t>(seg_total, 1), work_bytes);
    seg_pos = dalloc<int>(std::max<int64_t>(seg_total, 1), work_bytes);
    done = dalloc<int>(2 * (int64_t)N, work_bytes);  // done flags, then per-node tile counters
    next = dalloc<int>(1, work_bytes);
    err = dalloc<int>(1, work_bytes);
    GH_CUDA(cudaMemcpy(drow, f_drow.data(), sizeof(int64_t) * (N + 1), cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(pos_hash, f_pos_hash.data(), sizeof(int64_t) * (N + 1), cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(father, f_father.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(depth, f_depth.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(hld, f_hld.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
    hld_row = dalloc<int64_t>(N, work_bytes);
    hld_row_kernel<<<std::max(1, std::min(8192, (N + 255) / 256)), 256>>>(hld, drow, hld_row, N);
    GH_CUDA(cudaGetLastError());
    mark("allocations and uploads");
    {
      const size_t ksmem = (size_t)(max_m + 1) * sizeof(int);
      const int kdyn = enable_max_dynamic_smem(build_positions_kernel);
      GH_CHECK(ksmem <= (size_t)kdyn, H2H_ERR_DEVICE, "separator too large for the position-list staging");
      GH_CUDA(cudaMemset(err, 0, sizeof(int)));
      build_positions_kernel<<<std::max(1, std::min(N, nsm * 16)), 128, ksmem>>>(
          lists.off, lists.id, lists.w, depth, pos_hash, pos_pos, pos_id, pos_w, pos_src, err, N);
      GH_CUDA(cudaGetLastError());
      int e = 0;
      GH_CUDA(cudaMemcpy(&e, err, sizeof(int), cudaMemcpyDeviceToHost));
      GH_CHECK(e == 0, H2H_ERR_STATE, "an upper neighbour is not an ancestor in the tree");
    }
    mark("position lists");
    GH_CUDA(cudaMemcpy(seg_off, f_seg_off.data(), sizeof(int64_t) * (N + 1), cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(htop, f_htop.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(hpos, f_hpos.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
    root_path_segments_kernel<<<std::max(1, std::min(8192, (N + 255) / 256)), 256>>>(father, depth, htop, hpos,
                                                                                     seg_off, seg_top, seg_pos, N);
    GH_CUDA(cudaGetLastError());
    mark("root-path segments");
    build_tiles(pol);
    mark("tiles");
  } catch (...) {
    release_work();
    throw;
  }
}

FillPlan::~FillPlan() { release_work(); }

void FillPlan::release_work() {
  void *ps[] = {pos_w, pos_src, hld, htop, hpos, seg_off, seg_top, seg_pos, done, next, err, tiles, trace_t, hld_row};
  for (void *p : ps) cudaFree(p);
  trace_t = nullptr;
  pos_w = pos_src = hld = htop = hpos = seg_top = seg_pos = done = next = err = tiles = nullptr;
  hld_row = nullptr;
  seg_off = nullptr;
}

// Work items of the host passes over the forest: (graph, level, BFS range
// of at most kItemNodes nodes), graph by graph, levels in order.
namespace {
constexpr int kItemNodes = 32768;
struct LevelItem {
  int g, l, q0, q1;
};
std::vector<LevelItem> level_items(const std::vector<Graph *> &gs) {
  std::vector<LevelItem> items;
  for (int i = 0; i < (int)gs.size(); i++) {
    const Graph &g = *gs[i];
    for (int l = 0; l + 1 < (int)g.tree_hash.size(); l++)
      for (int q = g.tree_hash[l]; q < g.tree_hash[l + 1]; q += kItemNodes)
        items.push_back({i, l, q, std::min(q + kItemNodes, g.tree_hash[l + 1])});
  }
  return items;
}
int host_threads_of(const std::vector<Graph *> &gs) {
  int t = 1;
  for (const Graph *g : gs) t = std::max(t, g->threads);
  return t;
}
}  // namespace

std::vector<int> FillPlan::level_classes() const {
  int nlev = 0;
  for (const Graph *g : gs) nlev = std::max(nlev, (int)g->tree_hash.size() - 1);
  // nodes and min-plus updates per forest level, summed over items computed in parallel
  const std::vector<LevelItem> items = level_items(gs);
  std::vector<int64_t> iwork(items.size(), 0);
  {
    Pool pool(host_threads_of(gs));
    pool.parallel_for((int64_t)items.size(), 1, [&](int64_t lo, int64_t hi, int) {
      for (int64_t t = lo; t < hi; t++) {
        const LevelItem &it = items[t];
        const Graph &g = *gs[it.g];
        int64_t w = 0;
        for (int q = it.q0; q < it.q1; q++) {
          const int v = g.tree_bfs[q];
          w += (g.pos_hash[v + 1] - g.pos_hash[v] - 1) * (int64_t)g.depth[v];
        }
        iwork[t] = w;
      }
    });
  }
  std::vector<int64_t> width(nlev, 0), work(nlev, 0);
  for (size_t t = 0; t < items.size(); t++) {
    width[items[t].l] += items[t].q1 - items[t].q0;
    work[items[t].l] += iwork[t];
  }
  // narrow: fewer nodes than SMs, whatever their work (the critical path);
  // heavy: a wider level whose nodes average at least 2^18 min-plus updates
  // (GPUH2H_HEAVY_LEVEL_WORK overrides the figure)
  int64_t per_node = int64_t(1) << 18;
  if (const char *e = std::getenv("GPUH2H_HEAVY_LEVEL_WORK")) per_node = std::max(1LL, std::atoll(e));
  std::vector<int> cls(nlev, 0);
  for (int l = 0; l < nlev; l++)
    cls[l] = width[l] < nsm ? 0 : work[l] >= per_node * width[l] ? 2 : 1;
  return cls;
}

// Tiles in forest BFS order (level l of every graph, then level l + 1): a
// node's father always holds an earlier ticket, so the dataflow cannot wait
// on work no CTA has taken.  Two passes over the graphs in parallel: tile
// counts per (level, graph), then each graph writes its tiles at the
// offsets the counts give.
void FillPlan::build_tiles(const TilePolicy &pol) {
  const bool trace = std::getenv("GPUH2H_TRACE") != nullptr;
  Clock tclk;
  auto mark = [&](const char *what) {
    if (!trace) return;
    cudaDeviceSynchronize();
    std::fprintf(stderr, "[gpuh2h] tiles: %s %.3f ms\n", what, tclk.us() / 1e3);
    tclk.reset();
  };
  policy = pol;
  const int K = (int)gs.size();
  int nlev = 0;
  for (const Graph *g : gs) nlev = std::max(nlev, (int)g->tree_hash.size() - 1);
  const std::vector<int> lcls = level_classes();
  mark("level classes");
  auto tiles_of = [&](int wb, int m, int d, int &nt_node, int &cb, int &sc) {
    const int sb = TilePolicy::sep_bucket(m);
    if ((int64_t)m * d <= pol.small_work[wb][sb]) {
      nt_node = 1;
      cb = d;
      sc = std::max(m, 1);
      return true;  // one tile
    }
    cb = (pol.col_block[wb][sb] + 3) & ~3;  // the sweep takes columns four at a time
    sc = pol.sep_chunk[wb][sb];
    nt_node = ((d + cb - 1) / cb) * ((std::max(m, 1) + sc - 1) / sc);
    return false;
  };
  Pool pool(host_threads_of(gs));
  // pass 1 (items in parallel): every node's tile count and shape, tiles
  // per item, staging bounds
  const std::vector<LevelItem> items = level_items(gs);
  const int64_t nitems = (int64_t)items.size();
  std::vector<int, NoInit<int>> host((size_t)4 * N);  // every node's four entries are written below
  int *nfirst = host.data(), *nt = nfirst + N, *ncb = nfirst + 2 * N, *nsc = nfirst + 3 * N;
  std::vector<int64_t> icnt(nitems, 0);
  std::vector<int> imu(nitems, 1), imc(nitems, 1);
  pool.parallel_for(nitems, 1, [&](int64_t lo, int64_t hi, int) {
    for (int64_t t = lo; t < hi; t++) {
      const LevelItem &it = items[t];
      const Graph &g = *gs[it.g];
      const int vb = vbase[it.g], wb = lcls[it.l];
      int64_t c = 0;
      int mu = 1, mc = 1;
      for (int q = it.q0; q < it.q1; q++) {
        const int v = g.tree_bfs[q], V = vb + v, d = g.depth[v];
        const int m = (int)(g.pos_hash[v + 1] - g.pos_hash[v]) - 1;
        int nt_node, cb, sc;
        const bool one = tiles_of(wb, m, d, nt_node, cb, sc);
        nt[V] = nt_node;
        ncb[V] = cb;
        nsc[V] = sc;
        c += nt_node;
        mu = std::max(mu, one ? m : std::min(m, sc));
        mc = std::max(mc, one ? d : std::min(d, cb));
      }
      icnt[t] = c;
      imu[t] = mu;
      imc[t] = mc;
    }
  });
  // tickets: forest level by forest level, graphs in order inside a level,
  // BFS order inside a graph's level; the items of a (graph, level) are
  // consecutive in BFS order
  std::vector<std::vector<int64_t>> cnt(K);
  for (int i = 0; i < K; i++) cnt[i].assign(std::max(0, (int)gs[i]->tree_hash.size() - 1), 0);
  for (int64_t t = 0; t < nitems; t++) cnt[items[t].g][items[t].l] += icnt[t];
  std::vector<std::vector<int64_t>> off(K);
  int64_t total = 0;
  for (int i = 0; i < K; i++) off[i].assign(cnt[i].size(), 0);
  for (int l = 0; l < nlev; l++)
    for (int i = 0; i < K; i++)
      if (l < (int)cnt[i].size()) {
        off[i][l] = total;
        total += cnt[i][l];
      }
  ntiles = total;
  GH_CHECK(ntiles < INT32_MAX, H2H_ERR_ARG, "too many fill tiles");
  max_u = *std::max_element(imu.begin(), imu.end());
  max_c = *std::max_element(imc.begin(), imc.end());
  std::vector<int64_t> ibase(nitems, 0);
  for (int64_t t = 0; t < nitems; t++) {
    const bool first = t == 0 || items[t - 1].g != items[t].g || items[t - 1].l != items[t].l;
    ibase[t] = first ? off[items[t].g][items[t].l] : ibase[t - 1] + icnt[t - 1];
  }
  mark("pass 1");
  // pass 2 (items in parallel): every node's first ticket; the ticket ->
  // node array is expanded on the device
  pool.parallel_for(nitems, 1, [&](int64_t lo, int64_t hi, int) {
    for (int64_t t = lo; t < hi; t++) {
      const LevelItem &it = items[t];
      const Graph &g = *gs[it.g];
      const int vb = vbase[it.g];
      int64_t tk = ibase[t];
      for (int q = it.q0; q < it.q1; q++) {
        const int V = vb + g.tree_bfs[q];
        nfirst[V] = (int)tk;
        tk += nt[V];
      }
    }
  });
  const int64_t need = ntiles + 4 * (int64_t)N + (int64_t)(ntiles + nlev + 1);  // + chunk table bound
  if (need > tiles_cap) {
    cudaFree(tiles);
    tiles = nullptr;
    tiles_cap = 0;
    tiles = dalloc<int>(need, work_bytes);
    tiles_cap = need;
  }
  mark("pass 2 and allocation");
  // chunks: forest levels in ticket order.  A level with many times more
  // tiles than resident warps hands them out in groups (fewer atomics on the
  // counter); any other level one by one, so its tiles spread over warps.
  // When every level goes one by one there is no table (chunk k = tile k).
  // the table is built on the device from one (first chunk, first ticket,
  // step) row per level
  std::vector<int64_t> ltab;  // per level: first chunk, first ticket, step
  {
    const int64_t warps = (int64_t)nsm * 64;
    std::vector<int64_t> lt(nlev, 0);
    std::vector<int> step(nlev, 1);
    int64_t nc = 0;
    bool grouped = false;
    for (int l = 0; l < nlev; l++) {
      for (int i = 0; i < K; i++)
        if (l < (int)cnt[i].size()) lt[l] += cnt[i][l];
      step[l] = (int)std::max<int64_t>(1, std::min<int64_t>(8, lt[l] / (8 * warps)));
      grouped |= step[l] > 1;
      nc += (lt[l] + step[l] - 1) / step[l];
    }
    nchunks = grouped ? nc : ntiles;
    if (grouped) {
      ltab.resize(3 * (size_t)nlev);
      int64_t t = 0, k = 0;
      for (int l = 0; l < nlev; l++) {
        ltab[3 * l] = k;
        ltab[3 * l + 1] = t;
        ltab[3 * l + 2] = step[l];
        k += (lt[l] + step[l] - 1) / step[l];
        t += lt[l];
      }
      GH_CHECK(t == ntiles && k == nc, H2H_ERR_STATE, "fill chunks do not cover the tiles");
    }
  }
  mark("chunks");
  GH_CUDA(cudaMemcpy(tiles + ntiles, host.data(), sizeof(int) * 4 * (int64_t)N, cudaMemcpyHostToDevice));
  if (!ltab.empty()) {
    int64_t *d_ltab = nullptr;
    GH_CUDA(cudaMalloc(&d_ltab, sizeof(int64_t) * ltab.size()));
    cudaError_t e = cudaMemcpy(d_ltab, ltab.data(), sizeof(int64_t) * ltab.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
      chunk_table_kernel<<<std::max(1, std::min<int>(nsm * 8, (int)((nchunks + 255) / 256))), 256>>>(
          d_ltab, nlev, nchunks, ntiles, tiles + ntiles + 4 * (int64_t)N);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    cudaFree(d_ltab);
    GH_CUDA(e);
  }
  expand_tiles_kernel<<<std::max(1, std::min(8192, (N * 32 + 255) / 256)), 256>>>(tiles + ntiles, tiles + ntiles + N,
                                                                                  tiles, N);
  GH_CUDA(cudaGetLastError());
  mark("uploads and expansion");
  const int smem_dyn = enable_max_dynamic_smem(fill_flow_kernel);
  // one staging slice per warp (4 warps per 128-thread block)
  smem = 4 * ((size_t)((max_u + 1) & ~1) * 16 + (size_t)((std::max(max_segs, 1) + 1) & ~1) * 8);
  GH_CHECK(smem <= (size_t)smem_dyn, H2H_ERR_DEVICE, "separator or tree too large for the fill staging");
  int per_sm = 0;
  GH_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fill_flow_kernel, threads, smem));
  per_sm = std::max(1, per_sm);
  blocks = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)nsm * per_sm, ntiles));
}

void FillPlan::enqueue(cudaStream_t s, cudaEvent_t *fill_ev) {
  gather_pos_weights_kernel<<<std::max(1, std::min(8192, (N * 32 + 255) / 256)), 256, 0, s>>>(
      pos_hash, pos_src, lists.off, lists.w, pos_w, N);
  GH_CUDA(cudaGetLastError());
  // rows start at INT_MAX: split tiles combine with atomicMin; padding stays defined
  fill_int_kernel<<<1024, 256, 0, s>>>(dis, dis_total, INT_MAX);
  GH_CUDA(cudaGetLastError());
  GH_CUDA(cudaMemsetAsync(done, 0, sizeof(int) * 2 * (int64_t)N, s));
  GH_CUDA(cudaMemsetAsync(next, 0, sizeof(int), s));
  GH_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
  FlowArgs A;
  A.tile_node = tiles;
  A.ntiles = (int)ntiles;
  A.node_first = tiles + ntiles;
  A.node_ntiles = tiles + ntiles + N;
  A.node_cb = tiles + ntiles + 2 * (int64_t)N;
  A.node_sc = tiles + ntiles + 3 * (int64_t)N;
  A.chunk_start = nchunks == ntiles ? nullptr : tiles + ntiles + 4 * (int64_t)N;
  A.nchunks = (int)nchunks;
  A.node_cnt = done + N;
  A.father = father;
  A.depth = depth;
  A.drow = drow;
  A.dis = dis;
  A.pos_hash = pos_hash;
  A.pos_id = pos_id;
  A.pos_pos = pos_pos;
  A.pos_w = pos_w;
  A.hld_row = hld_row;
  A.seg_off = seg_off;
  A.seg_top = seg_top;
  A.seg_pos = seg_pos;
  A.done = done;
  A.next = next;
  A.err = err;
  A.spin_limit = spin_limit_cycles();
  A.max_u = max_u;
  A.max_segs = std::max(max_segs, 1);
  A.scalar_cols = scalar_cols;
  A.trace_t = nullptr;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  GH_CUDA(cudaStreamIsCapturing(s, &cs));
  const bool capturing = cs != cudaStreamCaptureStatusNone;
  if (std::getenv("GPUH2H_TRACE") && !capturing) {
    if (!trace_t) GH_CUDA(cudaMalloc(&trace_t, sizeof(unsigned long long) * std::max(N, 1)));
    GH_CUDA(cudaMemsetAsync(trace_t, 0, sizeof(unsigned long long) * std::max(N, 1), s));
    A.trace_t = trace_t;
  }
  // inside a capture an event record becomes a graph node only when external
  auto record = [&](cudaEvent_t e) {
    GH_CUDA(capturing ? cudaEventRecordWithFlags(e, s, cudaEventRecordExternal) : cudaEventRecord(e, s));
  };
  if (fill_ev) record(fill_ev[0]);
  fill_flow_kernel<<<blocks, threads, smem, s>>>(A);
  GH_CUDA(cudaGetLastError());
  if (fill_ev) record(fill_ev[1]);
}

// With GPUH2H_TRACE: where the last fill's time went, from the nodes'
// publish times -- per forest level the time from the previous level's last
// publish to its own (levels overlap in the dataflow; the spans add up to
// the fill), summed per tile class, and the ten longest levels.
void FillPlan::trace_report() {
  if (!trace_t) return;
  GH_CUDA(cudaDeviceSynchronize());
  std::vector<unsigned long long> t(N);
  std::vector<int> dep(N);
  GH_CUDA(cudaMemcpy(t.data(), trace_t, sizeof(unsigned long long) * N, cudaMemcpyDeviceToHost));
  GH_CUDA(cudaMemcpy(dep.data(), depth, sizeof(int) * N, cudaMemcpyDeviceToHost));
  const std::vector<int> cls = level_classes();
  const int nlev = (int)cls.size();
  std::vector<unsigned long long> last(nlev, 0);
  std::vector<int64_t> width(nlev, 0);
  unsigned long long t0 = ~0ull;
  for (int v = 0; v < N; v++) {
    const int l = dep[v] - 1;
    if (l < 0 || l >= nlev || t[v] == 0) continue;
    last[l] = std::max(last[l], t[v]);
    width[l]++;
    t0 = std::min(t0, t[v]);
  }
  if (t0 == ~0ull) return;
  double by_cls[3] = {0, 0, 0};
  std::vector<std::pair<double, int>> spans;
  unsigned long long prev = t0;
  for (int l = 0; l < nlev; l++) {
    if (!last[l]) continue;
    const double us = last[l] > prev ? (last[l] - prev) / 1e3 : 0.0;
    by_cls[cls[l]] += us;
    spans.push_back({us, l});
    prev = std::max(prev, last[l]);
  }
  std::fprintf(stderr, "[gpuh2h] fill trace: first to last publish %.3f ms; narrow levels %.3f, wide %.3f, heavy %.3f ms\n",
               (prev - t0) / 1e6, by_cls[0] / 1e3, by_cls[1] / 1e3, by_cls[2] / 1e3);
  std::sort(spans.rbegin(), spans.rend());
  for (size_t k = 0; k < spans.size() && k < 10; k++)
    std::fprintf(stderr, "[gpuh2h] fill trace: level %d (class %d, %lld nodes): %.1f us\n", spans[k].second,
                 cls[spans[k].second], (long long)width[spans[k].second], spans[k].first);
}

void FillPlan::check_error() {
  GH_CUDA(cudaDeviceSynchronize());
  int kerr = 0;
  GH_CUDA(cudaMemcpy(&kerr, err, sizeof(int), cudaMemcpyDeviceToHost));
  GH_CHECK(kerr == 0, H2H_ERR_DEVICE, "label fill: a dependency wait ran out (error code " + std::to_string(kerr) + ")");
}

void FillPlan::attach(bool first) {
  std::vector<int64_t> f_drow, f_pos_hash;
  if (first) {
    f_drow.resize(N + 1);
    f_pos_hash.resize(N + 1);
    GH_CUDA(cudaMemcpy(f_drow.data(), drow, sizeof(int64_t) * (N + 1), cudaMemcpyDeviceToHost));
    GH_CUDA(cudaMemcpy(f_pos_hash.data(), pos_hash, sizeof(int64_t) * (N + 1), cudaMemcpyDeviceToHost));
  }
  for (size_t i = 0; i < gs.size(); i++) {
    Graph &g = *gs[i];
    DeviceIndex &D = g.dev;
    const int vb = vbase[i];
    if (first) {
      D.release_labels();
      D.n = g.n;
      D.keep = storage;
      D.depth = depth + vb;
      D.father = father + vb;
      D.drow = drow + vb;
      D.pos_hash = pos_hash + vb;
      D.pos_pos = pos_pos;
      D.pos_id = pos_id;
      D.dis = dis;
      D.pos = f_pos_hash[vb + g.n] - f_pos_hash[vb];
      D.pos_base = f_pos_hash[vb];
      D.dis_padded = f_drow[vb + g.n] - f_drow[vb];
      D.err = dalloc_owned<int>(1, D);
      D.bytes += (int64_t)(g.n + 1) * 16 + (int64_t)g.n * 8 + D.pos * 8 + D.dis_padded * 4;
      g.drow_host.assign(f_drow.begin() + vb, f_drow.begin() + vb + g.n + 1);
    }
    g.max_label = -1;  // the largest label is computed when it is first asked for (label_max)
  }
}

// The largest finite label of g's rows, computed on first request (a pass
// over the labels, about 20 ms for the 6.26M-vertex graph's 115 GB) and
// kept; a rebuild resets it.
int64_t label_max(const Graph &gc) {
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  Graph &g = const_cast<Graph &>(gc);
  if (g.max_label >= 0 || !g.dev.dis || !g.dev.err) return std::max<int64_t>(g.max_label, 0);
  const int64_t r0 = g.drow_host.empty() ? 0 : g.drow_host[0];
  const int64_t r1 = g.drow_host.empty() ? g.dev.dis_padded : g.drow_host[g.n];
  int dev = 0, nsm = 1;
  GH_CUDA(cudaGetDevice(&dev));
  GH_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  GH_CUDA(cudaMemset(g.dev.err, 0, sizeof(int)));
  max_label_kernel<<<std::max(1, std::min<int>(nsm * 4, (int)((r1 - r0 + 255) / 256))), 256>>>(
      g.dev.dis + r0, r1 - r0, g.dev.err);
  GH_CUDA(cudaGetLastError());
  int mx = 0;
  GH_CUDA(cudaMemcpy(&mx, g.dev.err, sizeof(int), cudaMemcpyDeviceToHost));
  GH_CUDA(cudaMemset(g.dev.err, 0, sizeof(int)));
  g.max_label = mx;
  return mx;
}

// Autotuner of the forest fill's tile shapes.  Coordinate descent over the
// (level width x separator size) buckets that hold nodes: for each bucket in
// turn, first the one-tile threshold, then the column-block x separator-chunk
// split, each candidate timed as a whole fill (best of two runs) with the
// other buckets held; a candidate replaces the incumbent only when it is 2%
// faster.  Any policy gives the same labels: only the schedule changes.
std::string tile_policy_tune(FillPlan &plan, cudaStream_t s, int rounds) {
  bool used[TilePolicy::kWidth][TilePolicy::kSep] = {};
  {
    const std::vector<int> lcls = plan.level_classes();
    for (const Graph *g : plan.gs)
      for (int l = 0; l + 1 < (int)g->tree_hash.size(); l++)
        for (int q = g->tree_hash[l]; q < g->tree_hash[l + 1]; q++) {
          const int v = g->tree_bfs[q];
          used[lcls[l]][TilePolicy::sep_bucket((int)(g->pos_hash[v + 1] - g->pos_hash[v]) - 1)] = true;
        }
  }
  cudaEvent_t ev[2];
  GH_CUDA(cudaEventCreate(&ev[0]));
  GH_CUDA(cudaEventCreate(&ev[1]));
  auto time_policy = [&](const TilePolicy &p) -> float {
    try {
      plan.build_tiles(p);
    } catch (const Error &) {
      return 1e30f;  // staging does not fit: not a candidate
    }
    float best = 1e30f;
    for (int rep = 0; rep < 2; rep++) {
      plan.enqueue(s, ev);
      plan.check_error();
      float ms = 0;
      GH_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
      best = std::min(best, ms);
    }
    return best;
  };
  static const int kSmall[] = {0, 1 << 8, 1 << 10, 1 << 12, 1 << 14, 1 << 16};
  static const int kShape[][2] = {{32, 4}, {32, 8}, {32, 16}, {32, 32}, {64, 32}, {128, 256}};
  TilePolicy best = plan.policy;
  float best_ms = 0;
  try {
    best_ms = time_policy(best);
    for (int r = 0; r < rounds; r++)
      for (int wb = 0; wb < TilePolicy::kWidth; wb++)
        for (int sb = 0; sb < TilePolicy::kSep; sb++) {
          if (!used[wb][sb]) continue;
          for (int sw : kSmall) {
            if (sw == best.small_work[wb][sb]) continue;
            TilePolicy p = best;
            p.small_work[wb][sb] = sw;
            const float t = time_policy(p);
            if (t < best_ms * 0.98f) { best = p; best_ms = t; }
          }
          for (const auto &sh : kShape) {
            if (sh[0] == best.col_block[wb][sb] && sh[1] == best.sep_chunk[wb][sb]) continue;
            TilePolicy p = best;
            p.col_block[wb][sb] = sh[0];
            p.sep_chunk[wb][sb] = sh[1];
            const float t = time_policy(p);
            if (t < best_ms * 0.98f) { best = p; best_ms = t; }
          }
        }
    time_policy(best);  // leaves the tiles and the labels of the chosen policy
  } catch (...) {
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    throw;
  }
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  return best.str();
}

void fill_labels_gpu(Graph &g) {
  Clock clk;
  const int n = g.n;
  DeviceIndex &D = g.dev;
  // L4 runs as a dataflow over the tree; L3 (order-dependent, as shipped)
  // keeps the level-synchronous kernel that applies the reference's order.
  const bool flow = !uses_level_fill(g);
  if (flow) {
    TilePolicy pol = TilePolicy::for_height(g.tree_height);
    if (const char *e = std::getenv("GPUH2H_TILE_POLICY"))
      GH_CHECK(pol.parse(e), H2H_ERR_ARG, "GPUH2H_TILE_POLICY: expected 12 entries small_work/col_block/sep_chunk");
    FillPlan plan({&g}, pol, D.lists);
    GH_CUDA(cudaDeviceSynchronize());
    g.t.translate_labels = clk.us();
    clk.reset();
    cudaEvent_t ev[2];
    GH_CUDA(cudaEventCreate(&ev[0]));
    GH_CUDA(cudaEventCreate(&ev[1]));
    float ms = 0;
    try {
      plan.enqueue(0, ev);
      plan.check_error();
      plan.trace_report();
      GH_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
    } catch (...) {
      cudaEventDestroy(ev[0]);
      cudaEventDestroy(ev[1]);
      throw;
    }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    g.t.fill_gpu = (long long)(ms * 1000.0f);
    Clock tail;  // the per-graph view and the plan's work buffers count with the plan's host time
    plan.attach(true);
    plan.release_work();
    g.t.translate_labels += tail.us();
    return;
  }
  D.release_labels();
  D.n = n;
  D.pos_base = 0;
  // padded row offsets
  std::vector<int64_t> drow(n + 1, 0);
  for (int v = 0; v < n; v++) drow[v + 1] = drow[v] + ((g.depth[v] + 3) & ~3);
  D.dis_padded = drow[n];
  D.pos = g.pos_hash[n];
  const int nlev = (int)g.tree_hash.size() - 1;
  int64_t tmp_bytes = 0;
  D.drow = dalloc_owned<int64_t>(n + 1, D);
  D.dis = dalloc_owned<int>(D.dis_padded, D);
  D.pos_hash = dalloc_owned<int64_t>(n + 1, D);
  D.pos_pos = dalloc_owned<int>(D.pos, D);
  D.pos_id = dalloc_owned<int>(D.pos, D);
  D.father = dalloc_owned<int>(n, D);
  D.depth = dalloc_owned<int>(n, D);
  D.err = dalloc_owned<int>(1, D);
  int *d_pos_w = nullptr, *d_nodes = nullptr, *d_aux = nullptr;
  int64_t *d_chain[2] = {nullptr, nullptr};
  auto cleanup = [&]() {
    cudaFree(d_pos_w); cudaFree(d_nodes); cudaFree(d_aux); cudaFree(d_chain[0]); cudaFree(d_chain[1]);
  };
  try {
    d_pos_w = dalloc<int>(D.pos, tmp_bytes);
    d_nodes = dalloc<int>(n, tmp_bytes);
    d_aux = dalloc<int>(n, tmp_bytes);  // index of the node within its level
    std::vector<int> aux(n, 0);
    int64_t chain_max = 1;
    for (int l = 0; l < nlev; l++)
      for (int i = g.tree_hash[l]; i < g.tree_hash[l + 1]; i++) aux[g.tree_bfs[i]] = i - g.tree_hash[l];
    for (int l = 0; l < nlev; l++)
      chain_max = std::max<int64_t>(chain_max, (int64_t)(g.tree_hash[l + 1] - g.tree_hash[l]) * l);
    d_chain[0] = dalloc<int64_t>(chain_max, tmp_bytes);
    d_chain[1] = dalloc<int64_t>(chain_max, tmp_bytes);
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
    init_rows_kernel<<<std::max(1, std::min(65535, (n * 32 + 255) / 256)), 256>>>(D.drow, D.depth, D.pos_hash,
                                                                                  D.pos_pos, d_pos_w, D.dis, n);
    GH_CUDA(cudaGetLastError());
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
    GH_CUDA(cudaEventRecord(e1));
    GH_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    GH_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    g.t.fill_gpu = (long long)(ms * 1000.0f);
    g.max_label = -1;  // computed on first request (label_max)
  } catch (...) {
    cleanup();
    throw;
  }
  cleanup();
  g.drow_host.swap(drow);
}

// Copies the filled labels back into the reference's unpadded layout.
void upload_labels(Graph &g, const std::vector<int> &dis, const std::vector<int> &pos_id,
                   const std::vector<int> &pos_pos) {
  const int n = g.n;
  DeviceIndex &D = g.dev;
  D.release_labels();
  D.n = n;
  D.pos_base = 0;
  std::vector<int64_t> drow(n + 1, 0);
  for (int v = 0; v < n; v++) drow[v + 1] = drow[v] + ((g.depth[v] + 3) & ~3);
  D.dis_padded = drow[n];
  D.pos = g.pos_hash[n];
  D.drow = dalloc_owned<int64_t>(n + 1, D);
  D.dis = dalloc_owned<int>(D.dis_padded, D);
  D.pos_hash = dalloc_owned<int64_t>(n + 1, D);
  D.pos_pos = dalloc_owned<int>(D.pos, D);
  D.pos_id = dalloc_owned<int>(D.pos, D);
  D.father = dalloc_owned<int>(n, D);
  D.depth = dalloc_owned<int>(n, D);
  D.err = dalloc_owned<int>(1, D);
  GH_CUDA(cudaMemcpy(D.drow, drow.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice));
  GH_CUDA(cudaMemcpy(D.pos_hash, g.pos_hash.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice));
  if (D.pos) {
    GH_CUDA(cudaMemcpy(D.pos_pos, pos_pos.data(), sizeof(int) * D.pos, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(D.pos_id, pos_id.data(), sizeof(int) * D.pos, cudaMemcpyHostToDevice));
  }
  GH_CUDA(cudaMemcpy(D.father, g.father.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
  GH_CUDA(cudaMemcpy(D.depth, g.depth.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
  GH_CUDA(cudaMemset(D.err, 0, sizeof(int)));
  // rows into the padded layout through a page-locked staging buffer of at
  // most 64 Mi entries (padding entries are INT_MAX, as the fill leaves them)
  const int64_t kStage = int64_t(1) << 26;
  int *stage = nullptr;
  GH_CUDA(cudaMallocHost(&stage, sizeof(int) * std::min<int64_t>(std::max<int64_t>(D.dis_padded, 1), kStage)));
  try {
    int v = 0;
    while (v < n) {
      const int64_t p0 = drow[v];
      int w = v;
      while (w < n && drow[w + 1] - p0 <= kStage) w++;
      GH_CHECK(w > v, H2H_ERR_ARG, "a label row longer than the upload staging");
      for (int u = v; u < w; u++) {
        int *row = stage + (drow[u] - p0);
        std::copy(dis.begin() + g.dis_hash[u], dis.begin() + g.dis_hash[u] + g.depth[u], row);
        for (int64_t j = g.depth[u]; j < drow[u + 1] - drow[u]; j++) row[j] = INT_MAX;
      }
      GH_CUDA(cudaMemcpy(D.dis + p0, stage, sizeof(int) * (drow[w] - p0), cudaMemcpyHostToDevice));
      v = w;
    }
  } catch (...) {
    cudaFreeHost(stage);
    throw;
  }
  cudaFreeHost(stage);
  g.drow_host.swap(drow);
}

// Runs one of the reference's GPU fill mappings (mapping 0: a thread per
// (v, u) pair, plain_fill_level_kernel; 1: a thread per node,
// plain_node_fill_kernel) on the built graph into a scratch copy of the rows
// and compares it with the built labels.  The device time of the per-level
// launches and synchronisations goes to *ms; *mismatches receives the number
// of differing entries.
void fill_labels_plain(const Graph &g, int mapping, double *ms, int64_t *mismatches) {
  GH_CHECK(mapping == 0 || mapping == 1, H2H_ERR_ARG, "mapping must be 0 (pair per thread) or 1 (node per thread)");
  GH_CHECK(g.labelled && g.label_mode == H2H_LABEL_L4, H2H_ERR_STATE, "needs built L4 labels");
  const DeviceIndex &D = g.dev;
  const int n = g.n;
  const int64_t np = g.pos_hash[n];
  std::vector<int> pid(np), ppos(np);
  download_positions(g, pid.data(), ppos.data());
  // (v, k) pairs per tree level, k over v's entries other than v itself
  std::vector<int> pv;
  std::vector<int64_t> pk;
  std::vector<int64_t> lvl_off{0};
  const int nlev = (int)g.tree_hash.size() - 1;
  for (int l = 0; l < nlev; l++) {
    for (int q = g.tree_hash[l]; q < g.tree_hash[l + 1]; q++) {
      const int v = g.tree_bfs[q];
      for (int64_t k = g.pos_hash[v]; k < g.pos_hash[v + 1]; k++)
        if (pid[k] != v) { pv.push_back(v); pk.push_back(k); }
    }
    lvl_off.push_back((int64_t)pv.size());
  }
  int64_t tmp = 0;
  int *d_dis = nullptr, *d_pv = nullptr, *d_w = nullptr;
  int64_t *d_pk = nullptr, *d_drow = nullptr;
  int *d_depth = nullptr, *d_father = nullptr, *d_pos_pos = nullptr, *d_pos_id = nullptr, *d_bfs = nullptr;
  int64_t *d_pos_hash = nullptr;
  unsigned long long *d_bad = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  auto cleanup = [&]() {
    cudaFree(d_dis); cudaFree(d_pv); cudaFree(d_w); cudaFree(d_pk); cudaFree(d_drow); cudaFree(d_depth);
    cudaFree(d_father); cudaFree(d_pos_pos); cudaFree(d_pos_id); cudaFree(d_pos_hash); cudaFree(d_bad);
    cudaFree(d_bfs);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
  };
  try {
    const int64_t rows = g.drow_host[n] - g.drow_host[0];
    std::vector<int64_t> drow(n + 1);
    for (int v = 0; v <= n; v++) drow[v] = g.drow_host[v] - g.drow_host[0];
    std::vector<int> pw(np);
    {
      // shortcut weights per position entry from the device lists
      std::vector<int> xid(g.x_off[n]), xw(g.x_off[n]);
      if (g.x_off[n]) {
        GH_CUDA(cudaMemcpy(xid.data(), D.lists.id + D.x_base, sizeof(int) * g.x_off[n], cudaMemcpyDeviceToHost));
        GH_CUDA(cudaMemcpy(xw.data(), D.lists.w + D.x_base, sizeof(int) * g.x_off[n], cudaMemcpyDeviceToHost));
      }
      for (int v = 0; v < n; v++)  // lists are sorted by id: binary search
        for (int64_t k = g.pos_hash[v]; k < g.pos_hash[v + 1]; k++) {
          pw[k] = 0;
          if (pid[k] == v) continue;
          const auto b = xid.begin() + g.x_off[v], e = xid.begin() + g.x_off[v + 1];
          const auto it = std::lower_bound(b, e, pid[k] + D.id_base);
          if (it != e && *it == pid[k] + D.id_base) pw[k] = xw[it - xid.begin()];
        }
    }
    d_dis = dalloc<int>(rows, tmp);
    d_pv = dalloc<int>(std::max<size_t>(pv.size(), 1), tmp);
    d_pk = dalloc<int64_t>(std::max<size_t>(pk.size(), 1), tmp);
    d_drow = dalloc<int64_t>(n + 1, tmp);
    d_depth = dalloc<int>(n, tmp);
    d_father = dalloc<int>(n, tmp);
    d_pos_pos = dalloc<int>(std::max<int64_t>(np, 1), tmp);
    d_pos_id = dalloc<int>(std::max<int64_t>(np, 1), tmp);
    d_w = dalloc<int>(std::max<int64_t>(np, 1), tmp);
    d_pos_hash = dalloc<int64_t>(n + 1, tmp);
    d_bad = dalloc<unsigned long long>(1, tmp);
    d_bfs = dalloc<int>(std::max<size_t>(g.tree_bfs.size(), 1), tmp);
    if (!g.tree_bfs.empty())
      GH_CUDA(cudaMemcpy(d_bfs, g.tree_bfs.data(), sizeof(int) * g.tree_bfs.size(), cudaMemcpyHostToDevice));
    if (!pv.empty()) {
      GH_CUDA(cudaMemcpy(d_pv, pv.data(), sizeof(int) * pv.size(), cudaMemcpyHostToDevice));
      GH_CUDA(cudaMemcpy(d_pk, pk.data(), sizeof(int64_t) * pk.size(), cudaMemcpyHostToDevice));
    }
    GH_CUDA(cudaMemcpy(d_drow, drow.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_depth, g.depth.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_father, g.father.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_pos_pos, ppos.data(), sizeof(int) * np, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_pos_id, pid.data(), sizeof(int) * np, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_w, pw.data(), sizeof(int) * np, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_pos_hash, g.pos_hash.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemset(d_bad, 0, sizeof(unsigned long long)));
    GH_CUDA(cudaEventCreate(&e0));
    GH_CUDA(cudaEventCreate(&e1));
    GH_CUDA(cudaEventRecord(e0));
    // mallocH2HLabel_noHub's initial rows, then the levels in order
    init_rows_kernel<<<std::max(1, std::min(65535, (n * 32 + 255) / 256)), 256>>>(d_drow, d_depth, d_pos_hash,
                                                                                  d_pos_pos, d_w, d_dis, n);
    GH_CUDA(cudaGetLastError());
    GH_CUDA(cudaDeviceSynchronize());
    for (int l = 1; l < nlev; l++) {
      if (mapping == 1) {
        const int cnt = g.tree_hash[l + 1] - g.tree_hash[l];
        if (cnt == 0) continue;
        plain_node_fill_kernel<<<(cnt + 255) / 256, 256>>>(d_bfs + g.tree_hash[l], cnt, d_drow, d_depth, d_father,
                                                            d_pos_hash, d_pos_pos, d_pos_id, d_w, d_dis);
      } else {
        const int64_t a = lvl_off[l], b = lvl_off[l + 1];
        if (b == a) continue;
        const int cnt = (int)(b - a);
        plain_fill_level_kernel<<<(cnt + 255) / 256, 256>>>(d_pv + a, d_pk + a, cnt, d_drow, d_depth, d_father,
                                                             d_pos_pos, d_pos_id, d_w, d_dis);
      }
      GH_CUDA(cudaGetLastError());
      GH_CUDA(cudaDeviceSynchronize());
    }
    GH_CUDA(cudaEventRecord(e1));
    GH_CUDA(cudaEventSynchronize(e1));
    float t = 0;
    GH_CUDA(cudaEventElapsedTime(&t, e0, e1));
    if (ms) *ms = t;
    count_mismatch_kernel<<<1024, 256>>>(d_dis, D.dis + g.drow_host[0], rows, d_bad);
    GH_CUDA(cudaGetLastError());
    unsigned long long bad = 0;
    GH_CUDA(cudaMemcpy(&bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost));
    if (mismatches) *mismatches = (int64_t)bad;
  } catch (...) {
    cleanup();
    throw;
  }
  cleanup();
}

// Position lists in the reference layout with graph-local ids: the host
// copies (L3) or the graph's range of the device arrays (L4).
void download_positions(const Graph &g, int *pos_id, int *pos_pos) {
  const int64_t np = g.pos_hash.empty() ? 0 : g.pos_hash[g.n];
  if ((int64_t)g.pos_id.size() == np && np) {
    if (pos_id) std::copy(g.pos_id.begin(), g.pos_id.end(), pos_id);
    if (pos_pos) std::copy(g.pos_pos.begin(), g.pos_pos.end(), pos_pos);
    return;
  }
  GH_CHECK(g.dev.pos_id && g.dev.pos_pos && g.dev.pos == np, H2H_ERR_STATE, "position lists not on the device");
  if (!np) return;
  if (pos_pos) GH_CUDA(cudaMemcpy(pos_pos, g.dev.pos_pos + g.dev.pos_base, sizeof(int) * np, cudaMemcpyDeviceToHost));
  if (pos_id) {
    GH_CUDA(cudaMemcpy(pos_id, g.dev.pos_id + g.dev.pos_base, sizeof(int) * np, cudaMemcpyDeviceToHost));
    if (g.dev.id_base)
      for (int64_t k = 0; k < np; k++) pos_id[k] -= g.dev.id_base;
  }
}

// The graph's rows are [drow_host[0], drow_host[n]) of the device array
// (a batch's forest array holds other graphs' rows around them).
void download_labels(const Graph &g, int *dis_out) {
  const int n = g.n;
  const int64_t r0 = g.drow_host[0], r1 = g.drow_host[n];
  GH_CHECK(r1 - r0 == g.dev.dis_padded, H2H_ERR_STATE, "label rows and device index disagree");
  std::vector<int> tmp(r1 - r0);
  GH_CUDA(cudaMemcpy(tmp.data(), g.dev.dis + r0, sizeof(int) * (r1 - r0), cudaMemcpyDeviceToHost));
  for (int v = 0; v < n; v++)
    std::copy(tmp.begin() + (g.drow_host[v] - r0), tmp.begin() + (g.drow_host[v] - r0) + g.depth[v],
              dis_out + g.dis_hash[v]);
}

}  // namespace gh
