// query.cu -- batched H2H distance queries on the device-resident index, the
// work of H2HQuery_UsingLCA_D_noHub / H2HQuery_noLCA_D_noHub
// (kernel_functions.cu:1143-1296) and of the host single-pair queries
// (Query.cu:108-151).
//
// LCA by range minimum over the Euler tour: l, r = sorted firstAppeare,
// k = floor(log2(r - l + 1)) (31 - clz, the integer equal of the reference's
// (int)log2((double)...)), two sparse-table ids, the shallower wins.  Then:
//   LCA mode:   min over p in pos(LCA) of dis[x][p] + dis[y][p]
//   noLCA mode: min over j < depth(LCA) of dis[x][j] + dis[y][j]
// x == y answers 0 as in the reference.
#include <algorithm>
#include <climits>

#include "graph.h"

namespace gh {

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

struct QArgs {
  const int *x, *y;
  int *out;
  int64_t n;
  int nv;  // vertices; ids outside [0, nv) answer -1 without touching the index
  const int *first, *depth;
  const int64_t *rmq_hash;
  const int *rmq_id;
  const int64_t *pos_hash;
  const int *pos_pos;
  const int64_t *drow;
  const int *dis;
  int *bad;  // set to 1 when a pair holds an id outside [0, nv)
};

// G lanes cooperate on one query.  Every lane of the group resolves the LCA
// (same addresses, one transaction per load), then the lanes split the min.
template <int G, bool LCA_MODE>
__global__ void query_kernel(QArgs A) {
  const int lane = threadIdx.x & (G - 1);
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
  const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / G;
  for (int64_t q = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G; q < A.n; q += groups) {
    const int a = __ldg(A.x + q), b = __ldg(A.y + q);
    const bool valid = (unsigned)a < (unsigned)A.nv && (unsigned)b < (unsigned)A.nv;
    int res = !valid ? -1 : (a == b ? 0 : INT_MAX);
    if (!valid && lane == 0) atomicExch(A.bad, 1);
    if (valid && a != b) {
      const int fa = __ldg(A.first + a), fb = __ldg(A.first + b);
      const int l = min(fa, fb), r = max(fa, fb);
      const int k = 31 - __clz(r - l + 1);
      const int i1 = __ldg(A.rmq_id + __ldg(A.rmq_hash + l) + k);
      const int i2 = __ldg(A.rmq_id + __ldg(A.rmq_hash + r - (1 << k) + 1) + k);
      const int d1 = __ldg(A.depth + i1), d2 = __ldg(A.depth + i2);
      const int *rx = A.dis + __ldg(A.drow + a);
      const int *ry = A.dis + __ldg(A.drow + b);
      if (LCA_MODE) {
        const int lca = d1 <= d2 ? i1 : i2;
        const int64_t pb = __ldg(A.pos_hash + lca), pe = __ldg(A.pos_hash + lca + 1);
        for (int64_t t = pb + lane; t < pe; t += G) {
          const int p = __ldg(A.pos_pos + t);
          res = min(res, __ldg(rx + p) + __ldg(ry + p));
        }
      } else {
        const int dl = min(d1, d2);
        for (int j = lane; j < dl; j += G) res = min(res, __ldg(rx + j) + __ldg(ry + j));
      }
    }
    if (G > 1) {
      for (int o = G >> 1; o > 0; o >>= 1) res = min(res, __shfl_down_sync(gmask, res, o, G));
    }
    if (lane == 0) A.out[q] = res;
  }
}

// Warp-tiled batch: a warp owns TILE consecutive queries.  Phase 1: lane i
// < TILE resolves query i (ids, LCA through the sparse table, row bases, the
// position range) -- TILE independent dependent-load chains in flight.
// Phase 2: the whole warp walks each query's positions in turn with 4-way
// unrolled loads (position, then the two label entries) and a warp min
// (__reduce_min_sync); the owning lane keeps the answer and the answers
// leave in one coalesced store.  TILE = 32 for large batches; a batch too
// small to fill the GPU's resident warps takes a narrower tile, so more
// warps share its walks and the batch finishes sooner.
template <bool LCA_MODE, int TILE>
__global__ void __launch_bounds__(256, 8) query_tile_kernel(QArgs A) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t tile = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; tile * TILE < A.n; tile += nwarps) {
    const int64_t q = tile * TILE + lane;
    int res = INT_MAX, len = 0;
    int64_t pb = 0, bx = 0, by = 0;
    if (lane < TILE && q < A.n) {
      const int a = __ldg(A.x + q), b = __ldg(A.y + q);
      const bool valid = (unsigned)a < (unsigned)A.nv && (unsigned)b < (unsigned)A.nv;
      if (!valid) {
        res = -1;
        atomicExch(A.bad, 1);
      } else if (a == b) {
        res = 0;
      } else {
        const int fa = __ldg(A.first + a), fb = __ldg(A.first + b);
        bx = __ldg(A.drow + a);
        by = __ldg(A.drow + b);
        const int l = min(fa, fb), r = max(fa, fb);
        const int k = 31 - __clz(r - l + 1);
        const int i1 = __ldg(A.rmq_id + __ldg(A.rmq_hash + l) + k);
        const int i2 = __ldg(A.rmq_id + __ldg(A.rmq_hash + r - (1 << k) + 1) + k);
        const int d1 = __ldg(A.depth + i1), d2 = __ldg(A.depth + i2);
        if (LCA_MODE) {
          const int lca = d1 <= d2 ? i1 : i2;
          pb = __ldg(A.pos_hash + lca);
          len = (int)(__ldg(A.pos_hash + lca + 1) - pb);
        } else {
          len = min(d1, d2);
        }
      }
    }
#pragma unroll 1
    for (int s = 0; s < TILE; s++) {
      const int L = __shfl_sync(0xffffffffu, len, s);
      if (L == 0) continue;
      const int64_t PB = __shfl_sync(0xffffffffu, pb, s);
      const int *rx = A.dis + __shfl_sync(0xffffffffu, bx, s);
      const int *ry = A.dis + __shfl_sync(0xffffffffu, by, s);
      int m = INT_MAX;
      for (int t0 = 0; t0 < L; t0 += 128) {
        int p[4];
        bool ok[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int t = t0 + (u << 5) + lane;
          ok[u] = t < L;
          p[u] = ok[u] ? (LCA_MODE ? __ldg(A.pos_pos + PB + t) : t) : 0;
        }
        int xv[4], yv[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          xv[u] = ok[u] ? __ldg(rx + p[u]) : 0;
          yv[u] = ok[u] ? __ldg(ry + p[u]) : 0;
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
          if (ok[u]) m = min(m, xv[u] + yv[u]);
      }
      m = __reduce_min_sync(0xffffffffu, m);
      if (lane == s) res = m;
    }
    if (lane < TILE && q < A.n) A.out[q] = res;
  }
}

}  // namespace

// ---- compacted sparse table of the Euler tour (makeOULAAndRMQ,
// TreeStructure.cu:500-572), built on the GPU.  Row i of the table holds the
// shallowest-node ids of the windows [i, i + 2^j) for every j with
// i + 2^j - 1 < L, so it has floor(log2(L - i)) + 1 entries and starts at
//   RMQHash[i] = S(L) - S(L - i),  S(x) = sum_{t=1..x} (floor(log2 t) + 1)
//              = (k - 1) 2^k + 1 + (x - 2^k + 1)(k + 1),  k = floor(log2 x).
// Level j combines two level-(j-1) windows, the left one winning ties
// (depth <=, TreeStructure.cu:528); one launch per level covers the Euler
// tours of every graph given.
namespace {

struct RmqJob {
  const int *eid;    // Euler tour, vertex per position
  const int *depth;  // depth per vertex
  int64_t *hash;     // RMQHash [L]
  int *id;           // RMQ_ID  [S(L)]
  int64_t L;
};

__host__ __device__ inline int64_t rmq_prefix(int64_t x) {
  if (x <= 0) return 0;
  int k = 0;
  while ((int64_t(2) << k) <= x) k++;
  return ((int64_t)(k - 1) << k) + 1 + (x - (int64_t(1) << k) + 1) * (k + 1);
}

__device__ __forceinline__ int job_of(const int64_t *off, int njobs, int64_t p) {
  int lo = 0, hi = njobs - 1;  // last job with off[job] <= p
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= p) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void rmq_hash_kernel(const RmqJob *jobs, const int64_t *off, int njobs, int64_t total) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < total; p += (int64_t)gridDim.x * blockDim.x) {
    const int g = job_of(off, njobs, p);
    const int64_t i = p - off[g], L = jobs[g].L;
    jobs[g].hash[i] = rmq_prefix(L) - rmq_prefix(L - i);
  }
}

__global__ void rmq_level_kernel(const RmqJob *jobs, const int64_t *off, int njobs, int64_t total, int j) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < total; p += (int64_t)gridDim.x * blockDim.x) {
    const int g = job_of(off, njobs, p);
    const RmqJob J = jobs[g];
    const int64_t i = p - off[g];
    if (j == 0) {
      J.id[J.hash[i]] = J.eid[i];
    } else if (i + (int64_t(1) << j) - 1 < J.L) {
      const int a = J.id[J.hash[i] + j - 1];
      const int c = J.id[J.hash[i + (int64_t(1) << (j - 1))] + j - 1];
      J.id[J.hash[i] + j] = __ldg(J.depth + a) <= __ldg(J.depth + c) ? a : c;
    }
  }
}

}  // namespace

void build_rmq_gpu(const std::vector<Graph *> &gs) {
  Clock clk;
  const int K = (int)gs.size();
  std::vector<int64_t> off(K + 1, 0), voff(K + 1, 0);
  int levels = 0;
  for (int i = 0; i < K; i++) {
    const Graph &g = *gs[i];
    GH_CHECK((int64_t)g.euler_id.size() == g.euler_n && g.euler_n == 2 * (int64_t)g.n - 1, H2H_ERR_STATE,
             "Euler tour missing");
    off[i + 1] = off[i] + g.euler_n;
    voff[i + 1] = voff[i] + g.n;
    levels = std::max(levels, ilog2_floor(g.euler_n));
  }
  const int64_t total = off[K];
  int64_t tmp = 0;
  int *d_eid = nullptr, *d_depth = nullptr;
  int64_t *d_off = nullptr;
  RmqJob *d_jobs = nullptr;
  auto cleanup = [&]() { cudaFree(d_eid); cudaFree(d_depth); cudaFree(d_off); cudaFree(d_jobs); };
  try {
    d_eid = dalloc<int>(total, tmp);
    d_depth = dalloc<int>(voff[K], tmp);
    d_off = dalloc<int64_t>(K + 1, tmp);
    d_jobs = dalloc<RmqJob>(K, tmp);
    std::vector<RmqJob> jobs(K);
    for (int i = 0; i < K; i++) {
      Graph &g = *gs[i];
      DeviceIndex &D = g.dev;
      for (void *p : D.owned_rmq) cudaFree(p);
      D.owned_rmq.clear();
      D.bytes -= D.rmq_bytes;
      D.rmq_bytes = 0;
      D.euler = g.euler_n;
      g.rmq_total = rmq_prefix(g.euler_n);
      D.rmq = g.rmq_total;
      D.first = dalloc<int>(g.n, D.rmq_bytes);
      D.owned_rmq.push_back(D.first);
      D.rmq_hash = dalloc<int64_t>(D.euler, D.rmq_bytes);
      D.owned_rmq.push_back(D.rmq_hash);
      D.rmq_id = dalloc<int>(D.rmq, D.rmq_bytes);
      D.owned_rmq.push_back(D.rmq_id);
      D.bytes += D.rmq_bytes;
      GH_CUDA(cudaMemcpy(D.first, g.first.data(), sizeof(int) * g.n, cudaMemcpyHostToDevice));
      GH_CUDA(cudaMemcpy(d_eid + off[i], g.euler_id.data(), sizeof(int) * g.euler_n, cudaMemcpyHostToDevice));
      GH_CUDA(cudaMemcpy(d_depth + voff[i], g.depth.data(), sizeof(int) * g.n, cudaMemcpyHostToDevice));
      jobs[i] = RmqJob{d_eid + off[i], d_depth + voff[i], D.rmq_hash, D.rmq_id, g.euler_n};
    }
    GH_CUDA(cudaMemcpy(d_jobs, jobs.data(), sizeof(RmqJob) * K, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_off, off.data(), sizeof(int64_t) * (K + 1), cudaMemcpyHostToDevice));
    int dev = 0, nsm = 0;
    GH_CUDA(cudaGetDevice(&dev));
    GH_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)nsm * 8, (total + 255) / 256));
    rmq_hash_kernel<<<blocks, 256>>>(d_jobs, d_off, K, total);
    GH_CUDA(cudaGetLastError());
    for (int j = 0; j <= levels; j++) {
      rmq_level_kernel<<<blocks, 256>>>(d_jobs, d_off, K, total, j);
      GH_CUDA(cudaGetLastError());
    }
    GH_CUDA(cudaDeviceSynchronize());
  } catch (...) {
    cleanup();
    throw;
  }
  cleanup();
  const long long us = clk.us();
  for (Graph *g : gs) {
    std::vector<int>().swap(g->euler_id);
    g->t.tree += us / K;
  }
}

void upload_rmq(Graph &g, const std::vector<int64_t> &rmq_hash, const std::vector<int> &rmq_id) {
  DeviceIndex &D = g.dev;
  for (void *p : D.owned_rmq) cudaFree(p);
  D.owned_rmq.clear();
  D.bytes -= D.rmq_bytes;
  D.rmq_bytes = 0;
  D.euler = g.euler_n;
  D.rmq = g.rmq_total;
  D.first = dalloc<int>(g.n, D.rmq_bytes);
  D.owned_rmq.push_back(D.first);
  D.rmq_hash = dalloc<int64_t>(D.euler, D.rmq_bytes);
  D.owned_rmq.push_back(D.rmq_hash);
  D.rmq_id = dalloc<int>(D.rmq, D.rmq_bytes);
  D.owned_rmq.push_back(D.rmq_id);
  D.bytes += D.rmq_bytes;
  GH_CUDA(cudaMemcpy(D.first, g.first.data(), sizeof(int) * g.n, cudaMemcpyHostToDevice));
  GH_CUDA(cudaMemcpy(D.rmq_hash, rmq_hash.data(), sizeof(int64_t) * D.euler, cudaMemcpyHostToDevice));
  GH_CUDA(cudaMemcpy(D.rmq_id, rmq_id.data(), sizeof(int) * D.rmq, cudaMemcpyHostToDevice));
}

void download_rmq(const Graph &g, int64_t *rmq_hash, int *rmq_id) {
  GH_CHECK(g.dev.rmq_hash && g.dev.rmq_id, H2H_ERR_STATE, "sparse table not built");
  if (rmq_hash) GH_CUDA(cudaMemcpy(rmq_hash, g.dev.rmq_hash, sizeof(int64_t) * g.euler_n, cudaMemcpyDeviceToHost));
  if (rmq_id) GH_CUDA(cudaMemcpy(rmq_id, g.dev.rmq_id, sizeof(int) * g.rmq_total, cudaMemcpyDeviceToHost));
}

// The sparse table and firstAppeare are on the device since h2h_contract;
// labels since the fill.  Nothing is left to upload.
void upload_query_index(Graph &g) {
  GH_CHECK(g.dev.first && g.dev.rmq_hash && g.dev.rmq_id, H2H_ERR_STATE, "sparse table not built");
}

void run_query_batch(const Graph &g, const int *x, const int *y, int *out, int64_t n, int mode, cudaStream_t s,
                     int *bad) {
  if (n <= 0) return;
  const DeviceIndex &D = g.dev;
  QArgs A{x, y, out, n, g.n, D.first, D.depth, D.rmq_hash, D.rmq_id, D.pos_hash, D.pos_pos, D.drow, D.dis,
          bad ? bad : D.err};
  const int threads = 256;
  const int mi = mode == H2H_QUERY_LCA ? 0 : 1;
  using Kernel = void (*)(QArgs);
  static const Kernel kernels[2][4] = {
      {query_tile_kernel<true, 32>, query_tile_kernel<true, 16>, query_tile_kernel<true, 8>,
       query_tile_kernel<true, 4>},
      {query_tile_kernel<false, 32>, query_tile_kernel<false, 16>, query_tile_kernel<false, 8>,
       query_tile_kernel<false, 4>}};
  // device shape, looked up once (thread-safe static initialisation: the
  // server's worker and callers' threads may arrive together)
  struct Shape {
    int nsm = 1, per_sm[2] = {1, 1};  // resident 256-thread blocks per SM (all tile widths use 32 registers)
  };
  static const Shape shape = [] {
    Shape sh;
    int dev = 0;
    GH_CUDA(cudaGetDevice(&dev));
    GH_CUDA(cudaDeviceGetAttribute(&sh.nsm, cudaDevAttrMultiProcessorCount, dev));
    for (int k = 0; k < 2; k++) {
      GH_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&sh.per_sm[k], kernels[k][0], 256, 0));
      sh.per_sm[k] = std::max(1, sh.per_sm[k]);
    }
    return sh;
  }();
  const int nsm = shape.nsm;
  const int per_sm[2] = {shape.per_sm[0], shape.per_sm[1]};
  // narrowest tile whose warps still fit one wave of resident warps
  const int64_t resident_warps = (int64_t)nsm * per_sm[mi] * (threads / 32);
  int ti = 0, tile = 32;
  while (ti < 3 && ((n + tile / 2 - 1) / (tile / 2)) <= resident_warps) {
    tile /= 2;
    ti++;
  }
  const int64_t tiles = (n + tile - 1) / tile;
  // one wave of resident blocks, grid-striding over the tiles
  const int blocks = (int)std::min<int64_t>((tiles + 7) / 8, (int64_t)nsm * per_sm[mi]);
  kernels[mi][ti]<<<std::max(1, blocks), threads, 0, s>>>(A);
  GH_CUDA(cudaGetLastError());
}

void run_query_batch_plain(const Graph &g, const int *x, const int *y, int *out, int64_t n, int mode,
                           cudaStream_t s) {
  if (n <= 0) return;
  const DeviceIndex &D = g.dev;
  QArgs A{x, y, out, n, g.n, D.first, D.depth, D.rmq_hash, D.rmq_id, D.pos_hash, D.pos_pos, D.drow, D.dis, D.err};
  const int threads = 256;
  int blocks = (int)std::min<int64_t>((n + threads - 1) / threads, INT32_MAX);
  if (mode == H2H_QUERY_LCA) query_kernel<1, true><<<blocks, threads, 0, s>>>(A);
  else query_kernel<1, false><<<blocks, threads, 0, s>>>(A);
  GH_CUDA(cudaGetLastError());
}

}  // namespace gh
