// tree_gpu.cu -- the tree decomposition's structure and the fill's layout on
// the GPU, from the fathers the contraction picked:
//   getTreeStructure / OULADFS / makeOULAAndRMQ's tour (TreeStructure.cu:
//     102-262, 500-572): children in increasing id order (Childs), depths
//     (H2H_TreeHeight_Hash), firstAppeare and the Euler tour OULA_DFS_;
//   constructBFSTree's level order (H2HConsturction.cu:324-377): TreeBFS and
//     TreeHash;
//   the heavy-path layout and root-path segments the L4 fill reads its
//     ancestors from (labels.cu).
//
// The reference walks the tree recursively on the host.  Here every quantity
// is a closed form over subtree sizes and sums along root paths:
//   * children: a stable radix sort of (father, v) pairs, v ascending;
//   * subtree sizes: bottom-up, one thread per leaf climbing while it is the
//     last child of its father to arrive (one 64-bit word per node holds the
//     children still to come and the sizes already brought);
//   * a child c of p is entered in the tour at first(p) + 1 + 2 * (sizes of
//     the siblings before c), and p follows c's subtree at first(c) +
//     2 * size(c) - 1; the preorder index is (first + depth - 1) / 2;
//   * depth, first, heavy-path position and the count of heavy-path tops on
//     the root path are sums of per-node offsets along the root path:
//     pointer jumping, about log2(height) synchronous rounds;
//   * the level order is the preorder stably sorted by depth (nodes of one
//     depth appear in a breadth-first walk in the order a depth-first walk
//     with the same child order first reaches them).
// Every index a kernel writes through is checked against its array's size;
// a violation (only possible if the fathers are not one tree) sets an error
// word instead of writing.
#include <algorithm>
#include <cstring>

#include "graph.h"

namespace gh {

namespace {

// ------------------------------------------------------------------ scan

constexpr int kScanThreads = 1024, kScanItems = 4, kScanTile = kScanThreads * kScanItems;

template <typename T>
__global__ void __launch_bounds__(kScanThreads) scan_tile_kernel(const T *in, int64_t *out, int64_t n,
                                                                 int64_t *tile_sums) {
  __shared__ int64_t warp_tot[32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)tid * kScanItems;
  int64_t v[kScanItems];
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    v[k] = base + k < n ? (int64_t)in[base + k] : 0;
    s += v[k];
  }
  int64_t x = s;  // inclusive warp scan of the thread sums
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int64_t t = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    warp_tot[lane] = t;  // inclusive over warps
  }
  __syncthreads();
  int64_t run = x - s + (wid > 0 ? warp_tot[wid - 1] : 0);
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
  if (tid == kScanThreads - 1) tile_sums[blockIdx.x] = run;
}

__global__ void scan_add_kernel(int64_t *out, int64_t n, const int64_t *tile_offsets) {
  const int64_t add = tile_offsets[blockIdx.x];
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  for (int i = threadIdx.x; i < kScanTile; i += blockDim.x)
    if (base + i < n) out[base + i] += add;
}

// Device scratch of one tree build, freed together.
struct Workspace {
  std::vector<void *> p;
  template <typename T>
  T *get(int64_t n) {
    T *q = nullptr;
    GH_CUDA(cudaMalloc(&q, sizeof(T) * (size_t)std::max<int64_t>(n, 1)));
    p.push_back(q);
    return q;
  }
  ~Workspace() {
    for (void *q : p) cudaFree(q);
  }
};

// out[i] = sum of in[0 .. i) for i < n (tile sums scanned recursively).
template <typename T>
void exclusive_scan(const T *in, int64_t *out, int64_t n, Workspace &ws, cudaStream_t s) {
  if (n <= 0) return;
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  int64_t *sums = ws.get<int64_t>(tiles);
  scan_tile_kernel<T><<<(unsigned)tiles, kScanThreads, 0, s>>>(in, out, n, sums);
  GH_CUDA(cudaGetLastError());
  if (tiles > 1) {
    int64_t *offs = ws.get<int64_t>(tiles);
    exclusive_scan<int64_t>(sums, offs, tiles, ws, s);
    scan_add_kernel<<<(unsigned)tiles, 256, 0, s>>>(out, n, offs);
    GH_CUDA(cudaGetLastError());
  }
}

// ------------------------------------------------------------ radix sort
// Stable LSD radix sort of (uint32 key, int32 value) pairs, 8 bits a pass.
// A tile of 4,096 pairs is 8 warps x 16 rounds of 32 consecutive pairs; a
// pair's place in its digit's run is the digit's global offset for the tile
// (a scan over digit-major tile histograms) plus the pairs of that digit
// before it in the tile, counted warp by warp and round by round with
// __match_any_sync, so equal digits keep their input order.

constexpr int kRadixThreads = 256, kRadixRounds = 16, kRadixTile = kRadixThreads * kRadixRounds, kBins = 256;

__global__ void __launch_bounds__(kRadixThreads) radix_hist_kernel(const unsigned *keys, int64_t n, int shift,
                                                                   int *hist, int ntiles) {
  __shared__ int cnt[kBins];
  for (int b = threadIdx.x; b < kBins; b += blockDim.x) cnt[b] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kRadixTile;
  for (int i = threadIdx.x; i < kRadixTile; i += blockDim.x)
    if (base + i < n) atomicAdd(&cnt[(keys[base + i] >> shift) & (kBins - 1)], 1);
  __syncthreads();
  for (int b = threadIdx.x; b < kBins; b += blockDim.x) hist[(int64_t)b * ntiles + blockIdx.x] = cnt[b];
}

__global__ void __launch_bounds__(kRadixThreads) radix_scatter_kernel(const unsigned *kin, const int *vin,
                                                                      unsigned *kout, int *vout, int64_t n, int shift,
                                                                      const int64_t *offs, int ntiles) {
  __shared__ int64_t wpos[kRadixThreads / 32][kBins];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int b = lane; b < kBins; b += 32) wpos[w][b] = 0;
  __syncwarp();
  const int64_t wbase = (int64_t)blockIdx.x * kRadixTile + (int64_t)w * 32 * kRadixRounds;
  const unsigned lt = (1u << lane) - 1;
  for (int r = 0; r < kRadixRounds; r++) {  // per-warp digit counts
    const int64_t i = wbase + r * 32 + lane;
    const bool valid = i < n;
    const unsigned d = valid ? (kin[i] >> shift) & (kBins - 1) : kBins;
    const unsigned mask = __match_any_sync(0xffffffffu, d);
    if (valid && (mask & lt) == 0) wpos[w][d] += __popc(mask);
    __syncwarp();
  }
  __syncthreads();
  for (int b = threadIdx.x; b < kBins; b += blockDim.x) {  // warp starts inside the digit's run
    int64_t run = offs[(int64_t)b * ntiles + blockIdx.x];
    for (int ww = 0; ww < kRadixThreads / 32; ww++) {
      const int64_t c = wpos[ww][b];
      wpos[ww][b] = run;
      run += c;
    }
  }
  __syncthreads();
  for (int r = 0; r < kRadixRounds; r++) {
    const int64_t i = wbase + r * 32 + lane;
    const bool valid = i < n;
    const unsigned key = valid ? kin[i] : 0u;
    const unsigned d = valid ? (key >> shift) & (kBins - 1) : kBins;
    const unsigned mask = __match_any_sync(0xffffffffu, d);
    if (valid) {
      const int64_t pos = wpos[w][d] + __popc(mask & lt);
      if (pos >= 0 && pos < n) {
        kout[pos] = key;
        vout[pos] = vin[i];
      }
    }
    __syncwarp();
    if (valid && (mask & lt) == 0) wpos[w][d] += __popc(mask);
    __syncwarp();
  }
}

// Sorts keys/vals (n pairs, keys < 2^bits) stably by key; the result is in
// keys/vals.
void radix_sort_pairs(unsigned *keys, int *vals, int64_t n, int bits, Workspace &ws, cudaStream_t s) {
  if (n <= 1) return;
  const int ntiles = (int)((n + kRadixTile - 1) / kRadixTile);
  unsigned *k2 = ws.get<unsigned>(n);
  int *v2 = ws.get<int>(n);
  int *hist = ws.get<int>((int64_t)kBins * ntiles);
  int64_t *offs = ws.get<int64_t>((int64_t)kBins * ntiles);
  unsigned *ka = keys, *kb = k2;
  int *va = vals, *vb = v2;
  for (int shift = 0; shift < bits; shift += 8) {
    radix_hist_kernel<<<ntiles, kRadixThreads, 0, s>>>(ka, n, shift, hist, ntiles);
    GH_CUDA(cudaGetLastError());
    exclusive_scan<int>(hist, offs, (int64_t)kBins * ntiles, ws, s);
    radix_scatter_kernel<<<ntiles, kRadixThreads, 0, s>>>(ka, va, kb, vb, n, shift, offs, ntiles);
    GH_CUDA(cudaGetLastError());
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  if (ka != keys) {
    GH_CUDA(cudaMemcpyAsync(keys, ka, sizeof(unsigned) * n, cudaMemcpyDeviceToDevice, s));
    GH_CUDA(cudaMemcpyAsync(vals, va, sizeof(int) * n, cudaMemcpyDeviceToDevice, s));
  }
}

int bits_for(int64_t maxval) {
  int b = 1;
  while (b < 32 && (int64_t(1) << b) <= maxval) b++;
  return b;
}

// ------------------------------------------------------------ tree kernels

constexpr int kErrNotTree = 1;

__device__ __forceinline__ void flag_err(int *err) { atomicCAS(err, 0, kErrNotTree); }

__global__ void child_key_kernel(const int *father, int n, unsigned *key, int *val, int *cnt) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const int f = father[v];
    key[v] = f >= 0 && f < n ? (unsigned)f : (unsigned)n;  // the root sorts last
    val[v] = v;
    if (f >= 0 && f < n) atomicAdd(cnt + f, 1);
  }
}

// Subtree sizes: a thread starts at every leaf and climbs.  Each node has
// one 64-bit word: children still to arrive in the high half, the sizes
// they brought in the low half.  A child adds its size and takes one off
// the count in a single atomic; the child that sees the count reach zero
// knows the father's size from the value it got back and carries on.  One
// atomic per step (a chain as long as the tree is tall); every node is
// climbed past once, so the walk is O(n); a thread stops after n steps
// whatever the input.
__global__ void subtree_size_kernel(const int *father, const int *cnt, unsigned long long *word, int *size, int n,
                                    int *err) {
  for (int v0 = blockIdx.x * blockDim.x + threadIdx.x; v0 < n; v0 += gridDim.x * blockDim.x) {
    if (cnt[v0] != 0) continue;
    int v = v0;
    unsigned long long sz = 1;
    size[v] = 1;
    for (int step = 0; step < n; step++) {
      const int p = father[v];
      if (p < 0) break;
      if (p >= n) { flag_err(err); break; }
      const unsigned long long old = atomicAdd(word + p, sz - (1ull << 32));
      if ((old >> 32) != 1) break;  // a sibling is still climbing
      sz = (old & 0xffffffffull) + sz + 1;
      size[p] = (int)sz;
      v = p;
    }
  }
}

// Arrival words: the child count of every node in the high half.
__global__ void arrival_word_kernel(const int *cnt, unsigned long long *word, int n) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    word[v] = (unsigned long long)cnt[v] << 32;
}

// Per father, over its children in id order: the heavy child (largest
// subtree, the first one on ties), each child's tour offset 1 + 2 * (sizes of
// earlier siblings), its heavy-path offset (1 for the heavy child, else 1 +
// size(heavy) + sizes of earlier light siblings), whether it starts a heavy
// path, and its link up a heavy edge (the father when heavy, else itself).
__global__ void child_offsets_kernel(const int64_t *child_off, const int *childs, const int *size, int n, int root,
                                     int *off_first, int *off_hpos, int *seg_flag, int *hlink) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const int64_t b = child_off[p], e = child_off[p + 1];
    int best = -1, bs = 0;
    for (int64_t k = b; k < e; k++) {
      const int c = childs[k];
      if (size[c] > bs) { bs = size[c]; best = c; }
    }
    int64_t S = 0, L = 0;
    for (int64_t k = b; k < e; k++) {
      const int c = childs[k];
      off_first[c] = (int)(1 + 2 * S);
      S += size[c];
      if (c == best) {
        off_hpos[c] = 1;
      } else {
        off_hpos[c] = (int)(1 + bs + L);
        L += size[c];
      }
      seg_flag[c] = c != best;
      hlink[c] = c == best ? p : c;
    }
    if (p == root) {
      off_first[p] = 0;
      off_hpos[p] = 0;
      seg_flag[p] = 1;
      hlink[p] = p;
    }
  }
}

struct Jump {
  int *anc, *dep, *fst, *hp, *sg, *tl;
};

// One synchronous round of pointer jumping: every node adds its current
// ancestor's partial sums and jumps to that ancestor's ancestor; the heavy
// links jump likewise.  *more is set while any chain has not reached its top.
__global__ void jump_kernel(Jump a, Jump b, int n, int *more) {
  bool m = false;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const int u = a.anc[v];
    if (u >= 0 && u < n) {
      b.dep[v] = a.dep[v] + a.dep[u];
      b.fst[v] = a.fst[v] + a.fst[u];
      b.hp[v] = a.hp[v] + a.hp[u];
      b.sg[v] = a.sg[v] + a.sg[u];
      b.anc[v] = a.anc[u];
      m |= b.anc[v] >= 0;
    } else {
      b.dep[v] = a.dep[v];
      b.fst[v] = a.fst[v];
      b.hp[v] = a.hp[v];
      b.sg[v] = a.sg[v];
      b.anc[v] = -1;
    }
    const int t = a.tl[v];
    const int tt = t >= 0 && t < n ? a.tl[t] : t;
    b.tl[v] = tt;
    m |= tt != t;
  }
  if (__syncthreads_or(m) && threadIdx.x == 0) *more = 1;
}

// Euler tour, preorder, heavy-path order; every write index range-checked.
__global__ void place_kernel(const int *father, const int *size, const int *dep, const int *fst, const int *hp, int n,
                             int *euler, int *pre, int *hld, int *err) {
  const int64_t L = 2 * (int64_t)n - 1;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const int64_t f0 = fst[v];
    const int d = dep[v];
    if (f0 < 0 || f0 >= L || d < 1 || d > n || hp[v] < 0 || hp[v] >= n) { flag_err(err); continue; }
    euler[f0] = v;
    const int p = father[v];
    if (p >= 0) {
      const int64_t back = f0 + 2 * (int64_t)size[v] - 1;
      if (back < 0 || back >= L) { flag_err(err); continue; }
      euler[back] = p;
    }
    const int64_t pr = (f0 + d - 1) / 2;
    if (pr < 0 || pr >= n) { flag_err(err); continue; }
    pre[pr] = v;
    hld[hp[v]] = v;
  }
}

__global__ void level_key_kernel(const int *pre, const int *dep, int n, int height, unsigned *key, int *val,
                                 int *lvl_cnt, int *err) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int v = pre[i];
    if (v < 0 || v >= n || dep[v] < 1 || dep[v] > height) {  // the preorder is not a permutation
      flag_err(err);
      key[i] = 0;
      val[i] = 0;
      continue;
    }
    key[i] = (unsigned)(dep[v] - 1);
    val[i] = v;
    atomicAdd(lvl_cnt + dep[v] - 1, 1);
  }
}

__global__ void fill_value_kernel(int *a, int n, int value) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = value;
}

__global__ void max_kernel(const int *a, int n, int *out) {
  int m = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) m = max(m, a[i]);
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

template <typename T>
void download(std::vector<T> &h, const T *d, int64_t n) {
  h.resize(n);
  if (n) GH_CUDA(cudaMemcpy(h.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost));
}

}  // namespace

void build_tree_gpu(Graph &g) {
  Clock clk;
  const int n = g.n;
  GH_CHECK((int)g.father.size() == n && n >= 1, H2H_ERR_STATE, "fathers missing");
  g.head = g.elim[n - 1];
  int roots = 0;
  for (int v = 0; v < n; v++) {
    const int f = g.father[v];
    GH_CHECK(f >= -1 && f < n, H2H_ERR_STATE, "a father is out of range");
    roots += f < 0;
  }
  GH_CHECK(roots == 1 && g.father[g.head] < 0, H2H_ERR_STATE, "decomposition is not a single tree");
  int dev = 0, nsm = 0;
  GH_CUDA(cudaGetDevice(&dev));
  GH_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int grid = std::max(1, std::min(nsm * 8, (n + 255) / 256));
  cudaStream_t s = 0;
  Workspace ws;
  int *father = ws.get<int>(n), *cnt = ws.get<int>(n), *err = ws.get<int>(1), *more = ws.get<int>(1);
  GH_CUDA(cudaMemcpy(father, g.father.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
  GH_CUDA(cudaMemset(cnt, 0, sizeof(int) * n));
  GH_CUDA(cudaMemset(err, 0, sizeof(int)));
  // children in id order
  unsigned *key = ws.get<unsigned>(n);
  int *val = ws.get<int>(n);
  child_key_kernel<<<grid, 256, 0, s>>>(father, n, key, val, cnt);
  GH_CUDA(cudaGetLastError());
  radix_sort_pairs(key, val, n, bits_for(n), ws, s);
  int64_t *child_off = ws.get<int64_t>(n + 1);
  exclusive_scan<int>(cnt, child_off, n, ws, s);
  {
    // child_off[n] = child_off[n-1] + cnt[n-1]: one more element of the scan
    int64_t last = 0;
    int c_last = 0;
    GH_CUDA(cudaMemcpy(&last, child_off + n - 1, sizeof(int64_t), cudaMemcpyDeviceToHost));
    GH_CUDA(cudaMemcpy(&c_last, cnt + n - 1, sizeof(int), cudaMemcpyDeviceToHost));
    last += c_last;
    GH_CHECK(last == n - 1, H2H_ERR_STATE, "decomposition is not a single tree");
    GH_CUDA(cudaMemcpy(child_off + n, &last, sizeof(int64_t), cudaMemcpyHostToDevice));
  }
  const int *childs = val;  // the first n - 1 sorted values (the root's key sorts last)
  // subtree sizes
  unsigned long long *word = ws.get<unsigned long long>(n);
  int *size = ws.get<int>(n);
  arrival_word_kernel<<<grid, 256, 0, s>>>(cnt, word, n);
  GH_CUDA(cudaGetLastError());
  GH_CUDA(cudaMemset(size, 0, sizeof(int) * n));
  subtree_size_kernel<<<grid, 256, 0, s>>>(father, cnt, word, size, n, err);
  GH_CUDA(cudaGetLastError());
  {
    int sz_root = 0;
    GH_CUDA(cudaMemcpy(&sz_root, size + g.head, sizeof(int), cudaMemcpyDeviceToHost));
    GH_CHECK(sz_root == n, H2H_ERR_STATE, "decomposition is not a single tree");
  }
  // per-child offsets, then root-path sums by pointer jumping
  Jump A, B;
  for (Jump *J : {&A, &B}) {
    J->anc = ws.get<int>(n);
    J->dep = ws.get<int>(n);
    J->fst = ws.get<int>(n);
    J->hp = ws.get<int>(n);
    J->sg = ws.get<int>(n);
    J->tl = ws.get<int>(n);
  }
  child_offsets_kernel<<<grid, 256, 0, s>>>(child_off, childs, size, n, g.head, A.fst, A.hp, A.sg, A.tl);
  GH_CUDA(cudaGetLastError());
  GH_CUDA(cudaMemcpy(A.anc, father, sizeof(int) * n, cudaMemcpyDeviceToDevice));
  fill_value_kernel<<<grid, 256, 0, s>>>(A.dep, n, 1);  // every depth starts at one step
  GH_CUDA(cudaGetLastError());
  int rounds = 0;
  for (;;) {
    GH_CUDA(cudaMemsetAsync(more, 0, sizeof(int), s));
    jump_kernel<<<grid, 256, 0, s>>>(A, B, n, more);
    GH_CUDA(cudaGetLastError());
    std::swap(A, B);
    int m = 0;
    GH_CUDA(cudaMemcpy(&m, more, sizeof(int), cudaMemcpyDeviceToHost));
    if (!m) break;
    GH_CHECK(++rounds <= 40, H2H_ERR_STATE, "decomposition is not a single tree");
  }
  // tour, preorder, heavy-path order
  const int64_t L = 2 * (int64_t)n - 1;
  int *euler = ws.get<int>(L), *pre = ws.get<int>(n), *hld = ws.get<int>(n);
  GH_CUDA(cudaMemset(pre, 0xff, sizeof(int) * n));
  place_kernel<<<grid, 256, 0, s>>>(father, size, A.dep, A.fst, A.hp, n, euler, pre, hld, err);
  GH_CUDA(cudaGetLastError());
  int e = 0;
  GH_CUDA(cudaMemcpy(&e, err, sizeof(int), cudaMemcpyDeviceToHost));
  GH_CHECK(e == 0, H2H_ERR_STATE, "decomposition is not a single tree");
  // level order: the preorder stably sorted by depth
  int *hmax = ws.get<int>(1);
  GH_CUDA(cudaMemset(hmax, 0, sizeof(int)));
  max_kernel<<<grid, 256, 0, s>>>(A.dep, n, hmax);
  GH_CUDA(cudaGetLastError());
  int height = 0;
  GH_CUDA(cudaMemcpy(&height, hmax, sizeof(int), cudaMemcpyDeviceToHost));
  GH_CHECK(height >= 1 && height <= n, H2H_ERR_STATE, "decomposition is not a single tree");
  int *lvl_cnt = ws.get<int>(height);
  GH_CUDA(cudaMemset(lvl_cnt, 0, sizeof(int) * height));
  level_key_kernel<<<grid, 256, 0, s>>>(pre, A.dep, n, height, key, val, lvl_cnt, err);
  GH_CUDA(cudaGetLastError());
  GH_CUDA(cudaMemcpy(&e, err, sizeof(int), cudaMemcpyDeviceToHost));
  GH_CHECK(e == 0, H2H_ERR_STATE, "decomposition is not a single tree");
  radix_sort_pairs(key, val, n, bits_for(height - 1), ws, s);
  int64_t *lvl_off = ws.get<int64_t>(height);
  exclusive_scan<int>(lvl_cnt, lvl_off, height, ws, s);
  // root-path segment offsets and row offsets
  int64_t *seg_off = ws.get<int64_t>(n);
  exclusive_scan<int>(A.sg, seg_off, n, ws, s);
  int64_t *dis_hash = ws.get<int64_t>(n);
  exclusive_scan<int>(A.dep, dis_hash, n, ws, s);
  int *smax = ws.get<int>(1);
  GH_CUDA(cudaMemset(smax, 0, sizeof(int)));
  max_kernel<<<grid, 256, 0, s>>>(A.sg, n, smax);
  GH_CUDA(cudaGetLastError());
  GH_CUDA(cudaDeviceSynchronize());
  // host copies (the accessors, the index file and the fill plan read them)
  download(g.depth, A.dep, n);
  download(g.first, A.fst, n);
  download(g.euler_id, euler, L);
  download(g.tree_bfs, val, n);
  {
    std::vector<int64_t> lo;
    download(lo, lvl_off, height);
    g.tree_hash.resize(height + 1);
    for (int l = 0; l < height; l++) g.tree_hash[l] = (int)lo[l];
    g.tree_hash[height] = n;
  }
  download(g.hld, hld, n);
  download(g.htop, A.tl, n);
  download(g.hpos, A.hp, n);
  {
    std::vector<int> sg_last(1);
    download(g.seg_off, seg_off, n);
    GH_CUDA(cudaMemcpy(sg_last.data(), A.sg + n - 1, sizeof(int), cudaMemcpyDeviceToHost));
    g.seg_off.push_back(g.seg_off[n - 1] + sg_last[0]);
  }
  GH_CUDA(cudaMemcpy(&g.max_segs, smax, sizeof(int), cudaMemcpyDeviceToHost));
  {
    download(g.dis_hash, dis_hash, n);
    g.dis_hash.push_back(g.dis_hash[n - 1] + g.depth[n - 1]);
  }
  g.h2h_size = g.dis_hash[n];
  g.tree_height = height;
  g.euler_n = L;
  g.child_off.clear();
  g.childs.clear();
  g.tree_layout = true;
  g.t.tree = clk.us();
}

}  // namespace gh
