// contract.cu -- partition-level vertex elimination on the GPU, the work of
// makeCHPerHeight_2 / makeCHPerHeight_D_2 (kernel_functions.cu:309-553).
//
// The reference runs one thread per partition cell and, for each elimination,
// bubble-sorts the cell's remaining candidates by TDrank (degree + height,
// degree, id), bubble-sorts the eliminated vertex's list, rewrites every
// neighbour's list and scans lists linearly for fill-in.  The values it
// produces depend only on:
//   * the candidate picked at each step: the minimum of the TDrank order, a
//     strict total order because ids are unique -- so a block-wide argmin
//     over keys kept in shared memory picks the same vertex;
//   * the content of each list as a sequence: stable sorts by neighbour id
//     (rank sort on (id << 32 | position) keys gives the same permutation),
//     the duplicate merge carry (:339-351), the "recount" that leaves the
//     size unchanged when no valid entry remains (:353-360, :381-388), and
//     fill-in appends in the order the pair loop (:392-457) reaches them.
// Here one CTA owns a cell.  Per elimination: argmin over the candidate keys
// (shared memory), the eliminated vertex's list is staged and sorted in
// shared memory, then each warp takes whole neighbour lists: delete the
// back-edge, stable-sort, binary-search every other neighbour (first match =
// lower_bound on the sorted prefix) and append misses in neighbour order.
// Lists of different neighbours are disjoint, so warps never conflict.
// Lists longer than a warp buffer are handled by the whole CTA afterwards.
//
// Degree/height keys follow :462-476: a neighbour's height becomes
// max(height, HeightNow + 1) where HeightNow is the picked key's height, and
// the first pick of a cell uses the stale keys (input degree, height 0)
// written by makeAdjcentNode.
#include <algorithm>
#include <climits>
#include <cstring>

#include "graph.h"

namespace gh {

namespace {

constexpr uint32_t kIdxMask = 0xffffffffu;
constexpr int kErrOverflow = 1;  // a list outgrew its LUB capacity (reference corrupts memory)
constexpr int kErrEmpty = 2;     // eliminated vertex without neighbours (reference reads ID_hash[INT_MAX])
constexpr int kErrScratch = 3;   // a list outgrew the per-level staging bound

struct LevelArgs {
  int *slot_nbr;
  int *slot_w;
  const int64_t *slot_off;
  int *lsize;
  const int *cap;
  int *height;
  int *elim;              // candidate ids per cell range; rewritten in elimination order
  const int *deg0;        // input degree (stale first-pick key)
  const int *cell_start;
  const int *cell_count;
  int *cpos;              // vertex -> local candidate index while it is a candidate, else -1
  int *err;               // first error code (0 = none)
  int cell_lo;            // first cell index of the level
  int kmax;               // max candidates in a cell of this level
  int lmax;               // max list length in a cell of this level
  int wbuf;               // per-warp list buffer (entries)
  int keys_in_smem;       // candidate keys in shared memory (else scratch)
  int lists_in_smem;      // own-list + CTA sort buffers in shared memory (else scratch)
  char *scratch;          // global staging slab, per CTA stride bytes
  int64_t scratch_stride;
};

__device__ __forceinline__ void set_err(int *err, int code) { atomicCAS(err, 0, code); }

// Stable ascending sort of `key[0..s)` (distinct 64-bit keys) by a bitonic
// network over the next power of two; comparators that reach past s are
// skipped, which is the same as padding with +infinity.  `tid/nthr` span the
// cooperating threads; SYNC is __syncwarp or __syncthreads.
template <bool BLOCK>
__device__ void bitonic_sort(uint64_t *key, int s, int tid, int nthr) {
  if (s <= 1) return;
  int P = 1;
  while (P < s) P <<= 1;
  const int half_p = P >> 1;
  for (int k = 2; k <= P; k <<= 1) {
    const int hk = k >> 1;
    const int lg = __ffs(hk) - 1;
    for (int t = tid; t < half_p; t += nthr) {
      int lo = ((t >> lg) << (lg + 1)) + (t & (hk - 1));
      int hi = lo ^ (k - 1);
      if (hi < s) {
        uint64_t a = key[lo], b = key[hi];
        if (a > b) { key[lo] = b; key[hi] = a; }
      }
    }
    if (BLOCK) __syncthreads(); else __syncwarp();
    for (int m = k >> 2; m > 0; m >>= 1) {
      const int lm = __ffs(m) - 1;
      for (int t = tid; t < half_p; t += nthr) {
        int lo = ((t >> lm) << (lm + 1)) + (t & (m - 1));
        int hi = lo + m;
        if (hi < s) {
          uint64_t a = key[lo], b = key[hi];
          if (a > b) { key[lo] = b; key[hi] = a; }
        }
      }
      if (BLOCK) __syncthreads(); else __syncwarp();
    }
  }
}

__device__ __forceinline__ int key_id(uint64_t k) { return (int)(k >> 32); }

// lower_bound of id x in sorted keys[0..n)
__device__ __forceinline__ int lower_bound_id(const uint64_t *keys, int n, int x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (key_id(keys[mid]) < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

struct Cand {
  int *id, *deg, *third;
};

__device__ __forceinline__ bool key_less(int s1, int d1, int i1, int s2, int d2, int i2) {
  if (s1 != s2) return s1 < s2;
  if (d1 != d2) return d1 < d2;
  return i1 < i2;
}

// One neighbour list: delete v, stable sort, recount, fill-in against the
// eliminated vertex's sorted list (anbr/aw, c entries, own index iu).
// Runs on a warp (BLOCK=false) or on the whole CTA (BLOCK=true).
template <bool BLOCK>
__device__ void process_neighbour(const LevelArgs &A, int u, int wu, int iu, int v, int hnow, const int *anbr,
                                  const int *aw, int c, uint64_t *key, int *worig, int tid, int nthr, Cand cand,
                                  int *bcast) {
  const int64_t off = A.slot_off[u];
  const int s = A.lsize[u];
  // load with the back-edge to v replaced by INT_MAX (kernel_functions.cu:364-375)
  bool unsorted = false;
  for (int i = tid; i < s; i += nthr) {
    int nb = A.slot_nbr[off + i];
    if (nb == v) nb = INT_MAX;
    key[i] = ((uint64_t)(uint32_t)nb << 32) | (uint32_t)i;
    worig[i] = A.slot_w[off + i];
  }
  if (BLOCK) __syncthreads(); else __syncwarp();
  for (int i = tid; i + 1 < s; i += nthr)
    if (key_id(key[i]) > key_id(key[i + 1])) unsorted = true;
  if (BLOCK) unsorted = __syncthreads_or(unsorted);
  else unsorted = __any_sync(0xffffffffu, unsorted);
  if (unsorted) bitonic_sort<BLOCK>(key, s, tid, nthr);
  // write the sorted list back; valid entries form the prefix after the sort
  for (int i = tid; i < s; i += nthr) {
    uint64_t k = key[i];
    A.slot_nbr[off + i] = key_id(k);
    A.slot_w[off + i] = worig[k & kIdxMask];
  }
  const int cu = lower_bound_id(key, s, INT_MAX);
  const int size = cu > 0 ? cu : s;  // recount leaves the size unchanged when nothing valid remains
  if (BLOCK) __syncthreads(); else __syncwarp();
  // fill-in: every other neighbour x of v, in v's sorted order
  int appended = 0;
  for (int base = 0; base < c; base += nthr) {
    int i = base + tid;
    bool miss = false;
    int x = 0, len = 0;
    if (i < c && i != iu) {
      x = anbr[i];
      len = wu + aw[i];
      int p = lower_bound_id(key, size, x);
      if (p < size && key_id(key[p]) == x) {
        if (A.slot_w[off + p] > len) A.slot_w[off + p] = len;
      } else {
        miss = true;
      }
    }
    int rank, total;
    if (BLOCK) {
      // block-wide exclusive rank of misses
      const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
      unsigned bal = __ballot_sync(0xffffffffu, miss);
      if (lane == 0) bcast[wid] = __popc(bal);
      __syncthreads();
      int before = 0;
      total = 0;
      for (int w = 0; w < nw; w++) {
        if (w < wid) before += bcast[w];
        total += bcast[w];
      }
      rank = before + __popc(bal & ((1u << lane) - 1u));
      __syncthreads();
    } else {
      unsigned bal = __ballot_sync(0xffffffffu, miss);
      rank = __popc(bal & ((1u << tid) - 1u));
      total = __popc(bal);
    }
    if (miss) {
      int pos = size + appended + rank;
      if (pos >= A.cap[u]) {
        set_err(A.err, kErrOverflow);
      } else {
        A.slot_nbr[off + pos] = x;
        A.slot_w[off + pos] = len;
      }
    }
    appended += total;
  }
  if (tid == 0) {
    int ns = size + appended;
    A.lsize[u] = ns > A.cap[u] ? A.cap[u] : ns;
    int h = A.height[u];
    A.height[u] = (hnow + 1 > h) ? hnow + 1 : h;
    int p = A.cpos[u];
    if (p >= 0) {  // a remaining candidate of this cell: refresh its key
      cand.deg[p] = A.lsize[u];
      cand.third[p] = A.height[u];
    }
  }
  if (BLOCK) __syncthreads(); else __syncwarp();
}

__global__ void __launch_bounds__(256) contract_level_kernel(LevelArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int cell = A.cell_lo + blockIdx.x;
  const int start = A.cell_start[cell];
  const int k = A.cell_count[cell];
  if (k == 0) return;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int lane = tid & 31, wid = tid >> 5, nw = nthr >> 5;

  // ---- carve staging areas (shared memory, or this CTA's scratch slab)
  unsigned char *sp = smem;
  unsigned char *gp = (unsigned char *)A.scratch + (int64_t)blockIdx.x * A.scratch_stride;
  auto take = [&](bool in_smem, int64_t bytes) -> void * {
    bytes = (bytes + 15) & ~int64_t(15);
    void *r;
    if (in_smem) { r = sp; sp += bytes; } else { r = gp; gp += bytes; }
    return r;
  };
  __shared__ int bcast[32];
  __shared__ int s_red_sum[32], s_red_deg[32], s_red_id[32], s_red_pos[32];
  __shared__ int s_v, s_hnow, s_c, s_stop, s_nbig;
  Cand cand;
  cand.id = (int *)take(A.keys_in_smem, sizeof(int) * A.kmax);
  cand.deg = (int *)take(A.keys_in_smem, sizeof(int) * A.kmax);
  cand.third = (int *)take(A.keys_in_smem, sizeof(int) * A.kmax);
  int *anbr = (int *)take(A.lists_in_smem, sizeof(int) * A.lmax);
  int *aw = (int *)take(A.lists_in_smem, sizeof(int) * A.lmax);
  uint64_t *bkey = (uint64_t *)take(A.lists_in_smem, sizeof(uint64_t) * A.lmax);
  int *bw = (int *)take(A.lists_in_smem, sizeof(int) * A.lmax);
  int *big = (int *)take(A.lists_in_smem, sizeof(int) * A.lmax);  // deferred neighbour indices
  uint64_t *wkey = (uint64_t *)take(true, sizeof(uint64_t) * A.wbuf * nw) + (int64_t)wid * A.wbuf;
  int *ww = (int *)take(true, sizeof(int) * A.wbuf * nw) + (int64_t)wid * A.wbuf;

  for (int i = tid; i < k; i += nthr) {
    int v = A.elim[start + i];
    cand.id[i] = v;
    cand.deg[i] = A.deg0[v];
    cand.third[i] = 0;
    A.cpos[v] = i;
  }
  if (tid == 0) s_stop = 0;
  __syncthreads();

  for (int j = 0; j < k; j++) {
    // ---- 1. argmin of (deg + height, deg, id) over candidates [j, k)
    int bs = INT_MAX, bd = INT_MAX, bi = INT_MAX, bp = -1;
    for (int i = j + tid; i < k; i += nthr) {
      int d = cand.deg[i], t = cand.third[i], id = cand.id[i];
      if (bp < 0 || key_less(d + t, d, id, bs, bd, bi)) { bs = d + t; bd = d; bi = id; bp = i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      int os = __shfl_down_sync(0xffffffffu, bs, o), od = __shfl_down_sync(0xffffffffu, bd, o);
      int oi = __shfl_down_sync(0xffffffffu, bi, o), op = __shfl_down_sync(0xffffffffu, bp, o);
      if (op >= 0 && (bp < 0 || key_less(os, od, oi, bs, bd, bi))) { bs = os; bd = od; bi = oi; bp = op; }
    }
    if (lane == 0) { s_red_sum[wid] = bs; s_red_deg[wid] = bd; s_red_id[wid] = bi; s_red_pos[wid] = bp; }
    __syncthreads();
    if (tid == 0) {
      int rs = s_red_sum[0], rd = s_red_deg[0], ri = s_red_id[0], rp = s_red_pos[0];
      for (int w = 1; w < nw; w++) {
        if (s_red_pos[w] >= 0 && (rp < 0 || key_less(s_red_sum[w], s_red_deg[w], s_red_id[w], rs, rd, ri))) {
          rs = s_red_sum[w]; rd = s_red_deg[w]; ri = s_red_id[w]; rp = s_red_pos[w];
        }
      }
      // ---- 2. move the pick to position j
      int v = cand.id[rp];
      int hn = cand.third[rp];
      if (rp != j) {
        int u = cand.id[j];
        cand.id[rp] = u; cand.deg[rp] = cand.deg[j]; cand.third[rp] = cand.third[j];
        A.cpos[u] = rp;
        cand.id[j] = v; cand.deg[j] = rd; cand.third[j] = hn;
      }
      A.cpos[v] = -1;
      A.elim[start + j] = v;
      s_v = v;
      s_hnow = hn;
    }
    __syncthreads();
    const int v = s_v, hnow = s_hnow;
    // ---- 3. own list: stable sort, merge duplicates, compact (kernel_functions.cu:338-361)
    const int64_t voff = A.slot_off[v];
    const int sv = A.lsize[v];
    if (sv > A.lmax) { if (tid == 0) { set_err(A.err, kErrScratch); s_stop = 1; } }
    __syncthreads();
    if (s_stop) return;
    for (int i = tid; i < sv; i += nthr) {
      bkey[i] = ((uint64_t)(uint32_t)A.slot_nbr[voff + i] << 32) | (uint32_t)i;
      bw[i] = A.slot_w[voff + i];
    }
    __syncthreads();
    bitonic_sort<true>(bkey, sv, tid, nthr);
    bool dup = false;
    for (int i = tid; i < sv; i += nthr) {
      anbr[i] = key_id(bkey[i]);
      aw[i] = bw[bkey[i] & kIdxMask];
    }
    __syncthreads();
    for (int i = tid + 1; i < sv; i += nthr)
      if (anbr[i] == anbr[i - 1] && anbr[i] != INT_MAX) dup = true;
    dup = __syncthreads_or(dup);
    if (dup && tid == 0) {
      // carry merge then stable compaction (the second stable sort only moves the INT_MAX entries)
      for (int i = 1; i < sv; i++) {
        if (anbr[i] == anbr[i - 1] && anbr[i] != INT_MAX) {
          if (aw[i - 1] < aw[i]) aw[i] = aw[i - 1];
          anbr[i - 1] = INT_MAX;
        }
      }
      int c = 0;
      for (int i = 0; i < sv; i++) if (anbr[i] != INT_MAX) { anbr[c] = anbr[i]; aw[c] = aw[i]; c++; }
      for (int i = c; i < sv; i++) anbr[i] = INT_MAX;
    }
    __syncthreads();
    if (tid == 0) {
      int c = 0;
      while (c < sv && anbr[c] != INT_MAX) c++;  // valid entries form the prefix
      s_c = c;
      if (c == 0) { set_err(A.err, kErrEmpty); s_stop = 1; }
      else A.lsize[v] = c;
      s_nbig = 0;
    }
    __syncthreads();
    if (s_stop) return;
    const int c = s_c;
    for (int i = tid; i < c; i += nthr) { A.slot_nbr[voff + i] = anbr[i]; A.slot_w[voff + i] = aw[i]; }
    // ---- 4. neighbours, one warp each; long lists deferred to the CTA
    for (int i = wid; i < c; i += nw) {
      const int u = anbr[i];
      const int su = A.lsize[u];
      if (su > A.wbuf) {
        if (lane == 0) big[atomicAdd(&s_nbig, 1)] = i;
        continue;
      }
      process_neighbour<false>(A, u, aw[i], i, v, hnow, anbr, aw, c, wkey, ww, lane, 32, cand, nullptr);
    }
    __syncthreads();
    const int nbig = s_nbig;
    for (int b = 0; b < nbig; b++) {
      const int i = big[b];
      const int u = anbr[i];
      if (A.lsize[u] > A.lmax) {
        if (tid == 0) { set_err(A.err, kErrScratch); s_stop = 1; }
        __syncthreads();
        return;
      }
      process_neighbour<true>(A, u, aw[i], i, v, hnow, anbr, aw, c, bkey, bw, tid, nthr, cand, bcast);
    }
    // ---- 5. after the first pick every remaining key becomes live (:471-475)
    if (j == 0) {
      for (int i = 1 + tid; i < k; i += nthr) {
        int u = cand.id[i];
        cand.deg[i] = A.lsize[u];
        cand.third[i] = A.height[u];
      }
    }
    __syncthreads();
  }
}

__global__ void scatter_adjacency_kernel(const int *adj_off, const int *adj_v, const int *adj_w,
                                         const int64_t *slot_off, int *slot_nbr, int *slot_w, int n) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    int64_t o = slot_off[v];
    for (int e = adj_off[v]; e < adj_off[v + 1]; e++) {
      slot_nbr[o + (e - adj_off[v])] = adj_v[e];
      slot_w[o + (e - adj_off[v])] = adj_w[e];
    }
  }
}

__global__ void gather_lists_kernel(const int64_t *slot_off, const int *lsize, const int64_t *out_off,
                                    const int *slot_nbr, const int *slot_w, int *out_nbr, int *out_w, int n) {
  // one warp per vertex
  const int lane = threadIdx.x & 31;
  for (int64_t v = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; v < n;
       v += (gridDim.x * (int64_t)blockDim.x) >> 5) {
    int64_t so = slot_off[v], oo = out_off[v];
    int s = lsize[v];
    for (int i = lane; i < s; i += 32) {
      out_nbr[oo + i] = slot_nbr[so + i];
      out_w[oo + i] = slot_w[so + i];
    }
  }
}

template <typename T>
T *dalloc(size_t n) {
  T *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc(&p, n * sizeof(T));
  if (e != cudaSuccess) throw Error(H2H_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  return p;
}

}  // namespace

// Runs the partition levels H..C+1 and returns every vertex's list
// (elimination-time lists for eliminated vertices, current lists for the
// rest) in list order, plus the updated elimination order and heights.
void contract_partition_levels_gpu(Graph &g, std::vector<int64_t> &lst_off, std::vector<int> &lst_nbr,
                                   std::vector<int> &lst_w) {
  const int n = g.n;
  Clock clk;
  // per-cell bound on list lengths during the cell's level (makeAdjcentNode's
  // alive size + out-of-cell arcs, plus parallel-arc slack)
  const int64_t cells = (int64_t(1) << g.H) - 1;
  std::vector<int> level_of(n, 0);
  for (int h = g.H; h >= 1; h--) {
    const int64_t lo = (int64_t(1) << (h - 1)) - 1, hi = (int64_t(1) << h) - 2;
    for (int64_t c = lo; c <= hi; c++)
      for (int i = 0; i < g.cell_count[c]; i++) level_of[g.elim[g.cell_start[c] + i]] = h;
  }
  std::vector<int> dup(n, 0);
  {
    std::vector<int> tmp;
    for (int v = 0; v < n; v++) {
      tmp.assign(g.adj_v.begin() + g.adj_off[v], g.adj_v.begin() + g.adj_off[v + 1]);
      std::sort(tmp.begin(), tmp.end());
      dup[v] = (int)(tmp.size() - (std::unique(tmp.begin(), tmp.end()) - tmp.begin()));
    }
  }
  (void)cells;

  int *d_slot_nbr = dalloc<int>(g.lub), *d_slot_w = dalloc<int>(g.lub);
  int64_t *d_slot_off = dalloc<int64_t>(n);
  int *d_lsize = dalloc<int>(n), *d_cap = dalloc<int>(n), *d_height = dalloc<int>(n), *d_elim = dalloc<int>(n);
  int *d_deg0 = dalloc<int>(n), *d_cpos = dalloc<int>(n), *d_err = dalloc<int>(1);
  int *d_cell_start = dalloc<int>(g.cell_start.size()), *d_cell_count = dalloc<int>(g.cell_count.size());
  int *d_adj_off = dalloc<int>(n + 1), *d_adj_v = dalloc<int>(g.m), *d_adj_w = dalloc<int>(g.m);
  char *d_scratch = nullptr;
  int64_t scratch_bytes = 0;
  auto cleanup = [&]() {
    cudaFree(d_slot_nbr); cudaFree(d_slot_w); cudaFree(d_slot_off); cudaFree(d_lsize); cudaFree(d_cap);
    cudaFree(d_height); cudaFree(d_elim); cudaFree(d_deg0); cudaFree(d_cpos); cudaFree(d_err);
    cudaFree(d_cell_start); cudaFree(d_cell_count); cudaFree(d_adj_off); cudaFree(d_adj_v); cudaFree(d_adj_w);
    if (d_scratch) cudaFree(d_scratch);
  };
  try {
    std::vector<int> deg(n), minus1(n, -1), zeros(n, 0);
    for (int v = 0; v < n; v++) deg[v] = g.adj_off[v + 1] - g.adj_off[v];
    GH_CUDA(cudaMemcpy(d_slot_off, g.slot_off.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_lsize, deg.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_deg0, deg.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_cap, g.cap.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_height, zeros.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_cpos, minus1.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_elim, g.elim.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_cell_start, g.cell_start.data(), sizeof(int) * g.cell_start.size(), cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_cell_count, g.cell_count.data(), sizeof(int) * g.cell_count.size(), cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(d_adj_off, g.adj_off.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice));
    if (g.m) {
      GH_CUDA(cudaMemcpy(d_adj_v, g.adj_v.data(), sizeof(int) * g.m, cudaMemcpyHostToDevice));
      GH_CUDA(cudaMemcpy(d_adj_w, g.adj_w.data(), sizeof(int) * g.m, cudaMemcpyHostToDevice));
    }
    GH_CUDA(cudaMemset(d_err, 0, sizeof(int)));
    scatter_adjacency_kernel<<<std::max(1, std::min(4096, (n + 255) / 256)), 256>>>(d_adj_off, d_adj_v, d_adj_w, d_slot_off,
                                                                                   d_slot_nbr, d_slot_w, n);
    GH_CUDA(cudaGetLastError());
    GH_CUDA(cudaDeviceSynchronize());
    g.t.translate_lub = clk.us();
    clk.reset();

    const int smem_dyn = enable_max_dynamic_smem(contract_level_kernel);
    const int kThreads = 256, kWarps = kThreads / 32;
    for (int h = g.H; h > g.C; h--) {
      const int64_t lo = (int64_t(1) << (h - 1)) - 1, hi = (int64_t(1) << h) - 2;
      const int ncell = (int)(hi - lo + 1);
      int kmax = 1, lmax = 1;
      for (int64_t c = lo; c <= hi; c++) {
        kmax = std::max(kmax, g.cell_count[c]);
        // members of the cell at this level: vertices whose elimination level is <= h and that lie in the cut range
        int alive = 0;
        for (int i = g.cut_l[c]; i < g.cut_r[c]; i++) alive += level_of[g.part_ids[i]] <= h;
        for (int i = g.cut_l[c]; i < g.cut_r[c]; i++) {
          int v = g.part_ids[i];
          if (level_of[v] > h) continue;
          int out = 0;
          for (int e = g.adj_off[v]; e < g.adj_off[v + 1]; e++) {
            int u = g.adj_v[e];
            if (level_of[u] > h) continue;
            int iu = g.id_hash[u];
            if (iu < g.cut_l[c] || iu >= g.cut_r[c]) out++;
          }
          lmax = std::max(lmax, alive - 1 + out + dup[v]);
        }
      }
      LevelArgs A;
      A.slot_nbr = d_slot_nbr; A.slot_w = d_slot_w; A.slot_off = d_slot_off; A.lsize = d_lsize; A.cap = d_cap;
      A.height = d_height; A.elim = d_elim; A.deg0 = d_deg0; A.cell_start = d_cell_start;
      A.cell_count = d_cell_count; A.cpos = d_cpos; A.err = d_err; A.cell_lo = (int)lo;
      A.kmax = kmax; A.lmax = lmax;
      A.wbuf = std::min(lmax, 256);
      auto al = [](int64_t b) { return (b + 15) & ~int64_t(15); };
      int64_t keys_b = 3 * al(sizeof(int) * (int64_t)kmax);
      int64_t lists_b = al(4LL * lmax) * 2 + al(8LL * lmax) + al(4LL * lmax) * 2;
      int64_t warp_b = al(8LL * A.wbuf * kWarps) + al(4LL * A.wbuf * kWarps);
      const int64_t budget = smem_dyn;
      A.keys_in_smem = 1;
      A.lists_in_smem = 1;
      int64_t smem = keys_b + lists_b + warp_b;
      if (smem > budget) { A.lists_in_smem = 0; smem = keys_b + warp_b; }
      if (smem > budget) { A.keys_in_smem = 0; smem = warp_b; }
      GH_CHECK(smem <= budget, H2H_ERR_DEVICE, "contraction staging does not fit shared memory");
      int64_t stride = (A.keys_in_smem ? 0 : keys_b) + (A.lists_in_smem ? 0 : lists_b);
      stride = al(stride);
      if (stride * ncell > scratch_bytes) {
        if (d_scratch) cudaFree(d_scratch);
        d_scratch = nullptr;
        scratch_bytes = stride * ncell;
        GH_CUDA(cudaMalloc(&d_scratch, scratch_bytes));
      }
      A.scratch = d_scratch;
      A.scratch_stride = stride;
      contract_level_kernel<<<ncell, kThreads, (size_t)smem>>>(A);
      GH_CUDA(cudaGetLastError());
    }
    GH_CUDA(cudaDeviceSynchronize());
    int err = 0;
    GH_CUDA(cudaMemcpy(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost));
    GH_CHECK(err == 0, H2H_ERR_DEVICE,
             err == kErrOverflow ? "contraction: a list outgrew its LUB capacity"
             : err == kErrEmpty  ? "contraction: eliminated a vertex with an empty list (disconnected input)"
                                 : "contraction: list outgrew the staging bound");
    g.t.td_gpu = clk.us();
    clk.reset();
    // ---- copy back order, heights and compacted lists
    std::vector<int> lsize(n);
    g.height.resize(n);
    GH_CUDA(cudaMemcpy(g.elim.data(), d_elim, sizeof(int) * n, cudaMemcpyDeviceToHost));
    GH_CUDA(cudaMemcpy(lsize.data(), d_lsize, sizeof(int) * n, cudaMemcpyDeviceToHost));
    GH_CUDA(cudaMemcpy(g.height.data(), d_height, sizeof(int) * n, cudaMemcpyDeviceToHost));
    lst_off.assign(n + 1, 0);
    for (int v = 0; v < n; v++) lst_off[v + 1] = lst_off[v] + lsize[v];
    const int64_t tot = lst_off[n];
    int64_t *d_out_off = dalloc<int64_t>(n + 1);
    int *d_out_nbr = dalloc<int>(tot), *d_out_w = dalloc<int>(tot);
    GH_CUDA(cudaMemcpy(d_out_off, lst_off.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice));
    gather_lists_kernel<<<std::max(1, std::min(8192, (n * 32 + 255) / 256)), 256>>>(d_slot_off, d_lsize, d_out_off,
                                                                                   d_slot_nbr, d_slot_w, d_out_nbr,
                                                                                   d_out_w, n);
    cudaError_t e1 = cudaGetLastError();
    lst_nbr.resize(tot);
    lst_w.resize(tot);
    cudaError_t e2 = cudaMemcpy(lst_nbr.data(), d_out_nbr, sizeof(int) * tot, cudaMemcpyDeviceToHost);
    cudaError_t e3 = cudaMemcpy(lst_w.data(), d_out_w, sizeof(int) * tot, cudaMemcpyDeviceToHost);
    cudaFree(d_out_off); cudaFree(d_out_nbr); cudaFree(d_out_w);
    GH_CUDA(e1); GH_CUDA(e2); GH_CUDA(e3);
    g.t.translate_back = clk.us();
  } catch (...) {
    cleanup();
    throw;
  }
  cleanup();
}

}  // namespace gh
