// contract.cu -- partition-level vertex elimination on the GPU, the work of
// makeCHPerHeight_2 / makeCHPerHeight_D_2 (kernel_functions.cu:309-553).
//
// The reference runs one thread per partition cell and, for each elimination,
// bubble-sorts the cell's remaining candidates by TDrank (degree + height,
// degree, id), bubble-sorts the eliminated vertex's list, rewrites every
// neighbour's list and scans lists linearly for fill-in.  Its results depend
// only on:
//   * the candidate picked at each step: the minimum of the TDrank order, a
//     strict total order because ids are unique -- a block-wide argmin over
//     keys kept in shared memory picks the same vertex;
//   * each list as a sequence: stable sorts by neighbour id, the duplicate
//     merge carry of the eliminated vertex's list (:339-351), the "recount"
//     that leaves a size unchanged when no valid entry remains (:353-360,
//     :381-388), first-match fill-in updates and appends (:392-457).
// Every list is stable-sorted once up front and kept sorted: a stable sort
// of the reference's [sorted run][appended run] is exactly the sorted merge
// of the two runs, and every reader (next touch, own-list merge, the global
// heap's first-seen emplace) sees the same sequence.  A list whose valid
// entries all vanish keeps the reference's stale size as a prefix of junk
// entries (`ljunk`), and later appends land after them, as in the reference.
//
// One CTA owns a cell.  Per elimination: argmin over the candidate keys, the
// eliminated vertex's sorted list is staged in shared memory and merged,
// then each warp takes whole neighbour lists and rebuilds them with a
// merge-path union of (list minus v) and (the other neighbours), two linear
// walks per lane after one co-rank search; a match updates the first entry of
// that id (min weight), a miss inserts.  Warps never share a list.
//
// Keys follow :462-476: a neighbour's height becomes max(height, HeightNow+1)
// with HeightNow the picked key's height; the first pick of a cell uses the
// stale keys (input degree, height 0) written by makeAdjcentNode.
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "graph.h"

namespace gh {

namespace {

constexpr int kErrOverflow = 1;  // a list outgrew its LUB capacity (the reference corrupts memory)
constexpr int kErrEmpty = 2;     // eliminated a vertex without neighbours (the reference reads out of bounds)
constexpr int kErrStaging = 3;   // a list outgrew the per-level staging bound

struct LevelArgs {
  int *slot_nbr;
  int *slot_w;
  const int64_t *slot_off;
  int *lsize;             // list length, junk prefix included (CHTreeHash.first)
  int *ljunk;             // leading stale entries of the list
  const int *cap;
  int *height;            // CHInfo.second
  int *elim;              // candidate ids per cell range; rewritten in elimination order
  const int *deg0;        // input degree (stale first-pick key)
  const int *cell_start;
  const int *cell_count;
  int *cpos;              // vertex -> local candidate index while it is a candidate, else -1
  int *err;               // first error code (0 = none)
  int cell_lo;            // first cell index of the level
  int kmax;               // max candidates in a cell of this level
  int lmax;               // bound on valid list entries in a cell of this level
  int keys_in_smem;       // candidate keys in shared memory (else scratch)
  int lists_in_smem;      // list staging in shared memory (else scratch)
  char *scratch;          // global staging slab, scratch_stride bytes per CTA
  int64_t scratch_stride;
};

__device__ __forceinline__ void set_err(int *err, int code) { atomicCAS(err, 0, code); }

struct Cand {
  int *id, *deg, *third;
};

__device__ __forceinline__ bool key_less(int s1, int d1, int i1, int s2, int d2, int i2) {
  if (s1 != s2) return s1 < s2;
  if (d1 != d2) return d1 < d2;
  return i1 < i2;
}

// Q = the eliminated vertex's list without entry iu.
__device__ __forceinline__ int q_at(const int *a, int iu, int q) { return a[q < iu ? q : q + 1]; }

// Merge-path co-rank: number of P entries among the first k outputs of the
// stable merge of P and Q (ties take P first).
__device__ __forceinline__ int corank(const int *pid, int np, const int *aid, int iu, int nq, int k) {
  int lo = max(0, k - nq), hi = min(k, np);
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (pid[mid] <= q_at(aid, iu, k - 1 - mid)) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Rebuild neighbour u's list for the elimination of v (one warp):
//   P = valid entries of u's list except v (kernel_functions.cu:364-390),
//   output = P with the first entry of every matched id min-updated, plus the
//   unmatched members of Q inserted in order (:392-457).
__device__ void merge_neighbour(const LevelArgs &A, int u, int wu, int iu, int v, int hnow, const int *aid,
                                const int *aw, int c, int *pid, int *pw, int lane, Cand cand) {
  const int64_t off = A.slot_off[u];
  const int s = A.lsize[u];
  const int J = A.ljunk[u];
  // stage P with v removed (stable compaction)
  int np = 0;
  for (int base = J; base < s; base += 32) {
    const int idx = base + lane;
    int x = INT_MAX, w = 0;
    if (idx < s) { x = A.slot_nbr[off + idx]; w = A.slot_w[off + idx]; }
    const bool keep = idx < s && x != v;
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    if (keep) {
      const int pos = np + __popc(bal & ((1u << lane) - 1u));
      pid[pos] = x;
      pw[pos] = w;
    }
    np += __popc(bal);
  }
  __syncwarp();
  const int nq = c - 1;
  const int Jn = np > 0 ? 0 : s;  // nothing valid left: the reference keeps its stale size
  const int total_len = np + nq;
  const int seg = (total_len + 31) >> 5;
  const int k0 = min(lane * seg, total_len), k1 = min(k0 + seg, total_len);
  const int i0 = corank(pid, np, aid, iu, nq, k0);
  // pass 1: count outputs, apply matched updates to the first entry of the id
  int cnt = 0;
  {
    int i = i0, j = k0 - i0;
    for (int t = k0; t < k1; t++) {
      if (i < np && (j >= nq || pid[i] <= q_at(aid, iu, j))) {
        i++;
        cnt++;
      } else {
        const int x = q_at(aid, iu, j);
        if (i > 0 && pid[i - 1] == x) {
          int f = i - 1;
          while (f > 0 && pid[f - 1] == x) f--;
          atomicMin(pw + f, wu + q_at(aw, iu, j));
        } else {
          cnt++;
        }
        j++;
      }
    }
  }
  __syncwarp();
  int incl = cnt;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  const bool fits = Jn + total <= A.cap[u];
  if (fits) {
    int o = incl - cnt;
    int i = i0, j = k0 - i0;
    for (int t = k0; t < k1; t++) {
      if (i < np && (j >= nq || pid[i] <= q_at(aid, iu, j))) {
        A.slot_nbr[off + Jn + o] = pid[i];
        A.slot_w[off + Jn + o] = pw[i];
        o++;
        i++;
      } else {
        const int x = q_at(aid, iu, j);
        if (!(i > 0 && pid[i - 1] == x)) {
          A.slot_nbr[off + Jn + o] = x;
          A.slot_w[off + Jn + o] = wu + q_at(aw, iu, j);
          o++;
        }
        j++;
      }
    }
    for (int k = lane; k < Jn; k += 32) A.slot_nbr[off + k] = INT_MAX;
  }
  if (lane == 0) {
    if (!fits) set_err(A.err, kErrOverflow);
    const int ns = fits ? Jn + total : s;
    A.lsize[u] = ns;
    A.ljunk[u] = fits ? Jn : J;
    const int h = A.height[u];
    const int hn = (hnow + 1 > h) ? hnow + 1 : h;
    A.height[u] = hn;
    const int p = A.cpos[u];
    if (p >= 0) {  // a remaining candidate of this cell: refresh its key
      cand.deg[p] = ns;
      cand.third[p] = hn;
    }
  }
  __syncwarp();
}

__global__ void __launch_bounds__(512) contract_level_kernel(LevelArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int cell = A.cell_lo + blockIdx.x;
  const int start = A.cell_start[cell];
  const int k = A.cell_count[cell];
  if (k == 0) return;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int lane = tid & 31, wid = tid >> 5, nw = nthr >> 5;

  unsigned char *sp = smem;
  unsigned char *gp = (unsigned char *)A.scratch + (int64_t)blockIdx.x * A.scratch_stride;
  auto take = [&](bool in_smem, int64_t bytes) -> void * {
    bytes = (bytes + 15) & ~int64_t(15);
    void *r;
    if (in_smem) { r = sp; sp += bytes; } else { r = gp; gp += bytes; }
    return r;
  };
  __shared__ int s_red_sum[32], s_red_deg[32], s_red_id[32], s_red_pos[32];
  __shared__ int s_v, s_hnow, s_c, s_stop;
  Cand cand;
  cand.id = (int *)take(A.keys_in_smem, sizeof(int) * A.kmax);
  cand.deg = (int *)take(A.keys_in_smem, sizeof(int) * A.kmax);
  cand.third = (int *)take(A.keys_in_smem, sizeof(int) * A.kmax);
  int *aid = (int *)take(A.lists_in_smem, sizeof(int) * A.lmax);
  int *aw = (int *)take(A.lists_in_smem, sizeof(int) * A.lmax);
  int *pid = (int *)take(A.lists_in_smem, sizeof(int) * A.lmax * nw) + (int64_t)wid * A.lmax;
  int *pw = (int *)take(A.lists_in_smem, sizeof(int) * A.lmax * nw) + (int64_t)wid * A.lmax;

  for (int i = tid; i < k; i += nthr) {
    const int v = A.elim[start + i];
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
      const int d = cand.deg[i], t = cand.third[i], id = cand.id[i];
      if (bp < 0 || key_less(d + t, d, id, bs, bd, bi)) { bs = d + t; bd = d; bi = id; bp = i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const int os = __shfl_down_sync(0xffffffffu, bs, o), od = __shfl_down_sync(0xffffffffu, bd, o);
      const int oi = __shfl_down_sync(0xffffffffu, bi, o), op = __shfl_down_sync(0xffffffffu, bp, o);
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
      const int v = cand.id[rp];
      const int hn = cand.third[rp];
      if (rp != j) {
        const int u = cand.id[j];
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
    // ---- 3. own list: valid part is sorted; merge duplicates, drop junk (:338-361)
    const int64_t voff = A.slot_off[v];
    const int vJ = A.ljunk[v];
    const int sv = A.lsize[v] - vJ;
    if (sv > A.lmax) { if (tid == 0) { set_err(A.err, kErrStaging); s_stop = 1; } }
    __syncthreads();
    if (s_stop) return;
    for (int i = tid; i < sv; i += nthr) {
      aid[i] = A.slot_nbr[voff + vJ + i];
      aw[i] = A.slot_w[voff + vJ + i];
    }
    __syncthreads();
    bool dup = false;
    for (int i = tid + 1; i < sv; i += nthr)
      if (aid[i] == aid[i - 1]) dup = true;
    dup = __syncthreads_or(dup);
    if (tid == 0) {
      int c = sv;
      if (dup) {  // carry merge (the later entry keeps the smaller weight), then compaction
        for (int i = 1; i < sv; i++) {
          if (aid[i] == aid[i - 1] && aid[i] != INT_MAX) {
            if (aw[i - 1] < aw[i]) aw[i] = aw[i - 1];
            aid[i - 1] = INT_MAX;
          }
        }
        c = 0;
        for (int i = 0; i < sv; i++) if (aid[i] != INT_MAX) { aid[c] = aid[i]; aw[c] = aw[i]; c++; }
      }
      s_c = c;
      if (c == 0) { set_err(A.err, kErrEmpty); s_stop = 1; }
      else { A.lsize[v] = c; A.ljunk[v] = 0; }
    }
    __syncthreads();
    if (s_stop) return;
    const int c = s_c;
    for (int i = tid; i < c; i += nthr) { A.slot_nbr[voff + i] = aid[i]; A.slot_w[voff + i] = aw[i]; }
    // ---- 4. neighbours, one warp each
    for (int i = wid; i < c; i += nw) {
      const int u = aid[i];
      if (A.lsize[u] - A.ljunk[u] > A.lmax) {
        if (lane == 0) set_err(A.err, kErrStaging);
        continue;
      }
      merge_neighbour(A, u, aw[i], i, v, hnow, aid, aw, c, pid, pw, lane, cand);
    }
    __syncthreads();
    // ---- 5. after the first pick every remaining key becomes live (:471-475)
    if (j == 0) {
      for (int i = 1 + tid; i < k; i += nthr) {
        const int u = cand.id[i];
        cand.deg[i] = A.lsize[u];
        cand.third[i] = A.height[u];
      }
    }
    __syncthreads();
  }
}

__global__ void scatter_adjacency_kernel(const int *adj_off, const int *adj_v, const int *adj_w,
                                         const int64_t *slot_off, int *slot_nbr, int *slot_w, int n) {
  // input lists in file order, stable-sorted by neighbour id (insertion sort)
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const int64_t o = slot_off[v];
    const int b = adj_off[v], e = adj_off[v + 1];
    for (int i = b; i < e; i++) {
      const int x = adj_v[i], w = adj_w[i];
      int k = i - b;
      while (k > 0 && slot_nbr[o + k - 1] > x) {
        slot_nbr[o + k] = slot_nbr[o + k - 1];
        slot_w[o + k] = slot_w[o + k - 1];
        k--;
      }
      slot_nbr[o + k] = x;
      slot_w[o + k] = w;
    }
  }
}

__global__ void gather_lists_kernel(const int64_t *slot_off, const int *lsize, const int64_t *out_off,
                                    const int *slot_nbr, const int *slot_w, int *out_nbr, int *out_w, int n) {
  // one warp per vertex
  const int lane = threadIdx.x & 31;
  for (int64_t v = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; v < n;
       v += (gridDim.x * (int64_t)blockDim.x) >> 5) {
    const int64_t so = slot_off[v], oo = out_off[v];
    const int s = lsize[v];
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
  int *d_deg0 = dalloc<int>(n), *d_cpos = dalloc<int>(n), *d_err = dalloc<int>(1), *d_ljunk = dalloc<int>(n);
  int *d_cell_start = dalloc<int>(g.cell_start.size()), *d_cell_count = dalloc<int>(g.cell_count.size());
  int *d_adj_off = dalloc<int>(n + 1), *d_adj_v = dalloc<int>(g.m), *d_adj_w = dalloc<int>(g.m);
  char *d_scratch = nullptr;
  int64_t scratch_bytes = 0;
  auto cleanup = [&]() {
    cudaFree(d_slot_nbr); cudaFree(d_slot_w); cudaFree(d_slot_off); cudaFree(d_lsize); cudaFree(d_cap);
    cudaFree(d_height); cudaFree(d_elim); cudaFree(d_deg0); cudaFree(d_cpos); cudaFree(d_err); cudaFree(d_ljunk);
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
    GH_CUDA(cudaMemcpy(d_ljunk, zeros.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
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
    const bool trace = std::getenv("GPUH2H_TRACE") != nullptr;
    int nsm = 0, dev = 0;
    GH_CUDA(cudaGetDevice(&dev));
    GH_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
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
      A.kmax = kmax; A.lmax = lmax; A.ljunk = d_ljunk;
      auto al = [](int64_t b) { return (b + 15) & ~int64_t(15); };
      const int64_t keys_b = 3 * al(sizeof(int) * (int64_t)kmax);
      auto lists_bytes = [&](int nw) { return 2 * al(4LL * lmax) + 2 * al(4LL * lmax * nw); };
      const int64_t budget = smem_dyn;
      // few cells (top levels): 16 warps per cell; many cells: 8 warps, several CTAs per SM
      int nw = ncell < nsm ? 16 : 8;
      while (nw > 4 && keys_b + lists_bytes(nw) > budget) nw >>= 1;
      A.keys_in_smem = 1;
      A.lists_in_smem = 1;
      int64_t smem = keys_b + lists_bytes(nw);
      if (smem > budget) { A.lists_in_smem = 0; smem = keys_b; }
      if (smem > budget) { A.keys_in_smem = 0; smem = 0; }
      int64_t stride = (A.keys_in_smem ? 0 : keys_b) + (A.lists_in_smem ? 0 : lists_bytes(nw));
      stride = al(stride);
      if (stride * ncell > scratch_bytes) {
        if (d_scratch) cudaFree(d_scratch);
        d_scratch = nullptr;
        scratch_bytes = stride * ncell;
        GH_CUDA(cudaMalloc(&d_scratch, scratch_bytes));
      }
      A.scratch = d_scratch;
      A.scratch_stride = stride;
      cudaEvent_t ev0 = nullptr, ev1 = nullptr;
      if (trace) { cudaEventCreate(&ev0); cudaEventCreate(&ev1); cudaEventRecord(ev0); }
      contract_level_kernel<<<ncell, nw * 32, (size_t)smem>>>(A);
      GH_CUDA(cudaGetLastError());
      if (trace) {
        cudaEventRecord(ev1);
        cudaEventSynchronize(ev1);
        float ms = 0;
        cudaEventElapsedTime(&ms, ev0, ev1);
        std::fprintf(stderr, "[gpuh2h] contract level %d: %d cells x %d warps, kmax %d, lmax %d, smem %lld (keys %s, lists %s): %.3f ms\n",
                     h, ncell, nw, kmax, lmax, (long long)smem, A.keys_in_smem ? "smem" : "global",
                     A.lists_in_smem ? "smem" : "global", ms);
        cudaEventDestroy(ev0);
        cudaEventDestroy(ev1);
      }
    }
    GH_CUDA(cudaDeviceSynchronize());
    int err = 0;
    GH_CUDA(cudaMemcpy(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost));
    GH_CHECK(err == 0, H2H_ERR_DEVICE,
             err == kErrOverflow ? "contraction: a list outgrew its LUB capacity"
             : err == kErrEmpty ? "contraction: eliminated a vertex with an empty list (disconnected input)"
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
