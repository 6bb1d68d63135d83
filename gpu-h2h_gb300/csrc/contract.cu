// contract.cu -- vertex elimination on the GPU: the partition levels of
// makeCHPerHeight_2 / makeCHPerHeight_D_2 (kernel_functions.cu:309-553) and
// the global minimum-degree heap of TDInCPU / uploadCHset / CHUsingHeap_2
// (Traditional_H2H.cu:6-118, :216-351), both as one elimination kernel.
//
// The reference runs one thread per partition cell and, for each elimination,
// bubble-sorts the cell's remaining candidates by TDrank (degree + height,
// degree, id), bubble-sorts the eliminated vertex's list, rewrites every
// neighbour's list and scans lists linearly for fill-in; the top levels go to
// a std::set heap with hash-map adjacency on the host.  Its results depend
// only on:
//   * the vertex picked at each step: the minimum of the (degree + height,
//     degree, id) order, a strict total order because ids are unique -- a
//     block argmin over keys held in shared memory picks the same vertex;
//   * each list as a sequence: stable sorts by neighbour id, the duplicate
//     merge carry of the eliminated vertex's list (:339-351), the "recount"
//     that leaves a size unchanged when no valid entry remains (:353-360,
//     :381-388), first-match fill-in updates and appends (:392-457).
// Every list is stable-sorted once up front and kept sorted: a stable sort of
// the reference's [sorted run][appended run] is exactly the sorted merge of
// the two runs, and every reader (next touch, own-list merge, the heap's
// first-seen emplace) sees the same sequence.  A list whose valid entries
// all vanish keeps the reference's stale size as a prefix of junk entries
// (`ljunk`); later appends land after them, as in the reference.
//
// One thread-block cluster owns a cell (one CTA for the many small cells at
// the bottom, up to 16 CTAs for the few large cells near the top; a step of
// one cell -- the global order of a single graph -- runs instead as one
// cooperative launch over all SMs, cell_grid_kernel further down).  Per
// elimination the leader CTA takes the argmin and merges the eliminated
// vertex's own list in shared memory; after a cluster barrier every warp of
// every CTA rebuilds whole neighbour lists with a merge-path union of
// (list minus v) and (the other neighbours) -- one co-rank search and two
// linear walks per lane; a match min-updates the first entry of that id, a
// miss inserts -- and writes candidate keys back into the leader's shared
// memory.  Warps never share a list.
//
// Keys follow kernel_functions.cu:462-476: a neighbour's height becomes
// max(height, HeightNow + 1) with HeightNow the picked key's height; the
// first pick of a cell uses the stale keys (input degree, height 0) written
// by makeAdjcentNode, after which every key is live.  The global heap is the
// same loop over one "cell" holding every vertex of levels <= C, with live
// keys from the start (valid-entry count, height) and first-seen duplicate
// removal on entry (unordered_map::emplace), and empty lists stay empty.
#include <cooperative_groups.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <memory>
#include <queue>

#include "graph.h"
#include "pool.h"

namespace cg = cooperative_groups;

namespace gh {

namespace {

constexpr int kErrOverflow = 1;  // a list outgrew its LUB capacity (the reference corrupts memory)
constexpr int kErrEmpty = 2;     // eliminated a vertex without neighbours (the reference reads out of bounds)
constexpr int kErrStaging = 3;   // a list outgrew the per-level staging bound
constexpr int kErrTimeout = 4;   // a cell barrier wait ran out (cell_grid_kernel)
constexpr int kErrPick = 5;      // no candidate left to pick (inconsistent cell table)

struct ElimArgs {
  int *slot_nbr;
  int *slot_w;
  int64_t *slot_off;      // list start (a heap list that outgrows its range moves)
  int *lsize;             // list length, junk prefix included (CHTreeHash.first)
  int *ljunk;             // leading stale entries of the list
  int *cap;               // list capacity
  unsigned long long *pool_next;  // bump allocator over the slot arrays (heap mode)
  int64_t pool_size;
  int *height;            // CHInfo.second
  int *elim;              // candidate ids per cell range; rewritten in elimination order
  const int *key_deg0;    // first-pick degree key per vertex
  const int *key_h0;      // first-pick height key per vertex (nullptr = 0)
  const int *cell_start;
  const int *cell_count;
  int *cpos;              // vertex -> candidate index while it is a candidate of its cell, else -1
  int *err;               // first error code (0 = none)
  int cell_lo;            // first cell index of the launch
  int kmax;               // max candidates in a cell of this launch
  int lmax;               // bound on valid list entries in a cell of this launch
  int heap_mode;          // 1: global heap semantics (live keys, no refresh, no junk)
  int *pstage;            // non-null: per-warp merge buffers in global memory (2*lmax ints per warp)
};

__device__ __forceinline__ void set_err(int *err, int code) { atomicCAS(err, 0, code); }

struct Cand {
  int *id, *deg, *third;
};

// ints [at, at + n) of the arena, or -1 when it has no room (lane 0 asks,
// every lane gets the answer).
__device__ __forceinline__ int arena_take(int *next, int cap, int n, int lane) {
  int at = -1;
  if (lane == 0) {
    int cur = *(volatile int *)next;
    while (cur + n <= cap) {
      const int old = atomicCAS(next, cur, cur + n);
      if (old == cur) {
        at = cur;
        break;
      }
      cur = old;
    }
  }
  return __shfl_sync(0xffffffffu, at, 0);
}

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

// The duplicate merge of a picked vertex's own list (kernel_functions.cu:
// 338-361), by one warp.  The reference walks the list once: an entry equal
// to its predecessor takes the smaller of the two weights and the predecessor
// becomes INT_MAX, then the INT_MAX entries are compacted out.  So of every
// run of equal ids only the last entry stays, carrying the run's smallest
// weight, and entries that were INT_MAX already go too.  Here that is a
// segmented minimum over runs, 32 entries at a time (the run minimum crosses
// chunk boundaries in a register), and a stable compaction in place: an entry
// lands at or before its own index, after the warp has read the chunk and the
// entry that follows it.  Returns the new length in every lane.
__device__ int collapse_runs_warp(int *aid, int *aw, int sv, int lane) {
  int out = 0, last_id = INT_MAX, carry = INT_MAX;
  for (int base = 0; base < sv; base += 32) {
    const int i = base + lane;
    const bool valid = i < sv;
    const int x = valid ? aid[i] : INT_MAX;
    int w = valid ? aw[i] : INT_MAX;
    const int nx = i + 1 < sv ? aid[i + 1] : INT_MAX;
    const int px = __shfl_up_sync(0xffffffffu, x, 1);
    const int prev = lane == 0 ? last_id : px;
    const bool real = valid && x != INT_MAX;
    int f = !(real && x == prev && i > 0);  // head of a run
    if (lane == 0 && !f) w = min(w, carry);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int wy = __shfl_up_sync(0xffffffffu, w, o);
      const int fy = __shfl_up_sync(0xffffffffu, f, o);
      if (lane >= o) {
        if (!f) w = min(w, wy);
        f |= fy;
      }
    }
    const bool keep = real && (i + 1 >= sv || nx != x);
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    last_id = __shfl_sync(0xffffffffu, x, 31);
    carry = __shfl_sync(0xffffffffu, w, 31);
    __syncwarp();
    if (keep) {
      const int o = out + __popc(bal & ((1u << lane) - 1u));
      aid[o] = x;
      aw[o] = w;
    }
    out += __popc(bal);
    __syncwarp();
  }
  return out;
}

// What a merge needs to know about neighbour u, loaded in one round trip:
// list start, length (junk prefix included), junk prefix, capacity, height,
// candidate index.  Only the warp merging u writes these during an
// elimination (the candidate index changes only when u is picked).
struct NbrMeta {
  int64_t off;
  int s, J, cap, h, p;
};

// Mutable global data is read through L2 (ld.global.cg): other CTAs write it
// between barriers.
__device__ __forceinline__ NbrMeta load_meta(const ElimArgs &A, int u) {
  NbrMeta m;
  m.off = __ldcg(A.slot_off + u);
  m.s = __ldcg(A.lsize + u);
  m.J = __ldcg(A.ljunk + u);
  m.cap = __ldcg(A.cap + u);
  m.h = __ldcg(A.height + u);
  m.p = __ldcg(A.cpos + u);
  return m;
}

// Rebuild neighbour u's list for the elimination of v (one warp):
//   P = valid entries of u's list except v (kernel_functions.cu:364-390),
//   output = P with the first entry of every matched id min-updated, plus the
//   unmatched members of Q inserted in order (:392-457).
//
// kWide: the list is read with 128-bit loads, four per lane in flight (2 KB
// of ids and 2 KB of weights per warp per round trip instead of 512 B each):
// near the top of the order lists hold thousands of entries and the load is
// the merge's latency.  The slot arrays are padded by four entries, so a
// vector that starts inside the list never leaves the allocation.
// u's list minus v (P) into pid/pw by one warp; returns |P| in every lane.
// kWide: 128-bit loads, four per lane in flight (2 KB of ids and 2 KB of
// weights per warp per round trip instead of 512 B each); the slot arrays
// are padded by four entries, so a vector that starts inside the list never
// leaves the allocation.
template <bool kWide>
__device__ __forceinline__ int load_p(const ElimArgs &A, const NbrMeta &m, int v, int *pid, int *pw, int lane) {
  int np = 0;
  const int64_t off = m.off;
  const int s = m.s;
  const int J = m.J;
  if (kWide) {
    const int64_t lo = off + J, hi = off + s;
    for (int64_t base = lo & ~int64_t(3); base < hi; base += 4 * 32 * 4) {
      int4 xv[4], wv[4];
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const int64_t e = base + (int64_t)(r * 32 + lane) * 4;
        if (e < hi) {
          xv[r] = __ldcg(reinterpret_cast<const int4 *>(A.slot_nbr + e));
          wv[r] = __ldcg(reinterpret_cast<const int4 *>(A.slot_w + e));
        } else {
          xv[r] = make_int4(v, v, v, v);
          wv[r] = make_int4(0, 0, 0, 0);
        }
      }
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const int64_t e = base + (int64_t)(r * 32 + lane) * 4;
        const int xs[4] = {xv[r].x, xv[r].y, xv[r].z, xv[r].w};
        const int ws[4] = {wv[r].x, wv[r].y, wv[r].z, wv[r].w};
        bool keep[4];
        int kc = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
          keep[k] = e + k >= lo && e + k < hi && xs[k] != v;
          kc += keep[k];
        }
        int incl = kc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += y;
        }
        int pos = np + incl - kc;
#pragma unroll
        for (int k = 0; k < 4; k++)
          if (keep[k]) {
            pid[pos] = xs[k];
            pw[pos] = ws[k];
            pos++;
          }
        np += __shfl_sync(0xffffffffu, incl, 31);
      }
    }
  }
  // u's list minus v, loaded four warp-widths at a time so the L2 round trips overlap
  for (int base = J; !kWide && base < s; base += 128) {
    int x[4], w[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int idx = base + r * 32 + lane;
      x[r] = INT_MAX;
      w[r] = 0;
      if (idx < s) { x[r] = __ldcg(A.slot_nbr + off + idx); w[r] = __ldcg(A.slot_w + off + idx); }
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const bool keep = base + r * 32 + lane < s && x[r] != v;
      const unsigned bal = __ballot_sync(0xffffffffu, keep);
      if (keep) {
        const int pos = np + __popc(bal & ((1u << lane) - 1u));
        pid[pos] = x[r];
        pw[pos] = w[r];
      }
      np += __popc(bal);
    }
  }
  __syncwarp();
  return np;
}

//
// kTeam: T warps (tw = this warp's place among them) share the merge: the
// first stages P, then the merge path is cut into 32*T stretches, one per
// lane of the team, with a prefix of the warps' counts over `tsh` (12 ints
// of shared memory per team) and named barrier `bid` over the team's 32*T
// threads.  Every warp of the team takes the same branches (all depend on
// values the team shares), so each reaches every barrier.
template <bool kWide, bool kTeam = false>
__device__ __forceinline__ void merge_neighbour(const ElimArgs &A, int u, const NbrMeta &m, int wu, int iu, int v, int hnow,
                                const int *aid, const int *aw, int c, int *pid, int *pw, int lane, Cand cand,
                                int nslots, int T = 1, int tw = 0, int bid = 0, int *tsh = nullptr) {
  auto tsync = [&]() {
    if (kTeam)
      asm volatile("bar.sync %0, %1;" ::"r"(bid), "r"(32 * T) : "memory");
    else
      __syncwarp();
  };
  int64_t off = m.off;
  const int s = m.s;
  const int J = m.J;
  int np;
  if (kTeam) {
    if (tw == 0) {
      const int n0 = load_p<kWide>(A, m, v, pid, pw, lane);
      if (lane == 0) tsh[0] = n0;
    }
    tsync();
    np = tsh[0];
  } else {
    np = load_p<kWide>(A, m, v, pid, pw, lane);
  }
  const int L = kTeam ? 32 * T : 32, tl = kTeam ? 32 * tw + lane : lane;  // stretches, this lane's
  const int nq = c - 1;
  // nothing valid left: the partition kernel keeps its stale size, a heap map is empty
  const int Jn = (np > 0 || A.heap_mode) ? 0 : s;
  const int total_len = np + nq;
  const int seg = (total_len + L - 1) / L;
  const int k0 = min(tl * seg, total_len), k1 = min(k0 + seg, total_len);
  const int i0 = corank(pid, np, aid, iu, nq, k0);
  const int plast = max(0, np - 1), qlast = max(0, nq - 1);  // clamped load indices (in bounds when empty)
  // pass 1: count outputs, apply matched updates to the first entry of the
  // id.  Branch-free steps (the warp's lanes would otherwise run both sides
  // of every step): an exhausted list reads as INT_MAX (ids are below it,
  // and a step never finds both exhausted), the next P and Q ids are both
  // loaded and the taken side's kept, and the last P id taken and the first
  // index of its run stay in registers.  Q's ids are distinct (v's list is
  // sorted and its duplicates were merged), so a run of P receives at most
  // one update, from the one lane that meets its Q entry: a plain
  // read-min-write (a shared-memory atomic costs more), ordered before pass
  // 2's reads by the __syncwarp between the passes.  (A microbenchmark of
  // this walk on lists of 1,152 and 538 entries: 13.2k cycles per pass
  // against 17.3k with a branch per step.)
  int cnt = 0;
  {
    int i = i0, j = k0 - i0;
    int a = i < np ? pid[i] : INT_MAX;
    int b = j < nq ? q_at(aid, iu, j) : INT_MAX;
    int prev = i > 0 ? pid[i - 1] : INT_MIN, run = i - 1;  // the last P id taken and its run's first index
    if (i > 0)
      while (run > 0 && pid[run - 1] == prev) run--;
    for (int t = k0; t < k1; t++) {
      const bool tp = a <= b;
      const bool match = !tp && prev == b;
      if (match) {
        const int x = wu + q_at(aw, iu, j);
        if (x < pw[run]) pw[run] = x;
      }
      cnt += !match;
      run = (tp && a != prev) ? i : run;
      prev = tp ? a : prev;
      i += tp;
      j += !tp;
      const int na = pid[min(i, plast)];
      const int nb = q_at(aid, iu, min(j, qlast));
      a = i < np ? na : INT_MAX;
      b = j < nq ? nb : INT_MAX;
    }
  }
  __syncwarp();
  int incl = cnt;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  int total, before = 0;  // outputs of the merge, of the team's warps before this one
  if (kTeam) {
    if (lane == 31) tsh[1 + tw] = incl;
    tsync();  // also orders pass 1's updates before pass 2's reads across the team
    total = 0;
    for (int w = 0; w < T; w++) {
      const int x = tsh[1 + w];
      before += w < tw ? x : 0;
      total += x;
    }
  } else {
    total = __shfl_sync(0xffffffffu, incl, 31);
  }
  const int capu = m.cap;
  bool fits = Jn + total <= capu;
  if (!fits && A.heap_mode) {
    // the reference's heap adjacency is a hash map that grows freely: move the
    // list to a fresh range (the merge writes a full new copy anyway)
    int64_t fresh = -1;
    const int ncap = max(2 * capu, Jn + total);
    if (tl == 0) {
      const unsigned long long at = atomicAdd(A.pool_next, (unsigned long long)ncap);
      if ((int64_t)at + ncap <= A.pool_size) fresh = (int64_t)at;
    }
    if (kTeam) {
      if (tl == 0) {
        tsh[6] = (int)(fresh & 0xffffffffll);
        tsh[7] = (int)(fresh >> 32);
      }
      tsync();
      fresh = (int64_t)(((uint64_t)(unsigned)tsh[7] << 32) | (unsigned)tsh[6]);
    } else {
      fresh = __shfl_sync(0xffffffffu, fresh, 0);
    }
    if (fresh >= 0) {
      off = fresh;
      fits = true;
      if (tl == 0) {
        A.slot_off[u] = fresh;
        A.cap[u] = ncap;
      }
    }
  }
  if (fits && total == np && Jn == 0) {
    // no insert (every member of Q is already in P, as near the top of the
    // order): the output is P with its matched entries min-updated, written
    // contiguously
    for (int k = tl; k < np; k += L) {
      A.slot_nbr[off + k] = pid[k];
      A.slot_w[off + k] = pw[k];
    }
  } else if (fits) {
    // pass 2, branch-free as pass 1: write P's entries and the unmatched Q
    // entries of this lane's stretch
    int o = before + incl - cnt;
    int i = i0, j = k0 - i0;
    int a = i < np ? pid[i] : INT_MAX;
    int b = j < nq ? q_at(aid, iu, j) : INT_MAX;
    int prev = i > 0 ? pid[i - 1] : INT_MIN;
    for (int t = k0; t < k1; t++) {
      const bool tp = a <= b;
      const bool put = tp || prev != b;
      const int wv = tp ? pw[min(i, plast)] : wu + q_at(aw, iu, min(j, qlast));
      if (put) {
        A.slot_nbr[off + Jn + o] = tp ? a : b;
        A.slot_w[off + Jn + o] = wv;
      }
      o += put;
      prev = tp ? a : prev;
      i += tp;
      j += !tp;
      const int na = pid[min(i, plast)];
      const int nb = q_at(aid, iu, min(j, qlast));
      a = i < np ? na : INT_MAX;
      b = j < nq ? nb : INT_MAX;
    }
    for (int k = tl; k < Jn; k += L) A.slot_nbr[off + k] = INT_MAX;
  }
  if (tl == 0) {
    if (!fits) set_err(A.err, kErrOverflow);
    const int ns = fits ? Jn + total : s;
    A.lsize[u] = ns;
    A.ljunk[u] = fits ? Jn : J;
    const int h = m.h;
    const int hn = (hnow + 1 > h) ? hnow + 1 : h;
    A.height[u] = hn;
    const int p = m.p;
    if (p >= 0 && p < nslots) {  // a remaining candidate of this cell: refresh its key
      cand.deg[p] = ns;
      cand.third[p] = hn;
    }
  }
  tsync();  // the buffers are free again
}

// 48 registers: five 8-warp CTAs per SM for the many small cells at the
// bottom (left to itself the compiler takes 56 and fits four)
__global__ void __maxnreg__(48) elim_kernel(ElimArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  cg::cluster_group cluster = cg::this_cluster();
  const int CS = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int cell = A.cell_lo + (int)(blockIdx.x / CS);
  const int start = A.cell_start[cell];
  const int k = A.cell_count[cell];
  if (k == 0) return;  // uniform across the cluster
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int lane = tid & 31, wid = tid >> 5, nw = nthr >> 5;

  // identical layout in every CTA of the cluster; the leader's keys and
  // broadcast words are the shared copies
  unsigned char *sp = smem;
  auto take = [&](int64_t bytes) -> void * {
    bytes = (bytes + 15) & ~int64_t(15);
    void *r = sp;
    sp += bytes;
    return r;
  };
  __shared__ int s_red_sum[32], s_red_deg[32], s_red_id[32], s_red_pos[32];
  __shared__ int s_bc[4];  // v, HeightNow, |own list|, stop
  Cand mine;
  mine.id = (int *)take(sizeof(int) * A.kmax);
  mine.deg = (int *)take(sizeof(int) * A.kmax);
  mine.third = (int *)take(sizeof(int) * A.kmax);
  int *aid = (int *)take(sizeof(int) * A.lmax);
  int *aw = (int *)take(sizeof(int) * A.lmax);
  // this warp's merge buffers: in shared memory, or (lists too long for it)
  // its slab of the global staging; the merge is inlined once for each, so
  // the shared-memory copy uses shared-space loads and stores
  int *const gslab = A.pstage ? A.pstage + ((int64_t)blockIdx.x * nw + wid) * 2 * (int64_t)A.lmax : nullptr;
  int *spid = (int *)smem, *spw = (int *)smem;
  if (!A.pstage) {
    spid = (int *)take(sizeof(int) * A.lmax * nw) + (int64_t)wid * A.lmax;
    spw = (int *)take(sizeof(int) * A.lmax * nw) + (int64_t)wid * A.lmax;
  }
  Cand lead;  // the leader's keys through distributed shared memory
  lead.id = cluster.map_shared_rank(mine.id, 0);
  lead.deg = cluster.map_shared_rank(mine.deg, 0);
  lead.third = cluster.map_shared_rank(mine.third, 0);
  const int *lead_aid = cluster.map_shared_rank(aid, 0);
  const int *lead_aw = cluster.map_shared_rank(aw, 0);
  const int *lead_bc = cluster.map_shared_rank(s_bc, 0);

  if (rank == 0) {
    for (int i = tid; i < k; i += nthr) {
      const int v = A.elim[start + i];
      mine.id[i] = v;
      mine.deg[i] = A.key_deg0[v];
      mine.third[i] = A.key_h0 ? A.key_h0[v] : 0;
      A.cpos[v] = i;
    }
    if (tid == 0) s_bc[3] = 0;
  }
  cluster.sync();

  for (int j = 0; j < k; j++) {
    if (rank == 0) {
      // ---- 1. argmin of (deg + height, deg, id) over candidates [j, k)
      int bs = INT_MAX, bd = INT_MAX, bi = INT_MAX, bp = -1;
      for (int i = j + tid; i < k; i += nthr) {
        const int d = mine.deg[i], t = mine.third[i], id = mine.id[i];
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
        const int v = mine.id[rp];
        const int hn = mine.third[rp];
        if (rp != j) {
          const int u = mine.id[j];
          mine.id[rp] = u; mine.deg[rp] = mine.deg[j]; mine.third[rp] = mine.third[j];
          A.cpos[u] = rp;
          mine.id[j] = v; mine.deg[j] = rd; mine.third[j] = hn;
        }
        A.cpos[v] = -1;
        A.elim[start + j] = v;
        s_bc[0] = v;
        s_bc[1] = hn;
      }
      __syncthreads();
      // ---- 3. own list: valid part is sorted; merge duplicates, drop junk (:338-361)
      const int v = s_bc[0];
      const int64_t voff = __ldcg(A.slot_off + v);
      const int vJ = __ldcg(A.ljunk + v);
      const int sv = __ldcg(A.lsize + v) - vJ;
      if (sv <= A.lmax) {
        for (int i = tid; i < sv; i += nthr) {
          aid[i] = __ldcg(A.slot_nbr + voff + vJ + i);
          aw[i] = __ldcg(A.slot_w + voff + vJ + i);
        }
      }
      __syncthreads();
      bool dup = false;
      if (sv <= A.lmax)
        for (int i = tid + 1; i < sv; i += nthr)
          if (aid[i] == aid[i - 1]) dup = true;
      dup = __syncthreads_or(dup);
      int cn = sv;
      if (dup && sv <= A.lmax && wid == 0) cn = collapse_runs_warp(aid, aw, sv, lane);
      if (tid == 0) {
        if (sv > A.lmax) {
          set_err(A.err, kErrStaging);
          s_bc[3] = 1;
        } else {
          if (cn == 0 && !A.heap_mode) { set_err(A.err, kErrEmpty); s_bc[3] = 1; }
          else { A.lsize[v] = cn; A.ljunk[v] = 0; }
        }
        s_bc[2] = cn;
      }
      __syncthreads();
      const int c = s_bc[2];
      if (!s_bc[3])
        for (int i = tid; i < c; i += nthr) { A.slot_nbr[voff + i] = aid[i]; A.slot_w[voff + i] = aw[i]; }
    }
    cluster.sync();
    // ---- 4. neighbours: every warp of every CTA takes whole lists
    const int v = lead_bc[0], hnow = lead_bc[1], c = lead_bc[2];
    const int stop = lead_bc[3];
    if (!stop) {
      if (rank != 0) {
        for (int i = tid; i < c; i += nthr) { aid[i] = lead_aid[i]; aw[i] = lead_aw[i]; }
        __syncthreads();
      }
      for (int i = rank * nw + wid; i < c; i += CS * nw) {
        const int u = aid[i];
        const NbrMeta m = load_meta(A, u);
        if (m.s - m.J > A.lmax) {
          if (lane == 0) set_err(A.err, kErrStaging);
          continue;
        }
        if (gslab)
          merge_neighbour<false>(A, u, m, aw[i], i, v, hnow, aid, aw, c, gslab, gslab + A.lmax, lane, lead, k);
        else
          merge_neighbour<false>(A, u, m, aw[i], i, v, hnow, aid, aw, c, spid, spw, lane, lead, k);
      }
    }
    cluster.sync();  // no CTA leaves while a peer may still read the leader's shared memory
    if (stop) return;
    // ---- 5. after the first pick of a partition cell every key becomes live (:471-475)
    if (rank == 0 && j == 0 && !A.heap_mode) {
      for (int i = 1 + tid; i < k; i += nthr) {
        const int u = mine.id[i];
        mine.deg[i] = __ldcg(A.lsize + u);
        mine.third[i] = __ldcg(A.height + u);
      }
      __syncthreads();
    }
  }
}

// Elimination over all SMs: one cooperative launch runs one or more cells,
// each on its own range of blocks (one block per SM), without the cluster
// kernel's limit of 16 SMs per cell.  The few large cells near the top of the
// partition, and the global orders (one per graph), are long chains of
// eliminations whose neighbour merges want more SMs than that.
//
// Ownership: block r of a cell's nb blocks owns the vertices u with
// owner_of(u, nb) == r (a scrambled id mod nb).  It keeps the keys of the
// candidates it owns in shared memory (their slots in cpos), refreshes their
// keys and retires its picked candidate; the argmin of its candidates reads
// only shared memory.
// Per elimination:
//   every block of the cell reduces the cell's per-block argmins to the same
//   pick v (the key order is strict; the pick's height is its sum minus its
//   degree); the first block records it and writes back the previous pick's
//   compacted list (nobody reads that list any more); every block loads and
//   compacts v's list into its shared memory (the same code as the cluster
//   leader) and merges a share of v's neighbours: the ones it owns (their
//   keys updated in place), or -- in cells of 16+ blocks with at least two
//   merges per block -- an even range of v's list, a merge of a neighbour
//   owned elsewhere counting on the owner's counter, each owner waiting for
//   its count and then taking its candidates' keys from the merged lists;
//   then it publishes the argmin of its candidates            -- cell barrier
// Within a block, warps take merges from a shared counter (longest list
// first when they outnumber the warps, or teams of 2-4 warps per merge when
// they are few), with buffers cut from a shared-memory arena per pick.
// The cell barrier is a monotonic arrival counter in global memory (barrier
// t completes when it reaches t * nb); the launch is cooperative, so every
// block is resident, and a wait is bounded (the block records kErrTimeout and
// leaves).  Cells never wait on one another.  Same key order, list rules and
// results as the cluster kernel in both modes: partition cells take the
// first pick on stale keys and then refresh every key from the live lists; a
// global order has live keys from the start and lets lists run empty.
struct GridArgs {
  ElimArgs E;              // cell_lo = the launch's first cell; pstage, when set, holds the per-warp merge buffers
  const int *blk_cell;     // block -> cell of the launch (0-based)
  const int *cell_blk0;    // cell -> its first block; entry ncell = the block count
  int slice_max;           // most candidates one block owns (shared-memory key slots)
  int4 *partial;           // (deg + height, deg, id, slot) per block
  unsigned *bar;           // per cell: arrival counter
  long long spin_limit;    // bound on one barrier wait, in SM clock cycles
  int arena_ints;          // ints of shared memory handed out afresh at every pick (the owned-neighbour list first)
  int arena_merges;        // merges take their buffers from the arena (else from E.pstage)
  unsigned *done_cnt;      // per block: merges of the neighbours it owns finished in this pick (balance)
  int balance;             // split each pick's merges over the cell's blocks by work, not by owner
};

__device__ __forceinline__ void better(int &bs, int &bd, int &bi, int &bp, int s, int d, int i, int p) {
  if (p >= 0 && (bp < 0 || key_less(s, d, i, bs, bd, bi))) { bs = s; bd = d; bi = i; bp = p; }
}

// Block-wide argmin of (s, d, i, p) tuples; the result is valid in thread 0.
__device__ __forceinline__ void block_best(int &bs, int &bd, int &bi, int &bp, int *rs, int *rd, int *ri, int *rp) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    const int os = __shfl_down_sync(0xffffffffu, bs, o), od = __shfl_down_sync(0xffffffffu, bd, o);
    const int oi = __shfl_down_sync(0xffffffffu, bi, o), op = __shfl_down_sync(0xffffffffu, bp, o);
    better(bs, bd, bi, bp, os, od, oi, op);
  }
  if (lane == 0) { rs[wid] = bs; rd[wid] = bd; ri[wid] = bi; rp[wid] = bp; }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int w = 1; w < nw; w++) better(bs, bd, bi, bp, rs[w], rd[w], ri[w], rp[w]);
}

// The block of a cell's nb blocks that owns vertex u.  Ids are scrambled
// first (the murmur3 finaliser): separator vertices of a grid-like graph are
// often evenly spaced ids, and a plain u mod nb would pile them onto a few
// blocks.
__host__ __device__ __forceinline__ int owner_of(int u, int nb) {
  unsigned x = (unsigned)u;
  x ^= x >> 16;
  x *= 0x85ebca6bu;
  x ^= x >> 13;
  x *= 0xc2b2ae35u;
  x ^= x >> 16;
  return (int)(x % (unsigned)nb);
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Barrier t (target = t * nb) over the nb blocks of one cell.  False when the
// wait ran out or another block recorded an error: the caller leaves.
__device__ bool cell_barrier(unsigned *cnt, int nb, unsigned target, long long limit, int *err, int *s_flag) {
  __syncthreads();
  if (nb == 1) return true;
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();  // this block's writes before its arrival
    if (atomicAdd(cnt, 1u) + 1u == target) {
      __threadfence();  // the other blocks' writes
    } else {
      const long long t0 = clock64();
      while ((int)(ld_acquire_u32(cnt) - target) < 0) {
        if (*(volatile int *)err != 0) { ok = 0; break; }
        if (clock64() - t0 > limit) { set_err(err, kErrTimeout); ok = 0; break; }
      }
    }
    *s_flag = ok;
  }
  __syncthreads();
  return *s_flag != 0;
}

__global__ void __launch_bounds__(512, 1) cell_grid_kernel(GridArgs H) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_rs[32], s_rd[32], s_ri[32], s_rp[32];
  __shared__ int s_bc[4];  // v, height of the pick, |own list|, stop
  __shared__ int4 s_best;  // this block's argmin (a one-block cell reads it here)
  __shared__ int s_nmine, s_nslot, s_flag, s_ntake;
  const ElimArgs &A = H.E;
  const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = nthr >> 5;
  const int b = blockIdx.x;
  const int q = H.blk_cell[b];
  const int f = H.cell_blk0[q], nb = H.cell_blk0[q + 1] - f, r = b - f;
  const int start = A.cell_start[A.cell_lo + q], k = A.cell_count[A.cell_lo + q];
  if (k == 0) return;  // the whole cell leaves; nobody waits on its barrier
  unsigned *bar = H.bar + q;
  unsigned bar_target = 0;
  const int4 *partial = H.partial + f;
  const int lal = (A.lmax + 3) & ~3, sal = (H.slice_max + 3) & ~3;
  int *aid = (int *)smem;
  int *aw = aid + lal;
  int *cid = aw + lal;     // the candidates this block owns: id, degree key, height key, retired
  int *cdeg = cid + sal;
  int *ch = cdeg + sal;
  int *dead = ch + sal;
  // this warp's merge buffers: a pair sized to the list, cut from a
  // shared-memory arena that is handed out afresh at every pick, or its own
  // slab in global memory when the arena has no room left (a merge then
  // reads global memory, one round trip per step of a walk).  The merge is
  // inlined twice, so the shared-memory copy addresses its buffers as
  // shared memory (shared-space loads, not generic ones).
  if (A.pstage == nullptr) {  // the host always provides the global slabs
    if (tid == 0 && r == 0) set_err(A.err, kErrStaging);
    return;
  }
  int *const sbuf = dead + sal;
  int *const gpid = A.pstage + ((int64_t)b * nw + wid) * 2 * (int64_t)A.lmax;
  const bool pooled = H.arena_merges != 0;
  __shared__ int s_arena;  // pooled: arena ints taken in this pick
  __shared__ int s_team[16 * 12];  // per warp team: merge_neighbour's exchange, then the team's pair and ticket
  Cand cand;
  cand.id = cid;
  cand.deg = cdeg;
  cand.third = ch;
  // the candidates this block owns, with the first pick's keys (stale for a
  // partition cell, prepared for a global order)
  if (tid == 0) s_nslot = 0;
  __syncthreads();
  for (int i = tid; i < k; i += nthr) {
    const int v = A.elim[start + i];
    if (owner_of(v, nb) == r) {
      const int t = atomicAdd(&s_nslot, 1);
      if (t < H.slice_max) {
        cid[t] = v;
        cdeg[t] = A.key_deg0[v];
        ch[t] = A.key_h0 ? A.key_h0[v] : 0;
        dead[t] = 0;
        A.cpos[v] = t;
      }
    }
  }
  __syncthreads();
  const int ns = s_nslot;
  if (ns > H.slice_max) {  // the host sized the slots from the same vertex set
    if (tid == 0) set_err(A.err, kErrPick);
    return;
  }
  auto slice_best = [&]() {
    int bs = INT_MAX, bd = INT_MAX, bi = INT_MAX, bp = -1;
    for (int t = tid; t < ns; t += nthr)
      if (!dead[t]) better(bs, bd, bi, bp, cdeg[t] + ch[t], cdeg[t], cid[t], t);
    block_best(bs, bd, bi, bp, s_rs, s_rd, s_ri, s_rp);
    if (tid == 0) {
      s_best = make_int4(bs, bd, bi, bp);
      if (nb > 1) H.partial[b] = s_best;
    }
  };
  slice_best();
  bar_target += nb;
  if (!cell_barrier(bar, nb, bar_target, H.spin_limit, A.err, &s_flag)) return;
  int prev_v = -1, prev_c = 0;
  for (int j = 0; j < k; j++) {
    // ---- the pick
    {
      int bs = INT_MAX, bd = INT_MAX, bi = INT_MAX, bp = -1;
      if (nb == 1) {
        if (tid == 0) { bs = s_best.x; bd = s_best.y; bi = s_best.z; bp = s_best.w; }
      } else {
        for (int g = tid; g < nb; g += nthr) {
          const int4 t = __ldcg(partial + g);
          better(bs, bd, bi, bp, t.x, t.y, t.z, t.w);
        }
        block_best(bs, bd, bi, bp, s_rs, s_rd, s_ri, s_rp);
      }
      if (tid == 0) {
        s_nmine = 0;
        s_ntake = 0;
        s_bc[3] = bp < 0;  // j < k candidates remain, so a pick exists
        if (bp >= 0) {
          s_bc[0] = bi;
          s_bc[1] = bs - bd;
          if (r == 0) A.elim[start + j] = bi;
          if (owner_of(bi, nb) == r) {  // the owner retires the candidate
            dead[bp] = 1;
            A.cpos[bi] = -1;
          }
        } else if (r == 0) {
          set_err(A.err, kErrPick);
        }
      }
    }
    // the first block: the previous pick's list, read by nobody since the barrier
    if (r == 0 && prev_v >= 0) {
      const int64_t off = __ldcg(A.slot_off + prev_v);
      for (int i = tid; i < prev_c; i += nthr) { A.slot_nbr[off + i] = aid[i]; A.slot_w[off + i] = aw[i]; }
      if (tid == 0) { A.lsize[prev_v] = prev_c; A.ljunk[prev_v] = 0; }
    }
    __syncthreads();
    if (s_bc[3]) return;  // the same partials in every block of the cell: all leave
    const int v = s_bc[0], hnow = s_bc[1];
    const int64_t voff = __ldcg(A.slot_off + v);
    const int vJ = __ldcg(A.ljunk + v);
    const int sv = __ldcg(A.lsize + v) - vJ;
    if (sv > A.lmax) {  // every block of the cell sees the same sizes: all leave
      if (r == 0 && tid == 0) set_err(A.err, kErrStaging);
      return;
    }
    // ---- v's own list, valid part (every block the same copy): merge
    // duplicates, drop junk (kernel_functions.cu:338-361)
    for (int i = tid; i < sv; i += nthr) {
      aid[i] = __ldcg(A.slot_nbr + voff + vJ + i);
      aw[i] = __ldcg(A.slot_w + voff + vJ + i);
    }
    __syncthreads();
    bool dup = false;
    for (int i = tid + 1; i < sv; i += nthr)
      if (aid[i] == aid[i - 1]) dup = true;
    dup = __syncthreads_or(dup);
    int cn = sv;
    if (dup && wid == 0) cn = collapse_runs_warp(aid, aw, sv, lane);
    if (tid == 0) {
      if (cn == 0 && !A.heap_mode) {  // a partition cell never eliminates an isolated vertex
        if (r == 0) set_err(A.err, kErrEmpty);
        s_bc[3] = 1;
      }
      s_bc[2] = cn;
    }
    __syncthreads();
    if (s_bc[3]) return;
    const int c = s_bc[2];
    // balance: block r merges v's neighbours [r c / nb, (r + 1) c / nb) --
    // the same split in every block, from c and nb alone (the list sizes
    // change under other blocks' merges, so they cannot set it) -- and a
    // merge of a neighbour owned by another block counts on that owner's
    // counter; each owner takes its candidates' keys from the merged lists
    // once its count is in.  Every block then has c / nb merges, few enough
    // in a global order for warp teams.  Only cells of 16 or more blocks
    // and picks with at least two merges per block: elsewhere (the partition
    // levels of many cells, the short lists of a small graph's global order)
    // the owners' waits cost more than the split gains.  Otherwise a block
    // merges the neighbours it owns.
    const bool bal = H.balance != 0 && nb >= 16 && c >= 2 * nb;
    int lo_r = 0, hi_r = 0, cnt_own = 0;
    if (bal) {
      lo_r = (int)((int64_t)r * c / nb);
      hi_r = (int)((int64_t)(r + 1) * c / nb);
      int own = 0;
      for (int i = tid; i < c; i += nthr) own += owner_of(aid[i], nb) == r;
      for (int o = 16; o > 0; o >>= 1) own += __shfl_xor_sync(0xffffffffu, own, o);
      if (lane == 0) s_rd[wid] = own;
      __syncthreads();
      for (int w = 0; w < nw; w++) cnt_own += s_rd[w];
    }
    // the arena starts with this pick's list of the neighbours this block
    // merges (indices into aid, at most c), then room to order them by list
    // length; every merge of the last pick ended before the barrier
    const int c4 = (c + 3) & ~3;
    const bool room = 3 * c4 <= H.arena_ints;
    int *const mine = sbuf;
    int *const mlen = mine + c4;
    int *const order = mine + 2 * c4;
    if (tid == 0) s_arena = c4;
    // ---- the neighbours this block merges
    if (bal) {
      for (int t = tid; t < hi_r - lo_r; t += nthr) mine[t] = lo_r + t;
      if (tid == 0) s_nmine = hi_r - lo_r;
    } else {
      for (int i = tid; i < c; i += nthr)
        if (owner_of(aid[i], nb) == r) mine[atomicAdd(&s_nmine, 1)] = i;
    }
    __syncthreads();
    const int nm = s_nmine;
    // more merges than warps: hand them out longest list first, so a long
    // merge does not start last (the block's merges end with its slowest
    // warp, and the cell's step with its slowest block); the order changes
    // no result
    const bool lpt = room && nm > nw;
    if (lpt) {
      if (tid == 0) s_arena = 3 * c4;  // the merges start after the barriers below
      for (int t = tid; t < nm; t += nthr) {
        const int u = aid[mine[t]];  // merged by this block alone: its size is this pick's
        mlen[t] = __ldcg(A.lsize + u) - __ldcg(A.ljunk + u);
      }
      __syncthreads();
      for (int t = tid; t < nm; t += nthr) {
        const int lt = mlen[t];
        int rk = 0;
        for (int o = 0; o < nm; o++) {
          const int lo = mlen[o];
          rk += (lo > lt) || (lo == lt && o < t);
        }
        order[rk] = mine[t];
      }
      __syncthreads();
    }
    const int *const todo = lpt ? order : mine;
    // fewer merges than a quarter (a half) of the warps, as in a global
    // order: teams of 4 (2) warps share each merge, so the step's longest
    // merge runs on more lanes (team size, like nm, is the same in every warp
    // of the block)
    const int T = !pooled ? 1 : 4 * nm <= nw ? 4 : 2 * nm <= nw ? 2 : 1;
    if (T > 1) {
      const int team = wid / T, tw = wid - team * T, bid = 1 + team;
      int *const tsh = s_team + 12 * team;
      int *const tg = A.pstage + ((int64_t)b * nw + team * T) * 2 * (int64_t)A.lmax;  // the first warp's slab
      int tbase = 0, tcap = 0;  // the team's arena pair, held by its first warp
      for (;;) {
        // the first warp takes the ticket and, when the list outgrows the
        // team's pair, a new pair from the arena; the team reads both after
        // the barrier
        if (tw == 0) {
          int t = 0;
          if (lane == 0) t = atomicAdd(&s_ntake, 1);
          t = __shfl_sync(0xffffffffu, t, 0);
          if (t < nm) {
            const int u = aid[todo[t]];
            const int len = __ldcg(A.lsize + u) - __ldcg(A.ljunk + u);
            if (len <= A.lmax && len > tcap) {
              const int want = (len + 3) & ~3;
              const int at = arena_take(&s_arena, H.arena_ints, 2 * want, lane);
              if (at >= 0) {
                tbase = at;
                tcap = want;
              }
            }
          }
          if (lane == 0) {
            tsh[8] = tbase;
            tsh[9] = tcap;
            tsh[10] = t;
          }
        }
        asm volatile("bar.sync %0, %1;" ::"r"(bid), "r"(32 * T) : "memory");
        const int t = tsh[10], sb = tsh[8], scp = tsh[9];
        if (t >= nm) break;
        const int i = todo[t];
        const int u = aid[i];
        const NbrMeta m = load_meta(A, u);
        if (m.s - m.J > A.lmax) {  // the same m in every warp of the team
          if (tw == 0 && lane == 0) set_err(A.err, kErrStaging);
          // every warp has read the ticket before the first warp takes the next
          asm volatile("bar.sync %0, %1;" ::"r"(bid), "r"(32 * T) : "memory");
          continue;
        }
        // balance: the owner takes the keys from the merged list (nslots 0)
        if (m.s - m.J <= scp)
          merge_neighbour<true, true>(A, u, m, aw[i], i, v, hnow, aid, aw, c, sbuf + sb, sbuf + sb + scp, lane, cand,
                                      bal ? 0 : ns, T, tw, bid, tsh);
        else
          merge_neighbour<true, true>(A, u, m, aw[i], i, v, hnow, aid, aw, c, tg, tg + A.lmax, lane, cand,
                                      bal ? 0 : ns, T, tw, bid, tsh);
        if (bal && tw == 0 && lane == 0) {  // the team's writes precede (the merge ends at a team barrier)
          __threadfence();
          atomicAdd(H.done_cnt + f + owner_of(u, nb), 1u);
        }
      }
    }
    int wbase = 0, wcap = 0;  // this warp's arena pair in this pick
    // warps take the block's neighbours one at a time as they finish, so a
    // few long lists do not hold the block (and the cell's barrier) back
    for (; T == 1;) {
      int t = 0;
      if (lane == 0) t = atomicAdd(&s_ntake, 1);
      t = __shfl_sync(0xffffffffu, t, 0);
      if (t >= nm) break;
      const int i = todo[t];
      const int u = aid[i];
      const NbrMeta m = load_meta(A, u);
      if (m.s - m.J > A.lmax) {
        if (lane == 0) set_err(A.err, kErrStaging);
        continue;
      }
      int *sp = sbuf, scap = 0;
      bool in_smem = false;
      if (pooled) {
        const int len = m.s - m.J;
        if (len > wcap) {  // a fresh pair from the arena (the warp's old one stays unused)
          const int want = (len + 3) & ~3;
          const int at = arena_take(&s_arena, H.arena_ints, 2 * want, lane);
          if (at >= 0) {
            wbase = at;
            wcap = want;
          }
        }
        if (len <= wcap) {
          sp = sbuf + wbase;
          scap = wcap;
          in_smem = true;
        }
      }
      if (in_smem)
        merge_neighbour<true>(A, u, m, aw[i], i, v, hnow, aid, aw, c, sp, sp + scap, lane, cand, bal ? 0 : ns);
      else
        merge_neighbour<true>(A, u, m, aw[i], i, v, hnow, aid, aw, c, gpid, gpid + A.lmax, lane, cand,
                              bal ? 0 : ns);
      if (bal && lane == 0) {  // the warp's writes precede (the merge ends at __syncwarp)
        __threadfence();
        atomicAdd(H.done_cnt + f + owner_of(u, nb), 1u);
      }
    }
    __syncthreads();
    if (bal) {
      // every merge of a neighbour this block owns is done once its count is
      // in (every block merges its range before it waits here, so the waits
      // end); then the keys of its candidates among v's neighbours come from
      // the sizes and heights those merges wrote, and the count is cleared
      // for the next pick (the next increments follow the cell barrier)
      if (tid == 0) {
        unsigned *const cnt = H.done_cnt + b;
        const long long t0 = clock64();
        int ok = 1;
        while ((int)(ld_acquire_u32(cnt) - (unsigned)cnt_own) < 0) {
          if (*(volatile int *)A.err != 0) { ok = 0; break; }
          if (clock64() - t0 > H.spin_limit) { set_err(A.err, kErrTimeout); ok = 0; break; }
        }
        *cnt = 0u;
        s_flag = ok;
      }
      __syncthreads();
      if (!s_flag) return;
      for (int i = tid; i < c; i += nthr) {
        const int u = aid[i];
        if (owner_of(u, nb) == r) {
          const int p = __ldcg(A.cpos + u);
          if (p >= 0 && p < ns) {
            cdeg[p] = __ldcg(A.lsize + u);
            ch[p] = __ldcg(A.height + u);
          }
        }
      }
      __syncthreads();
    }
    // ---- after the first pick of a partition cell every key becomes live
    // (kernel_functions.cu:471-475); this block alone wrote its candidates' lists
    if (j == 0 && !A.heap_mode) {
      for (int t = tid; t < ns; t += nthr)
        if (!dead[t]) {
          const int u = cid[t];
          cdeg[t] = __ldcg(A.lsize + u);
          ch[t] = __ldcg(A.height + u);
        }
      __syncthreads();
    }
    // ---- the argmin of this block's candidates, keys final
    slice_best();
    prev_v = v;
    prev_c = c;
    bar_target += nb;
    if (!cell_barrier(bar, nb, bar_target, H.spin_limit, A.err, &s_flag)) return;
  }
  if (r == 0 && prev_v >= 0) {
    const int64_t off = __ldcg(A.slot_off + prev_v);
    for (int i = tid; i < prev_c; i += nthr) { A.slot_nbr[off + i] = aid[i]; A.slot_w[off + i] = aw[i]; }
    if (tid == 0) { A.lsize[prev_v] = prev_c; A.ljunk[prev_v] = 0; }
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

// Lists of the heap vertices as uploadCHset builds them (Traditional_H2H.cu:
// 43-75): valid entries in list order, first-seen entry of a duplicated
// neighbour kept; key = (number of valid entries, duplicates included;
// height).  One warp per vertex.
__global__ void prepare_heap_lists_kernel(const int *verts, int nv, const int64_t *slot_off, int *slot_nbr,
                                          int *slot_w, int *lsize, int *ljunk, const int *height, int *key_deg,
                                          int *key_h) {
  const int lane = threadIdx.x & 31;
  for (int64_t t = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; t < nv;
       t += (gridDim.x * (int64_t)blockDim.x) >> 5) {
    const int v = verts[t];
    const int64_t off = slot_off[v];
    const int J = ljunk[v], s = lsize[v];
    int c = 0;
    for (int base = J; base < s; base += 32) {
      const int idx = base + lane;
      int x = INT_MAX, w = 0, prev = INT_MIN;
      if (idx < s) {
        x = slot_nbr[off + idx];
        w = slot_w[off + idx];
        if (idx > J) prev = slot_nbr[off + idx - 1];
      }
      __syncwarp();
      const bool keep = idx < s && x != prev;
      const unsigned bal = __ballot_sync(0xffffffffu, keep);
      if (keep) {  // compaction never overtakes an unread entry: target <= source
        const int pos = c + __popc(bal & ((1u << lane) - 1u));
        slot_nbr[off + pos] = x;
        slot_w[off + pos] = w;
      }
      c += __popc(bal);
      __syncwarp();
    }
    if (lane == 0) {
      key_deg[v] = s - J;
      key_h[v] = height[v];
      lsize[v] = c;
      ljunk[v] = 0;
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

// rank[v] = position of v in the elimination order.
__global__ void rank_kernel(const int *elim, int *rank, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) rank[elim[i]] = i;
}

// father = the member of X(v) eliminated first (getTreeStructure,
// TreeStructure.cu:431-473: min rank over v's upper neighbours; -1 for the
// last vertex).  One warp per vertex; ranks are distinct.
__global__ void father_kernel(const int64_t *off, const int *id, const int *rank, int *father, int n) {
  const int lane = threadIdx.x & 31;
  for (int64_t v = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; v < n;
       v += (gridDim.x * (int64_t)blockDim.x) >> 5) {
    int best = INT_MAX, bid = -1;
    for (int64_t k = off[v] + lane; k < off[v + 1]; k += 32) {
      const int a = id[k], r = rank[a];
      if (r < best) { best = r; bid = a; }
    }
    const int m = __reduce_min_sync(0xffffffffu, best);
    const unsigned who = __ballot_sync(0xffffffffu, best == m && bid >= 0);
    const int f = who ? __shfl_sync(0xffffffffu, bid, __ffs(who) - 1) : -1;
    if (lane == 0) father[v] = f;
  }
}

// Device lists of a contraction (owned through ListStore::keep).
struct ListArrays {
  int64_t *off = nullptr;
  int *id = nullptr, *w = nullptr;
  ~ListArrays() {
    cudaFree(off);
    cudaFree(id);
    cudaFree(w);
  }
};

template <typename T>
T *dalloc(size_t n) {
  T *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc(&p, n * sizeof(T));
  if (e != cudaSuccess) throw Error(H2H_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  return p;
}

}  // namespace

namespace {

// Where a graph's global order starts: the vertices of the cells at levels
// C..1 (the tail of elim).
struct GraphLevels {
  int heap_start = 0, heap_n = 0;
};

GraphLevels graph_levels(const Graph &g) {
  GraphLevels L;
  int64_t heap_start = INT32_MAX;
  for (int h = g.C; h > 0; h--) {
    const int64_t lo = (int64_t(1) << (h - 1)) - 1, hi = (int64_t(1) << h) - 2;
    for (int64_t c = hi; c >= lo; c--) heap_start = std::min<int64_t>(heap_start, g.cell_start[c]);
  }
  GH_CHECK(heap_start != INT32_MAX, H2H_ERR_ARG, "ChangeToGlobalHeight must be >= 1");
  L.heap_start = (int)heap_start;
  L.heap_n = g.n - (int)heap_start;
  return L;
}

template <typename T>
T *palloc(size_t n, int64_t &bytes) {
  T *p = dalloc<T>(n);
  bytes += (int64_t)(std::max<size_t>(n, 1) * sizeof(T));
  return p;
}

}  // namespace

ElimPlan::ElimPlan(const std::vector<Graph *> &graphs) : gs(graphs) {
  const int K = (int)gs.size();
  GH_CHECK(K >= 1, H2H_ERR_ARG, "no graph to contract");
  const bool force_global_stage = std::getenv("GPUH2H_GLOBAL_STAGING") != nullptr;
  // with global staging, the shared memory left over is an arena of merge
  // buffers (GPUH2H_GRID_ARENA: 0 = every merge stages in global memory,
  // 1 = partition levels only, 2 = the global order too)
  int grid_arena = 2;
  if (const char *e = std::getenv("GPUH2H_GRID_ARENA")) grid_arena = std::max(0, std::min(2, std::atoi(e)));
  // cooperative steps: split each pick's merges over the cell's blocks by
  // work (GPUH2H_ELIM_BALANCE=0: each block merges the neighbours it owns)
  if (const char *e = std::getenv("GPUH2H_ELIM_BALANCE")) elim_balance = std::atoi(e) != 0;

  // cell list bounds come with the elimination sets (build_elimination_sets)
  std::vector<GraphLevels> L(K);
  int threads = 1;
  for (const Graph *g : gs) {
    threads = std::max(threads, g->threads);
    GH_CHECK(g->cell_bound.size() == g->cell_start.size(), H2H_ERR_STATE, "elimination sets not built");
  }
  for (int i = 0; i < K; i++) L[i] = graph_levels(*gs[i]);
  std::vector<int64_t> lbase(K);
  vbase.assign(K, 0);
  mbase.assign(K, 0);
  int64_t pool_extra = 1024;
  for (int i = 0; i < K; i++) {
    Graph &g = *gs[i];
    vbase[i] = N;
    mbase[i] = M;
    lbase[i] = lub;
    GH_CHECK((int64_t)N + g.n < INT32_MAX, H2H_ERR_ARG, "too many vertices in one batch");
    N += g.n;
    M += g.m;
    lub += g.lub;
    heap_total += L[i].heap_n;
    pool_extra += (int64_t)L[i].heap_n * std::min(L[i].heap_n, 8192);
    g.gpu_vertices = L[i].heap_start;
  }
  GH_CHECK(M < INT32_MAX, H2H_ERR_ARG, "too many arcs in one batch");
  // slot arrays: the LUB ranges, then a pool for global-order lists that
  // outgrow theirs
  pool_size = lub + pool_extra;
  // ---- forest arrays (written in full below, so not zero-filled first)
  std::vector<int64_t, NoInit<int64_t>> f_slot_off(N);
  std::vector<int, NoInit<int>> f_deg(N), f_cap(N), f_elim(N), f_adj_off(N + 1), f_adj_v(std::max<int64_t>(M, 1)),
      f_adj_w(std::max<int64_t>(M, 1)), f_heap(std::max(heap_total, 1));
  f_adj_v[0] = f_adj_w[0] = f_heap[0] = 0;  // defined when there is nothing to copy
  {
    std::vector<int> hbase(K, 0);
    for (int i = 1; i < K; i++) hbase[i] = hbase[i - 1] + L[i - 1].heap_n;
    auto verts = [&](int i, int64_t lo, int64_t hi) {
      const Graph &g = *gs[i];
      const int vb = vbase[i];
      for (int64_t v = lo; v < hi; v++) {
        f_slot_off[vb + v] = g.slot_off[v] + lbase[i];
        f_deg[vb + v] = g.adj_off[v + 1] - g.adj_off[v];
        f_cap[vb + v] = g.cap[v];
        f_elim[vb + v] = g.elim[v] + vb;
        f_adj_off[vb + v] = g.adj_off[v] + (int)mbase[i];
      }
    };
    auto arcs = [&](int i, int64_t lo, int64_t hi) {
      const Graph &g = *gs[i];
      const int vb = vbase[i];
      for (int64_t e = lo; e < hi; e++) {
        f_adj_v[mbase[i] + e] = g.adj_v[e] + vb;
        f_adj_w[mbase[i] + e] = g.adj_w[e];
      }
    };
    auto heap = [&](int i) {
      const Graph &g = *gs[i];
      for (int j = L[i].heap_start; j < g.n; j++) f_heap[hbase[i] + j - L[i].heap_start] = g.elim[j] + vbase[i];
    };
    Pool pool(threads);
    if (K >= threads) {  // a batch: a graph per task
      pool.parallel_for(K, 1, [&](int64_t lo, int64_t hi, int) {
        for (int64_t i = lo; i < hi; i++) {
          verts((int)i, 0, gs[i]->n);
          arcs((int)i, 0, gs[i]->m);
          heap((int)i);
        }
      });
    } else {  // few graphs: ranges of each graph's vertices and arcs per task
      for (int i = 0; i < K; i++) {
        pool.parallel_for(gs[i]->n, 1 << 16, [&](int64_t lo, int64_t hi, int) { verts(i, lo, hi); });
        pool.parallel_for(gs[i]->m, 1 << 17, [&](int64_t lo, int64_t hi, int) { arcs(i, lo, hi); });
        heap(i);
      }
    }
  }
  f_adj_off[N] = (int)M;
  // ---- launches.  Step s takes level H_i - s of every graph still above
  // C_i; the last step takes every graph's global order as one cell per
  // graph.  Within a step, cells are grouped by size class, each group is a
  // launch with its own cluster size (a large cell spreads its merges over up
  // to 16 CTAs), and the groups of a step run side by side on forked streams.
  // A step with few cells (or the global orders) instead runs as one
  // cooperative launch of cell_grid_kernel over all SMs.
  const int smem_dyn = enable_max_dynamic_smem(elim_kernel);
  const int smem_dyn_g = enable_max_dynamic_smem(cell_grid_kernel);
  const bool force_cluster = std::getenv("GPUH2H_CLUSTER_HEAP") != nullptr;
  GH_CUDA(cudaFuncSetAttribute(elim_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  int dev = 0;
  GH_CUDA(cudaGetDevice(&dev));
  GH_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  struct Cell {
    int start, count, lbound, cls;
  };
  auto size_class = [](int size) {
    return size >= 1024 ? 4 : size >= 512 ? 3 : size >= 256 ? 2 : size >= 128 ? 1 : 0;
  };
  std::vector<std::vector<Cell>> step_cells;
  std::vector<int> step_level;
  int steps = 0;
  for (int i = 0; i < K; i++) steps = std::max(steps, gs[i]->H - gs[i]->C);
  for (int st = 0; st < steps; st++) {
    std::vector<Cell> cells;
    int level = 0;
    for (int i = 0; i < K; i++) {
      const Graph &g = *gs[i];
      const int h = g.H - st;
      if (h <= g.C) continue;
      level = h;
      const int64_t lo = (int64_t(1) << (h - 1)) - 1, hi = (int64_t(1) << h) - 2;
      for (int64_t c = lo; c <= hi; c++) {
        const int cnt = g.cell_count[c], lb = g.cell_bound[c];
        cells.push_back({vbase[i] + g.cell_start[c], cnt, lb, size_class(std::max(cnt, lb))});
      }
    }
    if (cells.empty()) continue;
    step_cells.push_back(std::move(cells));
    step_level.push_back(K > 1 ? -(st + 1) : level);  // a step, not one graph's level
  }
  {
    std::vector<Cell> cells;
    for (int i = 0; i < K; i++)
      cells.push_back({vbase[i] + L[i].heap_start, L[i].heap_n, std::max(1, L[i].heap_n - 1),
                       size_class(L[i].heap_n)});
    step_cells.push_back(std::move(cells));
    step_level.push_back(0);
  }
  const int nsteps = (int)step_cells.size();
  std::vector<int> fcs, fcc;
  auto al = [](int64_t bb) { return (bb + 15) & ~int64_t(15); };
  int64_t pstage_ints = 0, partial_max = 0;
  std::vector<int> gmap;
  // Whole-step cooperative launch: one block per SM, for steps of at most
  // nsm / 2 cells (GPUH2H_GRID_CELLS overrides), where a cell gets two SMs
  // or more -- the cluster kernel caps a cell at 16 CTAs, and long lists
  // leave its CTAs room for only a few warps.  Measured on road graphs
  // against clusters: a single graph's global order 54 -> 33 ms (264k
  // vertices); the 3.6M-vertex graph's partition levels 1.78 -> 1.21 s
  // (level 3, 4 cells: 923 -> 474 ms; level 5, 16 cells: 379 -> 285 ms); a
  // 64-graph batch's partition steps 132 -> 123 ms and global orders 49 ->
  // 42 ms; steps of more cells than that ran slower.  Blocks go to cells
  // greedily by an estimate of the chain time, eliminations x (1 + merge
  // rounds x list length), merge rounds ~ 2 x list bound / warps.
  auto grid_launch = [&](const std::vector<Cell> &cells, int st, bool heap) -> bool {
    const int ncell = (int)cells.size();
    int max_cells = std::max(1, nsm / 2);
    if (const char *e = std::getenv("GPUH2H_GRID_CELLS")) max_cells = std::atoi(e);
    if (force_cluster || ncell > nsm || ncell > max_cells) return false;
    int lmax = 1, kmax = 1;
    for (const Cell &c : cells) {
      lmax = std::max(lmax, c.lbound);
      kmax = std::max(kmax, c.count);
    }
    // blocks per cell (16 warps each; the estimate only ranks cells)
    std::vector<int> nb(ncell, 1);
    auto est = [&](int c, int b) {
      const double lb = cells[c].lbound;
      return cells[c].count * (1.0 + std::max(1.0, 2.0 * lb / ((double)b * 16)) * (1.0 + lb / 256.0));
    };
    std::priority_queue<std::pair<double, int>> pq;
    for (int c = 0; c < ncell; c++) pq.push({est(c, 1), c});
    int used = ncell;
    while (used < nsm && !pq.empty()) {
      const auto [e, c] = pq.top();
      pq.pop();
      if (est(c, nb[c] + 1) >= e) continue;  // more blocks would not shorten this chain
      nb[c]++;
      used++;
      pq.push({est(c, nb[c]), c});
    }
    // candidate slots: block r of cell c owns the cell's vertices v with owner_of(v, nb) == r
    int slice_max = 1;
    {
      std::vector<int> cnt;
      for (int c = 0; c < ncell; c++) {
        cnt.assign(nb[c], 0);
        for (int i = 0; i < cells[c].count; i++) cnt[owner_of(f_elim[cells[c].start + i], nb[c])]++;
        for (int x : cnt) slice_max = std::max(slice_max, x);
      }
      int64_t arrivals = 0;
      for (int c = 0; c < ncell; c++) arrivals = std::max<int64_t>(arrivals, (int64_t)(cells[c].count + 1) * nb[c]);
      if (arrivals >= INT32_MAX) return false;  // the barrier counter compares as int
    }
    const int64_t own = 2 * al(4LL * lmax) + 4 * al(4LL * slice_max);
    if (own + al(4LL * lmax) > smem_dyn_g) return false;  // the arena holds at least the owned-neighbour list
    // 16 warps; the shared memory left over is an arena that each pick
    // carves into the pick's hash table, the warps' match bitmaps and buffer
    // pairs sized to the lists merged (near the top of the order a block
    // runs a handful of merges per pick, mostly of lists far shorter than
    // the longest); a merge that finds no room stages in global memory
    const int hw = 16;
    const bool gstage = true;
    const int arena = (int)(((smem_dyn_g - own) / 4) & ~int64_t(3));  // >= lmax ints (checked above)
    const bool arena_merges = grid_arena >= (heap ? 2 : 1);
    const int64_t hsmem = own + 4 * (int64_t)arena;
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, cell_grid_kernel, hw * 32, (size_t)hsmem) !=
            cudaSuccess ||
        per < 1) {
      cudaGetLastError();
      return false;
    }
    Launch Lc;
    Lc.step = st;
    Lc.level = step_level[st];
    Lc.heap = heap;
    Lc.lo = (int64_t)fcs.size();
    Lc.ncell = ncell;
    Lc.kmax = kmax;
    Lc.lmax = lmax;
    Lc.cs = 1;
    Lc.nw = hw;
    Lc.slots = used;
    Lc.smem = hsmem;
    Lc.global_stage = gstage;
    Lc.arena = arena;
    Lc.arena_merges = arena_merges;
    Lc.pstage_off = 0;
    Lc.grid = true;
    Lc.slice_max = slice_max;
    Lc.map_off = (int64_t)gmap.size();
    Lc.bar_off = grid_bar_words;
    for (const Cell &c : cells) {
      fcs.push_back(c.start);
      fcc.push_back(c.count);
    }
    for (int c = 0; c < ncell; c++)
      for (int i = 0; i < nb[c]; i++) gmap.push_back(c);
    for (int c = 0, b0 = 0; c <= ncell; c++) {
      gmap.push_back(b0);
      if (c < ncell) b0 += nb[c];
    }
    grid_bar_words += ncell;
    partial_max = std::max<int64_t>(partial_max, used);
    if (gstage) pstage_ints = std::max(pstage_ints, (int64_t)used * hw * 2 * (int64_t)lmax);
    launches.push_back(Lc);
    return true;
  };
  for (int st = 0; st < nsteps; st++) {
    const bool heap = st == nsteps - 1;
    std::vector<Cell> &cells = step_cells[st];
    if (grid_launch(cells, st, heap)) continue;
    std::stable_sort(cells.begin(), cells.end(), [](const Cell &x, const Cell &y) { return x.cls > y.cls; });
    int64_t step_pstage = 0;
    for (size_t g0 = 0; g0 < cells.size();) {
      size_t g1 = g0;
      while (g1 < cells.size() && cells[g1].cls == cells[g0].cls) g1++;
      Launch Lc;
      Lc.step = st;
      Lc.level = step_level[st];
      Lc.heap = heap;
      Lc.lo = (int64_t)fcs.size();
      Lc.ncell = (int)(g1 - g0);
      Lc.kmax = 1;
      Lc.lmax = 1;
      for (size_t c = g0; c < g1; c++) {
        fcs.push_back(cells[c].start);
        fcc.push_back(cells[c].count);
        Lc.kmax = std::max(Lc.kmax, cells[c].count);
        Lc.lmax = std::max(Lc.lmax, cells[c].lbound);
      }
      const int64_t keys_b = 3 * al(4LL * Lc.kmax);
      const int64_t own_b = keys_b + 2 * al(4LL * Lc.lmax);
      auto smem_for = [&](int w) { return own_b + 2 * al(4LL * Lc.lmax * w); };
      int nw = Lc.ncell * 4 < nsm ? 16 : 8;
      while (nw > 4 && smem_for(nw) > smem_dyn) nw >>= 1;
      // per-warp merge buffers move to global memory when they do not fit
      Lc.global_stage = smem_for(nw) > smem_dyn || force_global_stage;
      if (Lc.global_stage) nw = Lc.ncell * 4 < nsm ? 16 : 8;
      GH_CHECK(own_b <= smem_dyn, H2H_ERR_DEVICE,
               "elimination staging does not fit shared memory (candidate keys + eliminated list too large)");
      Lc.smem = Lc.global_stage ? own_b : smem_for(nw);
      Lc.nw = nw;
      // cluster size.  A cell eliminates serially; cs CTAs merge its lists
      // about cs^a times faster, while cs times more CTAs compete for the
      // resident slots.  Pick the cs that minimises waves(cs)^1.2 / cs^a with
      // waves = ceil(cells * cs / slots) (a later wave also waits for the
      // slowest cell of the one before).  Measured on road graphs: a = 0.8
      // above the bottom level; the bottom cells' vertices have few
      // neighbours when eliminated, so extra CTAs mostly add barriers (a = 0.3).
      const double alpha = st == 0 ? 0.3 : 0.8;
      int per_sm = 0;
      GH_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, elim_kernel, nw * 32, (size_t)Lc.smem));
      const int64_t slots = (int64_t)std::max(1, per_sm) * nsm;
      Lc.slots = (int)slots;
      int cs = 1;
      double best_cost = 1e300;
      for (int c = 1; c <= 16; c <<= 1) {
        const double waves = (double)((Lc.ncell * (int64_t)c + slots - 1) / slots);
        const double cost = std::pow(waves, 1.2) / std::pow((double)c, alpha);
        if (cost < best_cost * 0.999) { best_cost = cost; cs = c; }
      }
      for (;; cs >>= 1) {
        if (cs == 1) break;
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = cs;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cfg.blockDim = dim3(nw * 32);
        cfg.dynamicSmemBytes = (size_t)Lc.smem;
        cfg.gridDim = dim3(Lc.ncell * cs);
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, elim_kernel, &cfg) == cudaSuccess && nclusters > 0) break;
        cudaGetLastError();
      }
      Lc.cs = cs;
      Lc.grid = false;
      Lc.slice_max = 0;
      Lc.map_off = Lc.bar_off = 0;
      Lc.pstage_off = step_pstage;
      if (Lc.global_stage) step_pstage += (int64_t)Lc.ncell * cs * nw * 2 * (int64_t)Lc.lmax;
      launches.push_back(Lc);
      g0 = g1;
    }
    pstage_ints = std::max(pstage_ints, step_pstage);
  }
  {
    // side streams for the groups of a step beyond the first
    int most = 1;
    for (int st = 0; st < nsteps; st++) {
      int c = 0;
      for (const Launch &Lc : launches) c += Lc.step == st;
      most = std::max(most, c);
    }
    max_group = most;
  }
  // ---- device state
  try {
    slot_nbr = palloc<int>(pool_size + 4, bytes);  // + 4: a list's last 128-bit load stays inside
    slot_w = palloc<int>(pool_size + 4, bytes);
    pool_next = palloc<unsigned long long>(1, bytes);
    pool_first = palloc<unsigned long long>(1, bytes);
    slot_off = palloc<int64_t>(N, bytes);
    slot_off_init = palloc<int64_t>(N, bytes);
    lsize = palloc<int>(N, bytes);
    cap = palloc<int>(N, bytes);
    cap_init = palloc<int>(N, bytes);
    height = palloc<int>(N, bytes);
    elim = palloc<int>(N, bytes);
    elim_init = palloc<int>(N, bytes);
    deg0 = palloc<int>(N, bytes);
    deg_init = palloc<int>(N, bytes);
    h0 = palloc<int>(N, bytes);
    cpos = palloc<int>(N, bytes);
    err = palloc<int>(1, bytes);
    ljunk = palloc<int>(N, bytes);
    cell_start = palloc<int>(fcs.size(), bytes);
    cell_count = palloc<int>(fcc.size(), bytes);
    adj_off = palloc<int>(N + 1, bytes);
    adj_v = palloc<int>(std::max<int64_t>(M, 1), bytes);
    adj_w = palloc<int>(std::max<int64_t>(M, 1), bytes);
    heap_verts = palloc<int>(std::max(heap_total, 1), bytes);
    if (pstage_ints) pstage = palloc<int>(pstage_ints, bytes);
    if (!gmap.empty()) {
      hg_partial = palloc<int4>(2 * partial_max, bytes);  // per block: argmin, then (first word) merge count
      partial_cap = partial_max;
      grid_map = palloc<int>(gmap.size(), bytes);
      grid_bar = palloc<unsigned>(grid_bar_words, bytes);
      GH_CUDA(cudaMemcpy(grid_map, gmap.data(), sizeof(int) * gmap.size(), cudaMemcpyHostToDevice));
    }
    for (int k = 1; k < max_group; k++) {
      cudaStream_t st = nullptr;
      cudaEvent_t e = nullptr;
      GH_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
      side.push_back(st);
      GH_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      ev_join.push_back(e);
    }
    GH_CUDA(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    GH_CUDA(cudaMemcpy(slot_off_init, f_slot_off.data(), sizeof(int64_t) * N, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(deg_init, f_deg.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(cap_init, f_cap.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(elim_init, f_elim.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(cell_start, fcs.data(), sizeof(int) * fcs.size(), cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(cell_count, fcc.data(), sizeof(int) * fcc.size(), cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(adj_off, f_adj_off.data(), sizeof(int) * (N + 1), cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(adj_v, f_adj_v.data(), sizeof(int) * f_adj_v.size(), cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(adj_w, f_adj_w.data(), sizeof(int) * f_adj_w.size(), cudaMemcpyHostToDevice));
    if (heap_total)
      GH_CUDA(cudaMemcpy(heap_verts, f_heap.data(), sizeof(int) * heap_total, cudaMemcpyHostToDevice));
    const unsigned long long first_free = (unsigned long long)lub;
    GH_CUDA(cudaMemcpy(pool_first, &first_free, sizeof(first_free), cudaMemcpyHostToDevice));
  } catch (...) {
    release();
    throw;
  }
}

ElimPlan::~ElimPlan() { release(); }

void ElimPlan::release() {
  void *ps[] = {slot_nbr, slot_w, pool_next, pool_first, slot_off, slot_off_init, lsize, cap, cap_init, height, elim,
                elim_init, deg0, deg_init, h0, cpos, err, ljunk, cell_start, cell_count, adj_off, adj_v, adj_w,
                heap_verts, pstage};
  for (void *p : ps) cudaFree(p);
  cudaFree(hg_partial);
  cudaFree(grid_map);
  cudaFree(grid_bar);
  grid_map = nullptr;
  hg_partial = nullptr;
  grid_bar = nullptr;
  cudaFree(rank);
  cudaFree(father_dev);
  rank = father_dev = nullptr;
  for (cudaStream_t st : side) cudaStreamDestroy(st);
  for (cudaEvent_t e : ev_join) cudaEventDestroy(e);
  if (ev_fork) cudaEventDestroy(ev_fork);
  side.clear();
  ev_join.clear();
  ev_fork = nullptr;
  slot_nbr = slot_w = lsize = cap = cap_init = height = elim = elim_init = deg0 = deg_init = h0 = cpos = err = ljunk = nullptr;
  cell_start = cell_count = adj_off = adj_v = adj_w = heap_verts = pstage = nullptr;
  slot_off = slot_off_init = nullptr;
  pool_next = pool_first = nullptr;
}

void ElimPlan::set_weights(int gi, const int *w, cudaStream_t s) {
  GH_CHECK(gi >= 0 && gi < (int)gs.size(), H2H_ERR_ARG, "graph index out of range");
  const Graph &g = *gs[gi];
  if (g.m)
    GH_CUDA(cudaMemcpyAsync(adj_w + mbase[gi], w, sizeof(int) * g.m, cudaMemcpyHostToDevice, s));
}

void ElimPlan::launch_one(const Launch &Lc, cudaStream_t s, bool trace) {
  ElimArgs A;
  A.slot_nbr = slot_nbr; A.slot_w = slot_w; A.slot_off = slot_off; A.lsize = lsize; A.ljunk = ljunk;
  A.cap = cap; A.height = height; A.elim = elim; A.key_deg0 = deg0; A.key_h0 = Lc.heap ? h0 : nullptr;
  A.cell_start = cell_start; A.cell_count = cell_count; A.cpos = cpos; A.err = err;
  A.cell_lo = (int)Lc.lo; A.kmax = Lc.kmax; A.lmax = Lc.lmax; A.heap_mode = Lc.heap ? 1 : 0;
  A.pool_next = pool_next; A.pool_size = pool_size;
  A.pstage = Lc.global_stage ? pstage + Lc.pstage_off : nullptr;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = Lc.cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cfg.blockDim = dim3(Lc.nw * 32);
  cfg.dynamicSmemBytes = (size_t)Lc.smem;
  cfg.gridDim = dim3(Lc.ncell * Lc.cs);
  cfg.stream = s;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  if (trace) { cudaEventCreate(&ev0); cudaEventCreate(&ev1); cudaEventRecord(ev0, s); }
  if (Lc.grid) {
    GridArgs H;
    H.E = A;
    H.blk_cell = grid_map + Lc.map_off;
    H.cell_blk0 = grid_map + Lc.map_off + Lc.slots;
    H.slice_max = Lc.slice_max;
    H.partial = (int4 *)hg_partial;
    H.bar = grid_bar + Lc.bar_off;
    H.spin_limit = spin_limit_cycles();
    H.arena_ints = Lc.arena;
    H.arena_merges = Lc.arena_merges ? 1 : 0;
    H.done_cnt = reinterpret_cast<unsigned *>((int4 *)hg_partial + partial_cap);
    H.balance = elim_balance ? 1 : 0;
    GH_CUDA(cudaMemsetAsync(H.done_cnt, 0, sizeof(unsigned) * Lc.slots, s));
    cudaLaunchAttribute ca[1];
    ca[0].id = cudaLaunchAttributeCooperative;
    ca[0].val.cooperative = 1;
    cudaLaunchConfig_t cc = {};
    cc.attrs = ca;
    cc.numAttrs = 1;
    cc.blockDim = dim3(Lc.nw * 32);
    cc.gridDim = dim3(Lc.slots);
    cc.dynamicSmemBytes = (size_t)Lc.smem;
    cc.stream = s;
    GH_CUDA(cudaLaunchKernelEx(&cc, cell_grid_kernel, H));
  } else {
    GH_CUDA(cudaLaunchKernelEx(&cfg, elim_kernel, A));
  }
  if (trace) {
    cudaEventRecord(ev1, s);
    cudaEventSynchronize(ev1);
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0, ev1);
    char pool[64] = "";
    if (Lc.grid) std::snprintf(pool, sizeof pool, " (arena %d ints%s)", Lc.arena, Lc.arena_merges ? "" : ", lists only");
    std::fprintf(stderr,
                 "[gpuh2h] elim %s %d: %d cells x %d CTAs x %d warps, kmax %d, lmax %d, smem %lld, slots %d%s%s%s: %.3f ms\n",
                 Lc.heap ? "heap" : "level", Lc.level, Lc.ncell, Lc.cs, Lc.nw, Lc.kmax, Lc.lmax, (long long)Lc.smem,
                 Lc.slots, Lc.global_stage ? " (global merge staging)" : "", pool,
                 Lc.grid ? " (cooperative, slots = blocks)" : "", ms);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
  }
}

void ElimPlan::enqueue(cudaStream_t s, cudaEvent_t *heap_ev, bool trace) {
  // ---- reset to the input lists (relocation in the global order moves
  // lists and grows their capacity)
  GH_CUDA(cudaMemcpyAsync(slot_off, slot_off_init, sizeof(int64_t) * N, cudaMemcpyDeviceToDevice, s));
  GH_CUDA(cudaMemcpyAsync(cap, cap_init, sizeof(int) * N, cudaMemcpyDeviceToDevice, s));
  GH_CUDA(cudaMemcpyAsync(lsize, deg_init, sizeof(int) * N, cudaMemcpyDeviceToDevice, s));
  GH_CUDA(cudaMemcpyAsync(deg0, deg_init, sizeof(int) * N, cudaMemcpyDeviceToDevice, s));
  GH_CUDA(cudaMemcpyAsync(elim, elim_init, sizeof(int) * N, cudaMemcpyDeviceToDevice, s));
  GH_CUDA(cudaMemcpyAsync(pool_next, pool_first, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, s));
  GH_CUDA(cudaMemsetAsync(height, 0, sizeof(int) * N, s));
  GH_CUDA(cudaMemsetAsync(ljunk, 0, sizeof(int) * N, s));
  GH_CUDA(cudaMemsetAsync(cpos, 0xff, sizeof(int) * N, s));  // -1
  GH_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
  if (grid_bar_words) GH_CUDA(cudaMemsetAsync(grid_bar, 0, sizeof(unsigned) * grid_bar_words, s));
  scatter_adjacency_kernel<<<std::max(1, std::min(4096, (N + 255) / 256)), 256, 0, s>>>(
      adj_off, adj_v, adj_w, slot_off, slot_nbr, slot_w, N);
  GH_CUDA(cudaGetLastError());
  size_t li = 0;
  while (li < launches.size()) {
    size_t lj = li;
    while (lj < launches.size() && launches[lj].step == launches[li].step) lj++;
    if (launches[li].heap) {
      if (heap_ev) GH_CUDA(cudaEventRecord(heap_ev[0], s));
      if (heap_total) {
        prepare_heap_lists_kernel<<<std::max(1, std::min(4096, (heap_total * 32 + 255) / 256)), 256, 0, s>>>(
            heap_verts, heap_total, slot_off, slot_nbr, slot_w, lsize, ljunk, height, deg0, h0);
        GH_CUDA(cudaGetLastError());
      }
    }
    // the groups of one step are independent: fork them onto side streams
    if (lj - li > 1) GH_CUDA(cudaEventRecord(ev_fork, s));
    for (size_t k = li; k < lj; k++) {
      cudaStream_t ls = s;
      if (k > li) {
        ls = side[k - li - 1];
        GH_CUDA(cudaStreamWaitEvent(ls, ev_fork, 0));
      }
      launch_one(launches[k], ls, trace);
      if (k > li) GH_CUDA(cudaEventRecord(ev_join[k - li - 1], ls));
    }
    for (size_t k = li + 1; k < lj; k++) GH_CUDA(cudaStreamWaitEvent(s, ev_join[k - li - 1], 0));
    li = lj;
  }
  if (heap_ev) GH_CUDA(cudaEventRecord(heap_ev[1], s));
}

void ElimPlan::check_error() {
  GH_CUDA(cudaDeviceSynchronize());
  int e = 0;
  GH_CUDA(cudaMemcpy(&e, err, sizeof(int), cudaMemcpyDeviceToHost));
  GH_CHECK(e == 0, H2H_ERR_DEVICE,
           e == kErrOverflow ? "contraction: a list outgrew its LUB capacity"
           : e == kErrEmpty  ? "contraction: eliminated a vertex with an empty list (disconnected input)"
           : e == kErrTimeout ? "contraction: a cell barrier wait ran out"
           : e == kErrPick    ? "contraction: no candidate left to pick"
                              : "contraction: a list outgrew the staging bound");
}

void ElimPlan::build_lists() {
  int threads = 1;
  for (const Graph *g : gs) threads = std::max(threads, g->threads);
  Pool pool(threads);
  std::vector<int, NoInit<int>> f_lsize(N), f_elim(N), f_father(N);
  GH_CUDA(cudaMemcpy(f_lsize.data(), lsize, sizeof(int) * N, cudaMemcpyDeviceToHost));
  std::vector<int64_t, NoInit<int64_t>> off(N + 1);
  parallel_prefix(pool, N, off.data(), [&](int64_t v) { return (int64_t)f_lsize[v]; });
  const int64_t tot = off[N];
  auto la = std::make_shared<ListArrays>();
  la->off = dalloc<int64_t>(N + 1);
  la->id = dalloc<int>(std::max<int64_t>(tot, 1));
  la->w = dalloc<int>(std::max<int64_t>(tot, 1));
  lists.off = la->off;
  lists.id = la->id;
  lists.w = la->w;
  lists.total = tot;
  lists.keep = la;
  if (!rank) rank = palloc<int>(N, bytes);
  if (!father_dev) father_dev = palloc<int>(N, bytes);
  GH_CUDA(cudaMemcpy(lists.off, off.data(), sizeof(int64_t) * (N + 1), cudaMemcpyHostToDevice));
  enqueue_gather(0);
  rank_kernel<<<std::max(1, std::min(4096, (N + 255) / 256)), 256>>>(elim, rank, N);
  GH_CUDA(cudaGetLastError());
  father_kernel<<<std::max(1, std::min(8192, (N * 32 + 255) / 256)), 256>>>(lists.off, lists.id, rank, father_dev, N);
  GH_CUDA(cudaGetLastError());
  GH_CUDA(cudaMemcpy(f_elim.data(), elim, sizeof(int) * N, cudaMemcpyDeviceToHost));
  GH_CUDA(cudaMemcpy(f_father.data(), father_dev, sizeof(int) * N, cudaMemcpyDeviceToHost));
  for (size_t i = 0; i < gs.size(); i++) {
    Graph &g = *gs[i];
    const int vb = vbase[i];
    g.father.resize(g.n);
    g.x_off.resize(g.n + 1);
    pool.parallel_for(g.n, 1 << 16, [&](int64_t lo, int64_t hi, int) {
      for (int64_t v = lo; v < hi; v++) {
        g.elim[v] = f_elim[vb + v] - vb;
        g.father[v] = f_father[vb + v] < 0 ? -1 : f_father[vb + v] - vb;
        g.x_off[v + 1] = off[vb + v + 1] - off[vb];
      }
    });
    g.x_off[0] = 0;
    g.decomposition_size = g.x_off[g.n] + g.n;
    std::vector<int>().swap(g.x_id);
    std::vector<int>().swap(g.x_w);
    g.dev.lists = lists;
    g.dev.x_base = off[vb];
    g.dev.id_base = vb;
  }
}

void ElimPlan::enqueue_gather(cudaStream_t s) {
  gather_lists_kernel<<<std::max(1, std::min(8192, (N * 32 + 255) / 256)), 256, 0, s>>>(
      slot_off, lsize, lists.off, slot_nbr, slot_w, lists.id, lists.w, N);
  GH_CUDA(cudaGetLastError());
}

ListStore upload_lists(const std::vector<int64_t> &off, const std::vector<int> &id, const std::vector<int> &w) {
  ListStore L;
  auto la = std::make_shared<ListArrays>();
  const int64_t t = off.empty() ? 0 : off.back();
  la->off = dalloc<int64_t>(std::max<size_t>(off.size(), 1));
  la->id = dalloc<int>(std::max<int64_t>(t, 1));
  la->w = dalloc<int>(std::max<int64_t>(t, 1));
  L.off = la->off;
  L.id = la->id;
  L.w = la->w;
  L.total = t;
  L.keep = la;
  if (!off.empty()) GH_CUDA(cudaMemcpy(L.off, off.data(), sizeof(int64_t) * off.size(), cudaMemcpyHostToDevice));
  if (t) {
    GH_CUDA(cudaMemcpy(L.id, id.data(), sizeof(int) * t, cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemcpy(L.w, w.data(), sizeof(int) * t, cudaMemcpyHostToDevice));
  }
  return L;
}

void download_lists(Graph &g) {
  const ListStore &L = g.dev.lists;
  GH_CHECK(L.id && (int64_t)g.x_off.size() == g.n + 1, H2H_ERR_STATE, "not contracted");
  const int64_t t = g.x_off[g.n];
  g.x_id.resize(t);
  g.x_w.resize(t);
  if (t) {
    GH_CUDA(cudaMemcpy(g.x_id.data(), L.id + g.dev.x_base, sizeof(int) * t, cudaMemcpyDeviceToHost));
    GH_CUDA(cudaMemcpy(g.x_w.data(), L.w + g.dev.x_base, sizeof(int) * t, cudaMemcpyDeviceToHost));
  }
  if (g.dev.id_base)
    for (int64_t k = 0; k < t; k++) g.x_id[k] -= g.dev.id_base;
}

// Whole elimination of one graph on the GPU: partition levels H..C+1, then
// the global order over the vertices of levels <= C.  Fills g.elim
// (elimination order), g.father, g.x_off and g.gpu_vertices; the lists
// X(v)\{v} (sorted by id, the lists at elimination time) stay on the device.
void contract_gpu(Graph &g) {
  Clock clk;
  const bool trace = std::getenv("GPUH2H_TRACE") != nullptr;
  auto owned = std::make_unique<ElimPlan>(std::vector<Graph *>{&g});
  ElimPlan &plan = *owned;
  GH_CUDA(cudaDeviceSynchronize());
  g.t.translate_lub = clk.us();
  clk.reset();
  cudaEvent_t ev[2];
  GH_CUDA(cudaEventCreate(&ev[0]));
  GH_CUDA(cudaEventCreate(&ev[1]));
  long long heap_us = 0;
  try {
    plan.enqueue(0, ev, trace);
    plan.check_error();
    float hms = 0;
    GH_CUDA(cudaEventElapsedTime(&hms, ev[0], ev[1]));
    heap_us = (long long)(hms * 1000.0f);
  } catch (...) {
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    throw;
  }
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  g.t.td_gpu = clk.us() - heap_us;  // partition levels
  g.t.td_cpu = heap_us;             // global order over levels <= C (TDInCPUTime in the reference, on the GPU here)
  clk.reset();
  plan.build_lists();
  owned.reset();  // the elimination's device state is freed here, inside the timed phase
  g.t.translate_back = clk.us();
}

}  // namespace gh
