// noalloc.cu -- the L4 label fill for callers that cannot allocate device
// memory: h2h_fill_labels_l4_noalloc (include/gpuh2h.h).
//
// Some callers cannot call cudaMalloc: code that runs inside another
// framework's memory budget, embedded services whose device memory is
// partitioned up front, or plugins that may only use the buffers their host
// hands them.  This entry point takes every input and
// the output as caller-owned device buffers and keeps the fill's scratch (one
// "finished" flag per tree node, a work counter, an error word and the
// ancestor chain of every node) in one file-scope __device__ array of
// kScratchInts ints (32 MiB).  Every GPU that loads the library holds that
// array until the process exits.
//
// A first kernel checks every caller-passed offset, id and depth against the
// declared sizes and sets the error word before anything else is written;
// the fill kernel does no work once that word is set.  The fill itself is
// the dataflow form of the L4 label fill (labels.cu):
// persistent CTAs take nodes in the caller's order, wait for the father's
// flag (bounded spin with an error exit), stage the node's separator and
// ancestor rows in shared memory and compute each label column as the exact
// min-plus over the separator.  One CTA handles a whole node here.
#include <climits>
#include <mutex>

#include "graph.h"

namespace gh {

namespace {

constexpr int64_t kScratchInts = int64_t(8) << 20;  // 32 MiB: flags + counters + ancestor chains

__device__ __align__(256) int g_fill_scratch[kScratchInts];

struct NoAllocArgs {
  const int *order;
  int n;
  const int *father;
  const int *depth;
  const int64_t *pos_hash;
  const int *pos_id;
  const int *pos_pos;
  const int *pos_w;
  const int64_t *dis_hash;
  int *dis;
  int64_t total_label;
  int *done;   // scratch: n flags
  int *next;   // scratch: work counter
  int *err;    // scratch: error word (1 = wait ran out, 2 = inputs rejected by the validation)
  int *chain;  // scratch: ancestor ids per node, laid out like the labels
  long long spin_limit;
  int max_sep;
  int max_depth;
};

__device__ __forceinline__ int na_ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void na_st_release(int *p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int na_ld_relaxed(const int *p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Every access the fill makes is bounded by these checks: rows and position
// lists lie inside [0, total_label) and are non-empty, ids are in [0, n),
// a node's father is one level up (so its ancestor chain is exactly d-1
// long), and a position list is sorted, ends with the node itself and names
// proper ancestors at their own depths (so every label read stays inside the
// row it reads).  Any violation sets the error word to 2.
__global__ void __launch_bounds__(256) validate_noalloc_kernel(NoAllocArgs A) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (__ldg(A.dis_hash) < 0 || __ldg(A.dis_hash + A.n) > A.total_label || __ldg(A.pos_hash) < 0)
      atomicCAS(A.err, 0, 2);
  }
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += stride) {
    const int v = (int)i;
    bool ok = true;
    const int o = __ldg(A.order + v);
    ok &= o >= 0 && o < A.n;
    const int d = __ldg(A.depth + v);
    const int64_t r0 = __ldg(A.dis_hash + v), r1 = __ldg(A.dis_hash + v + 1);
    ok &= d >= 1 && d <= A.max_depth && r0 >= 0 && r1 >= r0 && d <= r1 - r0;
    const int f = __ldg(A.father + v);
    if (f < 0) ok &= f == -1 && d == 1;
    else ok &= f < A.n && __ldg(A.depth + f) == d - 1;
    const int64_t p0 = __ldg(A.pos_hash + v), p1 = __ldg(A.pos_hash + v + 1);
    const int64_t cnt = p1 - p0;
    ok &= p0 >= 0 && cnt >= 1 && cnt - 1 <= A.max_sep;
    if (ok) {
      int prev = -1;
      for (int64_t k = p0; k < p1 && ok; k++) {
        const int u = __ldg(A.pos_id + k), p = __ldg(A.pos_pos + k);
        ok &= u >= 0 && u < A.n && p > prev;
        if (ok) ok &= (k == p1 - 1) ? (u == v && p == d - 1) : (p < d - 1 && __ldg(A.depth + u) == p + 1);
        prev = p;
      }
    }
    if (!ok) atomicCAS(A.err, 0, 2);
  }
}

__global__ void __launch_bounds__(128) fill_noalloc_kernel(NoAllocArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_t, s_stop;
  const int tid = threadIdx.x, T = blockDim.x;
  int64_t *xs_row = (int64_t *)smem;            // [max_sep]
  int64_t *anc_row = xs_row + A.max_sep;        // [max_depth]
  int *xs_p = (int *)(anc_row + A.max_depth);   // [max_sep]
  int *xs_w = xs_p + A.max_sep;                 // [max_sep]
  if (na_ld_relaxed(A.err) != 0) return;  // the inputs failed validation: write nothing
  for (;;) {
    if (tid == 0) s_t = atomicAdd(A.next, 1);
    __syncthreads();
    const int t = s_t;
    if (t >= A.n) return;
    const int v = __ldg(A.order + t);
    const int d = __ldg(A.depth + v);
    const int f = __ldg(A.father + v);
    const int64_t pb = __ldg(A.pos_hash + v);
    const int m = (int)(__ldg(A.pos_hash + v + 1) - pb) - 1;
    if (tid == 0) {
      s_stop = 0;
      const bool row_fits = d >= 1 && d <= __ldg(A.dis_hash + v + 1) - __ldg(A.dis_hash + v);
      if (m < 0 || m > A.max_sep || d > A.max_depth || !row_fits || na_ld_relaxed(A.err) != 0) {
        atomicCAS(A.err, 0, 2);
        s_stop = 1;
      } else if (f >= 0) {
        const long long t0 = clock64();
        while (na_ld_acquire(A.done + f) == 0) {
          if (na_ld_relaxed(A.err) != 0 || clock64() - t0 > A.spin_limit) {
            atomicCAS(A.err, 0, 1);
            s_stop = 1;
            break;
          }
          __nanosleep(64);
        }
      }
    }
    __syncthreads();
    if (s_stop) return;
    const int64_t base = __ldg(A.dis_hash + v);
    for (int i = tid; i < m; i += T) {
      xs_p[i] = __ldg(A.pos_pos + pb + i);
      xs_w[i] = __ldg(A.pos_w + pb + i);
      xs_row[i] = __ldg(A.dis_hash + __ldg(A.pos_id + pb + i));
    }
    if (d >= 2) {
      const int64_t fb = __ldg(A.dis_hash + f);
      for (int j = tid; j < d - 1; j += T) {
        const int a = __ldcg(A.chain + fb + j);
        anc_row[j] = __ldg(A.dis_hash + a);
        A.chain[base + j] = a;
      }
    }
    if (tid == 0) {
      A.chain[base + d - 1] = v;
      A.dis[base + d - 1] = 0;
    }
    __syncthreads();
    for (int j = tid; j < d - 1; j += T) {
      int r = INT_MAX;
      const int64_t arow = anc_row[j];
      for (int i = 0; i < m; i++) {
        const int p = xs_p[i];
        int val;
        if (p > j) val = __ldcg(A.dis + xs_row[i] + j);
        else if (p == j) val = 0;
        else val = __ldcg(A.dis + arow + p);
        r = min(r, xs_w[i] + val);
      }
      A.dis[base + j] = r;
    }
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      na_st_release(A.done + v, 1);
    }
  }
}

std::mutex g_setup_mu;
int *g_scratch_ptr[128] = {nullptr};  // per device: address of g_fill_scratch

}  // namespace

}  // namespace gh

extern "C" int h2h_fill_labels_l4_noalloc(int n, const int *order, const int *father, const int *depth,
                                          const int64_t *pos_hash, const int *pos_id, const int *pos_pos,
                                          const int *pos_w, const int64_t *dis_hash, int64_t total_label, int *dis,
                                          int max_depth, int max_sep, void *stream) {
  using namespace gh;
  if (n <= 0 || !order || !father || !depth || !pos_hash || !pos_id || !pos_pos || !pos_w || !dis_hash || !dis) {
    set_last_error("h2h_fill_labels_l4_noalloc: null buffer or empty tree");
    return H2H_ERR_ARG;
  }
  if (total_label < n || max_depth < 1 || max_sep < 0) {
    set_last_error("h2h_fill_labels_l4_noalloc: inconsistent sizes");
    return H2H_ERR_ARG;
  }
  if ((int64_t)n + 2 + total_label > kScratchInts) {
    set_last_error("h2h_fill_labels_l4_noalloc: tree too large for the fixed scratch (n + label entries + 2 must be "
                   "<= 8388608)");
    return H2H_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 128) {
    set_last_error("h2h_fill_labels_l4_noalloc: no current device");
    return H2H_ERR_CUDA;
  }
  int *scratch = nullptr;
  {
    // once per device, with that device current: the host name of the array
    // is not a device address
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
      e = cudaGetSymbolAddress((void **)&g_scratch_ptr[dev], g_fill_scratch);
      if (e != cudaSuccess) {
        g_scratch_ptr[dev] = nullptr;
        set_last_error(std::string("h2h_fill_labels_l4_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        return H2H_ERR_CUDA;
      }
    }
    scratch = g_scratch_ptr[dev];
  }
  const size_t smem = (size_t)max_sep * 16 + (size_t)max_depth * 8;
  int optin = 0, nsm = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, fill_noalloc_kernel) != cudaSuccess || smem + fa.sharedSizeBytes > (size_t)optin) {
    set_last_error("h2h_fill_labels_l4_noalloc: max_depth/max_sep exceed the shared-memory staging");
    return H2H_ERR_ARG;
  }
  if (cudaFuncSetAttribute(fill_noalloc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(optin - fa.sharedSizeBytes)) != cudaSuccess) {
    set_last_error("h2h_fill_labels_l4_noalloc: cudaFuncSetAttribute failed");
    return H2H_ERR_CUDA;
  }
  // flags, counter and error word must start at zero; the chains are overwritten
  e = cudaMemsetAsync(scratch, 0, sizeof(int) * ((size_t)n + 2), s);
  if (e != cudaSuccess) {
    set_last_error(std::string("h2h_fill_labels_l4_noalloc: cudaMemsetAsync: ") + cudaGetErrorString(e));
    return H2H_ERR_CUDA;
  }
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fill_noalloc_kernel, 128, smem);
  NoAllocArgs A;
  A.order = order; A.n = n; A.father = father; A.depth = depth; A.pos_hash = pos_hash; A.pos_id = pos_id;
  A.pos_pos = pos_pos; A.pos_w = pos_w; A.dis_hash = dis_hash; A.dis = dis; A.total_label = total_label;
  A.done = scratch; A.next = scratch + n; A.err = scratch + n + 1; A.chain = scratch + n + 2;
  A.spin_limit = 4000000000LL;
  A.max_sep = max_sep;
  A.max_depth = max_depth;
  const int vblocks = (int)std::min<int64_t>((int64_t)nsm * 4, ((int64_t)n + 255) / 256);
  validate_noalloc_kernel<<<std::max(1, vblocks), 256, 0, s>>>(A);
  const int blocks = (int)std::min<int64_t>((int64_t)nsm * std::max(1, per_sm), n);
  fill_noalloc_kernel<<<std::max(1, blocks), 128, smem, s>>>(A);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(std::string("h2h_fill_labels_l4_noalloc: launch: ") + cudaGetErrorString(e));
    return H2H_ERR_CUDA;
  }
  int kerr = 0;
  e = cudaMemcpyAsync(&kerr, scratch + n + 1, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    set_last_error(std::string("h2h_fill_labels_l4_noalloc: ") + cudaGetErrorString(e));
    return H2H_ERR_CUDA;
  }
  if (kerr != 0) {
    set_last_error(kerr == 2 ? "h2h_fill_labels_l4_noalloc: inputs rejected before any write (an offset, id or "
                               "depth is out of range, a father is not one level up, a position list is not "
                               "sorted ending with its node, or a node exceeds max_depth/max_sep)"
                             : "h2h_fill_labels_l4_noalloc: a dependency wait ran out (order must list every "
                               "father before its children)");
    return H2H_ERR_DEVICE;
  }
  return H2H_OK;
}
