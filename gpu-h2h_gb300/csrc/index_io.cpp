// index_io.cpp -- h2h_save_index / h2h_load_index: the built index on disk,
// so a server restarts without a rebuild.  No counterpart in the reference,
// which rebuilds the labels on every run.
//
// Layout (little-endian, the host's byte order; both build hosts are):
//   "GPUH2HIX" | u32 version | u32 section count
//   header: i64 n, m, euler_n, rmq_total, x_total, pos_total, label_total,
//           max_label, decomposition_size; i32 H, C, label_mode, head,
//           tree_height, gpu_vertices, method, n_levels; u32 name length,
//           name bytes
//   sections, in a fixed order: u32 tag | u32 element size | u64 count | data
//     order, father, depth, first, rmq_hash, rmq_id, x_off, x_id, x_w,
//     dis_hash, pos_hash, pos_id, pos_pos, dis, tree_bfs, tree_hash
// Arrays are the reference's layouts (the ones the h2h_copy_* accessors
// return).  Loading validates sizes, offsets and id ranges before it touches
// the GPU, then uploads the index (labels into the padded device rows).
#include <cstdio>
#include <cstring>
#include <memory>

#include "gpuh2h.h"
#include "handle.h"

namespace {

constexpr char kMagic[8] = {'G', 'P', 'U', 'H', '2', 'H', 'I', 'X'};
constexpr uint32_t kVersion = 1;
enum Tag : uint32_t {
  kOrder = 1, kFather, kDepth, kFirst, kRmqHash, kRmqId, kXOff, kXId, kXW, kDisHash, kPosHash, kPosId, kPosPos,
  kDis, kTreeBfs, kTreeHash, kTagEnd
};

struct Header {
  int64_t n, m, euler_n, rmq_total, x_total, pos_total, label_total, max_label, decomposition_size;
  int32_t H, C, label_mode, head, tree_height, gpu_vertices, method, n_levels;
};

struct File {
  FILE *f = nullptr;
  std::string path;
  ~File() {
    if (f) std::fclose(f);
  }
  void write(const void *p, size_t bytes) {
    const char *c = (const char *)p;
    while (bytes) {
      const size_t k = std::fwrite(c, 1, std::min<size_t>(bytes, size_t(1) << 28), f);
      GH_CHECK(k > 0, H2H_ERR_IO, "write failed: " + path);
      c += k;
      bytes -= k;
    }
  }
  void read(void *p, size_t bytes) {
    char *c = (char *)p;
    while (bytes) {
      const size_t k = std::fread(c, 1, std::min<size_t>(bytes, size_t(1) << 28), f);
      GH_CHECK(k > 0, H2H_ERR_FORMAT, "file ends early: " + path);
      c += k;
      bytes -= k;
    }
  }
};

template <typename T>
void put_section(File &F, uint32_t tag, const T *data, uint64_t count) {
  const uint32_t es = sizeof(T);
  F.write(&tag, 4);
  F.write(&es, 4);
  F.write(&count, 8);
  if (count) F.write(data, sizeof(T) * count);
}

template <typename T>
void get_section(File &F, uint32_t tag, std::vector<T> &out, uint64_t expect) {
  uint32_t t = 0, es = 0;
  uint64_t count = 0;
  F.read(&t, 4);
  F.read(&es, 4);
  F.read(&count, 8);
  GH_CHECK(t == tag && es == sizeof(T), H2H_ERR_FORMAT, "unexpected section in " + F.path);
  GH_CHECK(count == expect, H2H_ERR_FORMAT, "section of the wrong size in " + F.path);
  out.resize(count);
  if (count) F.read(out.data(), sizeof(T) * count);
}

void check_offsets(const std::vector<int64_t> &off, int64_t total, const char *what) {
  GH_CHECK(!off.empty() && off.front() == 0 && off.back() == total, H2H_ERR_FORMAT,
           std::string(what) + ": offsets do not span the array");
  for (size_t i = 1; i < off.size(); i++)
    GH_CHECK(off[i] >= off[i - 1], H2H_ERR_FORMAT, std::string(what) + ": offsets decrease");
}

void check_ids(const std::vector<int> &a, int lo, int hi, const char *what) {
  for (int x : a) GH_CHECK(x >= lo && x < hi, H2H_ERR_FORMAT, std::string(what) + ": id out of range");
}

}  // namespace

extern "C" {

int h2h_save_index(const h2h_graph *h, const char *path) {
  if (!h || !path) { gh::set_last_error("null argument"); return H2H_ERR_ARG; }
  return gh::guarded([&] {
    gh::Graph &g = const_cast<gh::Graph &>(h->g);
    GH_CHECK(g.labelled, H2H_ERR_STATE, "labels not built");
    const int n = g.n;
    std::vector<int64_t> rmq_hash(g.euler_n);
    std::vector<int> rmq_id(g.rmq_total);
    gh::download_rmq(g, rmq_hash.data(), rmq_id.data());
    const bool had_lists = (int64_t)g.x_id.size() == g.x_off[n];
    if (!had_lists) gh::download_lists(g);
    const int64_t np = g.pos_hash[n];
    std::vector<int> pos_id(np), pos_pos(np), dis(g.dis_hash[n]);
    gh::download_positions(g, pos_id.data(), pos_pos.data());
    gh::download_labels(g, dis.data());
    File F;
    F.path = path;
    F.f = std::fopen(path, "wb");
    GH_CHECK(F.f, H2H_ERR_IO, std::string("cannot open ") + path);
    F.write(kMagic, 8);
    const uint32_t ver = kVersion, nsec = kTagEnd - 1;
    F.write(&ver, 4);
    F.write(&nsec, 4);
    Header hd{};
    hd.n = n;
    hd.m = g.m;
    hd.euler_n = g.euler_n;
    hd.rmq_total = g.rmq_total;
    hd.x_total = g.x_off[n];
    hd.pos_total = np;
    hd.label_total = g.dis_hash[n];
    hd.max_label = gh::label_max(g);
    hd.decomposition_size = g.decomposition_size;
    hd.H = g.H_cli;
    hd.C = g.C;
    hd.label_mode = g.label_mode;
    hd.head = g.head;
    hd.tree_height = g.tree_height;
    hd.gpu_vertices = g.gpu_vertices;
    hd.method = g.method;
    hd.n_levels = (int32_t)g.tree_hash.size() - 1;
    F.write(&hd, sizeof(hd));
    const uint32_t nl = (uint32_t)g.name.size();
    F.write(&nl, 4);
    F.write(g.name.data(), nl);
    put_section(F, kOrder, g.elim.data(), n);
    put_section(F, kFather, g.father.data(), n);
    put_section(F, kDepth, g.depth.data(), n);
    put_section(F, kFirst, g.first.data(), n);
    put_section(F, kRmqHash, rmq_hash.data(), g.euler_n);
    put_section(F, kRmqId, rmq_id.data(), g.rmq_total);
    put_section(F, kXOff, g.x_off.data(), n + 1);
    put_section(F, kXId, g.x_id.data(), g.x_off[n]);
    put_section(F, kXW, g.x_w.data(), g.x_off[n]);
    put_section(F, kDisHash, g.dis_hash.data(), n + 1);
    put_section(F, kPosHash, g.pos_hash.data(), n + 1);
    put_section(F, kPosId, pos_id.data(), np);
    put_section(F, kPosPos, pos_pos.data(), np);
    put_section(F, kDis, dis.data(), g.dis_hash[n]);
    put_section(F, kTreeBfs, g.tree_bfs.data(), g.tree_bfs.size());
    put_section(F, kTreeHash, g.tree_hash.data(), g.tree_hash.size());
    if (!had_lists && !gh::uses_level_fill(g)) {
      std::vector<int>().swap(g.x_id);
      std::vector<int>().swap(g.x_w);
    }
    GH_CHECK(std::fflush(F.f) == 0, H2H_ERR_IO, std::string("write failed: ") + path);
  });
}

int h2h_load_index(const char *path, h2h_graph **out) {
  if (out) *out = nullptr;
  if (!path || !out) { gh::set_last_error("null argument"); return H2H_ERR_ARG; }
  return gh::guarded([&] {
    File F;
    F.path = path;
    F.f = std::fopen(path, "rb");
    GH_CHECK(F.f, H2H_ERR_IO, std::string("cannot open ") + path);
    char magic[8];
    F.read(magic, 8);
    GH_CHECK(std::memcmp(magic, kMagic, 8) == 0, H2H_ERR_FORMAT, std::string("not an index file: ") + path);
    uint32_t ver = 0, nsec = 0;
    F.read(&ver, 4);
    F.read(&nsec, 4);
    GH_CHECK(ver == kVersion && nsec == kTagEnd - 1, H2H_ERR_FORMAT, "unsupported index version");
    Header hd{};
    F.read(&hd, sizeof(hd));
    GH_CHECK(hd.n >= 1 && hd.n < INT32_MAX && hd.euler_n == 2 * hd.n - 1 && hd.x_total >= 0 &&
                 hd.pos_total == hd.x_total + hd.n && hd.label_total >= hd.n && hd.rmq_total >= hd.euler_n &&
                 hd.head >= 0 && hd.head < hd.n && hd.n_levels >= 1 && hd.n_levels <= hd.n &&
                 (hd.label_mode == H2H_LABEL_L3 || hd.label_mode == H2H_LABEL_L4),
             H2H_ERR_FORMAT, "inconsistent index header");
    uint32_t nl = 0;
    F.read(&nl, 4);
    GH_CHECK(nl < 4096, H2H_ERR_FORMAT, "inconsistent index header");
    std::string name(nl, '\0');
    if (nl) F.read(&name[0], nl);
    auto hh = std::make_unique<h2h_graph>();
    gh::Graph &g = hh->g;
    const int n = (int)hd.n;
    g.name = name;
    g.n = n;
    g.m = hd.m;
    g.H_cli = g.H = hd.H;
    g.C = hd.C;
    g.method = hd.method;
    g.label_mode = hd.label_mode;
    g.head = hd.head;
    g.tree_height = hd.tree_height;
    g.gpu_vertices = hd.gpu_vertices;
    g.euler_n = hd.euler_n;
    g.rmq_total = hd.rmq_total;
    g.max_label = hd.max_label;
    g.decomposition_size = hd.decomposition_size;
    std::vector<int64_t> rmq_hash;
    std::vector<int> rmq_id, pos_id, pos_pos, dis;
    get_section(F, kOrder, g.elim, n);
    get_section(F, kFather, g.father, n);
    get_section(F, kDepth, g.depth, n);
    get_section(F, kFirst, g.first, n);
    get_section(F, kRmqHash, rmq_hash, hd.euler_n);
    get_section(F, kRmqId, rmq_id, hd.rmq_total);
    get_section(F, kXOff, g.x_off, n + 1);
    get_section(F, kXId, g.x_id, hd.x_total);
    get_section(F, kXW, g.x_w, hd.x_total);
    get_section(F, kDisHash, g.dis_hash, n + 1);
    get_section(F, kPosHash, g.pos_hash, n + 1);
    get_section(F, kPosId, pos_id, hd.pos_total);
    get_section(F, kPosPos, pos_pos, hd.pos_total);
    get_section(F, kDis, dis, hd.label_total);
    get_section(F, kTreeBfs, g.tree_bfs, n);
    get_section(F, kTreeHash, g.tree_hash, hd.n_levels + 1);
    // validation: everything the device index indexes with
    check_ids(g.elim, 0, n, "order");
    check_ids(g.father, -1, n, "father");
    for (int v = 0; v < n; v++)
      GH_CHECK(g.depth[v] >= 1 && g.depth[v] <= hd.tree_height, H2H_ERR_FORMAT, "depth out of range");
    check_ids(g.first, 0, (int)hd.euler_n, "firstAppeare");
    check_ids(rmq_id, 0, n, "RMQ_ID");
    for (int64_t i = 0; i < hd.euler_n; i++) {
      const int64_t need = (int64_t)gh::ilog2_floor(hd.euler_n - i) + 1;
      GH_CHECK(rmq_hash[i] >= 0 && rmq_hash[i] + need <= hd.rmq_total, H2H_ERR_FORMAT, "RMQHash out of range");
    }
    check_offsets(g.x_off, hd.x_total, "adjacency");
    check_ids(g.x_id, 0, n, "adjacency");
    check_offsets(g.dis_hash, hd.label_total, "dis_hash");
    check_offsets(g.pos_hash, hd.pos_total, "pos_hash");
    for (int v = 0; v < n; v++) {
      GH_CHECK(g.dis_hash[v + 1] - g.dis_hash[v] == g.depth[v], H2H_ERR_FORMAT, "label row length is not the depth");
      GH_CHECK(g.pos_hash[v + 1] - g.pos_hash[v] == g.x_off[v + 1] - g.x_off[v] + 1, H2H_ERR_FORMAT,
               "position list length does not match the adjacency");
      for (int64_t k = g.pos_hash[v]; k < g.pos_hash[v + 1]; k++)
        GH_CHECK(pos_pos[k] >= 0 && pos_pos[k] < g.depth[v], H2H_ERR_FORMAT, "position out of range");
    }
    check_ids(pos_id, 0, n, "pos_id");
    check_ids(g.tree_bfs, 0, n, "TreeBFS");
    GH_CHECK(g.tree_hash.front() == 0 && g.tree_hash.back() == n, H2H_ERR_FORMAT, "TreeHash does not span the tree");
    for (size_t i = 1; i < g.tree_hash.size(); i++)
      GH_CHECK(g.tree_hash[i] > g.tree_hash[i - 1], H2H_ERR_FORMAT, "TreeHash decreases");
    int64_t h2h = 0;
    for (int v = 0; v < n; v++) h2h += g.depth[v];
    g.h2h_size = h2h;
    // device index
    gh::upload_rmq(g, rmq_hash, rmq_id);
    g.dev.lists = gh::upload_lists(g.x_off, g.x_id, g.x_w);
    g.dev.x_base = 0;
    g.dev.id_base = 0;
    gh::upload_labels(g, dis, pos_id, pos_pos);
    if (!gh::uses_level_fill(g)) {
      std::vector<int>().swap(g.x_id);
      std::vector<int>().swap(g.x_w);
    }
    g.contracted = true;
    g.labelled = true;
    *out = hh.release();
  });
}

}  // extern "C"
