// io.cpp -- file formats of the reference: the Edge / ID / Cut loaders
// (Graph_Fundamental.cu:4-95), the CSV writers (GraphPartition.cu:252-265,
// TreeStructure.cu:54-99, Graph_Fundamental.cu:132-170, Query.cu:597-622).
// The synthetic road-graph generator that writes those formats is gen.cpp.
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <memory>
#include <cmath>
#include <cstring>
#include <fstream>
#include <numeric>

#include "graph.h"
#include "gpuh2h_tools.h"
#include "pool.h"

namespace gh {

namespace {

// A whole file in memory, read by several threads at once (pread of 16 MB
// pieces into an uninitialised buffer).
struct FileBytes {
  std::unique_ptr<char[]> data;
  size_t size = 0;
};

FileBytes read_file(const std::string &path, int threads) {
  const int fd = ::open(path.c_str(), O_RDONLY);
  if (fd < 0) throw Error(H2H_ERR_IO, "cannot open " + path);
  struct stat st;
  if (::fstat(fd, &st) != 0) {
    ::close(fd);
    throw Error(H2H_ERR_IO, "cannot stat " + path);
  }
  FileBytes f;
  f.size = st.st_size > 0 ? (size_t)st.st_size : 0;
  f.data.reset(new char[f.size + 1]);
  const size_t piece = size_t(16) << 20;
  const int64_t np = (int64_t)((f.size + piece - 1) / piece);
  std::atomic<bool> ok{true};
  auto read_pieces = [&](int64_t lo, int64_t hi, int) {
    for (int64_t k = lo; k < hi; k++) {
      size_t at = (size_t)k * piece;
      const size_t end = std::min(f.size, at + piece);
      while (at < end) {
        const ssize_t r = ::pread(fd, f.data.get() + at, end - at, (off_t)at);
        if (r <= 0) { ok = false; break; }
        at += (size_t)r;
      }
    }
  };
  if (np > 1 && threads > 1) {
    Pool pool(std::min<int64_t>(threads, np));
    pool.parallel_for(np, 1, read_pieces);
  } else {
    read_pieces(0, np, 0);
  }
  ::close(fd);
  if (!ok.load()) throw Error(H2H_ERR_IO, "short read on " + path);
  f.data[f.size] = 0;
  return f;
}

// Whitespace tokenizer with the istream >> semantics the reference relies on.
struct Cursor {
  const char *p, *e;
  std::string what;
  explicit Cursor(const std::string &s, std::string w) : p(s.data()), e(s.data() + s.size()), what(std::move(w)) {}
  explicit Cursor(const FileBytes &f, std::string w) : p(f.data.get()), e(f.data.get() + f.size), what(std::move(w)) {}
  void skip() {
    while (p < e && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t' || *p == '\v' || *p == '\f')) p++;
  }
  long long integer() {
    skip();
    bool neg = false;
    if (p < e && (*p == '-' || *p == '+')) neg = (*p++ == '-');
    if (p >= e || *p < '0' || *p > '9') throw Error(H2H_ERR_FORMAT, "expected an integer in " + what);
    long long v = 0;
    while (p < e && *p >= '0' && *p <= '9') v = v * 10 + (*p++ - '0');
    return neg ? -v : v;
  }
  void token() {  // a double field that the hot path never uses
    skip();
    const char *s = p;
    while (p < e && !(*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) p++;
    if (p == s) throw Error(H2H_ERR_FORMAT, "missing field in " + what);
  }
  void one_char() {  // `char s; Edge >> s` consumes exactly one non-blank character
    skip();
    if (p >= e) throw Error(H2H_ERR_FORMAT, "truncated " + what);
    p++;
  }
};

// The arcs of an Edge file in parallel, for files with one arc per line:
// the text after the header is cut into chunks at line starts, each chunk is
// parsed on its own (marker, u, v, w per arc) and must end on an arc
// boundary; the first m arcs are kept in file order, self loops dropped.
// Returns false (nothing kept) when the file needs the token-by-token reader:
// an arc spread over lines, fewer than m arcs, anything unparsable.  Ids and
// weights out of range still raise H2H_ERR_FORMAT.
bool parse_arcs_parallel(const Cursor &c0, long long m, int n, int threads, std::vector<int> &eu,
                         std::vector<int> &ev, std::vector<int> &ew) {
  const char *b = c0.p, *e = c0.e;
  if (m == 0 || threads < 2 || e - b < (1 << 20)) return false;
  const int T = threads;
  std::vector<const char *> cut(T + 1, e);
  cut[0] = b;
  for (int t = 1; t < T; t++) {
    const char *q = b + (e - b) * t / T;
    while (q < e && *q != '\n') q++;
    cut[t] = q < e ? q + 1 : e;
  }
  struct Part {
    std::vector<int> u, v, w;
    bool ok = true, range = true;
  };
  std::vector<Part> parts(T);
  Pool pool(T);
  pool.parallel_for(T, 1, [&](int64_t lo, int64_t hi, int) {
    for (int64_t t = lo; t < hi; t++) {
      Part &P = parts[t];
      static const std::string kEmpty;
      Cursor c(kEmpty, c0.what);
      c.p = cut[t];
      c.e = cut[t + 1];
      try {
        for (;;) {
          c.skip();
          if (c.p >= c.e) break;
          c.one_char();
          const long long a = c.integer(), bb = c.integer(), w = c.integer();
          if (a < 1 || a > n || bb < 1 || bb > n || w < 0 || w > INT32_MAX) { P.range = false; break; }
          P.u.push_back((int)a - 1);
          P.v.push_back((int)bb - 1);
          P.w.push_back((int)w);
          // an arc must end its line: the next non-blank character is on a new line
          const char *q = c.p;
          while (q < c.e && (*q == ' ' || *q == '\t' || *q == '\r')) q++;
          if (q < c.e && *q != '\n') { P.ok = false; break; }
        }
      } catch (const Error &) {
        P.ok = false;
      }
    }
  });
  long long total = 0;
  for (int t = 0; t < T; t++) {
    if (!parts[t].ok) return false;
    if (!parts[t].range) {
      // only an error if the bad arc is among the first m
      if (total + (long long)parts[t].u.size() < m)
        throw Error(H2H_ERR_FORMAT, "vertex id or weight out of range in " + c0.what);
      break;
    }
    total += (long long)parts[t].u.size();
    if (total >= m) break;
  }
  if (total < m) return false;
  // the first m arcs, self loops dropped, in file order: per part the arcs
  // it contributes and where they land, then the copies in parallel
  std::vector<long long> take(T, 0), keep(T, 0), at(T + 1, 0);
  long long left = m;
  for (int t = 0; t < T; t++) {
    take[t] = std::min<long long>(left, (long long)parts[t].u.size());
    left -= take[t];
  }
  pool.parallel_for(T, 1, [&](int64_t lo, int64_t hi, int) {
    for (int64_t t = lo; t < hi; t++) {
      long long k = 0;
      for (long long i = 0; i < take[t]; i++) k += parts[t].u[i] != parts[t].v[i];
      keep[t] = k;
    }
  });
  for (int t = 0; t < T; t++) at[t + 1] = at[t] + keep[t];
  eu.resize(at[T]);
  ev.resize(at[T]);
  ew.resize(at[T]);
  pool.parallel_for(T, 1, [&](int64_t lo, int64_t hi, int) {
    for (int64_t t = lo; t < hi; t++) {
      long long o = at[t];
      for (long long i = 0; i < take[t]; i++) {
        if (parts[t].u[i] == parts[t].v[i]) continue;  // self loops dropped
        eu[o] = parts[t].u[i];
        ev[o] = parts[t].v[i];
        ew[o] = parts[t].w[i];
        o++;
      }
    }
  });
  return true;
}

// The (position, vertex) pairs of an ID file in parallel, for files with one
// vertex per line ("idx lon lat vid"): chunks cut at line starts, each parsed
// on its own.  Returns false (nothing set) when the file needs the
// token-by-token reader -- a record spread over lines, fewer than n records,
// anything unparsable; positions or ids out of range raise H2H_ERR_FORMAT.
bool parse_ids_parallel(const Cursor &c0, int n, int threads, std::vector<int> &part_ids,
                        std::vector<int> &id_hash) {
  const char *b = c0.p, *e = c0.e;
  if (threads < 2 || e - b < (1 << 20)) return false;
  const int T = threads;
  std::vector<const char *> cut(T + 1, e);
  cut[0] = b;
  for (int t = 1; t < T; t++) {
    const char *q = b + (e - b) * t / T;
    while (q < e && *q != '\n') q++;
    cut[t] = q < e ? q + 1 : e;
  }
  struct Part {
    std::vector<int> hash, id;
    bool ok = true, range = true;
  };
  std::vector<Part> parts(T);
  Pool pool(T);
  pool.parallel_for(T, 1, [&](int64_t lo, int64_t hi, int) {
    for (int64_t t = lo; t < hi; t++) {
      Part &P = parts[t];
      static const std::string kEmpty;
      Cursor c(kEmpty, c0.what);
      c.p = cut[t];
      c.e = cut[t + 1];
      try {
        for (;;) {
          c.skip();
          if (c.p >= c.e) break;
          const long long hash = c.integer();
          c.token();
          c.token();
          const long long id = c.integer();
          if (hash < 0 || hash >= n || id < 0 || id >= n) { P.range = false; break; }
          P.hash.push_back((int)hash);
          P.id.push_back((int)id);
          const char *q = c.p;  // a record must end its line
          while (q < c.e && (*q == ' ' || *q == '\t' || *q == '\r')) q++;
          if (q < c.e && *q != '\n') { P.ok = false; break; }
        }
      } catch (const Error &) {
        P.ok = false;
      }
    }
  });
  long long total = 0;
  std::vector<long long> take(T, 0);
  for (int t = 0; t < T && total < n; t++) {
    if (!parts[t].ok) return false;
    take[t] = std::min<long long>(n - total, (long long)parts[t].hash.size());
    if (!parts[t].range && total + take[t] < n)
      throw Error(H2H_ERR_FORMAT, "index out of range in " + c0.what);
    total += take[t];
  }
  if (total < n) return false;
  // records of one position or id twice leave another unset: the caller's
  // permutation check rejects the file
  pool.parallel_for(T, 1, [&](int64_t lo, int64_t hi, int) {
    for (int64_t t = lo; t < hi; t++)
      for (long long i = 0; i < take[t]; i++) {
        part_ids[parts[t].hash[i]] = parts[t].id[i];
        id_hash[parts[t].id[i]] = parts[t].hash[i];
      }
  });
  return true;
}

}  // namespace

// Graph_D_H::Graph::Graph (Graph_Fundamental.cu:4-95).  Inputs that the
// reference would read out of bounds (ids outside [0,n), N mismatch between
// the ID and Edge files, short files) are rejected with H2H_ERR_FORMAT.
void load_graph(Graph &g, const std::string &edge, const std::string &idf, const std::string &cutf) {
  Clock clk;
  {
    const FileBytes s = read_file(idf, g.threads);
    Cursor c(s, idf);
    long long n = c.integer();
    GH_CHECK(n > 0 && n < INT32_MAX, H2H_ERR_FORMAT, "bad vertex count in " + idf);
    g.n = (int)n;
    g.part_ids.assign(g.n, -1);
    g.id_hash.assign(g.n, -1);
    if (!parse_ids_parallel(c, g.n, std::max(1, g.threads), g.part_ids, g.id_hash)) {
      std::fill(g.part_ids.begin(), g.part_ids.end(), -1);
      std::fill(g.id_hash.begin(), g.id_hash.end(), -1);
      for (int i = 0; i < g.n; i++) {                     // :27-31
        long long hash = c.integer();
        c.token();
        c.token();
        long long id = c.integer();
        GH_CHECK(hash >= 0 && hash < n && id >= 0 && id < n, H2H_ERR_FORMAT, "index out of range in " + idf);
        g.part_ids[hash] = (int)id;
        g.id_hash[id] = (int)hash;
      }
    }
    for (int i = 0; i < g.n; i++)
      GH_CHECK(g.part_ids[i] >= 0 && g.id_hash[i] >= 0, H2H_ERR_FORMAT, idf + " is not a permutation");
  }
  {
    const FileBytes s = read_file(edge, g.threads);
    Cursor c(s, edge);
    long long n2 = c.integer(), m = c.integer();
    GH_CHECK(n2 == g.n, H2H_ERR_FORMAT, "vertex count of " + edge + " differs from " + idf);
    GH_CHECK(m >= 0 && m < (1LL << 40), H2H_ERR_FORMAT, "bad arc count in " + edge);
    std::vector<int> eu, ev, ew;
    if (!parse_arcs_parallel(c, m, g.n, std::max(1, g.threads), eu, ev, ew)) {
      // the reference's stream semantics, one token at a time
      eu.clear(); ev.clear(); ew.clear();
      eu.reserve(m); ev.reserve(m); ew.reserve(m);
      for (long long i = 0; i < m; i++) {                 // :46-55
        c.one_char();
        long long a = c.integer(), b = c.integer(), w = c.integer();
        GH_CHECK(a >= 1 && a <= g.n && b >= 1 && b <= g.n, H2H_ERR_FORMAT, "vertex id out of range in " + edge);
        GH_CHECK(w >= 0 && w <= INT32_MAX, H2H_ERR_FORMAT, "weight out of range in " + edge);
        if (a == b) continue;                             // self loops dropped
        eu.push_back((int)a - 1); ev.push_back((int)b - 1); ew.push_back((int)w);
      }
    }
    g.m = (int64_t)eu.size();
    // adjList in file order (push_back): when the arcs already come grouped
    // by tail in increasing order, as Edge files are written, the lists are
    // the arc arrays themselves and the offsets the group starts (found in
    // parallel); otherwise a counting pass and a placement pass
    Pool pool(std::max(1, g.threads));
    std::atomic<bool> sorted{true};
    pool.parallel_for(g.m, 1 << 16, [&](int64_t lo, int64_t hi, int) {
      for (int64_t i = std::max<int64_t>(lo, 1); i < hi; i++)
        if (eu[i] < eu[i - 1]) { sorted = false; break; }
    });
    g.adj_off.assign(g.n + 1, 0);
    if (sorted.load()) {
      // adj_off[u] = the first arc whose tail is >= u
      pool.parallel_for(g.m + 1, 1 << 16, [&](int64_t lo, int64_t hi, int) {
        for (int64_t i = lo; i < hi; i++) {
          const int prev = i == 0 ? -1 : eu[i - 1];
          const int cur = i == g.m ? g.n : eu[i];
          for (int u = prev + 1; u <= cur; u++) g.adj_off[u] = (int)i;
        }
      });
      g.adj_v.swap(ev);
      g.adj_w.swap(ew);
    } else {
      std::vector<int> cnt(g.n + 1, 0);
      for (int a : eu) cnt[a]++;
      for (int i = 0; i < g.n; i++) g.adj_off[i + 1] = g.adj_off[i] + cnt[i];
      g.adj_v.resize(g.m);
      g.adj_w.resize(g.m);
      std::vector<int> fill(g.adj_off.begin(), g.adj_off.end() - 1);
      for (int64_t i = 0; i < g.m; i++) {                 // push_back keeps file order
        int k = fill[eu[i]]++;
        g.adj_v[k] = ev[i];
        g.adj_w[k] = ew[i];
      }
    }
  }
  {
    const FileBytes s = read_file(cutf, 1);
    Cursor c(s, cutf);
    long long hf = c.integer();
    GH_CHECK(hf >= 1 && hf <= 30, H2H_ERR_FORMAT, "bad partition height in " + cutf);
    g.H = (int)std::min<long long>(hf, g.H_cli);          // :66-69
    GH_CHECK(g.H >= 1, H2H_ERR_ARG, "partition height must be >= 1");
    const int64_t cells = (int64_t(1) << g.H) - 1;
    g.cut_l.resize(cells);
    g.cut_r.resize(cells);
    for (int64_t i = 0; i < cells; i++) {
      c.integer();
      long long l = c.integer(), r = c.integer();
      GH_CHECK(l >= 0 && r >= l && r <= g.n, H2H_ERR_FORMAT, "cut row out of range in " + cutf);
      g.cut_l[i] = (int)l;
      g.cut_r[i] = (int)r;
    }
  }
  g.t.load = clk.us();
}

// ----------------------------------------------------------------- CSV out

static bool file_exists(const std::string &p) {
  struct stat st;
  return ::stat(p.c_str(), &st) == 0;
}

static const char *kConstructHeader =
    "graphName,PartitionTreeHeight,changeHeight,ParititionTime,makePartitionRankTreeTime,AlllocateLUBTime,LUBSize,"
    "translateLUBToGPUTime,TDInGPUTime,translateBackAndMallocToCPUTime,vertexesConstructedInGPU,"
    "DecompositionTreeSize,TDInCPUTime,TDTREEHeight,,RMQsize,translateRMQTime,H2HLabelSize,,"
    "changeConstructDeviceSize,H2HmallocTime,H2HConstructBFSTreeTime,H2HTranslateBFSTreeTime,H2HUsingTime_CPU,"
    "H2HTranslateTime,H2HUsingTime_GPU,PartitionMethod,threadNum,contractDevice,parallelFine,constructDevice\n";

static std::string fmt_g(double v) {  // std::ostream default float formatting (precision 6)
  char b[64];
  std::snprintf(b, sizeof b, "%g", v);
  return b;
}

static const char *method_prefix(int method) {
  switch (method) {
    case 2: return "Minimum";
    case 3: return "metis";
    case 4: return "scotch";
    default: return "Latitude";
  }
}

const char *partition_file_prefix(int method) { return method_prefix(method); }

// GraphPartition.cu:252-265: one row per call, afs[h]/n for h = 1..H.
void write_partition_rate(const Graph &g, const std::string &dir) {
  std::string path = dir + "/" + method_prefix(g.method) + "PartitionRate.csv";
  FILE *f = std::fopen(path.c_str(), "a");
  if (!f) throw Error(H2H_ERR_IO, "cannot open " + path);
  std::string row = g.name + ",";
  for (size_t i = 1; i < g.layer_rate.size(); i++) row += fmt_g(g.layer_rate[i]) + ",";
  row += "\n";
  std::fputs(row.c_str(), f);
  std::fclose(f);
}

static std::string construct_row(const Graph &g, bool after_labels) {
  const double MB = 1024.0 * 1024.0;
  double lub_mb = (double)g.lub * 12.0 / MB;  // sizeof(myPair<int>) = 12 in the reference
  double dts = (double)g.decomposition_size * 12.0 / MB;
  double rmq_mb = 0, label_mb;
  if (after_labels) {                                  // mallocH2HLabel_noHub, H2HConsturction.cu:704-707
    rmq_mb = ((double)g.euler_n * 8 + (double)g.rmq_total * 4 + (double)g.n * 4) / MB;
    label_mb = ((double)(g.n + 1) * 8 * 2 + (double)(g.pos_hash.empty() ? 0 : g.pos_hash[g.n]) * 4 +
                (double)g.h2h_size * 4) / MB;
  } else {                                             // beforeH2H_noHub, TreeStructure.cu:69-70
    label_mb = ((double)8 * 2 * g.n + (double)g.decomposition_size * 4 + (double)g.h2h_size * 4) / MB;
  }
  const Timings &t = g.t;
  std::string r;
  r += g.name + "," + std::to_string(g.H) + "," + std::to_string(g.C) + ",0," + std::to_string(t.rank_tree) + "," +
       std::to_string(t.lub) + "," + fmt_g(lub_mb) + "," + std::to_string(t.translate_lub) + "," +
       std::to_string(t.td_gpu) + "," + std::to_string(t.translate_back) + "," + std::to_string(g.gpu_vertices) +
       "," + fmt_g(dts) + "," + std::to_string(t.td_cpu) + "," + std::to_string(g.tree_height) + ",," +
       fmt_g(rmq_mb) + ",0," + fmt_g(label_mb) + ",,64,";
  if (after_labels)
    r += std::to_string(t.malloc_labels) + "," + std::to_string(t.bfs) + ",0,0," + std::to_string(t.translate_labels) +
         "," + std::to_string(t.fill_gpu);
  else
    r += "0,0,0,0,0,0";
  r += "," + std::to_string(g.method) + "," + std::to_string(g.threads) + "," + std::to_string(g.contract_device) +
       "," + std::to_string(g.parallel_fine) + "," + std::to_string(g.construct_device) + "\n";
  return r;
}

static void append_csv(const std::string &path, const char *header, const std::string &row) {
  bool exists = file_exists(path);
  FILE *f = std::fopen(path.c_str(), "a");
  if (!f) throw Error(H2H_ERR_IO, "cannot open " + path + " (the reference needs the directory to exist too)");
  if (!exists) std::fputs(header, f);
  std::fputs(row.c_str(), f);
  std::fclose(f);
}

void write_contract_csv(const Graph &g, const std::string &root) {
  append_csv(root + "/ConstructInfo/" + g.name + "/contract.csv", kConstructHeader, construct_row(g, false));
}

void write_construct_info(const Graph &g, const std::string &root) {
  append_csv(root + "/ConstructInfo/" + g.name + "/constructInfo.csv", kConstructHeader, construct_row(g, true));
}

void write_query_result(const Graph &g, const std::string &root, int64_t qn, const int64_t *t19) {
  static const char *hdr =
      "queryNumber,sequence,multiThread-4,multiThread-6,multiThread-8,multiThread-10,multiThread-12,multiThread-14,"
      "multiThread-16,GPUnoLCA-64,GPUwithLCA-64,GPUnoLCA-128,GPUwithLCA-128,GPUnoLCA-256,GPUwithLCA-256,"
      "GPUnoLCA-512,GPUwithLCA-512,GPUnoLCA-1024,GPUwithLCA-1024,TreeHeight,changeHeight,PartitionMethod,"
      "contractDevice\n";
  std::string r = std::to_string(qn);
  for (int i = 0; i < 18; i++) r += "," + std::to_string(t19 ? t19[i] : 0);
  r += "," + std::to_string(g.H) + "," + std::to_string(g.C) + "," + std::to_string(g.method) + "," +
       std::to_string(g.contract_device) + "\n";
  append_csv(root + "/QueryResult/" + g.name + "/random.csv", hdr, r);
}

}  // namespace gh
