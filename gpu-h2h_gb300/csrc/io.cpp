// io.cpp -- file formats of the reference: the Edge / ID / Cut loaders
// (Graph_Fundamental.cu:4-95), the CSV writers (GraphPartition.cu:252-265,
// TreeStructure.cu:54-99, Graph_Fundamental.cu:132-170, Query.cu:597-622),
// and the seeded synthetic road-graph generator that writes those formats.
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <numeric>

#include "graph.h"
#include "gpuh2h_tools.h"
#include "pool.h"

namespace gh {

namespace {

std::string read_file(const std::string &path) {
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) throw Error(H2H_ERR_IO, "cannot open " + path);
  std::string s;
  std::fseek(f, 0, SEEK_END);
  long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  s.resize(sz > 0 ? (size_t)sz : 0);
  if (sz > 0 && std::fread(&s[0], 1, (size_t)sz, f) != (size_t)sz) {
    std::fclose(f);
    throw Error(H2H_ERR_IO, "short read on " + path);
  }
  std::fclose(f);
  return s;
}

// Whitespace tokenizer with the istream >> semantics the reference relies on.
struct Cursor {
  const char *p, *e;
  std::string what;
  explicit Cursor(const std::string &s, std::string w) : p(s.data()), e(s.data() + s.size()), what(std::move(w)) {}
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
    std::string s = read_file(idf);
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
    std::string s = read_file(edge);
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
    std::vector<int> cnt(g.n + 1, 0);
    for (int a : eu) cnt[a]++;
    g.m = (int64_t)eu.size();
    g.adj_off.assign(g.n + 1, 0);
    for (int i = 0; i < g.n; i++) g.adj_off[i + 1] = g.adj_off[i] + cnt[i];
    g.adj_v.resize(g.m);
    g.adj_w.resize(g.m);
    std::vector<int> fill(g.adj_off.begin(), g.adj_off.end() - 1);
    for (int64_t i = 0; i < g.m; i++) {                   // push_back keeps file order
      int k = fill[eu[i]]++;
      g.adj_v[k] = ev[i];
      g.adj_w[k] = ew[i];
    }
  }
  {
    std::string s = read_file(cutf);
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

// ------------------------------------------------------------- generator

namespace {

struct Rng {  // xoshiro256** seeded by splitmix64: same stream on every platform
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    uint64_t z = seed;
    for (int i = 0; i < 4; i++) {
      z += 0x9E3779B97F4A7C15ULL;
      uint64_t x = z;
      x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
      x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
      s[i] = x ^ (x >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t; s[3] = rotl(s[3], 45);
    return r;
  }
  uint64_t below(uint64_t m) { return (uint64_t)(((unsigned __int128)next() * m) >> 64); }
};

int64_t isqrt_round(int64_t s) {  // round(sqrt(s)), halves up, exact integer arithmetic
  if (s <= 0) return 0;
  int64_t r = (int64_t)std::sqrt((double)s);
  while (r * r > s) r--;
  while ((r + 1) * (r + 1) <= s) r++;
  return (s - r * r > r) ? r + 1 : r;
}

struct UF {
  std::vector<int> p;
  explicit UF(int n) : p(n) { std::iota(p.begin(), p.end(), 0); }
  int find(int x) {
    while (p[x] != x) { p[x] = p[p[x]]; x = p[x]; }
    return x;
  }
  bool unite(int a, int b) {
    a = find(a); b = find(b);
    if (a == b) return false;
    p[a] = b;
    return true;
  }
};

void mkdirs(const std::string &path) {
  std::string cur;
  for (size_t i = 0; i < path.size(); i++) {
    cur += path[i];
    if (path[i] == '/' && cur.size() > 1) ::mkdir(cur.c_str(), 0755);
  }
  ::mkdir(path.c_str(), 0755);
}

void put_milli(std::string &out, int64_t v) {  // v/1000 with three decimals, no float formatting
  if (v < 0) { out += '-'; v = -v; }
  out += std::to_string(v / 1000);
  out += '.';
  char b[4];
  std::snprintf(b, sizeof b, "%03d", (int)(v % 1000));
  out += b;
}

void write_text(const std::string &path, const std::string &s) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) throw Error(H2H_ERR_IO, "cannot write " + path);
  if (!s.empty() && std::fwrite(s.data(), 1, s.size(), f) != s.size()) {
    std::fclose(f);
    throw Error(H2H_ERR_IO, "short write on " + path);
  }
  std::fclose(f);
}

// k nearest peers of every point in pts (squared distance, ties by index), by bucket grid.
std::vector<std::vector<int>> knn(const std::vector<int64_t> &x, const std::vector<int64_t> &y,
                                  const std::vector<int> &pts, int k) {
  const int m = (int)pts.size();
  std::vector<std::vector<int>> res(m);
  if (m < 2) return res;
  int64_t minx = INT64_MAX, maxx = INT64_MIN, miny = INT64_MAX, maxy = INT64_MIN;
  for (int p : pts) { minx = std::min(minx, x[p]); maxx = std::max(maxx, x[p]); miny = std::min(miny, y[p]); maxy = std::max(maxy, y[p]); }
  int64_t w = maxx - minx + 1, h = maxy - miny + 1;
  int64_t cell = std::max<int64_t>(1, isqrt_round((w * h) / std::max(1, m / 2)));
  int64_t gx = w / cell + 1, gy = h / cell + 1;
  std::vector<std::vector<int>> bucket(gx * gy);
  for (int i = 0; i < m; i++) bucket[((y[pts[i]] - miny) / cell) * gx + (x[pts[i]] - minx) / cell].push_back(i);
  std::vector<std::pair<int64_t, int>> cand;
  for (int i = 0; i < m; i++) {
    int64_t cx = (x[pts[i]] - minx) / cell, cy = (y[pts[i]] - miny) / cell;
    cand.clear();
    for (int64_t r = 0;; r++) {
      for (int64_t by = cy - r; by <= cy + r; by++) {
        if (by < 0 || by >= gy) continue;
        for (int64_t bx = cx - r; bx <= cx + r; bx++) {
          if (bx < 0 || bx >= gx) continue;
          if (std::max(std::llabs(bx - cx), std::llabs(by - cy)) != r) continue;
          for (int j : bucket[by * gx + bx]) {
            if (j == i) continue;
            int64_t dx = x[pts[i]] - x[pts[j]], dy = y[pts[i]] - y[pts[j]];
            cand.push_back({dx * dx + dy * dy, j});
          }
        }
      }
      if ((int)cand.size() >= k) {
        std::sort(cand.begin(), cand.end());
        int64_t reach = r * cell;  // every unvisited point is at least this far
        if (cand[k - 1].first <= reach * reach) break;
      }
      if (r > gx + gy) break;
    }
    std::sort(cand.begin(), cand.end());
    for (int t = 0; t < (int)cand.size() && t < k; t++) res[i].push_back(pts[cand[t].second]);
  }
  return res;
}

}  // namespace

void generate_road(const h2h_gen_params &p, const std::string &root, const std::string &name, int64_t *n_arcs) {
  GH_CHECK(p.n >= 2 && p.n < (1LL << 30), H2H_ERR_ARG, "generator: n out of range");
  GH_CHECK(p.partition_height >= 1 && p.partition_height <= 30, H2H_ERR_ARG, "generator: bad partition height");
  const int n = (int)p.n;
  Rng rng(p.seed);
  int64_t cols = p.cols;
  if (cols <= 0) {
    double a = p.aspect_milli > 0 ? p.aspect_milli / 1000.0 : 1.0;
    cols = std::max<int64_t>(1, std::llround(std::sqrt((double)n / a)));
  }
  std::vector<int64_t> X(n), Y(n);
  const int64_t J = p.jitter_milli;
  for (int i = 0; i < n; i++) {
    X[i] = 1000 * (i % cols) + (int64_t)rng.below(2 * J + 1) - J;
    Y[i] = 1000 * (i / cols) + (int64_t)rng.below(2 * J + 1) - J;
  }
  auto wgt = [&](int a, int b) {
    int64_t dx = X[a] - X[b], dy = Y[a] - Y[b];
    return isqrt_round(dx * dx + dy * dy) + 1;
  };
  struct E { int a, b; int64_t w; };
  std::vector<E> base;  // grid + diagonal edges
  for (int i = 0; i < n; i++) {
    int64_t c = i % cols;
    if (c + 1 < cols && i + 1 < n) base.push_back({i, i + 1, 0});
    if (i + cols < n) base.push_back({i, (int)(i + cols), 0});
  }
  for (int i = 0; i < n; i++) {
    int64_t c = i % cols;
    if (c + 1 >= cols || i + cols + 1 >= n) continue;
    if ((int64_t)rng.below(1000) < p.diag_permille) {
      if (rng.below(2)) base.push_back({i, (int)(i + cols + 1), 0});
      else base.push_back({i + 1, (int)(i + cols), 0});
    }
  }
  for (auto &e : base) e.w = wgt(e.a, e.b);
  // highway tiers: nested random subsets, each vertex linked to its k nearest tier peers
  std::vector<E> hw;
  {
    std::vector<int> tier;
    int64_t cnt = (int64_t)n * p.hw_permille10 / 10000;
    std::vector<int> perm(n);
    std::iota(perm.begin(), perm.end(), 0);
    int64_t scale = p.hw_scale_milli > 0 ? p.hw_scale_milli : 400;
    for (int t = 0; t < p.hw_tiers; t++) {
      if (t == 0) {
        cnt = std::max<int64_t>(cnt, p.hw_k + 1);
        cnt = std::min<int64_t>(cnt, n);
        for (int64_t i = 0; i < cnt; i++) std::swap(perm[i], perm[i + (int64_t)rng.below(n - i)]);
        tier.assign(perm.begin(), perm.begin() + cnt);
      } else {
        int64_t c2 = std::max<int64_t>((int64_t)tier.size() / 5, p.hw_k + 1);
        if (c2 >= (int64_t)tier.size()) break;
        for (int64_t i = 0; i < c2; i++) std::swap(tier[i], tier[i + (int64_t)rng.below(tier.size() - i)]);
        tier.resize(c2);
        scale = scale * 3 / 4;
      }
      std::sort(tier.begin(), tier.end());
      auto nb = knn(X, Y, tier, p.hw_k);
      for (size_t i = 0; i < tier.size(); i++)
        for (int o : nb[i]) hw.push_back({tier[i], o, std::max<int64_t>(1, wgt(tier[i], o) * scale / 1000)});
    }
  }
  // random spanning tree over the base edges keeps the graph connected
  std::vector<int> idx(base.size());
  std::iota(idx.begin(), idx.end(), 0);
  for (size_t i = idx.size(); i > 1; i--) std::swap(idx[i - 1], idx[rng.below(i)]);
  UF uf(n);
  std::vector<char> in_tree(base.size(), 0);
  for (int e : idx) if (uf.unite(base[e].a, base[e].b)) in_tree[e] = 1;
  // a graph whose grid is not connected (tiny n) still gets connected by the highway/base tree
  std::vector<int> non_tree;
  for (int e : idx) if (!in_tree[e]) non_tree.push_back(e);
  // dedupe highway edges against base and each other
  auto key = [](int a, int b) { return a < b ? ((uint64_t)a << 32) | (uint32_t)b : ((uint64_t)b << 32) | (uint32_t)a; };
  std::vector<uint64_t> seen;
  seen.reserve(base.size() + hw.size());
  for (auto &e : base) seen.push_back(key(e.a, e.b));
  std::sort(seen.begin(), seen.end());
  std::vector<E> hw_u;
  {
    std::vector<uint64_t> hk;
    for (auto &e : hw) hk.push_back(key(e.a, e.b));
    std::vector<int> ord(hw.size());
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return hk[a] < hk[b]; });
    for (size_t i = 0; i < ord.size(); i++) {
      uint64_t k = hk[ord[i]];
      if (i > 0 && hk[ord[i - 1]] == k) continue;
      if (std::binary_search(seen.begin(), seen.end(), k)) continue;
      hw_u.push_back(hw[ord[i]]);
    }
  }
  int64_t drop;
  if (p.target_arcs > 0) drop = (int64_t)base.size() + (int64_t)hw_u.size() - p.target_arcs / 2;
  else drop = (int64_t)base.size() * p.drop_permille / 1000;
  drop = std::max<int64_t>(0, std::min<int64_t>(drop, (int64_t)non_tree.size()));
  std::vector<char> dropped(base.size(), 0);
  for (int64_t i = 0; i < drop; i++) dropped[non_tree[i]] = 1;  // non_tree is already in shuffled order
  std::vector<E> edges;
  for (size_t e = 0; e < base.size(); e++) if (!dropped[e]) edges.push_back(base[e]);
  for (auto &e : hw_u) edges.push_back(e);
  for (auto &e : edges) {
    if (p.weight_max > 0) e.w = std::min<int64_t>(e.w, p.weight_max);
    e.w = std::max<int64_t>(e.w, 1);
  }
  // arcs in both directions, sorted by (u, v)
  std::vector<std::pair<uint64_t, int64_t>> arcs;
  arcs.reserve(edges.size() * 2);
  for (auto &e : edges) {
    arcs.push_back({((uint64_t)e.a << 32) | (uint32_t)e.b, e.w});
    arcs.push_back({((uint64_t)e.b << 32) | (uint32_t)e.a, e.w});
  }
  std::sort(arcs.begin(), arcs.end());
  // latitude/longitude recursive median bisection, x first, ties by id
  const int H = p.partition_height;
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::vector<std::pair<int, int>> cells{{0, n}};
  std::string cut = std::to_string(H) + "\n";
  for (int h = 1; h <= H; h++) {
    std::vector<std::pair<int, int>> next;
    for (auto &c : cells) {
      cut += std::to_string(h) + " " + std::to_string(c.first) + " " + std::to_string(c.second) + "\n";
      if (h == H) continue;
      const std::vector<int64_t> &K = (h % 2 == 1) ? X : Y;
      std::sort(order.begin() + c.first, order.begin() + c.second, [&](int a, int b) {
        return K[a] != K[b] ? K[a] < K[b] : a < b;
      });
      int mid = c.first + (c.second - c.first) / 2;
      next.push_back({c.first, mid});
      next.push_back({mid, c.second});
    }
    cells.swap(next);
  }
  mkdirs(root + "/Graph/USA");
  mkdirs(root + "/Partition/" + name);
  std::string s;
  s.reserve(arcs.size() * 24 + 64);
  s += std::to_string(n) + " " + std::to_string(arcs.size()) + "\n";
  for (auto &a : arcs) {
    s += "a ";
    s += std::to_string((a.first >> 32) + 1);
    s += ' ';
    s += std::to_string((a.first & 0xffffffffu) + 1);
    s += ' ';
    s += std::to_string(a.second);
    s += '\n';
  }
  write_text(root + "/Graph/USA/" + name + "Edge.txt", s);
  s.clear();
  s += std::to_string(n) + "\n";
  for (int i = 0; i < n; i++) {
    s += "v " + std::to_string(i + 1) + " ";
    put_milli(s, X[i]);
    s += ' ';
    put_milli(s, Y[i]);
    s += '\n';
  }
  write_text(root + "/Graph/USA/" + name + "Node.txt", s);
  s.clear();
  s += std::to_string(n) + "\n";
  for (int i = 0; i < n; i++) {
    s += std::to_string(i) + " ";
    put_milli(s, X[order[i]]);
    s += ' ';
    put_milli(s, Y[order[i]]);
    s += ' ' + std::to_string(order[i]) + "\n";
  }
  write_text(root + "/Partition/" + name + "/LatitudeID.txt", s);
  write_text(root + "/Partition/" + name + "/LatitudeCut.txt", cut);
  if (n_arcs) *n_arcs = (int64_t)arcs.size();
}

void gen_uniform_pairs(int nv, int64_t n, uint64_t seed, int *x, int *y) {
  Rng r(seed);
  for (int64_t i = 0; i < n; i++) {
    x[i] = (int)r.below(nv);
    y[i] = (int)r.below(nv);
  }
}

void gen_local_pairs(const Graph &g, int64_t n, int hops, uint64_t seed, int *x, int *y) {
  Rng r(seed);
  for (int64_t i = 0; i < n; i++) {
    int s = (int)r.below(g.n), t = s;
    int steps = 1 + (int)r.below(hops > 0 ? hops : 1);
    for (int k = 0; k < steps; k++) {
      int deg = g.adj_off[t + 1] - g.adj_off[t];
      if (deg == 0) break;
      t = g.adj_v[g.adj_off[t] + (int)r.below(deg)];
    }
    x[i] = s;
    y[i] = t;
  }
}

}  // namespace gh
