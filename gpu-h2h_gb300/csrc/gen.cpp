// gen.cpp -- workload generators with no counterpart in the reference: a
// seeded synthetic road graph written in the reference's Edge / Node / ID /
// Cut formats (jittered grid, diagonals, highway tiers, a spanning tree that
// keeps it connected, latitude/longitude median bisection), uniform query
// pairs, and "local" pairs drawn by random walks over a graph's arcs.  All
// arithmetic is integer, so x86 and Arm hosts write the same bytes.
//
// Self-contained (standard library only): the library links it, and so does
// the oracle, so a CPU-only measurement can draw the same graph and pairs
// without loading the GPU library.
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "gen.h"

namespace gh {

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

void gen_default(h2h_gen_params *p) {  // the 64x64 test grid (4,096 vertices)
  std::memset(p, 0, sizeof(*p));
  p->n = 4096;
  p->cols = 64;
  p->aspect_milli = 1000;
  p->jitter_milli = 300;
  p->drop_permille = 100;
  p->diag_permille = 50;
  p->hw_k = 3;
  p->hw_scale_milli = 400;
  p->partition_height = 6;
  p->seed = 20240601;
}

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

void gen_local_pairs_csr(int nv, const int *off, const int *adj_v, int64_t n, int hops, uint64_t seed, int *x,
                         int *y) {
  Rng r(seed);
  for (int64_t i = 0; i < n; i++) {
    int s = (int)r.below(nv), t = s;
    int steps = 1 + (int)r.below(hops > 0 ? hops : 1);
    for (int k = 0; k < steps; k++) {
      int deg = off[t + 1] - off[t];
      if (deg == 0) break;
      t = adj_v[off[t] + (int)r.below(deg)];
    }
    x[i] = s;
    y[i] = t;
  }
}

}  // namespace gh
