/*
 * h2h_oracle.c -- plain-C restatement of the GPU-H2H hot path (CPU oracle).
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker for the CUDA implementation.
 * Nothing in the product library links or calls this file.
 *
 * Every function names the reference file:line it restates (paths are
 * relative to the reference project root).  Data layouts mirror the
 * reference where the order of operations depends on them (the LUB
 * adjacency, the candidate array of each partition cell, the heap key).
 */
#define _GNU_SOURCE
#include "h2h_oracle.h"

#include <limits.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct { int v, w; } arc_t;

typedef struct {           /* growable int vector */
  int *a;
  int64_t n, cap;
} ivec;

static void iv_push(ivec *v, int x) {
  if (v->n == v->cap) {
    v->cap = v->cap ? v->cap * 2 : 16;
    v->a = (int *)realloc(v->a, (size_t)v->cap * sizeof(int));
  }
  v->a[v->n++] = x;
}

/* Per-vertex ordered map nbr -> (w, hub) standing in for the reference's
 * unordered_map<int, pairs> CHAdjlist (Graph_D.cuh:496).  The reference
 * iterates the map in hash order; every use below is order-independent. */
typedef struct {
  int *nb, *w, *hub;
  int n, cap;
} amap;

static int am_find(const amap *m, int key) {
  int lo = 0, hi = m->n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (m->nb[mid] < key) lo = mid + 1; else hi = mid;
  }
  return (lo < m->n && m->nb[lo] == key) ? lo : -1;
}
static int am_lower(const amap *m, int key) {
  int lo = 0, hi = m->n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (m->nb[mid] < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}
/* emplace: insert only when absent (first-seen wins), as std::unordered_map::emplace */
static void am_emplace(amap *m, int key, int w, int hub) {
  int pos = am_lower(m, key);
  if (pos < m->n && m->nb[pos] == key) return;
  if (m->n == m->cap) {
    m->cap = m->cap ? m->cap * 2 : 8;
    m->nb = (int *)realloc(m->nb, (size_t)m->cap * sizeof(int));
    m->w = (int *)realloc(m->w, (size_t)m->cap * sizeof(int));
    m->hub = (int *)realloc(m->hub, (size_t)m->cap * sizeof(int));
  }
  memmove(m->nb + pos + 1, m->nb + pos, (size_t)(m->n - pos) * sizeof(int));
  memmove(m->w + pos + 1, m->w + pos, (size_t)(m->n - pos) * sizeof(int));
  memmove(m->hub + pos + 1, m->hub + pos, (size_t)(m->n - pos) * sizeof(int));
  m->nb[pos] = key; m->w[pos] = w; m->hub[pos] = hub;
  m->n++;
}
static void am_erase(amap *m, int key) {
  int pos = am_find(m, key);
  if (pos < 0) return;
  memmove(m->nb + pos, m->nb + pos + 1, (size_t)(m->n - pos - 1) * sizeof(int));
  memmove(m->w + pos, m->w + pos + 1, (size_t)(m->n - pos - 1) * sizeof(int));
  memmove(m->hub + pos, m->hub + pos + 1, (size_t)(m->n - pos - 1) * sizeof(int));
  m->n--;
}

struct or_graph {
  int n, H, C, threads;
  int64_t m;                 /* arcs kept (self loops dropped)           */
  /* loader (Graph_Fundamental.cu:4-95) */
  int *adj_off;              /* CSR of adjList in file order             */
  arc_t *adj;
  int *ne_id;                /* NE_P[idx].NodeID                          */
  int *id_hash;              /* ID_hash[vertex] = idx                     */
  or_pairs *ptree;           /* partition_Tree[2^H-1]                     */
  int64_t n_cells;
  or_pairs *chinfo_h;        /* CHInfo_H                                  */
  /* makeAdjcentNode (GraphPartition.cu:178-308) */
  or_tdrank *nonadj;
  int64_t nonadj_n;
  or_mypair *nanhash;
  or_mypair *chtree_hash;    /* indexed by partition idx                  */
  or_mypair *chtree;
  int64_t lub;
  /* GPU contraction state */
  unsigned char *visited;
  or_pairs *chinfo_d;
  /* CPU heap (Traditional_H2H.cu) */
  amap *chadj;
  or_pairs *chinfo;
  int gpu_vertices;
  /* tree (TreeStructure.cu) */
  int head;
  int *rank, *father, *child_cnt, *child_off, *childs;
  int *euler_id, *euler_depth;
  int64_t euler_n;
  int *first, *depth;
  int64_t h2h_size;
  int tree_height;
  int64_t *rmq_hash;
  int *rmq_id;
  int64_t rmq_n;
  /* labels (H2HConsturction.cu) */
  int64_t *dis_hash, *pos_hash;
  int *dis, *pos_id, *pos_pos;
  int64_t pos_n;
  int *tree_bfs, *tree_hash;
  int n_levels;
  char err[256];
};

const char *or_error(const or_graph *g) { return g ? g->err : "null graph"; }

/* ---------------------------------------------------------------- loader */
/* Graph_D_H::Graph::Graph (Graph_Fundamental.cu:4-95). */
or_graph *or_load(const char *edge_file, const char *id_file, const char *cut_file,
                  int partition_height, int change_height, int threads) {
  or_graph *g = (or_graph *)calloc(1, sizeof(or_graph));
  g->threads = threads > 0 ? threads : 1;
  g->C = change_height;
  FILE *f = fopen(id_file, "r");
  if (!f) { free(g); return NULL; }
  int n = 0;
  if (fscanf(f, "%d", &n) != 1) { fclose(f); free(g); return NULL; }
  g->ne_id = (int *)malloc(sizeof(int) * (size_t)n);
  g->id_hash = (int *)malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < n; i++) { g->ne_id[i] = -1; g->id_hash[i] = -1; }
  for (int i = 0; i < n; i++) {                     /* :27-31 */
    int hash, id; double la, gr;
    if (fscanf(f, "%d %lf %lf %d", &hash, &la, &gr, &id) != 4) { fclose(f); or_free(g); return NULL; }
    g->ne_id[hash] = id;
    g->id_hash[id] = hash;
  }
  fclose(f);
  f = fopen(edge_file, "r");
  if (!f) { or_free(g); return NULL; }
  long long mm = 0;
  int n2 = 0;
  if (fscanf(f, "%d %lld", &n2, &mm) != 2) { fclose(f); or_free(g); return NULL; }
  if (n2 != n) { fclose(f); or_free(g); return NULL; }
  g->n = n;
  int *cnt = (int *)calloc((size_t)n + 1, sizeof(int));
  int *eu = (int *)malloc(sizeof(int) * (size_t)mm), *ev = (int *)malloc(sizeof(int) * (size_t)mm),
      *ew = (int *)malloc(sizeof(int) * (size_t)mm);
  int64_t kept = 0;
  for (long long i = 0; i < mm; i++) {              /* :46-55 */
    char s[8]; int a, b, w;
    if (fscanf(f, "%7s %d %d %d", s, &a, &b, &w) != 4) { fclose(f); free(cnt); free(eu); free(ev); free(ew); or_free(g); return NULL; }
    if (a == b) continue;                            /* self loops dropped */
    eu[kept] = a - 1; ev[kept] = b - 1; ew[kept] = w; kept++;
    cnt[a - 1]++;
  }
  fclose(f);
  g->m = kept;
  g->adj_off = (int *)malloc(sizeof(int) * ((size_t)n + 1));
  g->adj_off[0] = 0;
  for (int i = 0; i < n; i++) g->adj_off[i + 1] = g->adj_off[i] + cnt[i];
  g->adj = (arc_t *)malloc(sizeof(arc_t) * (size_t)(kept ? kept : 1));
  for (int i = 0; i < n; i++) cnt[i] = g->adj_off[i];
  for (int64_t i = 0; i < kept; i++) {             /* push_back keeps file order */
    arc_t a = {ev[i], ew[i]};
    g->adj[cnt[eu[i]]++] = a;
  }
  free(cnt); free(eu); free(ev); free(ew);
  f = fopen(cut_file, "r");
  if (!f) { or_free(g); return NULL; }
  int hfile = 0;
  if (fscanf(f, "%d", &hfile) != 1) { fclose(f); or_free(g); return NULL; }
  g->H = hfile < partition_height ? hfile : partition_height;  /* :66-69 */
  g->n_cells = ((int64_t)1 << g->H) - 1;
  g->ptree = (or_pairs *)malloc(sizeof(or_pairs) * (size_t)g->n_cells);
  for (int64_t i = 0; i < g->n_cells; i++) {
    int h, l, r;
    if (fscanf(f, "%d %d %d", &h, &l, &r) != 3) { fclose(f); or_free(g); return NULL; }
    g->ptree[i].first = l; g->ptree[i].second = r;
  }
  fclose(f);
  g->chinfo_h = (or_pairs *)malloc(sizeof(or_pairs) * (size_t)n);   /* :85-91 */
  for (int i = 0; i < n; i++) { g->chinfo_h[i].first = g->adj_off[i + 1] - g->adj_off[i]; g->chinfo_h[i].second = 0; }
  g->visited = (unsigned char *)calloc((size_t)n, 1);
  return g;
}

void or_free(or_graph *g) {
  if (!g) return;
  free(g->adj_off); free(g->adj); free(g->ne_id); free(g->id_hash); free(g->ptree);
  free(g->chinfo_h); free(g->nonadj); free(g->nanhash); free(g->chtree_hash); free(g->chtree);
  free(g->visited); free(g->chinfo_d); free(g->chinfo);
  if (g->chadj) {
    for (int i = 0; i < g->n; i++) { free(g->chadj[i].nb); free(g->chadj[i].w); free(g->chadj[i].hub); }
    free(g->chadj);
  }
  free(g->rank); free(g->father); free(g->child_cnt); free(g->child_off); free(g->childs);
  free(g->euler_id); free(g->euler_depth); free(g->first); free(g->depth);
  free(g->rmq_hash); free(g->rmq_id); free(g->dis_hash); free(g->pos_hash); free(g->dis);
  free(g->pos_id); free(g->pos_pos); free(g->tree_bfs); free(g->tree_hash);
  free(g);
}

/* ------------------------------------------------- elimination sets + LUB */
/* Graph::makeAdjcentNode (GraphPartition.cu:178-308), goalHeight = 0. */
static int make_adjacent_node(or_graph *g) {
  const int n = g->n;
  unsigned char *alive = (unsigned char *)malloc((size_t)n), *alive_cp = (unsigned char *)malloc((size_t)n);
  int *place = (int *)malloc(sizeof(int) * (size_t)n);
  int *incell = (int *)malloc(sizeof(int) * (size_t)n);   /* cell membership stamp */
  int *outsz = (int *)malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < n; i++) { alive[i] = 1; place[i] = g->adj_off[i + 1] - g->adj_off[i]; incell[i] = -1; }
  g->nanhash = (or_mypair *)calloc((size_t)g->n_cells, sizeof(or_mypair));
  for (int64_t i = 0; i < g->n_cells; i++) { g->nanhash[i].NodeID = -1; }
  g->nonadj = (or_tdrank *)malloc(sizeof(or_tdrank) * (size_t)n);
  g->nonadj_n = 0;
  ivec members = {0};
  for (int h = g->H; h > 0; h--) {
    int64_t lo = ((int64_t)1 << (h - 1)) - 1, hi = ((int64_t)1 << h) - 2;
    memcpy(alive_cp, alive, (size_t)n);
    for (int64_t i = hi; i >= lo; i--) {             /* :202 high index to low */
      g->nanhash[i].first = (int)g->nonadj_n;
      g->nanhash[i].second = 0;
      g->nanhash[i].NodeID = 0;
      int l = g->ptree[i].first, r = g->ptree[i].second;
      members.n = 0;
      for (int j = l; j < r; j++) {                  /* std::map<int,int> subgraph: ordered by id */
        int id = g->ne_id[j];
        if (!alive[id]) continue;
        if (incell[id] == (int)i) continue;
        incell[id] = (int)i;
        iv_push(&members, id);
      }
      /* std::map iterates in increasing id */
      for (int64_t a = 1; a < members.n; a++) {
        int x = members.a[a]; int64_t b = a - 1;
        while (b >= 0 && members.a[b] > x) { members.a[b + 1] = members.a[b]; b--; }
        members.a[b + 1] = x;
      }
      int sz = (int)members.n;
      g->nanhash[i].second = sz;
      for (int64_t a = 0; a < members.n; a++) {      /* :219-230 */
        int id = members.a[a];
        int os = sz;
        for (int e = g->adj_off[id]; e < g->adj_off[id + 1]; e++) {
          int nb = g->adj[e].v;
          if (!alive[nb]) continue;
          if (incell[nb] != (int)i) os++;
        }
        outsz[id] = os;
      }
      for (int64_t a = 0; a < members.n; a++) {      /* :232-240 */
        int id = members.a[a];
        if (outsz[id] == g->nanhash[i].second) {
          alive_cp[id] = 0;
          g->nanhash[i].NodeID++;
          or_tdrank t = {g->adj_off[id + 1] - g->adj_off[id], id, 0, 0};
          g->nonadj[g->nonadj_n++] = t;
        }
        if (outsz[id] > place[id]) place[id] = outsz[id];
      }
      /* reset stamps so a vertex can be re-stamped by a later cell with the same index */
      for (int64_t a = 0; a < members.n; a++) incell[members.a[a]] = -1;
    }
    memcpy(alive, alive_cp, (size_t)n);
  }
  free(members.a);
  /* LUB allocation (:270-292): slots laid out in partition-array order. */
  g->chtree_hash = (or_mypair *)malloc(sizeof(or_mypair) * (size_t)n);
  int64_t total = 0;
  for (int i = 0; i < n; i++) total += place[g->ne_id[i]];
  g->lub = total;
  g->chtree = (or_mypair *)malloc(sizeof(or_mypair) * (size_t)(total ? total : 1));
  int64_t off = 0;
  int rc = 0;
  for (int i = 0; i < n; i++) {
    int id = g->ne_id[i];
    g->chtree_hash[i].first = 0;
    g->chtree_hash[i].second = place[id];
    g->chtree_hash[i].NodeID = (int)off;
    for (int s = 0; s < place[id]; s++) { or_mypair e = {-1, INT_MAX, 0}; g->chtree[off + s] = e; }
    for (int e = g->adj_off[id]; e < g->adj_off[id + 1]; e++) {
      if (g->chtree_hash[i].first >= g->chtree_hash[i].second) { rc = -1; break; }   /* :286-290 */
      or_mypair p = {-1, g->adj[e].v, g->adj[e].w};
      g->chtree[off + g->chtree_hash[i].first] = p;
      g->chtree_hash[i].first++;
    }
    off += place[id];
  }
  free(alive); free(alive_cp); free(place); free(incell); free(outsz);
  if (rc) snprintf(g->err, sizeof g->err, "LUB allocate error");
  return rc;
}

/* ------------------------------------------------ restated GPU cell kernel */
static int td_less(const or_tdrank *a, const or_tdrank *b) {   /* Graph_D.cuh:154-173 */
  if (a->third + a->first != b->third + b->first) return a->third + a->first < b->third + b->first;
  if (a->first != b->first) return a->first < b->first;
  return a->second < b->second;
}

/* tools::bobbleSortPairs (kernel_functions.cu:21-41): full passes, no early
 * exit.  TDrank::operator= leaves childSize in place, which is unused. */
static void bubble_td(or_tdrank *a, int left, int right) {
  for (int i = left; i <= right; i++)
    for (int j = left; j <= right - 1; j++)
      if (td_less(&a[j + 1], &a[j])) {
        int f = a[j].first, s = a[j].second, t = a[j].third;
        a[j].first = a[j + 1].first; a[j].second = a[j + 1].second; a[j].third = a[j + 1].third;
        a[j + 1].first = f; a[j + 1].second = s; a[j + 1].third = t;
      }
}

/* tools::bobbleSortmyPair (kernel_functions.cu:63-85): stable by .first,
 * stops after a pass without swaps. */
static void bubble_mp(or_mypair *a, int left, int right) {
  for (int i = left; i <= right; i++) {
    int swapped = 0;
    for (int j = left; j <= right - 1; j++)
      if (a[j + 1].first < a[j].first) {
        or_mypair t = a[j]; a[j] = a[j + 1]; a[j + 1] = t;
        swapped = 1;
      }
    if (!swapped) break;
  }
}

/* Body of makeCHPerHeight_D_2 for one partition cell (kernel_functions.cu:319-478). */
int or_contract_cell(int cell, or_tdrank *nonAdj, const int *ID_hash, or_mypair *CHTreeHash,
                     const or_mypair *NANHash, or_mypair *CHTree, unsigned char *visited,
                     or_pairs *CHInfo, int nv) {
  const int start = NANHash[cell].first;
  const int size = NANHash[cell].NodeID;
  for (int j = start; j < start + size; j++) {
    bubble_td(nonAdj, j, start + size - 1);                         /* :328 */
    const int v = nonAdj[j].second;
    visited[v] = 1;
    const int hv = ID_hash[v];
    const int base = CHTreeHash[hv].NodeID;
    int asz = CHTreeHash[hv].first;
    bubble_mp(CHTree, base, base + asz - 1);                         /* :338 */
    for (int k = base + 1; k < base + asz; k++) {                    /* :339-351 */
      if (CHTree[k].first == CHTree[k - 1].first && CHTree[k].first != INT_MAX) {
        if (CHTree[k - 1].second < CHTree[k].second) {
          CHTree[k].second = CHTree[k - 1].second;
          CHTree[k].NodeID = CHTree[k - 1].NodeID;
        }
        CHTree[k - 1].first = INT_MAX;
      }
    }
    bubble_mp(CHTree, base, base + asz - 1);                         /* :352 */
    for (int k = base; k < base + asz; k++) {                        /* :353-360 recount */
      if (CHTree[k].first == INT_MAX) break;
      CHTreeHash[hv].first = k - base + 1;
    }
    asz = CHTreeHash[hv].first;
    for (int k = base; k < base + asz; k++) {                        /* :364-390 delete back-edges */
      const int u = CHTree[k].first;
      if (u < 0 || u >= nv) return -1;                               /* reference reads ID_hash[INT_MAX] */
      const int hu = ID_hash[u];
      const int ub = CHTreeHash[hu].NodeID, us = CHTreeHash[hu].first;
      for (int q = ub; q < ub + us; q++)
        if (CHTree[q].first == v) CHTree[q].first = INT_MAX;
      bubble_mp(CHTree, ub, ub + us - 1);
      for (int k2 = ub; k2 < ub + us; k2++) {
        if (CHTree[k2].first == INT_MAX) break;
        CHTreeHash[hu].first = k2 - ub + 1;
      }
    }
    for (int k = base; k < base + asz; k++) {                        /* :392-457 fill-in */
      const int left = CHTree[k].first;
      for (int q = k + 1; q < base + asz; q++) {
        const int right = CHTree[q].first;
        if (left == right) continue;
        const int length = CHTree[k].second + CHTree[q].second;
        int leftHasRight = 0;
        const int hl = ID_hash[left], hr = ID_hash[right];
        for (int p = CHTreeHash[hl].NodeID; p < CHTreeHash[hl].NodeID + CHTreeHash[hl].first; p++) {
          if (CHTree[p].first == right) {
            leftHasRight = 1;
            if (CHTree[p].second > length) { CHTree[p].second = length; CHTree[p].NodeID = v; }
            break;
          }
        }
        for (int p = CHTreeHash[hr].NodeID; p < CHTreeHash[hr].NodeID + CHTreeHash[hr].first; p++) {
          if (CHTree[p].first == left) {
            if (CHTree[p].second > length) { CHTree[p].second = length; CHTree[p].NodeID = v; }
            break;
          }
        }
        if (!leftHasRight) {
          if (CHTreeHash[hl].first >= CHTreeHash[hl].second || CHTreeHash[hr].first >= CHTreeHash[hr].second)
            return -1;                                               /* LUB overflow: corrupts in the reference */
          int e = CHTreeHash[hl].NodeID + CHTreeHash[hl].first;
          CHTree[e].NodeID = v; CHTree[e].first = right; CHTree[e].second = length;
          CHTreeHash[hl].first++;
          e = CHTreeHash[hr].NodeID + CHTreeHash[hr].first;
          CHTree[e].NodeID = v; CHTree[e].first = left; CHTree[e].second = length;
          CHTreeHash[hr].first++;
        }
      }
    }
    for (int q = base; q < base + asz; q++) {                        /* :462-470 */
      if (CHTree[q].first == INT_MAX) continue;
      const int u = CHTree[q].first;
      const int hnow = nonAdj[j].third;
      CHInfo[u].first = CHTreeHash[ID_hash[u]].first;
      CHInfo[u].second = (hnow + 1 > CHInfo[u].second) ? hnow + 1 : CHInfo[u].second;
    }
    for (int k = j + 1; k < start + size; k++) {                     /* :471-475 */
      nonAdj[k].first = CHTreeHash[ID_hash[nonAdj[k].second]].first;
      nonAdj[k].third = CHInfo[nonAdj[k].second].second;
    }
  }
  return 0;
}

typedef struct {
  or_graph *g;
  int64_t lo, hi;
  int64_t next;            /* shared cell counter */
  pthread_mutex_t mu;
  int rc;
} cell_job;

static void *cell_worker(void *arg) {
  cell_job *job = (cell_job *)arg;
  or_graph *g = job->g;
  for (;;) {
    pthread_mutex_lock(&job->mu);
    int64_t c = job->next++;
    pthread_mutex_unlock(&job->mu);
    if (c > job->hi) break;
    int rc = or_contract_cell((int)c, g->nonadj, g->id_hash, g->chtree_hash, g->nanhash, g->chtree,
                              g->visited, g->chinfo_d, g->n);
    if (rc) { pthread_mutex_lock(&job->mu); job->rc = rc; pthread_mutex_unlock(&job->mu); }
  }
  return NULL;
}

/* makeCHPerHeight_2 (kernel_functions.cu:520-553): levels H..C+1, cells of a
 * level are independent (each touches only its own vertices' lists). */
static int contract_partition_levels(or_graph *g) {
  g->chinfo_d = (or_pairs *)malloc(sizeof(or_pairs) * (size_t)g->n);
  memcpy(g->chinfo_d, g->chinfo_h, sizeof(or_pairs) * (size_t)g->n);   /* translateBeforeCH, tanslate.cu:22 */
  for (int h = g->H; h > g->C; h--) {
    cell_job job;
    job.g = g; job.lo = ((int64_t)1 << (h - 1)) - 1; job.hi = ((int64_t)1 << h) - 2;
    job.next = job.lo; job.rc = 0;
    pthread_mutex_init(&job.mu, NULL);
    int nt = g->threads;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nt);
    for (int t = 0; t < nt; t++) pthread_create(&th[t], NULL, cell_worker, &job);
    for (int t = 0; t < nt; t++) pthread_join(th[t], NULL);
    free(th);
    pthread_mutex_destroy(&job.mu);
    if (job.rc) { snprintf(g->err, sizeof g->err, "partition contraction failed at level %d", h); return -1; }
  }
  memcpy(g->chinfo_h, g->chinfo_d, sizeof(or_pairs) * (size_t)g->n);   /* translateInTD, tanslate.cu:49 */
  return 0;
}

/* --------------------------------------------------------- global heap */
/* std::set<HostRank> ordered by (first+second, first, x) on CHInfo
 * (Graph_D.cuh:212-230); restated as an indexed binary heap. */
typedef struct { int *h; int *where; int n; const or_pairs *key; } vheap;

static int hr_less(const or_pairs *k, int a, int b) {
  if (k[a].first + k[a].second != k[b].first + k[b].second) return k[a].first + k[a].second < k[b].first + k[b].second;
  if (k[a].first != k[b].first) return k[a].first < k[b].first;
  return a < b;
}
static void vh_swap(vheap *q, int i, int j) {
  int a = q->h[i], b = q->h[j];
  q->h[i] = b; q->h[j] = a; q->where[b] = i; q->where[a] = j;
}
static void vh_up(vheap *q, int i) {
  while (i > 0) { int p = (i - 1) / 2; if (!hr_less(q->key, q->h[i], q->h[p])) break; vh_swap(q, i, p); i = p; }
}
static void vh_down(vheap *q, int i) {
  for (;;) {
    int l = 2 * i + 1, r = l + 1, s = i;
    if (l < q->n && hr_less(q->key, q->h[l], q->h[s])) s = l;
    if (r < q->n && hr_less(q->key, q->h[r], q->h[s])) s = r;
    if (s == i) break;
    vh_swap(q, i, s); i = s;
  }
}
static void vh_insert(vheap *q, int v) {
  if (q->where[v] >= 0) return;             /* std::set::insert of an equal key is a no-op */
  q->h[q->n] = v; q->where[v] = q->n; q->n++; vh_up(q, q->n - 1);
}
static void vh_erase(vheap *q, int v) {
  int i = q->where[v];
  if (i < 0) return;
  q->n--;
  if (i != q->n) { vh_swap(q, i, q->n); q->where[v] = -1; vh_up(q, i); vh_down(q, i); }
  else q->where[v] = -1;
}
static int vh_pop(vheap *q) { int v = q->h[0]; vh_erase(q, v); return v; }

/* Graph::uploadCHset (Traditional_H2H.cu:28-118) + CHUsingHeap_2 (:216-351). */
static int contract_global(or_graph *g) {
  const int n = g->n;
  g->chadj = (amap *)calloc((size_t)n, sizeof(amap));
  g->chinfo = (or_pairs *)malloc(sizeof(or_pairs) * (size_t)n);
  for (int i = 0; i < n; i++) { g->chinfo[i].first = -1; g->chinfo[i].second = -1; }
  vheap q;
  q.h = (int *)malloc(sizeof(int) * (size_t)n); q.where = (int *)malloc(sizeof(int) * (size_t)n);
  q.n = 0; q.key = g->chinfo;
  for (int i = 0; i < n; i++) q.where[i] = -1;
  int64_t tmp_index = INT_MAX;
  for (int h = g->C; h > 0; h--) {                                    /* :43-75 */
    int64_t lo = ((int64_t)1 << (h - 1)) - 1, hi = ((int64_t)1 << h) - 2;
    for (int64_t i = hi; i >= lo; i--) {
      int st = g->nanhash[i].first, sz = g->nanhash[i].NodeID;
      if (st < tmp_index) tmp_index = st;
      for (int j = st; j < st + sz; j++) {
        int v = g->nonadj[j].second;
        int hv = g->id_hash[v];
        int base = g->chtree_hash[hv].NodeID, asz = g->chtree_hash[hv].first;
        int cnt = 0;
        for (int k = base; k < base + asz; k++) {
          if (g->chtree[k].first == INT_MAX) continue;
          cnt++;
          am_emplace(&g->chadj[v], g->chtree[k].first, g->chtree[k].second, g->chtree[k].NodeID);
        }
        g->chinfo[v].first = cnt;
        g->chinfo[v].second = g->chinfo_h[v].second;
        vh_insert(&q, v);
      }
    }
  }
  for (int h = g->H; h > g->C; h--) {                                 /* :76-104 */
    int64_t lo = ((int64_t)1 << (h - 1)) - 1, hi = ((int64_t)1 << h) - 2;
    for (int64_t i = hi; i >= lo; i--) {
      int st = g->nanhash[i].first, sz = g->nanhash[i].NodeID;
      for (int j = st; j < st + sz; j++) {
        int v = g->nonadj[j].second;
        int hv = g->id_hash[v];
        int base = g->chtree_hash[hv].NodeID, asz = g->chtree_hash[hv].first;
        for (int k = base; k < base + asz; k++) {
          if (g->chtree[k].first == INT_MAX) continue;
          am_emplace(&g->chadj[v], g->chtree[k].first, g->chtree[k].second, g->chtree[k].NodeID);
        }
      }
    }
  }
  if (tmp_index == INT_MAX) tmp_index = g->nonadj_n;
  int64_t idx = tmp_index;
  g->gpu_vertices = (int)tmp_index;
  int *nei = (int *)malloc(sizeof(int) * (size_t)n), *neiw = (int *)malloc(sizeof(int) * (size_t)n);
  while (q.n > 0) {                                                   /* :222-323 */
    int v = vh_pop(&q);
    g->visited[v] = 1;
    amap *mv = &g->chadj[v];
    g->nonadj[idx].first = mv->n; g->nonadj[idx].second = v; g->nonadj[idx].third = g->chinfo[v].second;
    idx++;
    int d = mv->n;
    for (int i = 0; i < d; i++) { nei[i] = mv->nb[i]; neiw[i] = mv->w[i]; }
    for (int i = 0; i < d; i++) { am_erase(&g->chadj[nei[i]], v); vh_erase(&q, nei[i]); }
    for (int i = 0; i < d; i++) {
      int l = nei[i];
      for (int j = i + 1; j < d; j++) {
        int r = nei[j];
        int w = neiw[i] + neiw[j];
        amap *ml = &g->chadj[l], *mr = &g->chadj[r];
        int p = am_find(ml, r);
        if (p < 0) am_emplace(ml, r, w, v);
        else if (ml->w[p] > w) { ml->w[p] = w; ml->hub[p] = v; }
        p = am_find(mr, l);
        if (p < 0) am_emplace(mr, l, w, v);
        else if (mr->w[p] > w) { mr->w[p] = w; mr->hub[p] = v; }
      }
    }
    for (int i = 0; i < d; i++) {
      int u = nei[i];
      int hh = g->chinfo[v].second + 1 > g->chinfo[u].second ? g->chinfo[v].second + 1 : g->chinfo[u].second;
      g->chinfo[u].first = g->chadj[u].n;
      g->chinfo[u].second = hh;
      vh_insert(&q, u);
    }
  }
  free(nei); free(neiw); free(q.h); free(q.where);
  return 0;
}

/* ------------------------------------------------------------ tree + RMQ */
/* getrank, getTreeStructure, makeOULAAndRMQ, OULADFS (TreeStructure.cu:102-262). */
static int build_tree(or_graph *g) {
  const int n = g->n;
  g->rank = (int *)malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < n; i++) g->rank[i] = -1;
  for (int64_t i = 0; i < g->nonadj_n; i++) g->rank[g->nonadj[i].second] = (int)i;
  g->head = g->nonadj[g->nonadj_n - 1].second;
  g->father = (int *)malloc(sizeof(int) * (size_t)n);
  g->child_cnt = (int *)calloc((size_t)n, sizeof(int));
  g->child_off = (int *)malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < n; i++) {
    int fid = -1, tr = INT_MAX;
    for (int k = 0; k < g->chadj[i].n; k++) {
      int a = g->chadj[i].nb[k];
      if (tr > g->rank[a]) { tr = g->rank[a]; fid = a; }
    }
    g->father[i] = fid;
  }
  for (int i = 0; i < n; i++) if (g->father[i] != -1) g->child_cnt[g->father[i]]++;
  int t = 0;
  for (int i = 0; i < n; i++) { g->child_off[i] = t; t += g->child_cnt[i]; }
  g->childs = (int *)malloc(sizeof(int) * (size_t)(n > 1 ? n - 1 : 1));
  int *fill = (int *)calloc((size_t)n, sizeof(int));
  for (int i = 0; i < n; i++) {
    if (g->father[i] == -1) continue;
    int f = g->father[i];
    g->childs[g->child_off[f] + fill[f]] = i; fill[f]++;
  }
  free(fill);
  /* OULADFS, iterative form of the recursion at TreeStructure.cu:242-262 */
  g->first = (int *)malloc(sizeof(int) * (size_t)n);
  g->depth = (int *)malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < n; i++) { g->first[i] = -1; g->depth[i] = -1; }
  int64_t L = 2 * (int64_t)n - 1;
  g->euler_id = (int *)malloc(sizeof(int) * (size_t)L);
  g->euler_depth = (int *)malloc(sizeof(int) * (size_t)L);
  int *stk = (int *)malloc(sizeof(int) * (size_t)n), *cur = (int *)malloc(sizeof(int) * (size_t)n);
  unsigned char *vis = (unsigned char *)calloc((size_t)n, 1);
  int64_t e = 0;
  int sp = 0;
  g->h2h_size = 0; g->tree_height = 0;
  stk[sp] = g->head; cur[sp] = 0; sp++;
  g->euler_id[e] = g->head; g->euler_depth[e] = 1; g->first[g->head] = (int)e; e++;
  g->depth[g->head] = 1; g->h2h_size += 1; vis[g->head] = 1; g->tree_height = 1;
  while (sp > 0) {
    int v = stk[sp - 1];
    if (cur[sp - 1] < g->child_cnt[v]) {
      int c = g->childs[g->child_off[v] + cur[sp - 1]];
      cur[sp - 1]++;
      if (vis[c]) continue;
      int dd = sp + 1;
      g->euler_id[e] = c; g->euler_depth[e] = dd; g->first[c] = (int)e; e++;
      g->depth[c] = dd; g->h2h_size += dd; vis[c] = 1;
      if (dd > g->tree_height) g->tree_height = dd;
      stk[sp] = c; cur[sp] = 0; sp++;
    } else {
      sp--;
      if (sp > 0) {
        int p = stk[sp - 1];
        g->euler_id[e] = p; g->euler_depth[e] = sp; e++;
      }
    }
  }
  free(stk); free(cur); free(vis);
  g->euler_n = e;
  if (e != L) { snprintf(g->err, sizeof g->err, "tree is not spanning (euler %lld)", (long long)e); return -1; }
  /* dense sparse table then compaction (TreeStructure.cu:200-235) */
  int js = 0;
  while (((int64_t)2 << js) <= L) js++;                /* (int)log2((double)L) */
  int LS = js + 1;
  or_pairs *dense = (or_pairs *)malloc(sizeof(or_pairs) * (size_t)(LS * L));
  for (int64_t i = 0; i < LS * L; i++) { dense[i].first = -1; dense[i].second = -1; }
  for (int64_t i = 0; i < L; i++) { dense[i * LS].first = g->euler_depth[i]; dense[i * LS].second = g->euler_id[i]; }
  for (int j = 1; j <= js; j++) {
    int64_t dv = (int64_t)1 << (j - 1);
    for (int64_t i = 0; i + dv < L; i++) {
      if (dense[i * LS + j - 1].first <= dense[(i + dv) * LS + j - 1].first) dense[i * LS + j] = dense[i * LS + j - 1];
      else dense[i * LS + j] = dense[(i + dv) * LS + j - 1];
    }
  }
  g->rmq_hash = (int64_t *)malloc(sizeof(int64_t) * (size_t)L);
  int64_t tot = 0;
  for (int64_t i = 0; i < L; i++) for (int j = 0; j < LS; j++) { if (dense[i * LS + j].first == -1) break; tot++; }
  g->rmq_id = (int *)malloc(sizeof(int) * (size_t)tot);
  int64_t r = 0;
  for (int64_t i = 0; i < L; i++) {
    g->rmq_hash[i] = r;
    for (int j = 0; j < LS; j++) { if (dense[i * LS + j].first == -1) break; g->rmq_id[r++] = dense[i * LS + j].second; }
  }
  g->rmq_n = r;
  free(dense);
  return 0;
}

int or_contract(or_graph *g) {
  if (make_adjacent_node(g)) return -1;
  if (g->H != g->C) {                       /* main.cu:96: GPU levels only when H != C */
    if (contract_partition_levels(g)) return -1;
  }
  if (contract_global(g)) return -1;
  return build_tree(g);
}

/* ---------------------------------------------------------------- labels */
typedef struct { int v, p; } pp_t;
static int cmp_pos(const void *a, const void *b) { return ((const pp_t *)a)->p - ((const pp_t *)b)->p; }

/* mallocH2HLabel_noHub (H2HConsturction.cu:618-722) + constructBFSTree (:324-377). */
static int alloc_labels(or_graph *g) {
  const int n = g->n;
  g->dis_hash = (int64_t *)malloc(sizeof(int64_t) * ((size_t)n + 1));
  g->pos_hash = (int64_t *)malloc(sizeof(int64_t) * ((size_t)n + 1));
  int64_t pt = 0;
  for (int i = 0; i < n; i++) pt += g->chadj[i].n + 1;
  g->pos_n = pt;
  g->dis = (int *)malloc(sizeof(int) * (size_t)g->h2h_size);
  g->pos_id = (int *)malloc(sizeof(int) * (size_t)pt);
  g->pos_pos = (int *)malloc(sizeof(int) * (size_t)pt);
  int64_t dh = 0, ph = 0;
  pp_t *tmp = (pp_t *)malloc(sizeof(pp_t) * (size_t)(n + 1));
  for (int i = 0; i < n; i++) {
    g->dis_hash[i] = dh; g->pos_hash[i] = ph;
    int d = g->depth[i];
    for (int j = 0; j < d; j++) g->dis[dh + j] = INT_MAX;
    int c = 0;
    for (int k = 0; k < g->chadj[i].n; k++) {
      int a = g->chadj[i].nb[k];
      int p = g->depth[a] - 1;
      if (p >= d - 1 || p < 0) { free(tmp); snprintf(g->err, sizeof g->err, "neighbour %d of %d is not an ancestor", a, i); return -1; }
      tmp[c].v = a; tmp[c].p = p; c++;
      g->dis[dh + p] = g->chadj[i].w[k];
    }
    tmp[c].v = i; tmp[c].p = d - 1; c++;
    g->dis[dh + d - 1] = 0;
    qsort(tmp, (size_t)c, sizeof(pp_t), cmp_pos);   /* positions are distinct: any sort agrees with thrust::sort_by_key */
    for (int k = 0; k < c; k++) { g->pos_id[ph + k] = tmp[k].v; g->pos_pos[ph + k] = tmp[k].p; }
    dh += d; ph += c;
  }
  g->dis_hash[n] = dh; g->pos_hash[n] = ph;
  free(tmp);
  /* constructBFSTree: level order from the head, children in Childs order */
  g->tree_bfs = (int *)malloc(sizeof(int) * (size_t)n);
  g->tree_hash = (int *)malloc(sizeof(int) * ((size_t)n + 2));
  int nl = 0, qh = 0, qt = 0;
  g->tree_hash[nl++] = 0;
  g->tree_bfs[qt++] = g->head;
  g->tree_hash[nl++] = qt;
  while (qh < qt) {
    int lvl_end = qt;
    for (; qh < lvl_end; qh++) {
      int v = g->tree_bfs[qh];
      for (int k = 0; k < g->child_cnt[v]; k++) g->tree_bfs[qt++] = g->childs[g->child_off[v] + k];
    }
    if (qt > lvl_end) g->tree_hash[nl++] = qt;
  }
  g->n_levels = nl - 1;
  return 0;
}

typedef struct {
  or_graph *g;
  const int *nodes;
  int64_t count;
  int l4;
} fill_job;

/* Per-node body of makeH2HLabel_noHub_multiThred (H2HConsturction.cu:839-858);
 * with l4 the commented father-walk block (:850-857) runs as well. */
static void fill_node(or_graph *g, int v, int l4) {
  for (int64_t t = g->pos_hash[v + 1] - 2; t >= g->pos_hash[v]; t--) {
    int u = g->pos_id[t];
    int pos = g->pos_pos[t];
    int64_t iv = g->dis_hash[v], iu = g->dis_hash[u];
    int tl = g->dis[iv + pos];
    for (int j = pos - 1; j >= 0; j--) {
      int c = tl + g->dis[iu + j];
      if (c < g->dis[iv + j]) g->dis[iv + j] = c;
    }
    if (l4) {
      int64_t f = v;
      for (int j = (int)(g->dis_hash[v + 1] - g->dis_hash[v]) - 2; j > pos; j--) {
        f = g->father[f];
        int c = tl + g->dis[g->dis_hash[f] + pos];
        if (c < g->dis[iv + j]) g->dis[iv + j] = c;
      }
    }
  }
}

static void *fill_worker(void *arg) {
  fill_job *j = (fill_job *)arg;
  for (int64_t i = 0; i < j->count; i++) fill_node(j->g, j->nodes[i], j->l4);
  return NULL;
}

int or_build_labels(or_graph *g, int l4, int threads) {
  if (alloc_labels(g)) return -1;
  if (threads < 1) threads = 1;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
  fill_job *jobs = (fill_job *)malloc(sizeof(fill_job) * (size_t)threads);
  for (int lvl = 0; lvl < g->n_levels; lvl++) {           /* :813-871 level by level */
    int64_t s = g->tree_hash[lvl], e = g->tree_hash[lvl + 1];
    int64_t cnt = e - s;
    int64_t nt = threads < cnt ? threads : cnt;
    int64_t chunk = cnt / nt + 1;                          /* :821 */
    int64_t done = 0;
    int used = 0;
    for (int64_t t = 0; t < nt && done < cnt; t++) {
      int64_t c = chunk < cnt - done ? chunk : cnt - done;
      jobs[used].g = g; jobs[used].nodes = g->tree_bfs + s + done; jobs[used].count = c; jobs[used].l4 = l4;
      done += c; used++;
    }
    if (used == 1) fill_worker(&jobs[0]);
    else {
      for (int t = 0; t < used; t++) pthread_create(&th[t], NULL, fill_worker, &jobs[t]);
      for (int t = 0; t < used; t++) pthread_join(th[t], NULL);
    }
  }
  free(th); free(jobs);
  return 0;
}

/* --------------------------------------------------------------- queries */
static int ilog2(int x) { int k = 0; while ((2 << k) <= x) k++; return k; }

/* findLCA_noHub (H2HConsturction.cu:198-221) */
static int find_lca(const or_graph *g, int x, int y) {
  if (x == y) return x;
  int a = g->first[x], b = g->first[y];
  if (a > b) { int t = a; a = b; b = t; }
  int k = ilog2(b - a + 1);                  /* (int)log2((double)(b-a+1)) for b-a+1 >= 1 */
  int i1 = g->rmq_id[g->rmq_hash[a] + k];
  int i2 = g->rmq_id[g->rmq_hash[b - (1 << k) + 1] + k];
  return g->depth[i1] <= g->depth[i2] ? i1 : i2;
}

/* H2HDistancQuery_UsingLCA_noHub (Query.cu:108-122) */
int or_query_lca(const or_graph *g, int x, int y) {
  if (x == y) return 0;
  int lca = find_lca(g, x, y);
  int res = INT_MAX;
  for (int64_t i = g->pos_hash[lca]; i < g->pos_hash[lca + 1]; i++) {
    int t = g->dis[g->dis_hash[x] + g->pos_pos[i]] + g->dis[g->dis_hash[y] + g->pos_pos[i]];
    if (t < res) res = t;
  }
  return res;
}

/* H2HDistancQuery_noLCA_noHub (Query.cu:124-151) */
int or_query_nolca(const or_graph *g, int x, int y) {
  if (x == y) return 0;
  int fa = g->first[x], fb = g->first[y];
  int a = fa < fb ? fa : fb, b = fa < fb ? fb : fa;
  int k = ilog2(b - a + 1);
  int i1 = g->rmq_id[g->rmq_hash[a] + k];
  int i2 = g->rmq_id[g->rmq_hash[b - (1 << k) + 1] + k];
  int sz = g->depth[i2];
  if (g->depth[i1] <= g->depth[i2]) sz = g->depth[i1];
  int res = INT_MAX;
  for (int i = 0; i < sz; i++) {
    int t = g->dis[g->dis_hash[x] + i] + g->dis[g->dis_hash[y] + i];
    if (t < res) res = t;
  }
  return res;
}

typedef struct { const or_graph *g; const int *x, *y; int *out; int64_t s, e; int mode; } q_job;
static void *q_worker(void *arg) {
  q_job *j = (q_job *)arg;
  for (int64_t i = j->s; i < j->e; i++)
    j->out[i] = j->mode ? or_query_nolca(j->g, j->x[i], j->y[i]) : or_query_lca(j->g, j->x[i], j->y[i]);
  return NULL;
}

/* H2Hquery_bunch_MultiThread_noHub (Query.cu:172-202): contiguous chunks per thread. */
void or_query_batch(const or_graph *g, const int *x, const int *y, int *out, int64_t n, int mode, int threads) {
  if (threads < 1) threads = 1;
  int64_t chunk = n / threads + 1;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
  q_job *jobs = (q_job *)malloc(sizeof(q_job) * (size_t)threads);
  for (int t = 0; t < threads; t++) {
    int64_t s = t * chunk, e = (t + 1) * chunk;
    if (s > n) s = n;
    if (e > n) e = n;
    jobs[t].g = g; jobs[t].x = x; jobs[t].y = y; jobs[t].out = out; jobs[t].s = s; jobs[t].e = e; jobs[t].mode = mode;
    pthread_create(&th[t], NULL, q_worker, &jobs[t]);
  }
  for (int t = 0; t < threads; t++) pthread_join(th[t], NULL);
  free(th); free(jobs);
}

/* ------------------------------------------------------------- Dijkstra */
void or_dijkstra(const or_graph *g, int src, int *dist) {
  const int n = g->n;
  int *hp = (int *)malloc(sizeof(int) * (size_t)n), *where = (int *)malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < n; i++) { dist[i] = INT_MAX; where[i] = -1; }
  int hn = 0;
  dist[src] = 0; hp[hn] = src; where[src] = hn; hn++;
  while (hn > 0) {
    int v = hp[0];
    hn--; where[v] = -2;
    if (hn > 0) {
      hp[0] = hp[hn]; where[hp[0]] = 0;
      int i = 0;
      for (;;) {
        int l = 2 * i + 1, r = l + 1, s = i;
        if (l < hn && dist[hp[l]] < dist[hp[s]]) s = l;
        if (r < hn && dist[hp[r]] < dist[hp[s]]) s = r;
        if (s == i) break;
        int t = hp[i]; hp[i] = hp[s]; hp[s] = t; where[hp[i]] = i; where[hp[s]] = s; i = s;
      }
    }
    for (int e = g->adj_off[v]; e < g->adj_off[v + 1]; e++) {
      int u = g->adj[e].v;
      if (where[u] == -2) continue;
      int nd = dist[v] + g->adj[e].w;
      if (nd < dist[u]) {
        dist[u] = nd;
        int i = where[u];
        if (i < 0) { i = hn++; hp[i] = u; where[u] = i; }
        while (i > 0) {
          int p = (i - 1) / 2;
          if (dist[hp[p]] <= dist[hp[i]]) break;
          int t = hp[i]; hp[i] = hp[p]; hp[p] = t; where[hp[i]] = i; where[hp[p]] = p; i = p;
        }
      }
    }
  }
  free(hp); free(where);
}

/* ------------------------------------------------------------- accessors */
int or_n(const or_graph *g) { return g->n; }
int or_tree_height(const or_graph *g) { return g->tree_height; }
int64_t or_label_size(const or_graph *g) { return g->h2h_size; }
int64_t or_pos_size(const or_graph *g) { return g->pos_n; }
int64_t or_rmq_size(const or_graph *g) { return g->rmq_n; }
int64_t or_euler_size(const or_graph *g) { return g->euler_n; }
int or_n_levels(const or_graph *g) { return g->n_levels; }
int or_head(const or_graph *g) { return g->head; }
int64_t or_lub_size(const or_graph *g) { return g->lub; }
int or_gpu_vertices(const or_graph *g) { return g->gpu_vertices; }
void or_get_order(const or_graph *g, int *order) { for (int64_t i = 0; i < g->nonadj_n; i++) order[i] = g->nonadj[i].second; }
void or_get_father(const or_graph *g, int *f) { memcpy(f, g->father, sizeof(int) * (size_t)g->n); }
void or_get_depth(const or_graph *g, int *d) { memcpy(d, g->depth, sizeof(int) * (size_t)g->n); }
void or_get_first(const or_graph *g, int *f) { memcpy(f, g->first, sizeof(int) * (size_t)g->n); }
void or_get_rmq(const or_graph *g, int64_t *h, int *id) {
  memcpy(h, g->rmq_hash, sizeof(int64_t) * (size_t)g->euler_n);
  memcpy(id, g->rmq_id, sizeof(int) * (size_t)g->rmq_n);
}
void or_get_labels(const or_graph *g, int64_t *dh, int *dis, int64_t *ph, int *pid, int *ppos) {
  if (dh) memcpy(dh, g->dis_hash, sizeof(int64_t) * ((size_t)g->n + 1));
  if (dis) memcpy(dis, g->dis, sizeof(int) * (size_t)g->h2h_size);
  if (ph) memcpy(ph, g->pos_hash, sizeof(int64_t) * ((size_t)g->n + 1));
  if (pid) memcpy(pid, g->pos_id, sizeof(int) * (size_t)g->pos_n);
  if (ppos) memcpy(ppos, g->pos_pos, sizeof(int) * (size_t)g->pos_n);
}
void or_get_bfs(const or_graph *g, int *tb, int *th) {
  memcpy(tb, g->tree_bfs, sizeof(int) * (size_t)g->n);
  memcpy(th, g->tree_hash, sizeof(int) * ((size_t)g->n_levels + 1));
}
int64_t or_adj_total(const or_graph *g) { int64_t t = 0; for (int i = 0; i < g->n; i++) t += g->chadj[i].n; return t; }
void or_get_adj(const or_graph *g, int64_t *ah, int *aid, int *aw) {
  int64_t t = 0;
  for (int i = 0; i < g->n; i++) {
    ah[i] = t;
    for (int k = 0; k < g->chadj[i].n; k++) { aid[t] = g->chadj[i].nb[k]; aw[t] = g->chadj[i].w[k]; t++; }
  }
  ah[g->n] = t;
}

/* Input arcs in adjList order (file order, self loops dropped): off[n+1],
 * v[m].  The local-pair generator walks them. */
int64_t or_input_arcs(const or_graph *g) { return g->m; }
void or_get_input_arcs(const or_graph *g, int *off, int *v) {
  for (int i = 0; i <= g->n; i++) off[i] = g->adj_off[i];
  for (int64_t e = 0; e < g->m; e++) v[e] = g->adj[e].v;
}
