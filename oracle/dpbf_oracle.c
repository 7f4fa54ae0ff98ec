/*
 * CPU oracle for the exact group Steiner tree (GST) path: a plain-C
 * restatement of the reference's CPU DPBF solver and of the layered DP
 * formulation its GPU prototype follows.
 *
 * TEST INFRASTRUCTURE ONLY. The product (libgst) never links, loads or calls
 * this file; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg use it, as the checker.
 *
 * Data model (same as the reference's CSR_graph, csr_graph.hpp:29-65):
 *   row_ptr[V+1] (int64), col[nnz], w[nnz] (int32, already truncated from
 *   double as toCSR does at csr_graph.hpp:46); undirected edges appear in
 *   both rows. Groups: group_ptr[k+1], members[] (vertex IDs). Bit g of a
 *   group-set mask <=> group g (the reference uses the iteration order of an
 *   unordered_set, DPQ.cu:22-34; the optimal cost does not depend on it).
 *
 * Functions:
 *   oracle_dpbf      graph_v_of_v_idealID_DPBF_only_ec
 *                    (rucgraph/graph_v_of_v_idealID_DPBF_only_ec.h:133-323):
 *                    best-first search over states (v,p) keyed by cost,
 *                    seeded with T(v,p)=0 for every non-empty p inside v's
 *                    groups (:175-197), grow over the adjacency (:227-264),
 *                    merge with every disjoint p2 (:269-316), stop at the
 *                    first pop of the full mask (:217-223), tree rebuilt
 *                    from the recorded decisions (:90-129). The reference's
 *                    INT_MAX + cost overflow at :293 is not reproduced: an
 *                    absent T(v,p2) is skipped, which is what the reference
 *                    means by "cost inf".
 *   oracle_dp_table  the layered formulation of src/DP.cu:102-215 (merge
 *                    over submask splits, then shortest-path growth, masks
 *                    in increasing popcount): the exact fixpoint T(v,S) for
 *                    every vertex and mask, used to check full state tables.
 *   oracle_one_label_lb  lb0[v] = max_g dist(v, group g)
 *                    (src/DPQ.cu:361-403).
 */
#include <limits.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_INF INT32_MAX
#define ORC_LEAF INT32_MIN

enum { ORC_OK = 0, ORC_INFEASIBLE = 1, ORC_BAD_INPUT = -1, ORC_NOMEM = -3, ORC_TOO_SMALL = -2, ORC_STOPPED = 2 };

/* ---------------------------------------------------------------- heap --- */
/* Binary min-heap of state IDs keyed by cost[], with slot[] back-pointers
 * for decrease-key (the role boost::heap::fibonacci_heap::update plays). */
typedef struct {
  uint32_t *ids;
  int64_t n;
  int64_t *slot; /* -1: not in heap */
  const int32_t *key;
} heap_t;

static void heap_place(heap_t *h, int64_t i, uint32_t id) {
  h->ids[i] = id;
  h->slot[id] = i;
}
static void heap_up(heap_t *h, int64_t i) {
  uint32_t id = h->ids[i];
  int32_t k = h->key[id];
  while (i > 0) {
    int64_t p = (i - 1) >> 1;
    if (h->key[h->ids[p]] <= k) break;
    heap_place(h, i, h->ids[p]);
    i = p;
  }
  heap_place(h, i, id);
}
static void heap_down(heap_t *h, int64_t i) {
  uint32_t id = h->ids[i];
  int32_t k = h->key[id];
  for (;;) {
    int64_t c = 2 * i + 1;
    if (c >= h->n) break;
    if (c + 1 < h->n && h->key[h->ids[c + 1]] < h->key[h->ids[c]]) ++c;
    if (h->key[h->ids[c]] >= k) break;
    heap_place(h, i, h->ids[c]);
    i = c;
  }
  heap_place(h, i, id);
}
static void heap_push_or_decrease(heap_t *h, uint32_t id) {
  if (h->slot[id] >= 0) {
    heap_up(h, h->slot[id]);
  } else {
    h->ids[h->n] = id;
    h->slot[id] = h->n;
    h->n++;
    heap_up(h, h->n - 1);
  }
}
static uint32_t heap_pop(heap_t *h) {
  uint32_t top = h->ids[0];
  h->slot[top] = -1;
  h->n--;
  if (h->n > 0) {
    heap_place(h, 0, h->ids[h->n]);
    heap_down(h, 0);
  }
  return top;
}

/* ------------------------------------------------------------- helpers --- */
static int check_input(int32_t V, const int64_t *row_ptr, const int32_t *col, const int32_t *w, int32_t k,
                       const int32_t *group_ptr, const int32_t *members) {
  if (V < 1 || k < 1 || k > 20) return 0;
  if (row_ptr[0] != 0) return 0;
  for (int32_t v = 0; v < V; ++v)
    if (row_ptr[v + 1] < row_ptr[v]) return 0;
  for (int64_t e = 0; e < row_ptr[V]; ++e)
    if (col[e] < 0 || col[e] >= V || w[e] < 0) return 0;
  if (group_ptr[0] != 0) return 0;
  for (int32_t g = 0; g < k; ++g) {
    if (group_ptr[g + 1] < group_ptr[g]) return 0;
    for (int32_t i = group_ptr[g]; i < group_ptr[g + 1]; ++i)
      if (members[i] < 0 || members[i] >= V) return 0;
  }
  return 1;
}

/* groups(v) as a bit mask (graph_v_of_v_idealID_DPBF_vertex_group_set_ID, :43-59) */
static uint32_t *group_masks(int32_t V, int32_t k, const int32_t *group_ptr, const int32_t *members) {
  uint32_t *gm = (uint32_t *)calloc((size_t)V, sizeof(uint32_t));
  if (!gm) return NULL;
  for (int32_t g = 0; g < k; ++g)
    for (int32_t i = group_ptr[g]; i < group_ptr[g + 1]; ++i) gm[members[i]] |= 1u << g;
  return gm;
}

/* owner of CSR entry e: the v with row_ptr[v] <= e < row_ptr[v+1] */
static int32_t edge_owner(int32_t V, const int64_t *row_ptr, int64_t e) {
  int32_t lo = 0, hi = V - 1;
  while (lo < hi) {
    int32_t mid = lo + (hi - lo + 1) / 2;
    if (row_ptr[mid] <= e)
      lo = mid;
    else
      hi = mid - 1;
  }
  /* skip empty rows that share the same start */
  while (lo + 1 < V && row_ptr[lo + 1] <= e) ++lo;
  return lo;
}

/* Rebuild the tree of state (root, full) from parent codes:
 * code >= 0  grown over CSR entry `code` (owner -> this vertex),
 * code <  0  merged from p1 = -code and p ^ p1,
 * ORC_LEAF   single vertex (p inside its groups).
 * Emits (u, v, w) per grow step; vertices may repeat. */
static int backtrack(int32_t V, int32_t W, const int64_t *row_ptr, const int32_t *w, const int32_t *code,
                     int32_t root, int32_t full, int32_t *out_vertices, int32_t *out_nv, int32_t *out_edges,
                     int32_t *out_ne, int32_t cap) {
  int64_t stack_cap = 64, sp = 0;
  int64_t *stack = (int64_t *)malloc((size_t)stack_cap * sizeof(int64_t));
  if (!stack) return ORC_NOMEM;
  int32_t nv = 0, ne = 0;
  stack[sp++] = (int64_t)root * W + full;
  while (sp > 0) {
    int64_t s = stack[--sp];
    int32_t v = (int32_t)(s / W), p = (int32_t)(s % W);
    if (nv < cap) out_vertices[nv] = v;
    nv++;
    int32_t c = code[s];
    if (sp + 2 > stack_cap) {
      stack_cap *= 2;
      int64_t *ns = (int64_t *)realloc(stack, (size_t)stack_cap * sizeof(int64_t));
      if (!ns) {
        free(stack);
        return ORC_NOMEM;
      }
      stack = ns;
    }
    if (c == ORC_LEAF) {
      continue;
    } else if (c >= 0) {
      int32_t u = edge_owner(V, row_ptr, c);
      if (ne < cap) {
        out_edges[3 * ne + 0] = u;
        out_edges[3 * ne + 1] = v;
        out_edges[3 * ne + 2] = w[c];
      }
      ne++;
      stack[sp++] = (int64_t)u * W + p;
    } else {
      int32_t p1 = -c;
      stack[sp++] = (int64_t)v * W + p1;
      stack[sp++] = (int64_t)v * W + (p ^ p1);
    }
    if (nv > 64 * (int64_t)V + 64) break; /* defensive: a cycle would be a bug */
  }
  free(stack);
  *out_nv = nv;
  *out_ne = ne;
  return (nv > cap || ne > cap) ? ORC_TOO_SMALL : ORC_OK;
}

/* ---------------------------------------------------------- DPBF (heap) --- */
/*
 * Returns ORC_OK with *out_cost = optimal cost and the tree, ORC_INFEASIBLE
 * when no tree covers all groups, ORC_BAD_INPUT / ORC_NOMEM / ORC_TOO_SMALL
 * on errors, ORC_STOPPED when max_pops > 0 pops ran out first (used to time a
 * bounded sample). *out_pops counts popped states (the reference's
 * processed-state counter, DPQ.cu:675).
 */
int oracle_dpbf(int32_t V, const int64_t *row_ptr, const int32_t *col, const int32_t *w, int32_t k,
                const int32_t *group_ptr, const int32_t *members, int64_t max_pops, int32_t *out_cost,
                int32_t *out_root, int32_t *out_vertices, int32_t *out_nv, int32_t *out_edges, int32_t *out_ne,
                int32_t cap, int64_t *out_pops) {
  if (!check_input(V, row_ptr, col, w, k, group_ptr, members)) return ORC_BAD_INPUT;
  const int32_t W = 1 << k, full = W - 1;
  const int64_t S = (int64_t)V * W;
  if (S >= (int64_t)UINT32_MAX) return ORC_BAD_INPUT;
  int32_t *cost = (int32_t *)malloc((size_t)S * sizeof(int32_t));
  int32_t *code = (int32_t *)malloc((size_t)S * sizeof(int32_t));
  int64_t *slot = (int64_t *)malloc((size_t)S * sizeof(int64_t));
  uint32_t *ids = (uint32_t *)malloc((size_t)S * sizeof(uint32_t));
  uint32_t *gm = group_masks(V, k, group_ptr, members);
  int rc = ORC_INFEASIBLE;
  int64_t pops = 0;
  if (!cost || !code || !slot || !ids || !gm) {
    rc = ORC_NOMEM;
    goto done;
  }
  for (int64_t s = 0; s < S; ++s) {
    cost[s] = ORC_INF;
    slot[s] = -1;
  }
  heap_t h = {ids, 0, slot, cost};
  /* T(v,p) = 0 for every non-empty p inside groups(v)  (:175-197) */
  for (int32_t v = 0; v < V; ++v) {
    uint32_t g = gm[v];
    for (uint32_t p = g; p; p = (p - 1) & g) {
      int64_t s = (int64_t)v * W + p;
      cost[s] = 0;
      code[s] = ORC_LEAF;
      heap_push_or_decrease(&h, (uint32_t)s);
    }
  }
  while (h.n > 0) {
    if (max_pops > 0 && pops >= max_pops) {
      rc = ORC_STOPPED;
      break;
    }
    uint32_t s = heap_pop(&h);
    pops++;
    int32_t v = (int32_t)(s / (uint32_t)W), p = (int32_t)(s % (uint32_t)W);
    int32_t c = cost[s];
    if (p == full) { /* first pop of the full mask is optimal (:217-223) */
      *out_cost = c;
      *out_root = v;
      rc = backtrack(V, W, row_ptr, w, code, v, full, out_vertices, out_nv, out_edges, out_ne, cap);
      break;
    }
    /* grow (:227-264) */
    for (int64_t e = row_ptr[v]; e < row_ptr[v + 1]; ++e) {
      int64_t t = (int64_t)col[e] * W + p;
      int32_t cand = c + w[e];
      if (cand < cost[t]) {
        cost[t] = cand;
        code[t] = (int32_t)e;
        heap_push_or_decrease(&h, (uint32_t)t);
      }
    }
    /* merge with every non-empty p2 disjoint from p (:269-316) */
    int32_t comp = full ^ p;
    for (int32_t p2 = comp; p2; p2 = (p2 - 1) & comp) {
      int32_t c2 = cost[(int64_t)v * W + p2];
      if (c2 == ORC_INF) continue; /* absent T(v,p2) */
      int64_t t = (int64_t)v * W + (p | p2);
      int32_t cand = c + c2;
      if (cand < cost[t]) {
        cost[t] = cand;
        code[t] = -p;
        heap_push_or_decrease(&h, (uint32_t)t);
      }
    }
  }
done:
  if (out_pops) *out_pops = pops;
  free(cost);
  free(code);
  free(slot);
  free(ids);
  free(gm);
  return rc;
}

/* -------------------------------------------------- layered DP table --- */
/* Multi-source Dijkstra over one mask column: dist[] is both the seed
 * values and the result; code[] records the CSR entry of the last
 * improvement. */
static int column_dijkstra(int32_t V, const int64_t *row_ptr, const int32_t *col, const int32_t *w, int32_t *dist,
                           int32_t *code_col, uint32_t *ids, int64_t *slot) {
  heap_t h = {ids, 0, slot, dist};
  for (int32_t v = 0; v < V; ++v) {
    slot[v] = -1;
  }
  for (int32_t v = 0; v < V; ++v)
    if (dist[v] != ORC_INF) heap_push_or_decrease(&h, (uint32_t)v);
  while (h.n > 0) {
    uint32_t v = heap_pop(&h);
    int32_t c = dist[v];
    for (int64_t e = row_ptr[v]; e < row_ptr[v + 1]; ++e) {
      int32_t u = col[e];
      int32_t cand = c + w[e];
      if (cand < dist[u]) {
        dist[u] = cand;
        code_col[u] = (int32_t)e;
        heap_push_or_decrease(&h, (uint32_t)u);
      }
    }
  }
  return ORC_OK;
}

/*
 * Fills table[v*2^k + S] with the exact fixpoint T(v,S) (ORC_INF where no
 * tree exists; entry S=0 is left ORC_INF). Masks are processed in
 * increasing popcount; within a mask: T(v,S) = 0 if S inside groups(v),
 * else min over unordered splits S1|S2 of T(v,S1)+T(v,S2) (src/DP.cu:65-80),
 * then grown by shortest paths (the fixpoint of src/DP.cu:82-101).
 */
int oracle_dp_table(int32_t V, const int64_t *row_ptr, const int32_t *col, const int32_t *w, int32_t k,
                    const int32_t *group_ptr, const int32_t *members, int32_t *table) {
  if (!check_input(V, row_ptr, col, w, k, group_ptr, members)) return ORC_BAD_INPUT;
  const int32_t W = 1 << k;
  uint32_t *gm = group_masks(V, k, group_ptr, members);
  int32_t *dist = (int32_t *)malloc((size_t)V * sizeof(int32_t));
  int32_t *code_col = (int32_t *)malloc((size_t)V * sizeof(int32_t));
  uint32_t *ids = (uint32_t *)malloc((size_t)V * sizeof(uint32_t));
  int64_t *slot = (int64_t *)malloc((size_t)V * sizeof(int64_t));
  int rc = ORC_OK;
  if (!gm || !dist || !code_col || !ids || !slot) {
    rc = ORC_NOMEM;
    goto done;
  }
  for (int64_t s = 0; s < (int64_t)V * W; ++s) table[s] = ORC_INF;
  for (int32_t level = 1; level <= k; ++level) {
    for (int32_t S = 1; S < W; ++S) {
      if (__builtin_popcount((unsigned)S) != level) continue;
      int32_t low = S & -S;
      for (int32_t v = 0; v < V; ++v) {
        int32_t best = ((gm[v] & (uint32_t)S) == (uint32_t)S) ? 0 : ORC_INF;
        /* S1 holds the lowest bit of S: each unordered split once */
        for (int32_t s1 = (S - 1) & S; s1; s1 = (s1 - 1) & S) {
          if (!(s1 & low)) continue;
          int32_t a = table[(int64_t)v * W + s1], b = table[(int64_t)v * W + (S ^ s1)];
          if (a != ORC_INF && b != ORC_INF && a + b < best) best = a + b;
        }
        dist[v] = best;
      }
      column_dijkstra(V, row_ptr, col, w, dist, code_col, ids, slot);
      for (int32_t v = 0; v < V; ++v) table[(int64_t)v * W + S] = dist[v];
    }
  }
done:
  free(gm);
  free(dist);
  free(code_col);
  free(ids);
  free(slot);
  return rc;
}

/* lb0[v] = max over groups of dist(v, group)  (src/DPQ.cu:361-403);
 * ORC_INF when some group is unreachable from v. */
int oracle_one_label_lb(int32_t V, const int64_t *row_ptr, const int32_t *col, const int32_t *w, int32_t k,
                        const int32_t *group_ptr, const int32_t *members, int32_t *lb0) {
  if (!check_input(V, row_ptr, col, w, k, group_ptr, members)) return ORC_BAD_INPUT;
  int32_t *dist = (int32_t *)malloc((size_t)V * sizeof(int32_t));
  int32_t *code_col = (int32_t *)malloc((size_t)V * sizeof(int32_t));
  uint32_t *ids = (uint32_t *)malloc((size_t)V * sizeof(uint32_t));
  int64_t *slot = (int64_t *)malloc((size_t)V * sizeof(int64_t));
  if (!dist || !code_col || !ids || !slot) {
    free(dist);
    free(code_col);
    free(ids);
    free(slot);
    return ORC_NOMEM;
  }
  for (int32_t v = 0; v < V; ++v) lb0[v] = 0;
  for (int32_t g = 0; g < k; ++g) {
    for (int32_t v = 0; v < V; ++v) dist[v] = ORC_INF;
    for (int32_t i = group_ptr[g]; i < group_ptr[g + 1]; ++i) dist[members[i]] = 0;
    column_dijkstra(V, row_ptr, col, w, dist, code_col, ids, slot);
    for (int32_t v = 0; v < V; ++v)
      if (dist[v] > lb0[v]) lb0[v] = dist[v];
  }
  free(dist);
  free(code_col);
  free(ids);
  free(slot);
  return ORC_OK;
}
