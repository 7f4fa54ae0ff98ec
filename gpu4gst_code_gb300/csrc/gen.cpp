// Seeded synthetic GST instances (host only); see include/gst_gen.h.
#include "gst_gen.h"
#include "host_types.hpp"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <new>
#include <unordered_set>
#include <utility>
#include <vector>


namespace {

// xoshiro256** (Blackman & Vigna), seeded by splitmix64.
class Rng {
 public:
  explicit Rng(uint64_t seed) {
    for (auto& x : s_) {
      seed += 0x9E3779B97F4A7C15ull;
      uint64_t z = seed;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      x = z ^ (z >> 31);
    }
  }
  uint64_t next() {
    const uint64_t result = rotl(s_[1] * 5, 7) * 9;
    const uint64_t t = s_[1] << 17;
    s_[2] ^= s_[0];
    s_[3] ^= s_[1];
    s_[1] ^= s_[2];
    s_[0] ^= s_[3];
    s_[2] ^= t;
    s_[3] = rotl(s_[3], 45);
    return result;
  }
  // uniform in [0, n)
  uint64_t below(uint64_t n) { return (uint64_t)(((unsigned __int128)next() * n) >> 64); }
  // uniform in [lo, hi]
  int32_t range(int32_t lo, int32_t hi) { return lo + (int32_t)below((uint64_t)((int64_t)hi - lo + 1)); }
  // uniform in [0, 1) with 53 bits
  double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }

 private:
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t s_[4];
};

inline uint64_t edge_key(int32_t a, int32_t b) {
  if (a > b) std::swap(a, b);
  return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b;
}

// Undirected edge list -> CSR with both directions, rows sorted by neighbour.
gst_host_graph* to_csr(int32_t V, const std::vector<std::pair<int32_t, int32_t>>& edges,
                       const std::vector<int32_t>& weights) {
  auto* g = new (std::nothrow) gst_host_graph;
  if (!g) return nullptr;
  g->V = V;
  g->row_ptr.assign((size_t)V + 1, 0);
  for (auto& e : edges) {
    g->row_ptr[(size_t)e.first + 1]++;
    g->row_ptr[(size_t)e.second + 1]++;
  }
  for (int32_t v = 0; v < V; ++v) g->row_ptr[(size_t)v + 1] += g->row_ptr[v];
  const size_t nnz = (size_t)g->row_ptr[V];
  g->col.resize(nnz);
  g->w.resize(nnz);
  std::vector<int32_t> fill(g->row_ptr.begin(), g->row_ptr.end() - 1);
  for (size_t i = 0; i < edges.size(); ++i) {
    int32_t a = edges[i].first, b = edges[i].second;
    g->col[fill[a]] = b;
    g->w[fill[a]++] = weights[i];
    g->col[fill[b]] = a;
    g->w[fill[b]++] = weights[i];
  }
  std::vector<std::pair<int32_t, int32_t>> row;
  for (int32_t v = 0; v < V; ++v) {
    int32_t b = g->row_ptr[v], e = g->row_ptr[(size_t)v + 1];
    row.clear();
    for (int32_t i = b; i < e; ++i) row.emplace_back(g->col[i], g->w[i]);
    std::sort(row.begin(), row.end());
    for (int32_t i = b; i < e; ++i) {
      g->col[i] = row[i - b].first;
      g->w[i] = row[i - b].second;
    }
  }
  return g;
}

}  // namespace

extern "C" {

gst_host_graph* gst_gen_random_connected(int32_t V, int64_t E, int32_t wmin, int32_t wmax, uint64_t seed) {
  if (V < 1 || E < V - 1 || E > (int64_t)V * (V - 1) / 2 || wmin < 0 || wmax < wmin) return nullptr;
  if (2 * E >= INT32_MAX) return nullptr;
  Rng rng(seed);
  std::vector<std::pair<int32_t, int32_t>> edges;
  std::vector<int32_t> weights;
  edges.reserve((size_t)E);
  weights.reserve((size_t)E);
  std::unordered_set<uint64_t> present;
  present.reserve((size_t)E * 2);
  for (int32_t v = 1; v < V; ++v) {  // random recursive spanning tree
    int32_t u = (int32_t)rng.below((uint64_t)v);
    edges.emplace_back(u, v);
    weights.push_back(rng.range(wmin, wmax));
    present.insert(edge_key(u, v));
  }
  while ((int64_t)edges.size() < E) {  // uniform extra edges
    int32_t a = (int32_t)rng.below((uint64_t)V), b = (int32_t)rng.below((uint64_t)V);
    if (a == b || !present.insert(edge_key(a, b)).second) continue;
    edges.emplace_back(a, b);
    weights.push_back(rng.range(wmin, wmax));
  }
  return to_csr(V, edges, weights);
}

gst_host_graph* gst_gen_barabasi_albert(int32_t V, int32_t m, int32_t wmin, int32_t wmax, uint64_t seed) {
  if (m < 1 || V < m + 1 || wmin < 0 || wmax < wmin) return nullptr;
  const int64_t E = (int64_t)m * (m + 1) / 2 + (int64_t)(V - m - 1) * m;
  if (2 * E >= INT32_MAX) return nullptr;
  Rng rng(seed);
  std::vector<std::pair<int32_t, int32_t>> edges;
  std::vector<int32_t> weights;
  std::vector<int32_t> ends;  // each vertex once per incident edge
  edges.reserve((size_t)E);
  weights.reserve((size_t)E);
  ends.reserve((size_t)E * 2);
  for (int32_t a = 0; a <= m; ++a)
    for (int32_t b = a + 1; b <= m; ++b) {
      edges.emplace_back(a, b);
      weights.push_back(rng.range(wmin, wmax));
      ends.push_back(a);
      ends.push_back(b);
    }
  std::vector<int32_t> targets;
  for (int32_t v = m + 1; v < V; ++v) {
    targets.clear();
    while ((int32_t)targets.size() < m) {
      int32_t t = ends[rng.below(ends.size())];
      if (std::find(targets.begin(), targets.end(), t) == targets.end()) targets.push_back(t);
    }
    for (int32_t t : targets) {
      edges.emplace_back(t, v);
      weights.push_back(rng.range(wmin, wmax));
      ends.push_back(t);
      ends.push_back(v);
    }
  }
  return to_csr(V, edges, weights);
}

int32_t gst_host_graph_num_vertices(const gst_host_graph* g) { return g ? g->V : 0; }
int64_t gst_host_graph_num_entries(const gst_host_graph* g) { return g ? (int64_t)g->col.size() : 0; }
void gst_host_graph_copy(const gst_host_graph* g, int32_t* row_ptr, int32_t* col, int32_t* w) {
  std::copy(g->row_ptr.begin(), g->row_ptr.end(), row_ptr);
  std::copy(g->col.begin(), g->col.end(), col);
  std::copy(g->w.begin(), g->w.end(), w);
}
void gst_host_graph_free(gst_host_graph* g) { delete g; }

gst_host_groups* gst_gen_groups_uniform(int32_t V, int32_t k, int32_t size, uint64_t seed) {
  if (V < 1 || k < 1 || size < 1 || size > V) return nullptr;
  Rng rng(seed);
  auto* q = new (std::nothrow) gst_host_groups;
  if (!q) return nullptr;
  q->k = k;
  q->group_ptr.push_back(0);
  std::unordered_set<int32_t> chosen;
  for (int32_t g = 0; g < k; ++g) {
    chosen.clear();
    while ((int32_t)chosen.size() < size) {
      int32_t v = (int32_t)rng.below((uint64_t)V);
      if (chosen.insert(v).second) q->members.push_back(v);
    }
    q->group_ptr.push_back((int32_t)q->members.size());
  }
  return q;
}

gst_host_groups* gst_gen_groups_zipf_degree(const int32_t* row_ptr, const int32_t* col, int32_t V, int64_t nnz,
                                            int32_t k, double s, int32_t size_min, int32_t size_max,
                                            uint64_t seed) {
  if (!row_ptr || !col || V < 1 || nnz < 1 || k < 1 || s <= 1.0 || size_min < 1 || size_max < size_min)
    return nullptr;
  // Zipf(s) on {1,2,...}: P(n) = n^-s / zeta(s); mass at n >= size_max is
  // folded into size_max, mass below size_min into size_min (clipping).
  const int64_t N = 1 << 20;
  double zeta = 0.0;
  for (int64_t n = N - 1; n >= 1; --n) zeta += std::pow((double)n, -s);
  const double Nd = (double)N;  // Euler-Maclaurin tail from N
  zeta += std::pow(Nd, 1.0 - s) / (s - 1.0) + 0.5 * std::pow(Nd, -s) + s * std::pow(Nd, -s - 1.0) / 12.0;
  std::vector<double> cdf((size_t)size_max, 0.0);  // cdf[n-1] = P(X <= n), n < size_max
  double acc = 0.0;
  for (int32_t n = 1; n < size_max; ++n) {
    acc += std::pow((double)n, -s) / zeta;
    cdf[(size_t)n - 1] = acc;
  }
  Rng rng(seed);
  auto* q = new (std::nothrow) gst_host_groups;
  if (!q) return nullptr;
  q->k = k;
  q->group_ptr.push_back(0);
  // count vertices with at least one incident entry (eligible members)
  int64_t eligible = 0;
  for (int32_t v = 0; v < V; ++v) eligible += row_ptr[(size_t)v + 1] > row_ptr[v];
  std::unordered_set<int32_t> chosen;
  for (int32_t g = 0; g < k; ++g) {
    double u = rng.unit();
    int32_t n = size_max;
    for (int32_t i = 1; i < size_max; ++i)
      if (u < cdf[(size_t)i - 1]) {
        n = i;
        break;
      }
    n = std::max(n, size_min);
    if ((int64_t)n > eligible) n = (int32_t)eligible;
    chosen.clear();
    while ((int32_t)chosen.size() < n) {
      // col[e] for a uniform entry e: vertex v is hit with probability deg(v)/nnz
      int32_t v = col[rng.below((uint64_t)nnz)];
      if (chosen.insert(v).second) q->members.push_back(v);
    }
    q->group_ptr.push_back((int32_t)q->members.size());
  }
  return q;
}

int32_t gst_host_groups_k(const gst_host_groups* q) { return q ? q->k : 0; }
int64_t gst_host_groups_num_members(const gst_host_groups* q) { return q ? (int64_t)q->members.size() : 0; }
void gst_host_groups_copy(const gst_host_groups* q, int32_t* group_ptr, int32_t* members) {
  std::copy(q->group_ptr.begin(), q->group_ptr.end(), group_ptr);
  std::copy(q->members.begin(), q->members.end(), members);
}
void gst_host_groups_free(gst_host_groups* q) { delete q; }

}  // extern "C"
