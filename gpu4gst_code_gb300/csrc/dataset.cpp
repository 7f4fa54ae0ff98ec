// Readers of the reference's dataset files (include/gst_io.h).
#include <algorithm>
#include <cstdlib>
#include <fstream>
#include <map>
#include <new>
#include <set>
#include <string>
#include <utility>
#include <vector>

#include "gst_io.h"
#include "host_types.hpp"

namespace {

// The reference's parse_string (rucgraph/text_mining/parse_string.h): split
// on every occurrence of the delimiter, empty tokens kept.
std::vector<std::string> split(const std::string& s, char d) {
  std::vector<std::string> out;
  size_t start = 0;
  for (;;) {
    const size_t p = s.find(d, start);
    if (p == std::string::npos) {
      out.push_back(s.substr(start));
      return out;
    }
    out.push_back(s.substr(start, p - start));
    start = p + 1;
  }
}

void chomp(std::string& s) {
  while (!s.empty() && (s.back() == '\r' || s.back() == '\n')) s.pop_back();
}

bool to_long(const std::string& t, long long* v) {
  if (t.empty()) return false;
  char* end = nullptr;
  const long long x = std::strtoll(t.c_str(), &end, 10);
  if (end == t.c_str() || *end != '\0') return false;
  *v = x;
  return true;
}

// std::stod then int truncation, as the reference converts weights
bool to_trunc(const std::string& t, long long* v) {
  if (t.empty()) return false;
  char* end = nullptr;
  const double x = std::strtod(t.c_str(), &end);
  if (end == t.c_str() || *end != '\0' || !(x > -2147483648.0 && x < 2147483648.0)) return false;
  *v = (long long)x;
  return true;
}

gst_status bad(const std::string& path, size_t line, const std::string& what) {
  gst::set_last_error(path + ":" + std::to_string(line) + ": " + what);
  return GST_BAD_INPUT;
}

// rows of (neighbour, weight) -> CSR, rows sorted by neighbour ID
gst_host_graph* to_csr(std::vector<std::vector<std::pair<int32_t, int32_t>>>& rows) {
  auto* g = new (std::nothrow) gst_host_graph;
  if (!g) return nullptr;
  g->V = (int32_t)rows.size();
  g->row_ptr.assign(rows.size() + 1, 0);
  size_t n = 0;
  for (auto& r : rows) n += r.size();
  g->col.reserve(n);
  g->w.reserve(n);
  for (size_t v = 0; v < rows.size(); ++v) {
    std::stable_sort(rows[v].begin(), rows[v].end(),
                     [](const std::pair<int32_t, int32_t>& a, const std::pair<int32_t, int32_t>& b) {
                       return a.first < b.first;
                     });
    for (auto& e : rows[v]) {
      g->col.push_back(e.first);
      g->w.push_back(e.second);
    }
    g->row_ptr[v + 1] = (int32_t)g->col.size();
  }
  return g;
}

gst_host_groups* to_groups(const std::vector<std::vector<int32_t>>& lists) {
  auto* q = new (std::nothrow) gst_host_groups;
  if (!q) return nullptr;
  q->k = (int32_t)lists.size();
  q->group_ptr.assign(lists.size() + 1, 0);
  for (size_t i = 0; i < lists.size(); ++i) {
    q->members.insert(q->members.end(), lists[i].begin(), lists[i].end());
    q->group_ptr[i + 1] = (int32_t)q->members.size();
  }
  return q;
}

}  // namespace

extern "C" {

gst_status gst_read_graph_file(const char* path, gst_host_graph** out, int32_t* num_communities) {
  if (!path || !out) return bad("", 0, "path / out is NULL");
  *out = nullptr;
  std::ifstream f(path);
  if (!f.is_open()) return bad(path, 0, "cannot open");
  std::string line;
  if (!std::getline(f, line)) return bad(path, 1, "empty file");
  chomp(line);
  const auto head = split(line, ' ');
  long long V = 0, C = 0;
  if (head.size() < 3 || !to_trunc(head[0], &V) || !to_trunc(head[2], &C) || V < 1 || V > 2147483647LL)
    return bad(path, 1, "header must be 'V E C'");
  std::vector<std::vector<std::pair<int32_t, int32_t>>> rows((size_t)V);
  size_t ln = 1;
  while (std::getline(f, line)) {
    ++ln;
    chomp(line);
    const auto p = split(line, ' ');
    if (p.size() >= 2 && p[0] == "input_graph" && p[1] == "Vertex") {
      long long v = 0, nw = 0, c = 0;
      if (p.size() < 5 || !to_long(p[2], &v) || !to_trunc(p[3], &nw) || !to_trunc(p[4], &c) || v < 0 || v >= V)
        return bad(path, ln, "bad Vertex line");
    } else if (p.size() >= 2 && p[0] == "input_graph" && p[1] == "Edge") {
      long long a = 0, b = 0, ec = 0;
      if (p.size() < 5 || !to_long(p[2], &a) || !to_long(p[3], &b) || !to_trunc(p[4], &ec) || a < 0 || a >= V ||
          b < 0 || b >= V || ec < 0 || ec >= GST_COST_LIMIT)
        return bad(path, ln, "bad Edge line");
      rows[(size_t)a].push_back({(int32_t)b, (int32_t)ec});
      rows[(size_t)b].push_back({(int32_t)a, (int32_t)ec});
    }
  }
  gst_host_graph* g = to_csr(rows);
  if (!g) return GST_OOM;
  if (num_communities) *num_communities = (int32_t)C;
  *out = g;
  return GST_OK;
}

gst_status gst_read_groups_file(const char* path, gst_host_groups** out) {
  if (!path || !out) return bad("", 0, "path / out is NULL");
  *out = nullptr;
  std::ifstream f(path);
  if (!f.is_open()) return bad(path, 0, "cannot open");
  std::vector<std::vector<int32_t>> groups;
  std::string line;
  size_t ln = 0;
  while (std::getline(f, line)) {
    ++ln;
    chomp(line);
    if (line.empty()) continue;
    const auto p = split(line, ':');
    long long id = 0;
    if (p.size() < 2 || p[0].size() < 2 || !to_trunc(p[0].substr(1), &id) || id < 1 || id > (1LL << 30))
      return bad(path, ln, "expected 'g<id>:<members>'");
    if ((size_t)id > groups.size()) groups.resize((size_t)id);
    auto& g = groups[(size_t)id - 1];
    for (const auto& t : split(p[1], ' ')) {
      if (t.empty()) continue;  // tolerate a trailing space
      long long v = 0;
      if (!to_long(t, &v) || v < 0 || v > 2147483647LL) return bad(path, ln, "bad member '" + t + "'");
      g.push_back((int32_t)v);
    }
    std::sort(g.begin(), g.end());
  }
  gst_host_groups* q = to_groups(groups);
  if (!q) return GST_OOM;
  *out = q;
  return GST_OK;
}

gst_status gst_read_queries_file(const char* path, int32_t V, gst_host_groups** out) {
  if (!path || !out) return bad("", 0, "path / out is NULL");
  *out = nullptr;
  std::ifstream f(path);
  if (!f.is_open()) return bad(path, 0, "cannot open");
  std::vector<std::vector<int32_t>> queries;
  std::string line;
  size_t ln = 0;
  while (std::getline(f, line)) {
    ++ln;
    chomp(line);
    const auto p = split(line, ' ');
    std::vector<int32_t> q;
    for (size_t i = 0; i + 1 < p.size(); ++i) {  // the last token is ignored, as read_inquire does
      long long x = 0;
      if (!to_long(p[i], &x) || x - V < 0 || x - V > 2147483647LL) return bad(path, ln, "bad group value");
      q.push_back((int32_t)(x - V));
    }
    queries.push_back(std::move(q));
  }
  gst_host_groups* r = to_groups(queries);
  if (!r) return GST_OOM;
  *out = r;
  return GST_OK;
}

gst_status gst_read_gstp_instance(const char* path, gst_host_graph** graph, gst_host_groups** groups) {
  if (!path || !graph || !groups) return bad("", 0, "path / outputs are NULL");
  *graph = nullptr;
  *groups = nullptr;
  std::ifstream f(path);
  if (!f.is_open()) return bad(path, 0, "cannot open");
  std::map<std::pair<int32_t, int32_t>, int32_t> edges;  // add_edge replaces the weight
  std::vector<std::pair<long long, long long>> gedges;
  std::set<long long> gids;
  long long V = 0;
  std::string line;
  size_t ln = 0;
  while (std::getline(f, line)) {
    ++ln;
    chomp(line);
    const auto p = split(line, ' ');
    long long a = 0, b = 0, ec = 0;
    if (p.size() >= 3 && p[0] == "input_graph" && p[1] == "Vertex") {
      if (!to_long(p[2], &a) || a < 0 || a >= 2147483647LL) return bad(path, ln, "bad Vertex line");
      V = std::max(V, a + 1);
    } else if (p.size() >= 5 && p[0] == "input_graph" && p[1] == "Edge") {
      if (!to_long(p[2], &a) || !to_long(p[3], &b) || !to_trunc(p[4], &ec) || a < 0 || b < 0 ||
          a >= 2147483647LL || b >= 2147483647LL || ec < 0 || ec >= GST_COST_LIMIT)
        return bad(path, ln, "bad Edge line");
      V = std::max(V, std::max(a, b) + 1);
      edges[{(int32_t)std::min(a, b), (int32_t)std::max(a, b)}] = (int32_t)ec;
    } else if (p.size() >= 5 && p[0] == "group_graph" && p[1] == "Edge") {
      if (!to_long(p[2], &a) || !to_long(p[3], &b)) return bad(path, ln, "bad group Edge line");
      gedges.push_back({a, b});
    } else if (p.size() >= 2 && p[0] == "group_vertices") {
      if (!to_long(p[1], &a)) return bad(path, ln, "bad group_vertices line");
      gids.insert(a);
    }
  }
  std::vector<std::vector<std::pair<int32_t, int32_t>>> rows((size_t)V);
  for (auto& e : edges) {
    rows[(size_t)e.first.first].push_back({e.first.second, e.second});
    rows[(size_t)e.first.second].push_back({e.first.first, e.second});
  }
  std::map<long long, std::set<int32_t>> mem;
  for (long long gid : gids) mem[gid];
  for (auto& e : gedges) {
    if (mem.count(e.first) && e.second >= 0 && e.second < V) mem[e.first].insert((int32_t)e.second);
    else if (mem.count(e.second) && e.first >= 0 && e.first < V) mem[e.second].insert((int32_t)e.first);
  }
  std::vector<std::vector<int32_t>> lists;
  for (auto& kv : mem) lists.emplace_back(kv.second.begin(), kv.second.end());
  gst_host_graph* g = to_csr(rows);
  gst_host_groups* q = to_groups(lists);
  if (!g || !q) {
    gst_host_graph_free(g);
    gst_host_groups_free(q);
    return GST_OOM;
  }
  *graph = g;
  *groups = q;
  return GST_OK;
}

}  // extern "C"
