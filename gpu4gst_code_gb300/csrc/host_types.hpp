// Host-side objects shared by the generators (gen.cpp), the dataset readers
// (dataset.cpp) and the C ABI's error channel (engine.cu).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

struct gst_host_graph {
  int32_t V = 0;
  std::vector<int32_t> row_ptr, col, w;
};

struct gst_host_groups {
  int32_t k = 0;
  std::vector<int32_t> group_ptr, members;
};

namespace gst {
// Sets the text gst_last_error() returns on this thread (engine.cu).
void set_last_error(const std::string& msg);
}  // namespace gst
