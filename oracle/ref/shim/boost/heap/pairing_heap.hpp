// Stand-in for boost/heap/pairing_heap.hpp (oracle build only; see indexed_heap.hpp).
#pragma once
#include "indexed_heap.hpp"
namespace boost {
namespace heap {
template <class T>
using pairing_heap = gst_oracle_shim::indexed_heap<T>;
}  // namespace heap
}  // namespace boost
