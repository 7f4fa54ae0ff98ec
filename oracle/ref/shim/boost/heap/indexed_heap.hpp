// Stand-in for the two Boost.Heap containers the reference's CPU solvers use
// (boost::heap::fibonacci_heap and boost::heap::pairing_heap). The copy of
// Boost vendored with the reference is empty, and no system Boost exists, so
// the reference sources cannot be compiled without a replacement.
//
// This is TEST INFRASTRUCTURE for the oracle build only: it is compiled into
// oracle/_ref together with the reference's own headers and is never part of
// the product library.
//
// Only the members the reference calls are provided: push() returning a
// stable handle, top(), pop(), size(), empty() and update(handle, value).
// Ordering follows Boost.Heap: the container is a max-heap with respect to
// operator< of the element type (the reference defines operator< inversely to
// obtain a min-queue). Implementation: binary heap of pointers to nodes that
// live in a std::deque (stable addresses); each node records its heap slot so
// update() can sift in either direction in O(log n). Tie order between equal
// keys differs from Boost's, which can change WHICH optimal tree the reference
// returns but never its cost.
#pragma once
#include <cstddef>
#include <deque>
#include <utility>
#include <vector>

namespace gst_oracle_shim {

template <class T>
class indexed_heap {
 public:
  struct node {
    T value;
    std::size_t slot;
  };
  class handle_type {
   public:
    handle_type() : n_(nullptr) {}
    explicit handle_type(node* n) : n_(n) {}
    T& operator*() const { return n_->value; }
    node* n_;
  };

  handle_type push(const T& v) {
    node* n;
    if (!free_.empty()) {
      n = free_.back();
      free_.pop_back();
      n->value = v;
    } else {
      store_.push_back(node{v, 0});
      n = &store_.back();
    }
    n->slot = heap_.size();
    heap_.push_back(n);
    sift_up(n->slot);
    return handle_type(n);
  }
  const T& top() const { return heap_.front()->value; }
  void pop() {
    node* root = heap_.front();
    node* last = heap_.back();
    heap_.pop_back();
    if (!heap_.empty()) {
      heap_[0] = last;
      last->slot = 0;
      sift_down(0);
    }
    free_.push_back(root);
  }
  std::size_t size() const { return heap_.size(); }
  bool empty() const { return heap_.empty(); }
  void update(handle_type h, const T& v) {
    h.n_->value = v;
    sift_up(h.n_->slot);
    sift_down(h.n_->slot);
  }

 private:
  // a "ranks above" b  <=>  b < a   (max-heap on operator<)
  static bool above(const node* a, const node* b) { return b->value < a->value; }
  void place(std::size_t i, node* n) {
    heap_[i] = n;
    n->slot = i;
  }
  void sift_up(std::size_t i) {
    node* n = heap_[i];
    while (i > 0) {
      std::size_t parent = (i - 1) / 2;
      if (!above(n, heap_[parent])) break;
      place(i, heap_[parent]);
      i = parent;
    }
    place(i, n);
  }
  void sift_down(std::size_t i) {
    node* n = heap_[i];
    const std::size_t count = heap_.size();
    for (;;) {
      std::size_t child = 2 * i + 1;
      if (child >= count) break;
      if (child + 1 < count && above(heap_[child + 1], heap_[child])) ++child;
      if (!above(heap_[child], n)) break;
      place(i, heap_[child]);
      i = child;
    }
    place(i, n);
  }

  std::vector<node*> heap_;
  std::deque<node> store_;
  std::vector<node*> free_;
};

}  // namespace gst_oracle_shim
