// Stand-in for the one Boost.Heap type the reference CPU_HopHL code uses.
//
// TEST INFRASTRUCTURE ONLY: this header lets the reference's own header-only
// CPU implementation (CPU_HopHL/include/HBPLL/...) compile unmodified in a
// container without Boost, so that its output can serve as the parity oracle.
//
// The reference needs exactly this surface of boost::heap::fibonacci_heap<T>
// (CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels_generation.h:30,72,
// 79,100-104,188,194): push() returning a stable handle, top(), pop(),
// update(handle, value), size(), and a default-constructible handle_type.
// Boost's heaps are max-heaps under operator<, so top() is the element that is
// largest under operator<.  The reference's operator< (hop_constrained_two_hop_
// labels.h:42-52) is inverted, which makes top() the state with the smallest
// (distance, hop).
//
// This is an addressable binary heap, not a Fibonacci heap: the asymptotics
// differ, the order of pops among equal keys differs from Boost 1.85.0, and
// only the reference's `parent_vertex` choice on exact ties can depend on that
// order.  (hub, hop, distance) of every label does not.
#pragma once
#include <cstddef>
#include <deque>
#include <vector>

namespace boost {
namespace heap {

template <class T>
class fibonacci_heap {
  struct slot {
    T value;
    std::size_t pos;  // index in heap_, or npos once popped
  };
  std::deque<slot> store_;  // deque: element addresses stay valid on growth
  std::vector<slot*> heap_;

  void swap_at(std::size_t a, std::size_t b) {
    slot* t = heap_[a];
    heap_[a] = heap_[b];
    heap_[b] = t;
    heap_[a]->pos = a;
    heap_[b]->pos = b;
  }
  void sift_up(std::size_t i) {
    while (i > 0) {
      std::size_t p = (i - 1) / 2;
      if (!(heap_[p]->value < heap_[i]->value)) return;
      swap_at(i, p);
      i = p;
    }
  }
  void sift_down(std::size_t i) {
    for (;;) {
      std::size_t l = 2 * i + 1, r = l + 1, best = i;
      if (l < heap_.size() && heap_[best]->value < heap_[l]->value) best = l;
      if (r < heap_.size() && heap_[best]->value < heap_[r]->value) best = r;
      if (best == i) return;
      swap_at(i, best);
      i = best;
    }
  }

 public:
  using handle_type = slot*;

  handle_type push(const T& v) {
    store_.push_back(slot{v, heap_.size()});
    slot* s = &store_.back();
    heap_.push_back(s);
    sift_up(heap_.size() - 1);
    return s;
  }
  const T& top() const { return heap_.front()->value; }
  void pop() {
    swap_at(0, heap_.size() - 1);
    heap_.back()->pos = static_cast<std::size_t>(-1);
    heap_.pop_back();
    if (!heap_.empty()) sift_down(0);
  }
  void update(handle_type h, const T& v) {
    h->value = v;
    sift_up(h->pos);
    sift_down(h->pos);
  }
  std::size_t size() const { return heap_.size(); }
  bool empty() const { return heap_.empty(); }
};

}  // namespace heap
}  // namespace boost
