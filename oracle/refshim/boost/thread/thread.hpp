// boost::thread / boost::thread_group as the reference's EAR.cpp uses them.
// Threads of a group run one after another, in creation order, so that a
// replayed random tape is consumed deterministically.  TEST INFRASTRUCTURE
// ONLY (oracle/_ref).
#pragma once
#include "mutex.hpp"

namespace boost {
class thread {
 public:
  template <typename F>
  explicit thread(F f) {
    f();
  }
  void join() {}
};
class thread_group {
 public:
  template <typename F>
  void create_thread(F f) {
    f();
  }
  void join_all() {}
};
}  // namespace boost
