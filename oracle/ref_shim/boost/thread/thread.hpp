// boost/thread/thread.hpp stand-in: the thread_group TreadedRenderer uses
// (cell/ppu_renderer.cpp:129-142), over std::thread.
#pragma once
#include <thread>
#include <vector>

namespace boost {
class thread_group {
 public:
  template <class F>
  void create_thread(F f) { threads_.emplace_back(f); }
  void join_all() {
    for (auto& t : threads_) t.join();
    threads_.clear();
  }

 private:
  std::vector<std::thread> threads_;
};
}  // namespace boost
