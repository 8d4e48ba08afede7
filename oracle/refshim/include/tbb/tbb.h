// Single-process stand-in for the parts of Intel TBB that the reference's updater
// (Code/nomad/nb_main.cpp, pool.cpp, nb_data.cpp) uses: concurrent_queue, the two
// allocators and tick_count.  TEST INFRASTRUCTURE ONLY: it lets the unmodified
// reference sources compile into oracle/_ref/ so that the oracle can be checked
// against them.  The queue is a mutex-guarded deque with one extra knob for the
// driver (a pop budget, so that a one-thread run stops after an exact number of
// column visits); everything else behaves as TBB documents it.
#ifndef NOMAD_REFSHIM_TBB_H_
#define NOMAD_REFSHIM_TBB_H_

#include <atomic>
#include <chrono>
#include <deque>
#include <functional>
#include <mutex>

#include "tbb/cache_aligned_allocator.h"
#include "tbb/scalable_allocator.h"

namespace tbb {

template <typename T, typename A = cache_aligned_allocator<T>>
class concurrent_queue {
 public:
  concurrent_queue() = default;
  concurrent_queue(const concurrent_queue&) = delete;
  concurrent_queue& operator=(const concurrent_queue&) = delete;

  void push(const T& v) {
    std::lock_guard<std::mutex> g(m_);
    q_.push_back(v);
  }
  bool try_pop(T& out) {
    std::lock_guard<std::mutex> g(m_);
    if (pop_budget_ == 0) {
      refused_.store(true);
      return false;
    }
    if (q_.empty()) return false;
    out = q_.front();
    q_.pop_front();
    if (pop_budget_ > 0) --pop_budget_;
    return true;
  }
  long long unsafe_size() const {
    std::lock_guard<std::mutex> g(m_);
    return static_cast<long long>(q_.size());
  }
  bool empty() const { return unsafe_size() == 0; }
  void clear() {
    std::lock_guard<std::mutex> g(m_);
    q_.clear();
  }

  // Driver knobs (not TBB): after `budget` more successful pops every try_pop fails and
  // records that it was refused; a negative budget means unlimited.
  void shim_set_pop_budget(long long budget) {
    std::lock_guard<std::mutex> g(m_);
    pop_budget_ = budget;
    refused_.store(false);
  }
  bool shim_refused() const { return refused_.load(); }

 private:
  mutable std::mutex m_;
  std::deque<T> q_;
  long long pop_budget_ = -1;
  std::atomic<bool> refused_{false};
};

class tick_count {
 public:
  class interval_t {
   public:
    interval_t() : s_(0.0) {}
    explicit interval_t(double s) : s_(s) {}
    double seconds() const { return s_; }
    interval_t& operator+=(const interval_t& o) {
      s_ += o.s_;
      return *this;
    }

   private:
    double s_;
  };
  tick_count() : t_() {}
  static tick_count now() {
    tick_count t;
    t.t_ = std::chrono::steady_clock::now();
    return t;
  }
  friend interval_t operator-(const tick_count& a, const tick_count& b) {
    return interval_t(std::chrono::duration<double>(a.t_ - b.t_).count());
  }

 private:
  std::chrono::steady_clock::time_point t_;
};

}  // namespace tbb

#endif
