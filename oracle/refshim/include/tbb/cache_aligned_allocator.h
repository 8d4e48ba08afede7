// Stand-in for tbb::cache_aligned_allocator: 128-byte aligned, zero-filled storage, with
// the pre-C++20 construct/destroy members the reference calls (TEST INFRASTRUCTURE ONLY).
// Zero fill makes the fields the reference leaves unset after Pool::allocate (for
// instance ColumnData::source_, read as an index at nb_main.cpp:547) start at zero.
#ifndef NOMAD_REFSHIM_CACHE_ALIGNED_ALLOCATOR_H_
#define NOMAD_REFSHIM_CACHE_ALIGNED_ALLOCATOR_H_

#include <cstddef>
#include <cstring>
#include <new>
#include <utility>

namespace tbb {

template <typename T>
struct cache_aligned_allocator {
  using value_type = T;
  using pointer = T*;
  using const_pointer = const T*;
  using reference = T&;
  using const_reference = const T&;
  using size_type = std::size_t;
  using difference_type = std::ptrdiff_t;
  template <typename U>
  struct rebind {
    using other = cache_aligned_allocator<U>;
  };
  cache_aligned_allocator() noexcept = default;
  template <typename U>
  cache_aligned_allocator(const cache_aligned_allocator<U>&) noexcept {}
  T* allocate(std::size_t n) {
    const std::size_t bytes = n * sizeof(T) > 0 ? n * sizeof(T) : 1;
    void* p = ::operator new(bytes, std::align_val_t(128));
    std::memset(p, 0, bytes);
    return static_cast<T*>(p);
  }
  void deallocate(T* p, std::size_t) noexcept { ::operator delete(p, std::align_val_t(128)); }
  template <typename U, typename... Args>
  void construct(U* p, Args&&... args) {
    ::new (static_cast<void*>(p)) U(std::forward<Args>(args)...);
  }
  template <typename U>
  void destroy(U* p) {
    p->~U();
  }
};
template <typename T, typename U>
bool operator==(const cache_aligned_allocator<T>&, const cache_aligned_allocator<U>&) { return true; }
template <typename T, typename U>
bool operator!=(const cache_aligned_allocator<T>&, const cache_aligned_allocator<U>&) { return false; }

}  // namespace tbb

#endif
