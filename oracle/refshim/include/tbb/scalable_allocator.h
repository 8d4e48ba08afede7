// Stand-in for tbb::scalable_allocator: the standard allocator with the pre-C++20
// construct/destroy members the reference calls (TEST INFRASTRUCTURE ONLY).
#ifndef NOMAD_REFSHIM_SCALABLE_ALLOCATOR_H_
#define NOMAD_REFSHIM_SCALABLE_ALLOCATOR_H_

#include <cstddef>
#include <memory>
#include <new>
#include <utility>

namespace tbb {

template <typename T>
struct scalable_allocator {
  using value_type = T;
  using pointer = T*;
  using const_pointer = const T*;
  using reference = T&;
  using const_reference = const T&;
  using size_type = std::size_t;
  using difference_type = std::ptrdiff_t;
  template <typename U>
  struct rebind {
    using other = scalable_allocator<U>;
  };
  scalable_allocator() noexcept = default;
  template <typename U>
  scalable_allocator(const scalable_allocator<U>&) noexcept {}
  T* allocate(std::size_t n) { return static_cast<T*>(::operator new(n * sizeof(T))); }
  void deallocate(T* p, std::size_t) noexcept { ::operator delete(p); }
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
bool operator==(const scalable_allocator<T>&, const scalable_allocator<U>&) { return true; }
template <typename T, typename U>
bool operator!=(const scalable_allocator<T>&, const scalable_allocator<U>&) { return false; }

}  // namespace tbb

#endif
