// Test-only stand-in for the two Boost pool allocators the reference's
// seed/match sources name.  Backed by operator new; used only to compile the
// reference into the CPU oracle library.
#pragma once
#include <memory>
#include <cstddef>
namespace boost {
template <class T> struct fast_pool_allocator : std::allocator<T> {
  typedef T value_type;
  template <class U> struct rebind { typedef fast_pool_allocator<U> other; };
  fast_pool_allocator() {}
  template <class U> fast_pool_allocator(const fast_pool_allocator<U>&) {}
  using std::allocator<T>::allocate;
  using std::allocator<T>::deallocate;
  static T* allocate() { return static_cast<T*>(::operator new(sizeof(T))); }
  static void deallocate(T* p) { ::operator delete(p); }
};
template <class T> struct pool_allocator : fast_pool_allocator<T> {
  template <class U> struct rebind { typedef pool_allocator<U> other; };
  pool_allocator() {}
  template <class U> pool_allocator(const pool_allocator<U>&) {}
};
}
