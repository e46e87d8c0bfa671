// Test-only stand-in for the subset of boost::dynamic_bitset the reference's
// match and alignment classes call (test/set/flip/resize/size, search,
// shifts and comparison).  Bit 0 is the lowest bit, as in boost.
#pragma once
#include <vector>
#include <cstddef>
namespace boost {
template <class B = unsigned long, class A = void> class dynamic_bitset {
  std::vector<bool> v_;
 public:
  typedef std::size_t size_type;
  static const size_type npos = static_cast<size_type>(-1);
  dynamic_bitset() {}
  explicit dynamic_bitset(size_type n, unsigned long val = 0) : v_(n, false) {
    for (size_type i = 0; i < n && i < 64; ++i) v_[i] = (val >> i) & 1UL;
  }
  size_type size() const { return v_.size(); }
  bool test(size_type i) const { return v_[i]; }
  dynamic_bitset& set(size_type i, bool b = true) { v_[i] = b; return *this; }
  dynamic_bitset& set() { for (size_type i = 0; i < v_.size(); ++i) v_[i] = true; return *this; }
  dynamic_bitset& reset(size_type i) { v_[i] = false; return *this; }
  dynamic_bitset& reset() { for (size_type i = 0; i < v_.size(); ++i) v_[i] = false; return *this; }
  dynamic_bitset& flip() { v_.flip(); return *this; }
  dynamic_bitset& flip(size_type i) { v_[i] = !v_[i]; return *this; }
  void resize(size_type n, bool b = false) { v_.resize(n, b); }
  void clear() { v_.clear(); }
  void push_back(bool b) { v_.push_back(b); }
  bool operator[](size_type i) const { return v_[i]; }
  std::vector<bool>::reference operator[](size_type i) { return v_[i]; }
  size_type count() const { size_type c = 0; for (bool b : v_) c += b; return c; }
  bool any() const { return count() > 0; }
  bool none() const { return count() == 0; }
  bool operator==(const dynamic_bitset& o) const { return v_ == o.v_; }
  bool operator!=(const dynamic_bitset& o) const { return v_ != o.v_; }
  bool operator<(const dynamic_bitset& o) const { return v_ < o.v_; }
  dynamic_bitset& operator&=(const dynamic_bitset& o) { for (size_type i = 0; i < v_.size(); ++i) v_[i] = v_[i] && o.v_[i]; return *this; }
  dynamic_bitset& operator|=(const dynamic_bitset& o) { for (size_type i = 0; i < v_.size(); ++i) v_[i] = v_[i] || o.v_[i]; return *this; }
  dynamic_bitset& operator^=(const dynamic_bitset& o) { for (size_type i = 0; i < v_.size(); ++i) v_[i] = v_[i] != o.v_[i]; return *this; }
  dynamic_bitset& operator-=(const dynamic_bitset& o) { for (size_type i = 0; i < v_.size(); ++i) v_[i] = v_[i] && !o.v_[i]; return *this; }
  // bit i takes bit i+n (toward bit 0); the top n bits become 0
  dynamic_bitset& operator>>=(size_type n) {
    const size_type m = v_.size();
    for (size_type i = 0; i < m; ++i) v_[i] = i + n < m ? (bool)v_[i + n] : false;
    return *this;
  }
  // bit i takes bit i-n (away from bit 0); the low n bits become 0
  dynamic_bitset& operator<<=(size_type n) {
    const size_type m = v_.size();
    for (size_type i = m; i-- > 0;) v_[i] = i >= n ? (bool)v_[i - n] : false;
    return *this;
  }
  dynamic_bitset operator>>(size_type n) const { dynamic_bitset r(*this); r >>= n; return r; }
  dynamic_bitset operator<<(size_type n) const { dynamic_bitset r(*this); r <<= n; return r; }
  dynamic_bitset operator~() const { dynamic_bitset r(*this); r.flip(); return r; }
  size_type find_first() const { return find_from(0); }
  size_type find_next(size_type i) const { return find_from(i + 1); }
  void swap(dynamic_bitset& o) { v_.swap(o.v_); }
  bool empty() const { return v_.empty(); }
  size_type num_blocks() const { return (v_.size() + 63) / 64; }

 private:
  size_type find_from(size_type i) const {
    for (; i < v_.size(); ++i)
      if (v_[i]) return i;
    return npos;
  }

 public:
};
template <class B, class A>
dynamic_bitset<B, A> operator&(const dynamic_bitset<B, A>& x, const dynamic_bitset<B, A>& y) { dynamic_bitset<B, A> r(x); r &= y; return r; }
template <class B, class A>
dynamic_bitset<B, A> operator|(const dynamic_bitset<B, A>& x, const dynamic_bitset<B, A>& y) { dynamic_bitset<B, A> r(x); r |= y; return r; }
template <class B, class A>
dynamic_bitset<B, A> operator^(const dynamic_bitset<B, A>& x, const dynamic_bitset<B, A>& y) { dynamic_bitset<B, A> r(x); r ^= y; return r; }
template <class B, class A>
dynamic_bitset<B, A> operator-(const dynamic_bitset<B, A>& x, const dynamic_bitset<B, A>& y) { dynamic_bitset<B, A> r(x); r -= y; return r; }
template <class B, class A>
void swap(dynamic_bitset<B, A>& x, dynamic_bitset<B, A>& y) { x.swap(y); }
}
