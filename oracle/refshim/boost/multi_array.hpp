// Test-only stand-in for the part of boost::multi_array the reference's
// libMems headers use (element access by [i][j][k], extents, resize, shape),
// so those headers compile for the oracle build.  Not product code.
#pragma once
#include <array>
#include <cstddef>
#include <vector>

namespace boost {
namespace mashim {
template <std::size_t K>
struct extent_gen {
  std::array<std::size_t, K> e{};
  extent_gen<K + 1> operator[](std::size_t n) const {
    extent_gen<K + 1> r;
    for (std::size_t i = 0; i < K; ++i) r.e[i] = e[i];
    r.e[K] = n;
    return r;
  }
};
template <class T, std::size_t N>
struct view {
  T* p;
  const std::size_t* ext;
  const std::size_t* stride;
  view<T, N - 1> operator[](std::size_t i) const { return view<T, N - 1>{p + i * stride[0], ext + 1, stride + 1}; }
  std::size_t size() const { return ext[0]; }
};
template <class T>
struct view<T, 1> {
  T* p;
  const std::size_t* ext;
  const std::size_t* stride;
  T& operator[](std::size_t i) const { return p[i]; }
  std::size_t size() const { return ext[0]; }
};
}  // namespace mashim

static const mashim::extent_gen<0> extents;

template <class T, std::size_t N>
class multi_array {
 public:
  typedef T element;
  typedef std::size_t size_type;
  multi_array() { ext_.fill(0); stride_.fill(0); }
  explicit multi_array(const mashim::extent_gen<N>& g) { resize(g); }
  multi_array& resize(const mashim::extent_gen<N>& g) {
    std::vector<T> old;
    old.swap(data_);
    const std::array<std::size_t, N> oext = ext_, ostride = stride_;
    ext_ = g.e;
    std::size_t n = 1;
    for (std::size_t k = N; k-- > 0;) {
      stride_[k] = n;
      n *= ext_[k];
    }
    data_.assign(n, T());
    if (!old.empty()) copy_overlap(old, oext, ostride);
    return *this;
  }
  auto operator[](std::size_t i) { return index(data_.data(), i); }
  auto operator[](std::size_t i) const { return index(const_cast<T*>(data_.data()), i); }
  const std::size_t* shape() const { return ext_.data(); }
  std::size_t size() const { return ext_[0]; }
  std::size_t num_elements() const { return data_.size(); }
  std::size_t num_dimensions() const { return N; }
  T* data() { return data_.data(); }
  const T* data() const { return data_.data(); }
  T* origin() { return data_.data(); }

 private:
  template <std::size_t M = N>
  typename std::enable_if<(M > 1), mashim::view<T, N - 1>>::type index(T* base, std::size_t i) const {
    return mashim::view<T, N - 1>{base + i * stride_[0], ext_.data() + 1, stride_.data() + 1};
  }
  template <std::size_t M = N>
  typename std::enable_if<(M == 1), T&>::type index(T* base, std::size_t i) const { return base[i]; }
  void copy_overlap(std::vector<T>& old, const std::array<std::size_t, N>& oext,
                    const std::array<std::size_t, N>& ostride) {
    std::array<std::size_t, N> lim, idx{};
    for (std::size_t k = 0; k < N; ++k) lim[k] = oext[k] < ext_[k] ? oext[k] : ext_[k];
    for (std::size_t k = 0; k < N; ++k)
      if (lim[k] == 0) return;
    for (;;) {
      std::size_t so = 0, sn = 0;
      for (std::size_t k = 0; k < N; ++k) {
        so += idx[k] * ostride[k];
        sn += idx[k] * stride_[k];
      }
      data_[sn] = old[so];
      std::size_t k = N;
      while (k-- > 0) {
        if (++idx[k] < lim[k]) break;
        idx[k] = 0;
        if (k == 0) return;
      }
    }
  }
  std::vector<T> data_;
  std::array<std::size_t, N> ext_{};
  std::array<std::size_t, N> stride_{};
};
}  // namespace boost
