// Test-only stand-in for boost::tuple on top of std::tuple (with boost's
// member get<N>()), for the reference's libMems sources in the oracle build.
// Not product code.
#pragma once
#include <cstddef>
#include <tuple>
#include <type_traits>
#include <utility>

namespace boost {
template <class... T>
struct tuple : std::tuple<T...> {
  using std::tuple<T...>::tuple;
  tuple() = default;
  tuple(const std::tuple<T...>& t) : std::tuple<T...>(t) {}
  template <std::size_t N>
  typename std::tuple_element<N, std::tuple<T...>>::type& get() {
    return std::get<N>(static_cast<std::tuple<T...>&>(*this));
  }
  template <std::size_t N>
  const typename std::tuple_element<N, std::tuple<T...>>::type& get() const {
    return std::get<N>(static_cast<const std::tuple<T...>&>(*this));
  }
};
template <class... T>
tuple<typename std::decay<T>::type...> make_tuple(T&&... t) {
  return tuple<typename std::decay<T>::type...>(std::forward<T>(t)...);
}
using std::get;
using std::tie;
namespace tuples {
using boost::make_tuple;
using boost::tuple;
using std::get;
}  // namespace tuples
}  // namespace boost

namespace std {
template <class... T>
struct tuple_size<boost::tuple<T...>> : tuple_size<std::tuple<T...>> {};
template <std::size_t N, class... T>
struct tuple_element<N, boost::tuple<T...>> : tuple_element<N, std::tuple<T...>> {};
}  // namespace std
