// Test-only stand-in for boost::tuple on top of std::tuple, for the
// reference's libMems sources in the oracle build.  Not product code.
#pragma once
#include <tuple>

namespace boost {
using std::get;
using std::make_tuple;
using std::tie;
using std::tuple;
namespace tuples {
using std::get;
using std::make_tuple;
using std::tuple;
}  // namespace tuples
}  // namespace boost
