// Test-only stand-in; see compile_only_graph.hpp.
#pragma once
#include "boost/graph/compile_only_graph.hpp"
