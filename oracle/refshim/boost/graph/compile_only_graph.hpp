// Test-only stand-in for the few boost::graph names the reference's
// ProgressiveAligner.cpp (findMidpoint) and Backbone.cpp use, so that those
// sources compile for the oracle build.  Compile-only: the oracle's drivers
// never reach that code, and every stand-in function aborts if called.
// Not product code.
#pragma once
#include <cstdlib>
#include <utility>

namespace boost {
struct vecS {};
struct listS {};
struct undirectedS {};
struct directedS {};
struct bidirectionalS {};
struct no_property {};
struct edge_weight_t {};
struct edge_color_t {};
struct vertex_index_t {};
enum default_color_type { white_color, gray_color, black_color };
struct on_tree_edge {};
static const edge_weight_t edge_weight = {};
static const edge_color_t edge_color = {};

template <class Tag, class T, class Base = no_property>
struct property {};

template <class G>
struct graph_traits {
  typedef int vertex_descriptor;
  typedef int* edge_iterator;
  typedef int* vertex_iterator;
  typedef int* out_edge_iterator;
  typedef std::size_t vertices_size_type;
};

template <class A = vecS, class B = vecS, class C = directedS, class VP = no_property, class EP = no_property,
          class GP = no_property, class EL = listS>
struct adjacency_list {
  typedef int vertex_descriptor;
  adjacency_list() {}
  explicit adjacency_list(std::size_t) {}
  template <class It>
  adjacency_list(It, It, std::size_t) {}
};

struct compile_only_map {
  int& operator[](int) const { std::abort(); }
};
template <class G, class Tag>
struct property_map {
  typedef compile_only_map type;
  typedef compile_only_map const_type;
};

template <class G, class Tag>
compile_only_map get(Tag, G&) { std::abort(); }
template <class G>
std::pair<int*, int*> edges(const G&) { std::abort(); }
template <class G>
std::pair<int*, int*> vertices(const G&) { std::abort(); }
template <class G>
std::size_t num_vertices(const G&) { std::abort(); }
template <class G>
int vertex(std::size_t, const G&) { std::abort(); }
template <class G, class V>
std::pair<int, bool> add_edge(V, V, G&) { std::abort(); }
template <class G, class D>
bool johnson_all_pairs_shortest_paths(G&, D&) { std::abort(); }

struct compile_only_params {
  template <class T>
  compile_only_params visitor(const T&) const { return *this; }
  template <class T>
  compile_only_params edge_color_map(const T&) const { return *this; }
  template <class T>
  compile_only_params vertex_color_map(const T&) const { return *this; }
};
template <class V>
compile_only_params root_vertex(V) { return compile_only_params(); }
template <class T>
int make_dfs_visitor(const T&) { return 0; }
template <class P, class Tag>
int record_predecessors(P, Tag) { return 0; }
template <class P, class Tag>
int record_distances(P, Tag) { return 0; }
template <class G, class P>
void undirected_dfs(const G&, const P&) { std::abort(); }
}  // namespace boost
