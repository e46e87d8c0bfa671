// Test-only stand-in, force-included into the reference's Aligner.cpp alone.
//
// Two comparators there (MatchLeftEndComparator, LabeledMemComparator)
// declare a copy constructor that takes a non-const reference, which
// today's std::sort cannot move.  These overloads are found first for calls
// made inside namespace mems and hand std::sort a copyable handle that calls
// the comparator in place: std::sort sees the same comparison results, so the
// sorted order is the one std::sort would give with the comparator itself.
#pragma once
#include <algorithm>

namespace mems {
class MatchLeftEndComparator;
class LabeledMemComparator;

template <class C>
struct RefCmpShim {
  C* c;
  template <class A, class B>
  bool operator()(const A& a, const B& b) const {
    return (*c)(a, b);
  }
};

template <class It>
void sort(It first, It last, MatchLeftEndComparator& c) {
  std::sort(first, last, RefCmpShim<MatchLeftEndComparator>{&c});
}

template <class It>
void sort(It first, It last, LabeledMemComparator& c) {
  std::sort(first, last, RefCmpShim<LabeledMemComparator>{&c});
}
}  // namespace mems
