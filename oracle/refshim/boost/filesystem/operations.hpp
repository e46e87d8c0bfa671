// Test-only stand-in for the boost::filesystem calls in the reference's
// Files.h (path decomposition, remove, exists).
#pragma once
#include <string>
#include <cstdio>
#include <sys/stat.h>
namespace boost { namespace filesystem {
class path {
  std::string s_;
 public:
  path() {}
  path(const std::string& s) : s_(s) {}
  path(const char* s) : s_(s) {}
  std::string string() const { return s_; }
  path branch_path() const { size_t p = s_.rfind('/'); return p == std::string::npos ? path("") : path(s_.substr(0, p)); }
  path parent_path() const { return branch_path(); }
  path leaf() const { size_t p = s_.rfind('/'); return p == std::string::npos ? path(s_) : path(s_.substr(p + 1)); }
  path filename() const { return leaf(); }
  path& operator/=(const std::string& o) { if (!s_.empty() && s_.back() != '/') s_ += '/'; s_ += o; return *this; }
  path& operator/=(const path& o) { return *this /= o.s_; }
  void clear() { s_.clear(); }
  bool empty() const { return s_.empty(); }
};
inline bool remove(const path& p) { return std::remove(p.string().c_str()) == 0; }
inline bool exists(const path& p) { struct stat st; return ::stat(p.string().c_str(), &st) == 0; }
}}
