// Test-only stand-in for boost::iostreams::mapped_file_source (read-only
// mmap of a whole file), used by the reference's file-backed sorted mer list.
#pragma once
#include <string>
#include <cstddef>
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>
namespace boost { namespace iostreams {
class mapped_file_source {
  const char* d_ = nullptr; std::size_t n_ = 0;
 public:
  mapped_file_source() {}
  explicit mapped_file_source(const std::string& f) { open(f); }
  ~mapped_file_source() { close(); }
  void open(const std::string& f) {
    close();
    int fd = ::open(f.c_str(), O_RDONLY); if (fd < 0) return;
    struct stat st; if (fstat(fd, &st) != 0 || st.st_size == 0) { ::close(fd); return; }
    void* p = mmap(nullptr, st.st_size, PROT_READ, MAP_PRIVATE, fd, 0); ::close(fd);
    if (p == MAP_FAILED) return; d_ = static_cast<const char*>(p); n_ = st.st_size;
  }
  // Maps len bytes starting at offset (offset must be page aligned, as in Boost).
  void open(const std::string& f, std::size_t len, unsigned long long offset) {
    close();
    int fd = ::open(f.c_str(), O_RDONLY); if (fd < 0) return;
    void* p = mmap(nullptr, len, PROT_READ, MAP_PRIVATE, fd, (off_t)offset); ::close(fd);
    if (p == MAP_FAILED) return; d_ = static_cast<const char*>(p); n_ = len;
  }
  void close() { if (d_) munmap(const_cast<char*>(d_), n_); d_ = nullptr; n_ = 0; }
  bool is_open() const { return d_ != nullptr; }
  const char* data() const { return d_; }
  std::size_t size() const { return n_; }
};
}}
