// Test infrastructure: a stand-in for the parts of the OCCA API that the
// reference's host ogs headers name (libs/ogs, include/memory.hpp,
// include/platform.hpp), so that the reference's own host operator
// (libs/ogs/ogsOperator.cpp) compiles without OCCA for the oracle's
// cross-check and the CPU timing.  No device memory, kernels or streams
// exist behind it: the reference's device paths are compiled, never called.
#pragma once
#include <cstddef>
#include <cstring>
#include <map>
#include <sstream>
#include <string>
#include <vector>

namespace occa {

class dtype_t {};
namespace dtype {
template <class T>
inline const dtype_t& get() {
  static const dtype_t d;
  return d;
}
}  // namespace dtype

// Property trees: every key and assignment accepted and dropped.
class json {
 public:
  json() = default;
  json& operator[](const std::string&) { return *this; }
  const json& operator[](const std::string&) const { return *this; }
  template <class T>
  json& operator=(const T&) { return *this; }
  template <class T>
  T get(const std::string&, const T& fallback) const { return fallback; }
  bool has(const std::string&) const { return false; }
};

class memory {
 public:
  memory() = default;
  bool isInitialized() const { return false; }
  void* ptr() const { return nullptr; }
  void setDtype(const dtype_t&) {}
  size_t size() const { return 0; }
  size_t length() const { return 0; }
  memory operator+(std::ptrdiff_t) const { return memory(); }
  memory slice(std::ptrdiff_t, std::ptrdiff_t = -1) const { return memory(); }
  void copyFrom(const void*, size_t = 0, size_t = 0, const json& = json()) {}
  void copyFrom(const memory&, size_t = 0, size_t = 0, size_t = 0, const json& = json()) {}
  void copyTo(void*, size_t = 0, size_t = 0, const json& = json()) const {}
  void copyTo(memory&, size_t = 0, size_t = 0, size_t = 0, const json& = json()) const {}
  void free() {}
};

class stream {};

class kernel {
 public:
  bool isInitialized() const { return false; }
  template <class... A>
  void operator()(A&&...) const {}
};

class device {
 public:
  template <class T>
  memory malloc(size_t, const void* = nullptr, const json& = json()) { return memory(); }
  template <class T>
  memory malloc(size_t, const json&) { return memory(); }
  void finish() {}
  std::string mode() const { return "Serial"; }
};

inline int getDeviceCount(const std::string&) { return 0; }
namespace env {
inline void setOccaCacheDir(const std::string&) {}
}  // namespace env

}  // namespace occa
