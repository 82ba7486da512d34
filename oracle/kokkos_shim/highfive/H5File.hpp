// HighFive stand-in for the oracle's reference build: just enough declarations
// for the reference headers to parse.  Creating a file, groups and datasets is
// accepted -- so the reference's HDF5_Writer still produces its XDMF sidecar,
// which is plain text -- and reading throws.  Datasets are written nowhere
// unless TECS_SHIM_DUMP names a directory: each dataset's bytes then go to
// <dir>/<group>.<dataset>.bin (the fixtures of whole reference programs), and
// with TECS_SHIM_STOP_AFTER=K the program exits after its K-th group.
#pragma once
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

namespace HighFive {
namespace details {
template <class T, class Enable = void>
struct inspector {
  using type = T;
  using base_type = T;
  using hdf5_type = T;
  static constexpr std::size_t ndim = 0;
  static constexpr std::size_t min_ndim = 0;
  static constexpr std::size_t max_ndim = 0;
  static constexpr bool is_trivially_nestable = std::is_arithmetic_v<T>;
  static constexpr bool is_trivially_copyable = std::is_trivially_copyable_v<T>;
  static std::size_t getRank(const T&) { return 0; }
  static std::vector<std::size_t> getDimensions(const T&) { return {}; }
  static void prepare(T&, const std::vector<std::size_t>&) {}
  static hdf5_type* data(T& v) { return &v; }
  static const hdf5_type* data(const T& v) { return &v; }
  template <class It>
  static void serialize(const T& v, const std::vector<std::size_t>&, It m) { *m = v; }
  template <class It>
  static void unserialize(const It& m, const std::vector<std::size_t>&, T& v) { v = *m; }
};
}  // namespace details

class DataSpace {
 public:
  std::vector<std::size_t> getDimensions() const { return {}; }
};

class DataSet {
 public:
  DataSpace getSpace() const { return {}; }
  template <class T>
  void read(T&) const { throw std::runtime_error("HighFive stand-in: no file I/O in the oracle build"); }
  template <class T>
  void write(const T&) { throw std::runtime_error("HighFive stand-in: no file I/O in the oracle build"); }
};

namespace shim {
inline const char* dump_dir() { return std::getenv("TECS_SHIM_DUMP"); }
inline int& groups_made() {
  static int n = 0;
  return n;
}
// ends the program once the group after the K-th is begun (the K-th is complete then)
inline void count_group() {
  const char* k = std::getenv("TECS_SHIM_STOP_AFTER");
  if (k && ++groups_made() > std::atoi(k)) std::exit(0);
}
template <class T>
void dump(const std::string& group, const std::string& name, const T& data) {
  const char* dir = dump_dir();
  if (!dir) return;
  if constexpr (requires { data.data(); data.extent(0); }) {
    using V = std::remove_cv_t<std::remove_pointer_t<decltype(data.data())>>;
    const std::string path = std::string(dir) + "/" + group + "." + name + ".bin";
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return;
    std::fwrite(data.data(), sizeof(V), data.extent(0), f);
    std::fclose(f);
  }
}
}  // namespace shim

class Group {
 public:
  Group() = default;
  explicit Group(const std::string& name) : name_(name) {}
  template <class T>
  DataSet createDataSet(const std::string& name, const T& data) {
    shim::dump(name_, name, data);
    return {};
  }
  DataSet getDataSet(const std::string&) const {
    throw std::runtime_error("HighFive stand-in: no file I/O in the oracle build");
  }

 private:
  std::string name_;
};

class File : public Group {
 public:
  enum class AccessMode { ReadOnly, ReadWrite, Truncate, Excl, Debug, Create, Overwrite, OpenOrCreate };
  File(const std::string&, AccessMode = AccessMode::ReadOnly) {}
  Group createGroup(const std::string& name) {
    shim::count_group();
    return Group(name);
  }
  void flush() {}
};
}  // namespace HighFive
