// HighFive stand-in for the oracle's reference build: just enough declarations
// for the reference headers to parse.  Creating a file, groups and datasets is
// accepted and writes nothing -- so the reference's HDF5_Writer still produces
// its XDMF sidecar, which is plain text -- and reading throws.
#pragma once
#include <cstddef>
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

class Group {
 public:
  template <class T>
  DataSet createDataSet(const std::string&, const T&) {
    return {};
  }
  DataSet getDataSet(const std::string&) const {
    throw std::runtime_error("HighFive stand-in: no file I/O in the oracle build");
  }
};

class File : public Group {
 public:
  enum class AccessMode { ReadOnly, ReadWrite, Truncate, Excl, Debug, Create, Overwrite, OpenOrCreate };
  File(const std::string&, AccessMode = AccessMode::ReadOnly) {}
  Group createGroup(const std::string&) { return {}; }
  void flush() {}
};
}  // namespace HighFive
