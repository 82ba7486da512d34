// tecs/hdf5_reader.hpp -- io::HDF5_Reader of the C++20 drop-in layer: reads
// datasets of an HDF5 file into views, as the reference's reader does
// (include/io/hdf5_reader.hpp:28-72, over HighFive).  libhdf5 is absent, so
// this is an own reader of the format's parts that such files use: the
// version-0 superblock with 8-byte offsets, symbol-table groups (B-tree v1,
// symbol nodes, local heap), version-1 object headers with continuation
// blocks, and contiguous or compact datasets of little-endian IEEE floats or
// integers of 1 to 8 bytes.  Values are converted to the view's scalar type
// as HighFive converts them on read.
#ifndef TECS_CXX_HDF5_READER_HPP
#define TECS_CXX_HDF5_READER_HPP

#include <cstdint>
#include <cstring>
#include <fstream>
#include <iterator>
#include <map>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "view.hpp"

namespace tecs {
namespace io {

class HDF5_Reader {
 public:
  explicit HDF5_Reader(const std::string& path) {
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::runtime_error("cannot open " + path);
    b_.assign(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
    static const unsigned char sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    if (b_.size() < 96 || std::memcmp(b_.data(), sig, 8) != 0) throw std::runtime_error(path + ": not an HDF5 file");
    if (b_[8] != 0) throw std::runtime_error(path + ": superblock version not supported");
    if (b_[13] != 8 || b_[14] != 8) throw std::runtime_error(path + ": only 8-byte offsets and lengths");
    root_ = u64(64);
  }

  // the dataset's dimensions (hdf5_reader.hpp:50-53)
  std::vector<std::size_t> get_dataset_dimensions(const std::string& name) const {
    return dataset(name).dims;
  }

  // the dataset's values into the view's host array (row-major, as many as
  // the view holds), then to its device array (hdf5_reader.hpp:66-71)
  template <typename T>
  void read_dataset(const std::string& name, View<T> out) const {
    const Dataset d = dataset(name);
    std::size_t count = 1;
    for (std::size_t e : d.dims) count *= e;
    using S = scalar_of<T>;
    constexpr std::size_t per = sizeof(T) / sizeof(S);
    const std::size_t room = std::size_t(out.extent(0)) * per;
    if (count > room) count = room;
    S* dst = reinterpret_cast<S*>(out.data());
    for (std::size_t k = 0; k < count; ++k) dst[k] = convert<S>(d, k);
    out.unconditional_sync_device();
  }

 private:
  struct Dataset {
    std::vector<std::size_t> dims;
    int cls = 0;  // 0 integer, 1 float
    bool is_signed = false;
    unsigned size = 0;
    const unsigned char* data = nullptr;  // null: never written (zeros)
  };

  template <typename T>
  static auto scalar_tag() {
    if constexpr (std::is_arithmetic_v<T>) return T{};
    else return typename T::value_type{};
  }
  template <typename T>
  using scalar_of = decltype(scalar_tag<T>());

  std::uint64_t u64(std::size_t at) const { return rd<std::uint64_t>(at); }
  template <typename U>
  U rd(std::size_t at) const {
    if (at + sizeof(U) > b_.size()) throw std::runtime_error("HDF5 file truncated");
    U v;
    std::memcpy(&v, b_.data() + at, sizeof v);
    return v;
  }

  // (type, body offset, body size) of an object header's messages
  std::vector<std::tuple<unsigned, std::size_t, std::size_t>> messages(std::size_t addr) const {
    if (b_.at(addr) != 1) throw std::runtime_error("object header version not supported");
    std::vector<std::pair<std::size_t, std::size_t>> blocks{{addr + 16, rd<std::uint32_t>(addr + 8)}};
    std::vector<std::tuple<unsigned, std::size_t, std::size_t>> out;
    for (std::size_t q = 0; q < blocks.size(); ++q) {
      std::size_t off = blocks[q].first;
      const std::size_t end = off + blocks[q].second;
      while (off + 8 <= end) {
        const unsigned type = rd<std::uint16_t>(off);
        const std::size_t size = rd<std::uint16_t>(off + 2);
        if (type == 0x0010) blocks.push_back({u64(off + 8), u64(off + 16)});
        else out.emplace_back(type, off + 8, size);
        off += 8 + size;
      }
    }
    return out;
  }
  std::size_t message(std::size_t addr, unsigned type) const {
    for (const auto& m : messages(addr))
      if (std::get<0>(m) == type) return std::get<1>(m);
    return 0;
  }

  std::map<std::string, std::size_t> group(std::size_t ohdr) const {
    const std::size_t st = message(ohdr, 0x0011);
    if (!st) throw std::runtime_error("not a symbol-table group");
    const std::size_t btree = u64(st), heap = u64(st + 8);
    if (std::memcmp(b_.data() + heap, "HEAP", 4) != 0) throw std::runtime_error("bad local heap");
    const std::size_t names = u64(heap + 24);
    std::map<std::string, std::size_t> out;
    std::vector<std::size_t> todo{btree};
    while (!todo.empty()) {
      const std::size_t node = todo.back();
      todo.pop_back();
      if (std::memcmp(b_.data() + node, "TREE", 4) != 0) throw std::runtime_error("bad B-tree node");
      const unsigned level = b_.at(node + 5), entries = rd<std::uint16_t>(node + 6);
      for (unsigned k = 0; k < entries; ++k) {
        const std::size_t child = u64(node + 24 + 16 * std::size_t(k) + 8);
        if (level > 0) {
          todo.push_back(child);
          continue;
        }
        if (std::memcmp(b_.data() + child, "SNOD", 4) != 0) throw std::runtime_error("bad symbol table node");
        const unsigned symbols = rd<std::uint16_t>(child + 6);
        for (unsigned e = 0; e < symbols; ++e) {
          const std::size_t at = child + 8 + 40 * std::size_t(e);
          const char* name = reinterpret_cast<const char*>(b_.data() + names + u64(at));
          out[std::string(name)] = u64(at + 8);
        }
      }
    }
    return out;
  }

  Dataset dataset(const std::string& path) const {
    std::size_t addr = root_;
    std::size_t start = 0;
    while (start < path.size()) {
      std::size_t slash = path.find('/', start);
      if (slash == std::string::npos) slash = path.size();
      if (slash > start) {
        const auto entries = group(addr);
        const auto it = entries.find(path.substr(start, slash - start));
        if (it == entries.end()) throw std::runtime_error("no dataset " + path);
        addr = it->second;
      }
      start = slash + 1;
    }
    Dataset d;
    const std::size_t space = message(addr, 0x0001), type = message(addr, 0x0003), layout = message(addr, 0x0008);
    if (!space || !type || !layout) throw std::runtime_error(path + " is not a dataset");
    const unsigned version = b_.at(space), rank = b_.at(space + 1);
    const std::size_t first = space + (version == 1 ? 8 : 4);
    for (unsigned k = 0; k < rank; ++k) d.dims.push_back(u64(first + 8 * std::size_t(k)));
    d.cls = b_.at(type) & 0x0F;
    if (b_.at(type + 1) & 0x01) throw std::runtime_error(path + ": big-endian data not supported");
    d.is_signed = (b_.at(type + 1) & 0x08) != 0;
    d.size = rd<std::uint32_t>(type + 4);
    if ((d.cls != 0 && d.cls != 1) || (d.cls == 1 && d.size != 4 && d.size != 8) || d.size == 0 || d.size > 8)
      throw std::runtime_error(path + ": datatype not supported");
    if (b_.at(layout) != 3) throw std::runtime_error(path + ": layout message version not supported");
    std::size_t count = 1;
    for (std::size_t e : d.dims) count *= e;
    if (b_.at(layout + 1) == 1) {  // contiguous
      const std::uint64_t at = u64(layout + 2);
      if (at != ~std::uint64_t(0)) {
        if (at + count * d.size > b_.size()) throw std::runtime_error(path + ": data beyond the file");
        d.data = b_.data() + at;
      }
    } else if (b_.at(layout + 1) == 0) {  // compact
      if (rd<std::uint16_t>(layout + 2) < count * d.size) throw std::runtime_error(path + ": short compact data");
      d.data = b_.data() + layout + 4;
    } else {
      throw std::runtime_error(path + ": chunked datasets are not supported");
    }
    return d;
  }

  template <typename S>
  static S convert(const Dataset& d, std::size_t k) {
    if (!d.data) return S(0);
    const unsigned char* p = d.data + k * d.size;
    if (d.cls == 1) {
      if (d.size == 4) {
        float v;
        std::memcpy(&v, p, 4);
        return static_cast<S>(v);
      }
      double v;
      std::memcpy(&v, p, 8);
      return static_cast<S>(v);
    }
    std::uint64_t raw = 0;
    std::memcpy(&raw, p, d.size);
    if (d.is_signed && d.size < 8 && (raw >> (8 * d.size - 1)) & 1u) raw |= ~std::uint64_t(0) << (8 * d.size);
    return d.is_signed ? static_cast<S>(static_cast<std::int64_t>(raw)) : static_cast<S>(raw);
  }

  std::vector<unsigned char> b_;
  std::size_t root_ = 0;
};

}  // namespace io
}  // namespace tecs

#endif  // TECS_CXX_HDF5_READER_HPP
