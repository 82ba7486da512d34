// tecs/hdf5_writer.hpp -- snapshot writer of the C++20 drop-in layer.
//
// io::HDF5_Writer<Config> keeps the reference's writer interface
// (include/io/hdf5_writer.hpp:66-79 constructor, :306-321 write, :335-347
// write_static): "<path>.h5" holds one group "t<step>" per write with one
// dataset per view, named by the view's label and shaped [active_count,
// components] (float32 for VectorN / Polarity_, uint32 for Link).  libhdf5 is
// not a dependency: the file is written directly in the subset of the HDF5
// format the library uses for such files -- version 0 superblock, version 1
// object headers, symbol-table groups (version 1 B-tree, symbol table nodes,
// local heaps), contiguous datasets with dataspace v1, datatype v1, fill
// value v2 and layout v3 messages -- with the same byte layout as
// tecs_gb300/h5.py's writer.  The file takes any number of writes: the root
// group's B-tree gains levels (32 children per node) as its symbol table nodes
// (8 groups each) grow, and its name heap moves to a segment twice the size
// when it fills.  With Settings::write_xmf (the default) it also
// writes the reference's XDMF sidecar "<path>.xmf" (hdf5_writer.hpp:134-287)
// for visualisation tools: one temporal collection, a uniform grid per write
// with the first view as geometry, the other views as node attributes (links
// as polyline topology) and the static group in every grid.
#ifndef TECS_CXX_HDF5_WRITER_HPP
#define TECS_CXX_HDF5_WRITER_HPP

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

namespace tecs {

template <typename T>
class View;
struct Link;
template <typename Scalar, int dimensions>
struct VectorN;
template <typename Scalar>
struct Polarity_;

namespace io {
namespace h5detail {

constexpr std::uint64_t kUndef = ~std::uint64_t(0);
constexpr unsigned kLeafK = 4, kInternalK = 16;
constexpr unsigned kSnodEntries = 2 * kLeafK;
constexpr std::size_t kEntrySize = 40;
constexpr std::size_t kSnodSize = 8 + kSnodEntries * kEntrySize;
constexpr std::size_t kBtreeSize = 24 + (2 * kInternalK + 1) * 8 + 2 * kInternalK * 8;
constexpr std::size_t kRootHeapData = 8192;

inline std::size_t pad8(std::size_t n) { return (n + 7) & ~std::size_t(7); }

using Bytes = std::vector<unsigned char>;

template <typename T>
void put(Bytes& b, T v) {  // little-endian on every host this builds for
  unsigned char raw[sizeof(T)];
  std::memcpy(raw, &v, sizeof(T));
  b.insert(b.end(), raw, raw + sizeof(T));
}
inline void zeros(Bytes& b, std::size_t n) { b.insert(b.end(), n, 0); }

inline Bytes msg(std::uint16_t type, Bytes body, unsigned char flags = 0) {
  zeros(body, pad8(body.size()) - body.size());
  Bytes m;
  put<std::uint16_t>(m, type);
  put<std::uint16_t>(m, static_cast<std::uint16_t>(body.size()));
  put<std::uint8_t>(m, flags);
  zeros(m, 3);
  m.insert(m.end(), body.begin(), body.end());
  return m;
}

inline Bytes dataspace(std::uint64_t rows, std::uint64_t cols) {
  Bytes b;
  put<std::uint8_t>(b, 1); put<std::uint8_t>(b, 2); put<std::uint8_t>(b, 1);
  zeros(b, 5);
  put(b, rows); put(b, cols);  // dimensions
  put(b, rows); put(b, cols);  // maximum dimensions
  return msg(0x0001, b);
}

// float32 (IEEE little endian), or a 32-bit integer (signed or not)
enum class Kind { u32, f32, i32 };
inline Bytes datatype(Kind kind) {
  Bytes b;
  if (kind == Kind::f32) {
    b = {0x11, 0x20, 0x1F, 0x00};
    put<std::uint32_t>(b, 4);
    put<std::uint16_t>(b, 0); put<std::uint16_t>(b, 32);
    put<std::uint8_t>(b, 23); put<std::uint8_t>(b, 8); put<std::uint8_t>(b, 0); put<std::uint8_t>(b, 23);
    put<std::uint32_t>(b, 127);
  } else {
    b = {0x10, static_cast<unsigned char>(kind == Kind::i32 ? 0x08 : 0x00), 0x00, 0x00};
    put<std::uint32_t>(b, 4);
    put<std::uint16_t>(b, 0); put<std::uint16_t>(b, 32);
  }
  return msg(0x0003, b, 1);
}

inline Bytes fill_value() {
  Bytes b = {2, 2, 2, 1};
  put<std::uint32_t>(b, 0);
  return msg(0x0005, b, 1);
}

inline Bytes layout_contiguous(std::uint64_t addr, std::uint64_t size) {
  Bytes b = {3, 1};
  put(b, addr); put(b, size);
  return msg(0x0008, b);
}

inline Bytes symbol_table_msg(std::uint64_t btree, std::uint64_t heap) {
  Bytes b;
  put(b, btree); put(b, heap);
  return msg(0x0011, b);
}

inline Bytes object_header(const std::vector<Bytes>& messages, std::size_t min_size = 0) {
  Bytes body;
  for (const auto& m : messages) body.insert(body.end(), m.begin(), m.end());
  std::uint16_t n = static_cast<std::uint16_t>(messages.size());
  if (body.size() < min_size) {  // a NIL message pads the header as the library does
    std::size_t pad = min_size - body.size();
    if (pad < 8) pad += 8;
    put<std::uint16_t>(body, 0);
    put<std::uint16_t>(body, static_cast<std::uint16_t>(pad - 8));
    put<std::uint8_t>(body, 0);
    zeros(body, 3);
    zeros(body, pad - 8);
    ++n;
  }
  Bytes h;
  put<std::uint8_t>(h, 1); put<std::uint8_t>(h, 0);
  put<std::uint16_t>(h, n);
  put<std::uint32_t>(h, 1);
  put<std::uint32_t>(h, static_cast<std::uint32_t>(body.size()));
  zeros(h, 4);
  h.insert(h.end(), body.begin(), body.end());
  return h;
}

inline Bytes entry(std::uint64_t name_off, std::uint64_t ohdr) {
  Bytes b;
  put(b, name_off); put(b, ohdr);
  put<std::uint32_t>(b, 0); put<std::uint32_t>(b, 0);
  zeros(b, 16);
  return b;
}
inline Bytes entry(std::uint64_t name_off, std::uint64_t ohdr, std::uint64_t btree, std::uint64_t heap) {
  Bytes b;
  put(b, name_off); put(b, ohdr);
  put<std::uint32_t>(b, 1); put<std::uint32_t>(b, 0);
  put(b, btree); put(b, heap);
  return b;
}

inline Bytes snod(const std::vector<Bytes>& entries) {
  Bytes b = {'S', 'N', 'O', 'D', 1, 0};
  put<std::uint16_t>(b, static_cast<std::uint16_t>(entries.size()));
  for (const auto& e : entries) b.insert(b.end(), e.begin(), e.end());
  zeros(b, kSnodSize - b.size());
  return b;
}

inline Bytes btree(const std::vector<std::uint64_t>& keys, const std::vector<std::uint64_t>& children,
                   unsigned level = 0, std::uint64_t left = kUndef, std::uint64_t right = kUndef) {
  Bytes b = {'T', 'R', 'E', 'E', 0, static_cast<unsigned char>(level)};
  put<std::uint16_t>(b, static_cast<std::uint16_t>(children.size()));
  put(b, left); put(b, right);
  for (std::size_t k = 0; k < children.size(); ++k) { put(b, keys[k]); put(b, children[k]); }
  put(b, keys[children.size()]);
  zeros(b, kBtreeSize - b.size());
  return b;
}

inline Bytes heap_header(std::uint64_t data_size, std::uint64_t free_off, std::uint64_t data_addr) {
  Bytes b = {'H', 'E', 'A', 'P', 0, 0, 0, 0};
  put(b, data_size); put(b, free_off); put(b, data_addr);
  return b;
}

// local heap data segment: NUL-terminated names padded to 8 bytes
struct Heap {
  std::size_t size;
  Bytes data = Bytes(8, 0);  // offset 0: the empty name
  explicit Heap(std::size_t s) : size(s) {}
  bool fits(const std::string& name) const { return data.size() + pad8(name.size() + 1) + 16 <= size; }
  std::uint64_t add(const std::string& name) {
    const std::uint64_t off = data.size();
    data.insert(data.end(), name.begin(), name.end());
    data.push_back(0);
    zeros(data, pad8(name.size() + 1) - (name.size() + 1));
    if (data.size() + 16 > size) throw std::runtime_error("group name heap full");
    return off;
  }
  // the segment from `start` and the free-list head; full = false stops after the free block's header
  // (what changes when a name is added to a segment whose rest is zero)
  std::pair<Bytes, std::uint64_t> segment(std::size_t start = 0, bool full = true) const {
    Bytes out(data.begin() + static_cast<std::ptrdiff_t>(start), data.end());
    const std::size_t free = size - data.size();
    if (free >= 16) {
      put<std::uint64_t>(out, 1);  // one free block, the last in the list
      put<std::uint64_t>(out, free);
      if (full) zeros(out, free - 16);
      return {out, data.size()};
    }
    zeros(out, free);
    return {out, kUndef};
  }
};

struct Dataset {
  std::string name;
  const void* data;
  std::uint64_t rows, cols;
  Kind kind;
};

// An append-only HDF5 file of groups of 2-D datasets.
class File {
 public:
  explicit File(const std::string& path) : path_(path), heap_(kRootHeapData) {
    f_ = std::fopen(path.c_str(), "wb+");
    if (!f_) throw std::runtime_error("cannot create " + path);
    root_ohdr_ = 96;
    root_btree_ = root_ohdr_ + 40;
    root_heap_ = root_btree_ + kBtreeSize;
    root_heap_data_ = root_heap_ + 32;
    eof_ = root_heap_data_ + kRootHeapData;
    write_root();
  }
  File(const File&) = delete;
  File& operator=(const File&) = delete;
  ~File() {
    if (!f_) return;
    write_at(0, superblock());
    std::fclose(f_);
    std::error_code ec;  // the file ends at the last allocation
    std::filesystem::resize_file(path_, eof_, ec);
  }

  void write_group(const std::string& group, const std::vector<Dataset>& datasets) {
    if (groups_.count(group)) throw std::runtime_error("group " + group + " exists");
    if (datasets.size() > kSnodEntries) throw std::runtime_error("at most 8 datasets per group");
    std::vector<Dataset> ds = datasets;
    std::sort(ds.begin(), ds.end(), [](const Dataset& a, const Dataset& b) { return a.name < b.name; });
    std::size_t heap_bytes = 8 + 16;
    for (const auto& d : ds) heap_bytes += pad8(d.name.size() + 1);
    Heap gheap(pad8(heap_bytes));
    std::map<std::string, std::uint64_t> name_off;
    for (const auto& d : datasets) name_off[d.name] = gheap.add(d.name);  // heap order = call order
    std::vector<Bytes> entries;
    for (const auto& d : ds) {
      const std::uint64_t bytes = d.rows * d.cols * 4;
      const std::uint64_t data_addr = alloc(std::max<std::uint64_t>(bytes, 1));
      write_raw(data_addr, d.data, bytes);
      const Bytes oh = object_header({dataspace(d.rows, d.cols), datatype(d.kind), fill_value(),
                                      layout_contiguous(bytes ? data_addr : kUndef, bytes)},
                                     216);
      const std::uint64_t oaddr = alloc(oh.size());
      write_at(oaddr, oh);
      entries.push_back(entry(name_off[d.name], oaddr));
    }
    const std::uint64_t sn = alloc(kSnodSize);
    write_at(sn, snod(entries));
    const std::uint64_t bt = alloc(kBtreeSize);
    write_at(bt, btree({0, ds.empty() ? 0 : name_off[ds.back().name]}, {sn}));
    const auto [seg, free] = gheap.segment();
    const std::uint64_t heap = alloc(32);
    const std::uint64_t heap_data = alloc(seg.size());
    write_at(heap, heap_header(seg.size(), free, heap_data));
    write_at(heap_data, seg);
    const Bytes goh = object_header({symbol_table_msg(bt, heap)}, 24);
    const std::uint64_t gaddr = alloc(goh.size());
    write_at(gaddr, goh);
    const bool moved = !heap_.fits(group);
    if (moved) {  // a name segment twice the size at the end of the file
      while (!heap_.fits(group)) heap_.size *= 2;
      root_heap_data_ = alloc(heap_.size);
    }
    const std::uint64_t group_name = heap_.add(group);
    groups_[group] = {group_name, gaddr, bt, heap};
    const auto at = std::lower_bound(order_.begin(), order_.end(), group);
    const std::size_t first = static_cast<std::size_t>(at - order_.begin());
    order_.insert(at, group);
    write_root(first, moved ? 0 : group_name);
    std::fflush(f_);
  }

 private:
  struct Group {
    std::uint64_t name_off, ohdr, btree, heap;
  };

  void write_at(std::uint64_t addr, const Bytes& b) { write_raw(addr, b.data(), b.size()); }
  void write_raw(std::uint64_t addr, const void* p, std::uint64_t n) {
    if (!n) return;
    if (std::fseek(f_, static_cast<long>(addr), SEEK_SET) != 0 || std::fwrite(p, 1, n, f_) != n)
      throw std::runtime_error("HDF5 write failed");
  }
  std::uint64_t alloc(std::uint64_t size) {
    const std::uint64_t a = eof_;
    eof_ = pad8(eof_ + size);
    return a;
  }

  Bytes superblock() const {
    Bytes b = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n', 0, 0, 0, 0, 0, 8, 8, 0};
    put<std::uint16_t>(b, kLeafK);
    put<std::uint16_t>(b, kInternalK);
    put<std::uint32_t>(b, 0);
    put<std::uint64_t>(b, 0); put(b, kUndef); put(b, eof_); put(b, kUndef);
    const Bytes e = entry(0, root_ohdr_, root_btree_, root_heap_);
    b.insert(b.end(), e.begin(), e.end());
    return b;
  }

  // The root group's metadata: its entries in name order in symbol table nodes of 8 (those before the
  // node holding entry `first` are unchanged and not rewritten), a B-tree of 32 children per node that
  // gains levels as the nodes grow (the root node stays at its fixed address), the name heap (from offset
  // `heap_from`; 0: all of it).
  void write_root(std::size_t first = 0, std::uint64_t heap_from = 0) {
    const std::size_t n = order_.size();
    const std::size_t nchunks = std::max<std::size_t>(1, (n + kSnodEntries - 1) / kSnodEntries);
    while (snods_.size() < nchunks) snods_.push_back(alloc(kSnodSize));
    for (std::size_t k = first / kSnodEntries; k < nchunks; ++k) {
      std::vector<Bytes> chunk;
      for (std::size_t i = k * kSnodEntries; i < std::min(n, (k + 1) * kSnodEntries); ++i) {
        const Group& g = groups_.at(order_[i]);
        chunk.push_back(entry(g.name_off, g.ohdr, g.btree, g.heap));
      }
      write_at(snods_[k], snod(chunk));
    }
    // each child's largest name (heap offset); a node's keys: the bound left of its first child, then these
    std::vector<std::uint64_t> children(snods_.begin(), snods_.begin() + nchunks), maxkey;
    for (std::size_t k = 0; k < nchunks; ++k)
      maxkey.push_back(n ? groups_.at(order_[std::min(n, (k + 1) * kSnodEntries) - 1]).name_off : 0);
    unsigned level = 0;
    constexpr std::size_t width = 2 * kInternalK;
    while (children.size() > width) {
      const std::size_t count = (children.size() + width - 1) / width;
      if (nodes_.size() <= level) nodes_.emplace_back();
      auto& addrs = nodes_[level];
      while (addrs.size() < count) addrs.push_back(alloc(kBtreeSize));
      std::vector<std::uint64_t> up;
      for (std::size_t j = 0; j < count; ++j) {
        const std::size_t lo = j * width, hi = std::min(children.size(), lo + width);
        std::vector<std::uint64_t> keys = {j ? maxkey[lo - 1] : 0};
        keys.insert(keys.end(), maxkey.begin() + lo, maxkey.begin() + hi);
        write_at(addrs[j], btree(keys, std::vector<std::uint64_t>(children.begin() + lo, children.begin() + hi), level,
                                 j ? addrs[j - 1] : kUndef, j + 1 < count ? addrs[j + 1] : kUndef));
        up.push_back(maxkey[hi - 1]);
      }
      children.assign(addrs.begin(), addrs.begin() + count);
      maxkey = up;
      ++level;
    }
    std::vector<std::uint64_t> keys = {0};
    keys.insert(keys.end(), maxkey.begin(), maxkey.end());
    write_at(root_btree_, btree(keys, children, level));
    const auto [seg, free] = heap_.segment(heap_from, heap_from == 0);
    write_at(root_heap_, heap_header(heap_.size, free, root_heap_data_));
    write_at(root_heap_data_ + heap_from, seg);
    write_at(root_ohdr_, object_header({symbol_table_msg(root_btree_, root_heap_)}));
    write_at(0, superblock());
  }

  std::FILE* f_ = nullptr;
  std::filesystem::path path_;
  Heap heap_;
  std::map<std::string, Group> groups_;
  std::vector<std::string> order_;  // group names in name order
  std::vector<std::uint64_t> snods_;
  std::vector<std::vector<std::uint64_t>> nodes_;  // B-tree nodes below the root, per level (leaf level first)
  std::uint64_t root_ohdr_ = 0, root_btree_ = 0, root_heap_ = 0, root_heap_data_ = 0, eof_ = 0;
};

template <typename T>
struct ViewShape;
template <typename S, int D>
struct ViewShape<VectorN<S, D>> {
  static_assert(std::is_same_v<S, float> || std::is_same_v<S, unsigned> || std::is_same_v<S, int>,
                "float32, uint32 or int32 views");
  static constexpr std::uint64_t cols = D;
  static constexpr Kind kind = std::is_same_v<S, float> ? Kind::f32 : std::is_same_v<S, int> ? Kind::i32 : Kind::u32;
};
template <typename S>
struct ViewShape<Polarity_<S>> {
  static constexpr std::uint64_t cols = 2;
  static constexpr Kind kind = Kind::f32;
};
template <>
struct ViewShape<Link> {
  static constexpr std::uint64_t cols = 2;
  static constexpr Kind kind = Kind::u32;
};
template <>
struct ViewShape<float> {
  static constexpr std::uint64_t cols = 1;
  static constexpr Kind kind = Kind::f32;
};
template <>
struct ViewShape<unsigned> {
  static constexpr std::uint64_t cols = 1;
  static constexpr Kind kind = Kind::u32;
};
template <>
struct ViewShape<int> {
  static constexpr std::uint64_t cols = 1;
  static constexpr Kind kind = Kind::i32;
};

}  // namespace h5detail

template <typename SimulationConfig>
class HDF5_Writer {
 public:
  static constexpr bool writes = true;
  // field names as the reference's (the second keeps its spelling)
  struct Settings {
    bool write_xmf = true;
    std::size_t buffer_treshold = 65536;  // XDMF text kept before writing it out
  };

  HDF5_Writer(const std::string& path, const Settings& settings = {})
      : xmf_threshold_(settings.buffer_treshold), filename_(std::filesystem::path(path).filename().string()) {
    const std::filesystem::path p(path + ".h5");
    if (p.has_parent_path()) std::filesystem::create_directories(p.parent_path());
    file_ = std::make_unique<h5detail::File>(p.string());
    if (settings.write_xmf) {
      xmf_.open(path + ".xmf", std::ios::out | std::ios::trunc);
      xmf_buf_ = "<?xml version=\"1.0\"?>\n<Xdmf Version=\"3.0\">\n\t<Domain>\n"
                 "\t\t<Grid Name=\"Agents\" GridType=\"Collection\" CollectionType=\"Temporal\">\n";
    }
  }
  HDF5_Writer(const HDF5_Writer&) = delete;
  HDF5_Writer& operator=(const HDF5_Writer&) = delete;
  ~HDF5_Writer() {
    if (!xmf_.is_open()) return;
    xmf_buf_ += "\t\t</Grid>\n\t</Domain>\n</Xdmf>\n";
    xmf_.write(xmf_buf_.data(), static_cast<std::streamsize>(xmf_buf_.size()));
    xmf_.close();
  }

  // one group "t<step>" with one dataset per non-empty view (hdf5_writer.hpp:306-321)
  template <typename T0, typename... Ts>
  void write(double time, unsigned step, const View<T0>& first, const View<Ts>&... rest) {
    const std::string group = "t" + std::to_string(step);
    write_group(group, first, rest...);
    if (!xmf_.is_open()) return;
    // with active links the grid's topology is the links' polylines, else the cells as vertices
    bool links = false;
    [[maybe_unused]] auto is_link = [&](const auto& v) {  // unused when only the geometry is written
      using T = typename std::decay_t<decltype(v)>::value_type;
      if constexpr (std::is_same_v<T, Link>) links = links || v.get_active_count() != 0;
    };
    (is_link(rest), ...);
    xmf_grid_open(time, group, first, links);
    (xmf_item(xmf_buf_, group, rest), ...);
    xmf_buf_ += xmf_static_;
    xmf_buf_ += "\t\t\t</Grid>\n";
    if (xmf_buf_.size() > xmf_threshold_) {
      xmf_.write(xmf_buf_.data(), static_cast<std::streamsize>(xmf_buf_.size()));
      xmf_buf_.clear();
    }
  }

  // the "static" group, once (hdf5_writer.hpp:335-347); in every later XDMF grid
  template <typename... Ts>
  void write_static(const View<Ts>&... views) {
    if (static_written_) throw std::runtime_error("Static data has already been written. You can only write to static data once.");
    static_written_ = true;
    write_group("static", views...);
    if (xmf_.is_open()) (xmf_item(xmf_static_, "static", views), ...);
  }

 private:
  template <typename T>
  static std::string active_rows(const View<T>& v) {
    return std::to_string(v.get_active_count());
  }

  template <typename T>
  void xmf_grid_open(double time, const std::string& group, const View<T>& geometry, bool links) {
    constexpr int D = SimulationConfig::dimensions;
    std::string& b = xmf_buf_;
    b += "\t\t\t<Grid Name=\"" + group + "\" GridType=\"Uniform\">\n\t\t\t\t<Time Value=\"";
    b += std::to_string(time);
    if (!links) b += "\"/>\n\t\t\t\t<Topology TopologyType=\"Polyvertex\" NumberOfElements=\"" + active_rows(geometry);
    b += "\"/>\n\t\t\t\t<Geometry GeometryType=\"";
    b += D == 1 ? "X" : (D == 2 ? "XY" : "XYZ");
    b += "\">\n\t\t\t\t\t<DataItem Format=\"HDF\" Dimensions=\"" + active_rows(geometry) + " " + std::to_string(D);
    b += "\">\n\t\t\t\t\t\t" + filename_ + ".h5:" + group + "/" + geometry.label();
    b += "\n\t\t\t\t\t</DataItem>\n\t\t\t\t</Geometry>\n";
  }

  // a node attribute, or the links' polyline topology (hdf5_writer.hpp:210-262)
  template <typename T>
  void xmf_item(std::string& b, const std::string& group, const View<T>& v) const {
    if (v.extent(0) == 0) return;
    std::string dims = active_rows(v) + " ";
    int cols = 0;
    if constexpr (requires { T::dimensions; }) cols = int(T::dimensions);
    else if constexpr (requires { T::components; }) cols = int(T::components);
    if (cols) dims += std::to_string(cols) + " ";
    const char* type = !cols ? "Scalar" : (cols == 2 || cols == 3) ? "Vector" : cols == 9 ? "Tensor" : "Matrix";
    if constexpr (std::is_same_v<T, Link>) {
      b += "\t\t\t\t<Topology TopologyType=\"Polyline\" NumberOfElements=\"" + active_rows(v) + "\">\n";
      b += "\t\t\t\t\t<DataItem Format=\"HDF\" DataType=\"UInt32\"";
    } else {
      b += "\t\t\t\t<Attribute Name=\"" + v.label() + "\" AttributeType=\"" + type + "\" Center=\"Node\">\n";
      b += "\t\t\t\t\t<DataItem Format=\"HDF\"";
    }
    b += " Dimensions=\"" + dims + "\">\n\t\t\t\t\t\t" + filename_ + ".h5:" + group + "/" + v.label();
    b += "\n\t\t\t\t\t</DataItem>\n";
    b += std::is_same_v<T, Link> ? "\t\t\t\t</Topology>\n" : "\t\t\t\t</Attribute>\n";
  }

  template <typename... Ts>
  void write_group(const std::string& group, const View<Ts>&... views) {
    std::vector<h5detail::Dataset> ds;
    auto one = [&](const auto& v) {
      using T = typename std::decay_t<decltype(v)>::value_type;
      if (v.get_active_count() == 0) return;
      // the host copy, with what device code wrote (hdf5_writer.hpp:120-129)
      std::decay_t<decltype(v)> h = v;
      h.sync_host();
      ds.push_back({v.label(), static_cast<const void*>(v.data()), v.get_active_count(), h5detail::ViewShape<T>::cols,
                    h5detail::ViewShape<T>::kind});
    };
    (one(views), ...);
    file_->write_group(group, ds);
  }

  std::size_t xmf_threshold_;
  std::string filename_;
  std::unique_ptr<h5detail::File> file_;
  std::ofstream xmf_;
  std::string xmf_buf_, xmf_static_;
  bool static_written_ = false;
};

}  // namespace io
}  // namespace tecs

#endif  // TECS_CXX_HDF5_WRITER_HPP
