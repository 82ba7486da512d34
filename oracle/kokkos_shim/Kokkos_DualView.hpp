// Kokkos_DualView.hpp -- host-only DualView for the oracle's Kokkos shim: the
// host and device views are the same allocation, so every sync is a no-op.
#pragma once
#include "Kokkos_Core.hpp"

namespace Kokkos {
template <class DataType, class... Props>
class DualView {
 public:
  using t_dev = View<DataType, Props...>;
  using t_host = t_dev;
  using t_dev_const = t_dev;
  using t_host_const = t_dev;
  using value_type = typename t_dev::value_type;
  using non_const_value_type = typename t_dev::non_const_value_type;
  using memory_space = HostSpace;
  using execution_space = Serial;
  using host_mirror_space = HostSpace;

  t_dev d_view;
  t_host h_view;

  DualView() = default;
  DualView(const std::string& label, std::size_t n0) : d_view(label, n0), h_view(d_view) {}

  const t_dev& view_device() const { return d_view; }
  const t_host& view_host() const { return h_view; }
  template <class Space>
  const t_dev& view() const { return d_view; }

  std::size_t extent(int d) const { return d_view.extent(d); }
  std::size_t size() const { return d_view.size(); }

  void modify_device() { dev_mod_ = true; }
  void modify_host() { host_mod_ = true; }
  void clear_sync_state() { dev_mod_ = host_mod_ = false; }
  bool need_sync_host() const { return dev_mod_; }
  bool need_sync_device() const { return host_mod_; }
  void sync_host() { dev_mod_ = false; }
  void sync_device() { host_mod_ = false; }
  template <class Space>
  void sync() { clear_sync_state(); }
  template <class Space>
  void modify() {}

  void resize(std::size_t n) {
    Kokkos::resize(d_view, n);
    h_view = d_view;
  }
  void realloc(std::size_t n) {
    Kokkos::realloc(d_view, n);
    h_view = d_view;
  }

 private:
  bool dev_mod_ = false, host_mod_ = false;
};

template <class D1, class... P1, class D2, class... P2>
void deep_copy(DualView<D1, P1...>& dst, const DualView<D2, P2...>& src) {
  deep_copy(dst.d_view, src.d_view);
}
}  // namespace Kokkos
