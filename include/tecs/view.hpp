// tecs/view.hpp -- View<T> and DeviceVar<T> of the C++20 drop-in layer.
//
// The reference's tecs::View (include/types/view.hpp:47-266) is a
// Kokkos::DualView with an active count and a flag that device code sets
// when it writes; DeviceVar (include/types/device_var.hpp:38-134) is one
// device value.  Here both are handles to a host array and a device array on
// the GPU (allocated through the C ABI, so a program built by g++ holds
// them too).  Indexing a View reads the host array on the host and the device
// array in device code, and marks the side it was reached from as modified,
// as the reference's operator() does; sync_host, sync_device and auto_sync
// move the data the way the reference's do.  Copies are shallow (a device
// lambda captures a handle, not the data).
//
// A DeviceVar's value is read and written from both sides: device code
// reaches the device copy, host code the host copy.  The Simulation marks
// every DeviceVar as possibly changed on the device whenever it has run user
// code there, so a host read fetches the device value first; a host write
// through data() makes the host copy the newer one, and the Simulation sends
// such values to the device before it next runs user code there.
#ifndef TECS_CXX_VIEW_HPP
#define TECS_CXX_VIEW_HPP

#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include "../tecs_gpu.h"
#include "vector.hpp"

namespace tecs {

namespace detail {

// device memory through the C ABI; null when no device is present (a
// host-only handle, enough for programs that never reach the device)
inline void* device_alloc(std::size_t bytes) {
  void* p = nullptr;
  if (tecs_device_alloc(0, bytes ? bytes : 16, &p) != 0) return nullptr;
  return p;
}
inline void device_copy(void* dst, const void* src, std::size_t bytes) {
  if (bytes && tecs_device_copy(dst, src, bytes) != 0) throw std::runtime_error(tecs_last_error());
}

// Count of the times user code ran on the device (DeviceVar values may have
// changed there since a host copy was taken), and the values whose host copy
// is newer.
struct DeviceVarState {
  virtual ~DeviceVarState() = default;
  virtual void push() = 0;  // host copy -> device when the host copy is newer
  std::uint64_t epoch = 0;  // device_epoch() when the host copy was last made current
  bool host_newer = false;
};
inline std::uint64_t& device_epoch_ref() {
  static std::uint64_t e = 1;
  return e;
}
inline std::uint64_t device_epoch() { return device_epoch_ref(); }
inline std::mutex& registry_mutex() {
  static std::mutex m;
  return m;
}
inline std::set<DeviceVarState*>& registry() {
  static std::set<DeviceVarState*> r;
  return r;
}
// before user code runs on the device: every value written on the host is sent
inline void push_device_vars() {
  std::lock_guard<std::mutex> lock(registry_mutex());
  for (DeviceVarState* s : registry())
    if (s->host_newer) s->push();
}
// after user code ran on the device: host copies may be stale
inline void device_ran_user_code() { ++device_epoch_ref(); }

template <typename T>
struct ViewStorage {
  std::string label;
  std::vector<T> host;
  T* device = nullptr;
  unsigned* device_modified = nullptr;  // device flag set by device-side indexing
  bool host_modified = false;
  // a source that may hold newer data than either array (a simulation's
  // state): when stale is set, refresh brings the arrays up to date before
  // the view is read on the host or synchronised
  bool stale = false;
  std::function<void()> refresh;
  ~ViewStorage() {
    if (device) tecs_device_free(device);
    if (device_modified) tecs_device_free(device_modified);
  }
};
}  // namespace detail

template <typename T>
class View {
 public:
  using value_type = T;
  using non_const_value_type = std::remove_const_t<T>;

  View() : View(std::string("tecs::View default"), 0u) {}
  View(const std::string& label, unsigned active_count_) : View(label, active_count_, active_count_) {}
  View(const std::string& label, unsigned active_count_, unsigned capacity) : active_count(active_count_) {
    st_ = std::make_shared<detail::ViewStorage<T>>();
    st_->label = label;
    st_->host.assign(capacity, T{});
    st_->device = static_cast<T*>(detail::device_alloc(std::size_t(capacity) * sizeof(T)));
    st_->device_modified = static_cast<unsigned*>(detail::device_alloc(sizeof(unsigned)));
    if (st_->device && capacity) {
      // the device array starts as the host one (value-initialised)
      detail::device_copy(st_->device, st_->host.data(), std::size_t(capacity) * sizeof(T));
    }
    if (st_->device_modified) {
      const unsigned zero = 0u;
      detail::device_copy(st_->device_modified, &zero, sizeof zero);
    }
    bind();
  }

  // element i: the host array on the host, the device array in device code,
  // each marking its side as modified (view.hpp:112-129)
  TECS_HD T& operator()(int i) const {
#if defined(__CUDA_ARCH__)
    *dmod_ = 1u;
    return d_[i];
#else
    if (*stale_) refresh();
    *hmod_ = true;
    return h_[i];
#endif
  }
  TECS_HD T& access(int i) const {
#if defined(__CUDA_ARCH__)
    return d_[i];
#else
    if (*stale_) refresh();
    return h_[i];
#endif
  }
  TECS_HD T& read(int i) const { return access(i); }
  TECS_HD T& write(int i) const { return (*this)(i); }

  TECS_HD unsigned get_capacity() const { return cap_; }
  TECS_HD std::size_t extent(int) const { return cap_; }
  TECS_HD int rank() const { return 1; }
  unsigned get_active_count() const { return active_count; }
  void set_active_count(unsigned value) { active_count = value; }
  std::string label() const { return st_->label; }
  T* data() const {
    if (*stale_) refresh();
    return h_;
  }
  T* device_data() const { return d_; }

  // device -> host when device code wrote the view (view.hpp:139-148)
  void sync_host() {
    if (st_->stale) refresh();
    if (device_flag()) {
      copy_to_host();
      clear_device_flag();
    }
  }
  // host -> device when host code wrote the view
  void sync_device() {
    if (st_->stale) refresh();
    if (st_->host_modified) copy_to_device();
  }
  void unconditional_sync_device() {
    if (st_->stale) refresh();
    copy_to_device();
  }
  void unconditional_sync_host() {
    if (st_->stale) refresh();
    copy_to_host();
    clear_device_flag();
  }
  // whichever side was written is copied to the other (view.hpp:166-176)
  void auto_sync() {
    if (st_->stale) refresh();
    if (device_flag()) {
      copy_to_host();
      clear_device_flag();
    } else if (st_->host_modified) {
      copy_to_device();
    }
  }
  void deep_copy(const T& value) {
    for (auto& v : st_->host) v = value;
    copy_to_device();
    clear_device_flag();
  }
  void deep_copy(const View& src) {
    const std::size_t n = std::min<std::size_t>(cap_, src.cap_);
    for (std::size_t k = 0; k < n; ++k) st_->host[k] = src.st_->host[k];
    copy_to_device();
    clear_device_flag();
  }
  // a new capacity, the first values kept (view.hpp:190-195)
  void resize(unsigned capacity) {
    std::vector<T> h(capacity, T{});
    for (std::size_t k = 0; k < std::min<std::size_t>(capacity, st_->host.size()); ++k) h[k] = st_->host[k];
    st_->host.swap(h);
    if (st_->device) tecs_device_free(st_->device);
    st_->device = static_cast<T*>(detail::device_alloc(std::size_t(capacity) * sizeof(T)));
    bind();
    copy_to_device();
  }

  // for the Simulation: the source this view mirrors, and the flags
  void set_refresh(std::function<void()> f) { st_->refresh = std::move(f); }
  void set_stale(bool v) { st_->stale = v; }
  T* host_array() const { return h_; }
  bool host_modified() const { return st_->host_modified; }
  void set_host_modified(bool v) { st_->host_modified = v; }
  bool device_flag() const {
    if (!st_->device_modified) return false;
    unsigned f = 0u;
    detail::device_copy(&f, st_->device_modified, sizeof f);
    return f != 0u;
  }
  void clear_device_flag() {
    if (!st_->device_modified) return;
    const unsigned zero = 0u;
    detail::device_copy(st_->device_modified, &zero, sizeof zero);
  }
  void copy_to_host() {
    if (st_->device) detail::device_copy(h_, st_->device, std::size_t(cap_) * sizeof(T));
  }
  void copy_to_device() {
    if (st_->device) detail::device_copy(st_->device, h_, std::size_t(cap_) * sizeof(T));
    st_->host_modified = false;
  }

  unsigned active_count = 0;

 private:
  void refresh() const {
    if (st_->refresh) st_->refresh();
    st_->stale = false;
  }
  void bind() {
    h_ = st_->host.data();
    d_ = st_->device;
    hmod_ = &st_->host_modified;
    stale_ = &st_->stale;
    dmod_ = st_->device_modified;
    cap_ = static_cast<unsigned>(st_->host.size());
  }
  std::shared_ptr<detail::ViewStorage<T>> st_;
  T* h_ = nullptr;
  T* d_ = nullptr;
  bool* hmod_ = nullptr;
  bool* stale_ = nullptr;
  unsigned* dmod_ = nullptr;
  unsigned cap_ = 0;
};

template <typename T>
class DeviceVar {
  struct State : detail::DeviceVarState {
    T host{};
    T* device = nullptr;
    void push() override {
      if (device) detail::device_copy(device, &host, sizeof(T));
      host_newer = false;
    }
    void pull() {
      if (device) detail::device_copy(&host, device, sizeof(T));
      epoch = detail::device_epoch();
    }
    ~State() override {
      {
        std::lock_guard<std::mutex> lock(detail::registry_mutex());
        detail::registry().erase(this);
      }
      if (device) tecs_device_free(device);
    }
  };

 public:
  DeviceVar() : DeviceVar(T{}) {}
  explicit DeviceVar(const std::string&) : DeviceVar(T{}) {}
  DeviceVar(const std::string&, const T& value) : DeviceVar(value) {}
  DeviceVar(const T& value) {
    st_ = std::make_shared<State>();
    st_->host = value;
    st_->device = static_cast<T*>(detail::device_alloc(sizeof(T)));
    st_->push();
    st_->epoch = detail::device_epoch();
    {
      std::lock_guard<std::mutex> lock(detail::registry_mutex());
      detail::registry().insert(st_.get());
    }
    d_ = st_->device;
  }

  // the value: the device copy in device code; on the host the newer of the
  // two copies (device_var.hpp:67-84)
  TECS_HD operator T() const {
#if defined(__CUDA_ARCH__)
    return *d_;
#else
    current();
    return st_->host;
#endif
  }
  DeviceVar& operator=(const T& value) {
    st_->host = value;
    st_->push();
    st_->epoch = detail::device_epoch();
    return *this;
  }
  // the device copy in device code; on the host the host copy, which then
  // counts as the newer one (the caller may write through it)
  TECS_HD T* data() const {
#if defined(__CUDA_ARCH__)
    return d_;
#else
    current();
    st_->host_newer = true;
    return &st_->host;
#endif
  }

 private:
  void current() const {
    if (!st_->host_newer && st_->epoch != detail::device_epoch()) st_->pull();
  }
  std::shared_ptr<State> st_;
  T* d_ = nullptr;
};

}  // namespace tecs

#endif  // TECS_CXX_VIEW_HPP
