// Kokkos_Sort.hpp -- BinOp1D / BinSort for the oracle's Kokkos shim.
// Semantics follow Kokkos's documentation: keys are binned by
// int((key - min) * max_bins / (max - min)) (an integer key range not wider
// than the bin count maps one key per bin); bin_offsets is the exclusive scan
// of the bin counts; the permutation lists each bin's members in the order the
// binning loop meets them, which for a serial loop is ascending index.
#pragma once
#include <vector>

#include "Kokkos_Core.hpp"

namespace Kokkos {
template <class KeyView>
struct BinOp1D {
  int max_bins_ = 0;
  double mul_ = 0.0;
  double min_ = 0.0;
  BinOp1D() = default;
  BinOp1D(int max_bins, typename KeyView::const_value_type min, typename KeyView::const_value_type max)
      : max_bins_(max_bins + 1),
        mul_((double)max_bins / ((double)max - (double)min)),
        min_((double)min) {
    if (std::is_integral_v<typename KeyView::non_const_value_type> && ((double)max - (double)min) <= (double)max_bins)
      mul_ = 1.0;
  }
  template <class V>
  int bin(const V& keys, int i) const {
    return (int)(mul_ * ((double)keys(i) - min_));
  }
  int max_bins() const { return max_bins_; }
};

template <class KeyView, class BinOp>
class BinSort {
 public:
  using offset_type = View<unsigned*>;
  BinSort() = default;
  BinSort(const KeyView& keys, int begin, int end, BinOp op, bool = false)
      : keys_(keys), begin_(begin), end_(end), op_(op) {}
  template <class Exec>
  BinSort(const Exec&, const KeyView& keys, int begin, int end, BinOp op, bool = false)
      : BinSort(keys, begin, end, op) {}

  void create_permute_vector() {
    const int nb = op_.max_bins();
    offsets_ = offset_type("Kokkos::SortImpl::BinSortFunctor::bin_offsets", nb > 0 ? nb : 0);
    perm_ = offset_type("PermuteVector", end_ - begin_ > 0 ? end_ - begin_ : 0);
    std::vector<unsigned> count(nb > 0 ? nb : 0, 0u);
    for (int i = begin_; i < end_; ++i) count[op_.bin(keys_, i)]++;
    unsigned acc = 0;
    for (int b = 0; b < nb; ++b) {
      offsets_(b) = acc;
      acc += count[b];
      count[b] = 0;
    }
    for (int i = begin_; i < end_; ++i) {
      const int b = op_.bin(keys_, i);
      perm_(offsets_(b) + count[b]++) = (unsigned)i;
    }
  }
  template <class Exec>
  void create_permute_vector(const Exec&) {
    create_permute_vector();
  }
  offset_type get_permute_vector() const { return perm_; }
  offset_type get_bin_offsets() const { return offsets_; }

 private:
  KeyView keys_;
  int begin_ = 0, end_ = 0;
  BinOp op_;
  offset_type offsets_, perm_;
};
}  // namespace Kokkos
