// Serial Kokkos-subset shim (test infrastructure only): BinOp3D and BinSort
// as called by ExaMiniMD src/binning_types/binning_kksort.{h,cpp}.
//
// BinOp3D::bin: per-dimension truncation int((x_d - min_d) * nbin_d/(max_d - min_d)),
// flattened with x slowest and z fastest (the decode in
// binning_kksort.cpp:61-63 assumes this order).
// BinSort::create_permute_vector: count, exclusive scan, then fill each bin
// in ascending source index (serial atomics resolve in loop order).
#ifndef EMD_KOKKOS_SHIM_SORT_HPP
#define EMD_KOKKOS_SHIM_SORT_HPP
#include "Kokkos_Core.hpp"

namespace Kokkos {

template <class KeyViewType>
struct BinOp3D {
  int max_bins_[3] = {0, 0, 0};
  double mul_[3] = {0, 0, 0};
  double min_[3] = {0, 0, 0};
  BinOp3D() {}
  template <class I, class F>
  BinOp3D(I max_bins[], F min[], F max[]) {
    for (int d = 0; d < 3; ++d) {
      max_bins_[d] = int(max_bins[d]);
      mul_[d] = double(max_bins[d]) / (double(max[d]) - double(min[d]));
      min_[d] = double(min[d]);
    }
  }
  template <class V>
  int bin(const V& keys, const int& i) const {
    const int ix = int((double(keys(i, 0)) - min_[0]) * mul_[0]);
    const int iy = int((double(keys(i, 1)) - min_[1]) * mul_[1]);
    const int iz = int((double(keys(i, 2)) - min_[2]) * mul_[2]);
    return ix * max_bins_[1] * max_bins_[2] + iy * max_bins_[2] + iz;
  }
  int max_bins() const { return max_bins_[0] * max_bins_[1] * max_bins_[2]; }
};

template <class KeyViewType, class BinSortOp, class ExecutionSpace = DefaultExecutionSpace, class SizeType = int>
class BinSort {
 public:
  using bin_count_type = View<const int*>;
  using offset_type = View<const SizeType*>;
  using permute_type = View<SizeType*>;

 private:
  KeyViewType keys_;
  BinSortOp op_;
  View<int*> bin_count_;
  View<SizeType*> bin_offsets_;
  View<SizeType*> sort_order_;

 public:
  BinSort() {}
  BinSort(const KeyViewType& keys, BinSortOp op, bool = false) : keys_(keys), op_(op) {}

  void create_permute_vector() {
    const int nbins = op_.max_bins();
    const long n = long(keys_.extent(0));
    bin_count_ = View<int*>("Kokkos::SortImpl::BinSortFunctor::bin_count", nbins);
    bin_offsets_ = View<SizeType*>("Kokkos::SortImpl::BinSortFunctor::bin_offsets", nbins);
    sort_order_ = View<SizeType*>("Kokkos::SortImpl::BinSortFunctor::sort_order", n);
    for (long i = 0; i < n; ++i) bin_count_(op_.bin(keys_, int(i)))++;
    SizeType off = 0;
    for (int b = 0; b < nbins; ++b) {
      bin_offsets_(b) = off;
      off += bin_count_(b);
    }
    std::vector<int> fill(size_t(nbins), 0);
    for (long i = 0; i < n; ++i) {
      const int b = op_.bin(keys_, int(i));
      sort_order_(bin_offsets_(b) + fill[size_t(b)]++) = SizeType(i);
    }
  }

  // values(i, ...) <- values(sort_order(i), ...) for i < n
  template <class V>
  void sort(const V& values) const {
    const size_t n = sort_order_.extent(0);
    const size_t inner = V::Rank > 1 ? values.extent(1) : 1;
    using T = typename V::non_const_value_type;
    std::vector<T> tmp(n * inner);
    for (size_t i = 0; i < n; ++i)
      for (size_t c = 0; c < inner; ++c) tmp[i * inner + c] = get(values, size_t(sort_order_(i)), c);
    for (size_t i = 0; i < n; ++i)
      for (size_t c = 0; c < inner; ++c) get(values, i, c) = tmp[i * inner + c];
  }

  permute_type get_permute_vector() const { return sort_order_; }
  bin_count_type get_bin_count() const { return bin_count_; }
  offset_type get_bin_offsets() const { return bin_offsets_; }

 private:
  template <class V>
  static typename V::value_type& get(const V& v, size_t i, size_t c) {
    return const_cast<typename V::value_type&>(v.ptr_[i * v.str_[0] + (V::Rank > 1 ? c * v.str_[1] : 0)]);
  }
};

}  // namespace Kokkos
#endif
