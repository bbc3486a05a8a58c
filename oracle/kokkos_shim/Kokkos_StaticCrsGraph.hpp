// Serial Kokkos-subset shim (test infrastructure only): the StaticCrsGraph
// container that ExaMiniMD's NeighListCSR derives from
// (src/neighbor_types/neighbor_csr.h:82-120): entries + row_map views.
#ifndef EMD_KOKKOS_SHIM_CRS_HPP
#define EMD_KOKKOS_SHIM_CRS_HPP
#include "Kokkos_Core.hpp"

namespace Kokkos {
template <class DataType, class Arg1Type, class Arg2Type = void, class Arg3Type = void, typename SizeType = size_t>
class StaticCrsGraph {
 public:
  using entries_type = View<DataType*, Arg1Type>;
  using row_map_type = View<const SizeType*, Arg1Type>;
  entries_type entries;
  row_map_type row_map;
  StaticCrsGraph() {}
  StaticCrsGraph(const StaticCrsGraph&) = default;
  StaticCrsGraph& operator=(const StaticCrsGraph&) = default;
  template <class EntriesType, class RowMapType>
  StaticCrsGraph(const EntriesType& e, const RowMapType& r) : entries(e), row_map(r) {}
  SizeType numRows() const { return row_map.extent(0) ? SizeType(row_map.extent(0) - 1) : 0; }
};
}  // namespace Kokkos
#endif
