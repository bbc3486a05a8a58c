// Row access shared by the force kernels.  CSR rows are contiguous.  2D
// rows are column-major in groups of four entries: entries 4q..4q+3 of row
// i form one int4 at int4 index q*stride + i, so a warp of consecutive rows
// loads four entries per lane in one coalesced 512-byte access (the
// column-major LayoutLeft of the reference's Neighbor2D view on a GPU, with
// 16-byte granules).
#pragma once

namespace emd {

__host__ __device__ __forceinline__ size_t quad_index(int i, int k, int stride) {
  return (((size_t)(k >> 2) * stride + i) << 2) + (k & 3);
}

struct ListView {
  const int* entries;
  const int* offsets;     // CSR row starts (N+1)
  const int* num_neighs;  // row lengths
  int stride;             // 2D leading dimension; 0 for CSR
};

template <bool TWO_D>
struct Row {
  const int* p;
  int n;
  int stride;
  __device__ __forceinline__ Row(const ListView& L, int i) {
    n = L.num_neighs[i];
    if (TWO_D) {
      p = L.entries + 4 * (size_t)i;
      stride = L.stride;
    } else {
      p = L.entries + L.offsets[i];
      stride = 1;
    }
  }
  __device__ __forceinline__ int operator[](int k) const {
    return TWO_D ? __ldg(p + (((size_t)(k >> 2) * stride) << 2) + (k & 3)) : __ldg(p + k);
  }
};

}  // namespace emd
