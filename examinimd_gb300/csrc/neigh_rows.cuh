// Row access shared by the force kernels: CSR rows are contiguous, 2D rows
// are column-major with leading dimension `stride` (LayoutLeft, as the
// reference's Neighbor2D view on a GPU).
#pragma once

namespace emd {

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
      p = L.entries + i;
      stride = L.stride;
    } else {
      p = L.entries + L.offsets[i];
      stride = 1;
    }
  }
  __device__ __forceinline__ int operator[](int k) const { return __ldg(p + (size_t)k * stride); }
};

}  // namespace emd
