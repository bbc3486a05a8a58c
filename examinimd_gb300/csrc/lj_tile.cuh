// Tiled neighbour rows of the mixed-precision LJ force.
//
// A tile is a run of whole interior bins along z in one (bx, by) column of
// the binning grid, at most kTileAtoms binned particles (more only when a
// single bin holds more).  Its stage is the union of the 3 x 3 columns
// around it over bins bz0 - 1 .. bz1 + 1: nine segments, each a contiguous
// range of the binning's permutation (bins along z are consecutive bin
// indices).  The force kernel copies a tile's stage into shared memory once
// per step as FP32 positions relative to each particle's bin centre, with the
// x and y bin shift towards the tile's column already added, and its rows
// address neighbours by their byte offset in that array: 16-bit entries,
// eight per 16-byte granule, entry k of row i at uint16 index
// ((k >> 3) * stride + i) * 8 + (k & 7) (column-major like the other rows).
//
// A list is built in this format when every tile's stage fits kTileStageMax
// particles; otherwise the packed 32-bit format (j << 6 | stencil code)
// serves the force instead.
#pragma once
#include <cuda_runtime.h>

namespace emd {

constexpr int kTileAtoms = 256;      // particles binned into a tile's own bins (two per force thread)
constexpr int kTileThreads = 128;    // threads of a force CTA
constexpr int kTileStageMax = 4096;  // staged particles per tile (entries are 16-bit byte offsets)

struct __align__(16) TileDesc {
  int bx, by, bz0, bz1;  // column and z range of the tile's own bins
  int seg[9];            // permutation index where segment r = (dx + 1) * 3 + (dy + 1) starts
  int base[10];          // stage index where segment r starts; base[9] = staged total
  int own0, nown;        // stage index and count of the particles binned into the tile's own bins
  int pad[5];
};
static_assert(sizeof(TileDesc) == 128, "one 128-byte line per tile");

// Everything a kernel needs to turn a tiled entry of row i back into j.
struct TileView {
  const TileDesc* tiles;
  const int* tile_of_bin;  // per bin of the build's grid (-1 outside interior bins)
  const int* abin;         // bin of every particle at the build
  const int* perm;         // the build's permutation (copied: a later binning may overwrite its own)
  const unsigned short* rows;
  int stride;
};

__host__ __device__ __forceinline__ size_t tile_entry_index(int i, int k, int stride) {
  return (((size_t)(k >> 3) * stride + i) << 3) + (k & 7);
}

// stage index -> particle, with the tile's segment table
__device__ __forceinline__ int tile_stage_particle(const TileDesc& t, const int* perm, int s) {
  int r = 0;
#pragma unroll
  for (int q = 1; q < 9; ++q) r += (s >= t.base[q]) ? 1 : 0;
  return perm[t.seg[r] + (s - t.base[r])];
}

// j of entry k of row i (slow path: energy, adjoint, list read-back)
struct TileRow {
  const TileView& V;
  const TileDesc* t;
  int i;
  __device__ __forceinline__ TileRow(const TileView& v, int i_) : V(v), i(i_) {
    t = V.tiles + V.tile_of_bin[V.abin[i]];
  }
  __device__ __forceinline__ int operator[](int k) const {
    const int s = int(V.rows[tile_entry_index(i, k, V.stride)]) >> 4;
    return tile_stage_particle(*t, V.perm, s);
  }
};

}  // namespace emd
