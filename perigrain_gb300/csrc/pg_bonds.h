// Internal interface of the GPU bond-list builder (pg_bonds.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

namespace pg {

// Device scratch of one bond build. `cells` is the capacity of the cell arrays.
struct BondScratch {
  unsigned long long* box;  // [6] ordered-key bounding box
  uint32_t* cell_count;     // [cells]
  uint32_t* cell_start;     // [cells + 1]
  uint32_t* key;            // [n]
  uint32_t* rank;           // [n]
  uint32_t* sorted;         // [n]
  uint32_t* pcount;         // [n]
  uint32_t* poff;           // [n + 1]
  uint32_t* tile_sum;       // [bond_scan_tiles(max(cells, n))]
  uint32_t* done;           // [1]
  int32_t* error;           // [1]
  uint32_t cells;
};

// Entries per tile of the bond builder's exclusive scan (1024 threads x 4 entries).
constexpr uint32_t BOND_SCAN_TILE = 4096;
// Grid cells of a bond build over n nodes, and scan tiles of a scan over len entries (both also
// usable where a scratch size must be known at compile time).
constexpr uint32_t bond_grid_cells_c(uint32_t n) { return 4u * n + 64u; }
constexpr uint32_t bond_scan_tiles_c(uint32_t len) { return ((len ? len : 1u) + BOND_SCAN_TILE - 1u) / BOND_SCAN_TILE; }

uint32_t bond_grid_cells(uint32_t n);
// Exclusive scan of in[0..len) into out[0..len], out[len] = total, on stream st. tile_sum holds
// bond_scan_tiles(len) words; *done must be 0 (and is 0 again when the scan ends).
cudaError_t scan_u32_dev(const uint32_t* in, uint32_t len, uint32_t* out, uint32_t* tile_sum, uint32_t* done,
                         cudaStream_t st);
uint32_t bond_scan_tiles(uint32_t len);
int run_bond_build(const double* pos, uint32_t n, uint32_t dim, double delta, uint32_t* pairs, uint64_t capacity,
                   uint64_t* n_pairs, cudaStream_t st, const BondScratch& S, std::string* err);

}  // namespace pg
