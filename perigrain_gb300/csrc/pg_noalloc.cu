// pg_build_bonds_noalloc: the GPU bond-list builder for callers that cannot allocate device
// memory. Such callers include code running while a CUDA graph is captured on the stream (a
// cudaMalloc there breaks the capture), allocator hooks and memory-pool managers that must not
// re-enter the allocator, and embedders whose device memory is fully reserved up front (for
// example a host application that hands the GPU to this library with a fixed budget). It computes
// exactly what pg_build_bonds computes, with its scratch in one file-scope device array instead
// of cudaMalloc'd memory.
//
// The array holds the scratch of one grain of up to PG_NOALLOC_MAX_NODES nodes (about 1.7 MB);
// every GPU that loads the library keeps it until the process exits. Calls share it: two calls
// that overlap on the GPU (different streams, or different host threads on one device) race and
// must be serialised by the caller. Whatever a call needs zeroed (cell counts, flags, the
// bounding box) is cleared by that call, so each call starts from a clean scratch even though the
// array keeps the previous call's contents.
//
// Its address is looked up once per device with cudaGetSymbolAddress, with that device current,
// on the first call made on the device; make that first call before capturing a stream.
#include <cuda_runtime.h>

#include <string>

#include "../../include/perigrain.h"
#include "pg_bonds.h"

namespace {

constexpr uint32_t kMaxNodes = PG_NOALLOC_MAX_NODES;
constexpr uint32_t kCells = 4u * kMaxNodes + 64u;  // = pg::bond_grid_cells(kMaxNodes)
constexpr uint32_t kTiles = (kCells + 4095u) / 4096u;
constexpr size_t kWords = 12 + (size_t)kCells * 2 + 1 + (size_t)kMaxNodes * 5 + 1 + kTiles + 2;

__device__ __align__(256) uint32_t g_bond_scratch[kWords];

constexpr int kMaxDevices = 64;
uint32_t* g_scratch_addr[kMaxDevices] = {nullptr};
thread_local std::string g_err;

}  // namespace

extern "C" int pg_build_bonds_noalloc(const double* pos, uint32_t n, uint32_t dim, double delta, uint32_t* pairs,
                                      uint64_t capacity, uint64_t* n_pairs, void* stream) {
  if (!n_pairs || (n && !pos) || (dim != 2 && dim != 3) || (capacity && !pairs)) {
    g_err = "bad arguments";
    return PG_EINVAL;
  }
  *n_pairs = 0;
  if (n > kMaxNodes) {
    g_err = "pg_build_bonds_noalloc handles at most " + std::to_string(kMaxNodes) + " nodes per call, got " +
            std::to_string(n) + " (use pg_build_bonds)";
    return PG_EINVAL;
  }
  if (n < 2) return PG_OK;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    g_err = e != cudaSuccess ? cudaGetErrorString(e) : "device index out of range";
    return PG_ECUDA;
  }
  if (!g_scratch_addr[dev]) {
    // host code may not use the symbol itself as an address: ask the runtime for this device's copy
    uint32_t* p = nullptr;
    e = cudaGetSymbolAddress((void**)&p, g_bond_scratch);
    if (e != cudaSuccess || !p) {
      g_err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return PG_ECUDA;
    }
    g_scratch_addr[dev] = p;
  }
  pg::BondScratch S;
  S.cells = pg::bond_grid_cells(n);
  const uint32_t tiles = pg::bond_scan_tiles(S.cells > n ? S.cells : n);
  uint32_t* w = g_scratch_addr[dev];
  S.box = (unsigned long long*)w;  // 256-byte aligned start
  w += 12;
  S.cell_count = w;
  w += S.cells;
  S.cell_start = w;
  w += S.cells + 1;
  S.key = w;
  w += n;
  S.rank = w;
  w += n;
  S.sorted = w;
  w += n;
  S.pcount = w;
  w += n;
  S.poff = w;
  w += n + 1;
  S.tile_sum = w;
  w += tiles;
  S.done = w;
  w += 1;
  S.error = (int32_t*)w;
  std::string err;
  const int rc = pg::run_bond_build(pos, n, dim, delta, pairs, capacity, n_pairs, (cudaStream_t)stream, S, &err);
  if (rc) g_err = err;
  return rc;
}

extern "C" const char* pg_noalloc_last_error(void) { return g_err.c_str(); }
