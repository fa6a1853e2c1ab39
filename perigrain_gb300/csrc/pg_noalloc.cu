// pg_build_bonds_noalloc: the GPU bond-list builder for callers that cannot allocate device
// memory. Such callers include allocator hooks and memory-pool managers (a cudaMalloc from inside
// them would re-enter the allocator they implement), and embedders whose device memory is fully
// reserved up front (a host application that hands the GPU to this library with a fixed budget,
// or a process sharing a GPU under a hard memory quota). It computes exactly what pg_build_bonds
// computes, with its scratch in one file-scope device array instead of cudaMalloc'd memory, and
// calls no cudaMalloc, cudaFree or other allocating routine.
//
// The array holds the scratch of one grain of up to PG_NOALLOC_MAX_NODES nodes (about 1.7 MB);
// every GPU that loads the library keeps it until the process exits. Calls share it: two calls
// that overlap on the GPU (different streams, or different host threads on one device) race and
// must be serialised by the caller. Whatever a call needs zeroed (cell counts, flags, the
// bounding box, the scan's ticket) is cleared by that call, so each call starts from a clean
// scratch even though the array keeps the previous call's contents.
//
// In host code the array's name is only a host-side stand-in, not a device address. Its device
// address is looked up with cudaGetSymbolAddress once per device, with that device current, by the
// first call made on the device; make that first call before any stream capture. The address is
// cached for the life of the CUDA context: after cudaDeviceReset the cached address is stale, so a
// process that resets a device must not call this entry point on it again.
#include <cuda_runtime.h>

#include <atomic>
#include <string>

#include "../../include/perigrain.h"
#include "pg_bonds.h"

namespace {

constexpr uint32_t kMaxNodes = PG_NOALLOC_MAX_NODES;
constexpr uint32_t kCells = pg::bond_grid_cells_c(kMaxNodes);
constexpr uint32_t kTiles = pg::bond_scan_tiles_c(kCells > kMaxNodes ? kCells : kMaxNodes);
// box (6 x u64) + counts + starts + 5 per-node arrays (+1 for the offsets' total) + tile sums +
// ticket + error word
constexpr size_t kWords = 12 + (size_t)kCells + ((size_t)kCells + 1) + (size_t)kMaxNodes * 5 + 1 + kTiles + 1 + 1;

__device__ __align__(256) uint32_t g_bond_scratch[kWords];

constexpr int kMaxDevices = 64;
std::atomic<uint32_t*> g_scratch_addr[kMaxDevices];
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
  uint32_t* base = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!base) {
    // set-up on this device: host code may not use the symbol itself as an address, so ask the
    // runtime for the current device's copy (two threads doing this at once store the same value)
    uint32_t* p = nullptr;
    e = cudaGetSymbolAddress((void**)&p, g_bond_scratch);
    if (e != cudaSuccess || !p) {
      g_err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return PG_ECUDA;
    }
    g_scratch_addr[dev].store(p, std::memory_order_release);
    base = p;
  }
  pg::BondScratch S;
  S.cells = pg::bond_grid_cells(n);
  const uint32_t tiles = pg::bond_scan_tiles(S.cells > n ? S.cells : n);
  uint32_t* w = base;
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
  w += 1;
  if ((size_t)(w - base) > kWords) {  // cannot happen for n <= kMaxNodes (sizes are monotone in n)
    g_err = "internal: scratch layout exceeds the static array";
    return PG_EINVAL;
  }
  std::string err;
  const int rc = pg::run_bond_build(pos, n, dim, delta, pairs, capacity, n_pairs, (cudaStream_t)stream, S, &err);
  if (rc) g_err = err;
  return rc;
}

extern "C" const char* pg_noalloc_last_error(void) { return g_err.c_str(); }
