// GPU bond-list builder: the Connectivity of one grain -- all node pairs (i, j), i < j, with
// sqrt(sum((p_j - p_i)^2)) <= delta, in lexicographic order. The reference builds it in Python
// over all n(n-1)/2 pairs (exp_dict.py:171-222: itertools.combinations + single_bond); here a
// uniform grid of cell >= delta restricts each node to the 3^dim surrounding cells.
//
// Passes (all on the caller's stream): bounding box -> cell key and count -> exclusive scan
// (cell starts) -> scatter -> per-node count of partners j > i -> exclusive scan (row offsets)
// -> per-node write of its partners in ascending j. Compiled with --fmad=false so the distance is
// the same IEEE computation numpy performs, and the pair set is identical to the reference's.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>

#include "../../include/perigrain.h"
#include "pg_bonds.h"
#include "pg_sqrt_threshold.h"
#include "pg_device.cuh"

namespace pg {

constexpr int BT = 256;               // threads per block
constexpr int SCAN_T = 1024;          // scan block
constexpr int SCAN_TILE_B = SCAN_T * 4;
static_assert(SCAN_TILE_B == (int)BOND_SCAN_TILE, "scan tile of the bond builder and its declared size differ");
constexpr int MAX_PARTNERS = 4096;    // partners j > i of one node (the row is sorted in place)

struct BondGrid {
  double origin[3];
  double inv_cell;
  uint32_t dims[3];
};

// Bounding box of the positions as ordered keys: each block folds its nodes with warp reductions
// and shared memory, then one atomic per block and bound (a per-thread atomic on the same six words
// serialised in L2: 54 us for 20k nodes).
__global__ void __launch_bounds__(BT) kb_box(const double* pos, uint32_t n, uint32_t dim, unsigned long long* box) {
  __shared__ unsigned long long red[6][BT / 32];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long mn[3], mx[3];
  for (uint32_t c = 0; c < 3; ++c) {
    mn[c] = ~0ull;
    mx[c] = 0ull;
    if (c < dim && i < n) {
      mn[c] = dbl_to_ordered(pos[(size_t)i * dim + c]);
      mx[c] = mn[c];
    }
    mn[c] = warp_min_u64(mn[c]);
    mx[c] = warp_max_u64(mx[c]);
  }
  if (lane == 0)
    for (uint32_t c = 0; c < 3; ++c) {
      red[c][warp] = mn[c];
      red[3 + c][warp] = mx[c];
    }
  __syncthreads();
  if (warp == 0) {
    const uint32_t nw = blockDim.x >> 5;
    for (uint32_t c = 0; c < dim; ++c) {
      const unsigned long long a = warp_min_u64(lane < nw ? red[c][lane] : ~0ull);
      const unsigned long long b = warp_max_u64(lane < nw ? red[3 + c][lane] : 0ull);
      if (lane == 0) {
        atomicMin(&box[c], a);
        atomicMax(&box[3 + c], b);
      }
    }
  }
}

__device__ __forceinline__ uint32_t bond_cell_of(const double* p, uint32_t dim, const BondGrid& g, int32_t* cc) {
  for (uint32_t c = 0; c < 3; ++c) cc[c] = 0;
  for (uint32_t c = 0; c < dim; ++c) {
    double f = floor((p[c] - g.origin[c]) * g.inv_cell);
    int32_t v = (f < 0) ? 0 : (f >= (double)(g.dims[c] - 1) ? (int32_t)g.dims[c] - 1 : (int32_t)f);
    cc[c] = v;
  }
  return ((uint32_t)cc[2] * g.dims[1] + (uint32_t)cc[1]) * g.dims[0] + (uint32_t)cc[0];
}

__global__ void kb_key(const double* pos, uint32_t n, uint32_t dim, BondGrid g, BondScratch S) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int32_t cc[3];
  const uint32_t k = bond_cell_of(pos + (size_t)i * dim, dim, g, cc);
  S.key[i] = k;
  S.rank[i] = atomicAdd(&S.cell_count[k], 1u);
}

__device__ __forceinline__ uint32_t blk_excl(uint32_t v, uint32_t* ws, uint32_t* total) {
  const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) ws[wid] = x;
  __syncthreads();
  if (wid == 0) {
    const uint32_t nw = blockDim.x >> 5;
    uint32_t s = lane < nw ? ws[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= (uint32_t)o) s += y;
    }
    if (lane < nw) ws[lane] = s;
  }
  __syncthreads();
  const uint32_t base = wid ? ws[wid - 1] : 0;
  if (total) *total = ws[(blockDim.x >> 5) - 1];
  __syncthreads();
  return base + x - v;
}

// exclusive scan of in[0..len) into out[0..len], out[len] = total; tile sums in tsum, done flag
__global__ void kb_scan_tiles(const uint32_t* in, uint32_t len, uint32_t* tsum, uint32_t* done) {
  __shared__ uint32_t ws[32];
  __shared__ bool last;
  const uint32_t base = blockIdx.x * SCAN_TILE_B + threadIdx.x * 4;
  uint32_t s = 0;
  for (int k = 0; k < 4; ++k)
    if (base + k < len) s += in[base + k];
  uint32_t tot;
  blk_excl(s, ws, &tot);
  if (threadIdx.x == 0) {
    tsum[blockIdx.x] = tot;
    __threadfence();
    last = (atomicAdd(done, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  uint32_t carry = 0;
  for (uint32_t b0 = 0; b0 < gridDim.x; b0 += SCAN_T) {
    const uint32_t i = b0 + threadIdx.x;
    const uint32_t v = i < gridDim.x ? ((volatile uint32_t*)tsum)[i] : 0;
    uint32_t t2;
    const uint32_t ex = blk_excl(v, ws, &t2);
    if (i < gridDim.x) tsum[i] = carry + ex;
    carry += t2;
  }
  if (threadIdx.x == 0) *done = 0;
}

__global__ void kb_scan_final(const uint32_t* in, uint32_t len, const uint32_t* tsum, uint32_t* out) {
  __shared__ uint32_t ws[32];
  const uint32_t base = blockIdx.x * SCAN_TILE_B + threadIdx.x * 4;
  uint32_t v[4], s = 0;
  for (int k = 0; k < 4; ++k) {
    v[k] = base + k < len ? in[base + k] : 0;
    s += v[k];
  }
  uint32_t ex = blk_excl(s, ws, nullptr) + tsum[blockIdx.x];
  for (int k = 0; k < 4; ++k) {
    if (base + k < len) out[base + k] = ex;
    ex += v[k];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[len] = ex;
}

__global__ void kb_scatter(uint32_t n, BondScratch S) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) S.sorted[S.cell_start[S.key[i]] + S.rank[i]] = i;
}

// Visit every partner j > i of node i within delta, in the grid's cell order: f(j). The test
// sqrt(s) <= delta is made as s <= s_max, s_max = sqrt_le_max(delta): the same outcome for every s.
template <class F>
__device__ __forceinline__ void for_partners(const double* pos, uint32_t i, uint32_t dim, double s_max,
                                             const BondGrid& g, const BondScratch& S, F f) {
  int32_t cc[3];
  const double* pi = pos + (size_t)i * dim;
  bond_cell_of(pi, dim, g, cc);
  const int z0 = dim == 3 ? max(cc[2] - 1, 0) : 0, z1 = dim == 3 ? min(cc[2] + 1, (int)g.dims[2] - 1) : 0;
  const int y0 = max(cc[1] - 1, 0), y1 = min(cc[1] + 1, (int)g.dims[1] - 1);
  const int x0 = max(cc[0] - 1, 0), x1 = min(cc[0] + 1, (int)g.dims[0] - 1);
  for (int z = z0; z <= z1; ++z)
    for (int y = y0; y <= y1; ++y) {
      const uint32_t row = ((uint32_t)z * g.dims[1] + (uint32_t)y) * g.dims[0];
      const uint32_t b0 = S.cell_start[row + x0], b1 = S.cell_start[row + x1 + 1];
      for (uint32_t b = b0; b < b1; ++b) {
        const uint32_t j = S.sorted[b];
        if (j <= i) continue;
        const double* pj = pos + (size_t)j * dim;
        double s = (pj[0] - pi[0]) * (pj[0] - pi[0]);
        for (uint32_t c = 1; c < dim; ++c) s = s + (pj[c] - pi[c]) * (pj[c] - pi[c]);
        if (!(s <= s_max)) continue;
        f(j);
      }
    }
}

// WRITE = false: count node i's partners j > i. WRITE = true: write row i (pairs (i, j), j
// ascending) at its offset: the partners go to the row in visit order and are sorted there; a row
// that crosses `capacity` gets its smallest partners that fit, picked one at a time.
template <bool WRITE>
__global__ void kb_pairs(const double* pos, uint32_t n, uint32_t dim, double s_max, BondGrid g, BondScratch S,
                         uint32_t* pairs, uint64_t capacity) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (!WRITE) {
    uint32_t cnt = 0;
    for_partners(pos, i, dim, s_max, g, S, [&](uint32_t) { ++cnt; });
    S.pcount[i] = cnt;
    if (cnt > (uint32_t)MAX_PARTNERS) atomicCAS(S.error, 0, (int32_t)PG_ECAPACITY);
    return;
  }
  const uint64_t off = S.poff[i];
  const uint32_t cnt = S.pcount[i];
  if (cnt == 0 || off >= capacity) return;
  if (off + cnt <= capacity) {
    uint32_t k = 0;
    for_partners(pos, i, dim, s_max, g, S, [&](uint32_t j) {
      if (k < cnt) pairs[2 * (off + k) + 1] = j;
      ++k;
    });
    // insertion sort of the row by j
    for (uint32_t a = 1; a < cnt; ++a) {
      const uint32_t v = pairs[2 * (off + a) + 1];
      uint32_t b = a;
      while (b > 0 && pairs[2 * (off + b - 1) + 1] > v) {
        pairs[2 * (off + b) + 1] = pairs[2 * (off + b - 1) + 1];
        --b;
      }
      pairs[2 * (off + b) + 1] = v;
    }
    for (uint32_t a = 0; a < cnt; ++a) pairs[2 * (off + a)] = i;
  } else {
    uint32_t prev = i;
    for (uint64_t k = off; k < capacity; ++k) {
      uint32_t best = 0xffffffffu;
      for_partners(pos, i, dim, s_max, g, S, [&](uint32_t j) {
        if (j > prev && j < best) best = j;
      });
      pairs[2 * k] = i;
      pairs[2 * k + 1] = best;
      prev = best;
    }
  }
}

static inline uint32_t cdivb(uint64_t a, uint32_t b) { return (uint32_t)((a + b - 1) / b); }

static cudaError_t scan_u32(const uint32_t* in, uint32_t len, uint32_t* out, const BondScratch& S,
                            cudaStream_t st) {
  const uint32_t tiles = cdivb(len ? len : 1, SCAN_TILE_B);
  kb_scan_tiles<<<tiles, SCAN_T, 0, st>>>(in, len, S.tile_sum, S.done);
  kb_scan_final<<<tiles, SCAN_T, 0, st>>>(in, len, S.tile_sum, out);
  return cudaGetLastError();
}

cudaError_t scan_u32_dev(const uint32_t* in, uint32_t len, uint32_t* out, uint32_t* tile_sum, uint32_t* done,
                         cudaStream_t st) {
  const uint32_t tiles = cdivb(len ? len : 1, SCAN_TILE_B);
  kb_scan_tiles<<<tiles, SCAN_T, 0, st>>>(in, len, tile_sum, done);
  kb_scan_final<<<tiles, SCAN_T, 0, st>>>(in, len, tile_sum, out);
  return cudaGetLastError();
}

uint32_t bond_grid_cells(uint32_t n) { return bond_grid_cells_c(n); }
uint32_t bond_scan_tiles(uint32_t len) { return bond_scan_tiles_c(len); }

int run_bond_build(const double* pos, uint32_t n, uint32_t dim, double delta, uint32_t* pairs, uint64_t capacity,
                   uint64_t* n_pairs, cudaStream_t st, const BondScratch& S, std::string* err) {
  *n_pairs = 0;
  if (n < 2) return PG_OK;
  // 1. bounding box
  unsigned long long init[6] = {~0ull, ~0ull, ~0ull, 0ull, 0ull, 0ull};
  cudaError_t e = cudaMemcpyAsync(S.box, init, sizeof init, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    kb_box<<<cdivb(n, BT), BT, 0, st>>>(pos, n, dim, S.box);
    e = cudaGetLastError();
  }
  unsigned long long box[6];
  if (e == cudaSuccess) e = cudaMemcpyAsync(box, S.box, sizeof box, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    *err = cudaGetErrorString(e);
    return PG_ECUDA;
  }
  // 2. grid: cells >= delta (1 + 1e-6), at most S.cells cells
  BondGrid g;
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0}, ext = 0;
  for (uint32_t c = 0; c < dim; ++c) {
    lo[c] = ordered_to_dbl(box[c]);
    hi[c] = ordered_to_dbl(box[3 + c]);
    if (!std::isfinite(lo[c]) || !std::isfinite(hi[c])) {
      *err = "non-finite node position";
      return PG_EINVAL;
    }
    ext = std::fmax(ext, hi[c] - lo[c]);
  }
  double cell = delta > 0 ? delta * (1 + 1e-6) : std::fmax(ext, 1e-300) / 64;
  const double s_max = sqrt_le_max(delta);
  for (int it = 0; it < 200; ++it) {
    uint64_t cells = 1;
    for (uint32_t c = 0; c < dim; ++c) cells *= (uint64_t)((hi[c] - lo[c]) / cell) + 1;
    if (cells <= S.cells) break;
    cell *= 1.25;
  }
  g.inv_cell = 1.0 / cell;
  uint64_t cells = 1;
  for (uint32_t c = 0; c < 3; ++c) {
    g.origin[c] = c < dim ? lo[c] : 0.0;
    g.dims[c] = c < dim ? (uint32_t)((hi[c] - lo[c]) / cell) + 1 : 1;
    cells *= g.dims[c];
  }
  if (cells > S.cells) {
    *err = "bond grid does not fit its scratch";
    return PG_ECAPACITY;
  }
  const uint32_t C = (uint32_t)cells;
  // 3. counting sort by cell
  e = cudaMemsetAsync(S.cell_count, 0, (size_t)C * 4, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(S.done, 0, 4, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(S.error, 0, 4, st);
  if (e == cudaSuccess) {
    kb_key<<<cdivb(n, BT), BT, 0, st>>>(pos, n, dim, g, S);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = scan_u32(S.cell_count, C, S.cell_start, S, st);
  if (e == cudaSuccess) {
    kb_scatter<<<cdivb(n, BT), BT, 0, st>>>(n, S);
    e = cudaGetLastError();
  }
  // 4. count partners, row offsets, write rows
  if (e == cudaSuccess) {
    kb_pairs<false><<<cdivb(n, BT), BT, 0, st>>>(pos, n, dim, s_max, g, S, pairs, capacity);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = scan_u32(S.pcount, n, S.poff, S, st);
  if (e == cudaSuccess) {
    kb_pairs<true><<<cdivb(n, 128), 128, 0, st>>>(pos, n, dim, s_max, g, S, pairs, capacity);
    e = cudaGetLastError();
  }
  uint32_t total = 0;
  int32_t derr = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&total, S.poff + n, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&derr, S.error, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    *err = cudaGetErrorString(e);
    return PG_ECUDA;
  }
  *n_pairs = total;
  if (derr) {
    *err = "a node has more than 4096 partners j > i within delta";
    return PG_ECAPACITY;
  }
  if (total > capacity) {
    *err = "pair buffer too small: " + std::to_string(total) + " pairs";
    return PG_ECAPACITY;
  }
  return PG_OK;
}

}  // namespace pg

// ---------------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------------
namespace {
thread_local std::string g_bond_err;
}

extern "C" const char* pg_bond_last_error(void) { return g_bond_err.c_str(); }

extern "C" int pg_build_bonds(const double* pos, uint32_t n, uint32_t dim, double delta, uint32_t* pairs,
                              uint64_t capacity, uint64_t* n_pairs, void* stream) {
  using namespace pg;
  if (!n_pairs || (n && !pos) || (dim != 2 && dim != 3) || (capacity && !pairs)) {
    g_bond_err = "bad arguments";
    return PG_EINVAL;
  }
  *n_pairs = 0;
  if (n < 2) return PG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  BondScratch S;
  S.cells = bond_grid_cells(n);
  const uint32_t tiles = bond_scan_tiles(S.cells > n ? S.cells : n);
  void* block = nullptr;
  const size_t words = 12 + (size_t)S.cells * 2 + 1 + (size_t)n * 5 + 1 + tiles + 2;
  cudaError_t e = cudaMalloc(&block, words * 4 + 64);
  if (e != cudaSuccess) {
    g_bond_err = cudaGetErrorString(e);
    return PG_ENOMEM;
  }
  uint32_t* w = (uint32_t*)block;
  S.box = (unsigned long long*)w;
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
  int rc = run_bond_build(pos, n, dim, delta, pairs, capacity, n_pairs, st, S, &err);
  cudaStreamSynchronize(st);
  cudaFree(block);
  if (rc) g_bond_err = err;
  return rc;
}
