// Device code shared by the FP64 (pg_kernels.cu) and mixed-precision (pg_kernels_mixed.cu)
// translation units: vector loads/stores, the cell-start scan, the counting-sort scatter, the
// torque centroid, bounding-box predicates and the per-step finalize kernel. Kernels here are
// `static` so each translation unit carries its own copy.
#pragma once
#include <cuda_runtime.h>

#include <cmath>

#include "pg_device.cuh"

namespace pg {

template <int D>
struct Lay {
  static constexpr int S = (D == 2) ? 2 : 4;   // doubles per node vector
  static constexpr int SF = (D == 2) ? 2 : 4;  // floats per node vector (curf)
};

template <int D>
__device__ __forceinline__ void ldv(const double* a, uint32_t i, double (&v)[D]) {
  if constexpr (D == 2) {
    double2 t = reinterpret_cast<const double2*>(a)[i];
    v[0] = t.x;
    v[1] = t.y;
  } else {
    const double2* p = reinterpret_cast<const double2*>(a + 4ull * i);
    double2 t0 = p[0], t1 = p[1];
    v[0] = t0.x;
    v[1] = t0.y;
    v[2] = t1.x;
  }
}
template <int D>
__device__ __forceinline__ void stv(double* a, uint32_t i, const double (&v)[D]) {
  if constexpr (D == 2) {
    reinterpret_cast<double2*>(a)[i] = make_double2(v[0], v[1]);
  } else {
    double2* p = reinterpret_cast<double2*>(a + 4ull * i);
    p[0] = make_double2(v[0], v[1]);
    p[1] = make_double2(v[2], 0.0);
  }
}
template <int D>
__device__ __forceinline__ void ldf(const float* a, uint32_t i, float (&v)[D]) {
  if constexpr (D == 2) {
    float2 t = reinterpret_cast<const float2*>(a)[i];
    v[0] = t.x;
    v[1] = t.y;
  } else {
    float4 t = reinterpret_cast<const float4*>(a)[i];
    v[0] = t.x;
    v[1] = t.y;
    v[2] = t.z;
  }
}

__device__ __forceinline__ void set_status(int32_t* st, int32_t code) { atomicCAS(st, 0, code); }

// Programmatic dependent launch. Every kernel of a step starts with pdl_enter(), which waits until
// the previous kernel in the stream has finished and its writes are visible; launched with
// programmatic stream serialization, the kernel's blocks are scheduled while the previous kernel's
// last blocks drain instead of after it. (No early launch_dependents: letting the next kernel's
// blocks in while the current one still runs measured slower.) A no-op for a kernel launched
// without the attribute.
__device__ __forceinline__ void pdl_enter() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Launch k<<<g, b, smem, s>>>(args...), with programmatic stream serialization when `pdl`.
template <class... KArgs, class... Args>
inline void launch_k(void (*k)(KArgs...), dim3 g, dim3 b, size_t smem, cudaStream_t s, bool pdl, Args... args) {
  if (!pdl) {
    k<<<g, b, smem, s>>>(args...);
    return;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = g;
  cfg.blockDim = b;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k, args...);
}

// Mask recording: append this node's contact entries to rec_ent (one atomic per warp; the whole
// warp must call this) and store its offset, count and wall bits. On overflow of rec_cap the
// node's list is stored empty and PG_ECAPACITY raised, so the host can grow the buffer and redo.
__device__ __forceinline__ void record_masks(const Dev& P, uint32_t d, bool act, uint32_t lane,
                                             const uint32_t* rent, uint32_t nrec, uint32_t wbits) {
  const uint32_t full = 0xffffffffu;
  uint32_t incl = nrec;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(full, incl, o);
    if (lane >= (uint32_t)o) incl += y;
  }
  const uint32_t tot = __shfl_sync(full, incl, 31);
  uint32_t base = 0;
  if (lane == 31 && tot) base = atomicAdd(P.rec_n, tot);
  base = __shfl_sync(full, base, 31);
  if (!act) return;
  const uint32_t o = base + incl - nrec;
  if ((uint64_t)o + nrec <= (uint64_t)P.rec_cap) {
    for (uint32_t i = 0; i < nrec; ++i) P.rec_ent[o + i] = rent[i];
    P.rec_off[d] = o;
    P.rec_cnt[d] = (uint8_t)nrec;
  } else {
    set_status(P.status, PG_ECAPACITY);
    P.rec_off[d] = 0;
    P.rec_cnt[d] = 0;
  }
  P.rec_wall[d] = wbits;
}

// Gait clamps of run_timeloop_worm (timeloop.h:1213-1244) on the node with grain-local index li:
// vel = acc = 0 for nodes 0 and 3 (phase 0) or 1 and 2 (phase 1), then no y motion for nodes 0-3.
template <int D, class TA, class TV>
__device__ __forceinline__ void worm_clamp(uint32_t li, uint32_t phase, TA (&a)[D], TV (&v)[D]) {
  if ((phase == 0 && (li == 0 || li == 3)) || (phase == 1 && (li == 1 || li == 2))) {
    for (int c = 0; c < D; ++c) {
      a[c] = 0;
      v[c] = 0;
    }
  }
  if (li < 4) {
    a[1] = 0;
    v[1] = 0;
  }
}

// Tape of the step (REC with rec_x): the CurrPos and velocity node d's forces saw, and (first
// threads) the wall positions and the step number.
template <int D>
__device__ __forceinline__ void record_tape(const Dev& P, uint32_t d, bool act, uint32_t t, const double (&x)[D],
                                            const double (&v)[D]) {
  if (act) {
    stv<D>(P.rec_x, d, x);
    stv<D>(P.rec_v, d, v);
  }
  constexpr uint32_t NS = 2 * D;
  if (d < P.I * NS) P.rec_w[d] = P.inst[d / NS].wall[d % NS];
  if (d == 0) *P.rec_t = t;
}

// ---------------------------------------------------------------------------------------------
// Exclusive scan of cell_count -> cell_start (reduce-then-scan, last block scans tile sums).
// ---------------------------------------------------------------------------------------------
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_PER = 16;  // four uint4 loads per thread
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_PER;

__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* warp_sums, uint32_t* total) {
  const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t x = v;
  for (int off = 1; off < 32; off <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= (uint32_t)off) x += y;
  }
  if (lane == 31) warp_sums[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint32_t nw = blockDim.x >> 5;
    uint32_t s = lane < nw ? warp_sums[lane] : 0;
    for (int off = 1; off < 32; off <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, s, off);
      if (lane >= (uint32_t)off) s += y;
    }
    if (lane < nw) warp_sums[lane] = s;
  }
  __syncthreads();
  uint32_t base = wid ? warp_sums[wid - 1] : 0;
  if (total) *total = warp_sums[(blockDim.x >> 5) - 1];
  return base + x - v;
}

// With candidate lists the grid is rebuilt only on rebuild steps; the grid kernels return at once
// on the other steps.
__device__ __forceinline__ bool grid_idle(const Dev& P) { return P.cand_q && !*P.rebuild; }

static __global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const Dev P) {
  pdl_enter();
  __shared__ uint32_t ws[32];
  __shared__ bool last;
  if (grid_idle(P)) return;
  const uint32_t tile = blockIdx.x;
  const uint32_t base = tile * SCAN_TILE + threadIdx.x * SCAN_PER;
  uint32_t s = 0;
  if (base + SCAN_PER <= P.table_total) {
    const uint4* q = reinterpret_cast<const uint4*>(P.cell_count + base);
    uint4 v[SCAN_PER / 4];
    for (int k = 0; k < SCAN_PER / 4; ++k) v[k] = q[k];
    for (int k = 0; k < SCAN_PER / 4; ++k) s += v[k].x + v[k].y + v[k].z + v[k].w;
  } else {
    for (int k = 0; k < SCAN_PER; ++k) {
      uint32_t i = base + k;
      if (i < P.table_total) s += P.cell_count[i];
    }
  }
  uint32_t tot;
  block_excl_scan(s, ws, &tot);
  if (threadIdx.x == 0) {
    P.scan_tile_sum[tile] = tot;
    __threadfence();
    uint32_t ticket = atomicAdd(P.scan_done, 1u);
    last = (ticket == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // last block: exclusive scan of the tile sums in place
  const uint32_t ntiles = gridDim.x;
  uint32_t carry = 0;
  for (uint32_t b0 = 0; b0 < ntiles; b0 += SCAN_THREADS) {
    uint32_t i = b0 + threadIdx.x;
    uint32_t v = i < ntiles ? ((volatile uint32_t*)P.scan_tile_sum)[i] : 0;
    uint32_t t2;
    uint32_t ex = block_excl_scan(v, ws, &t2);
    __syncthreads();
    if (i < ntiles) P.scan_tile_sum[i] = carry + ex;
    carry += t2;
    __syncthreads();
  }
  if (threadIdx.x == 0) *P.scan_done = 0;
}

static __global__ void __launch_bounds__(SCAN_THREADS) k_scan_final(const Dev P) {
  pdl_enter();
  __shared__ uint32_t ws[32];
  if (grid_idle(P)) return;
  const uint32_t tile = blockIdx.x;
  const uint32_t base = tile * SCAN_TILE + threadIdx.x * SCAN_PER;
  uint32_t v[SCAN_PER];
  uint32_t s = 0;
  const bool full = base + SCAN_PER <= P.table_total;
  if (full) {
    const uint4* q4 = reinterpret_cast<const uint4*>(P.cell_count + base);
    for (int k = 0; k < SCAN_PER / 4; ++k) {
      const uint4 q = q4[k];
      v[4 * k] = q.x;
      v[4 * k + 1] = q.y;
      v[4 * k + 2] = q.z;
      v[4 * k + 3] = q.w;
    }
  } else {
    for (int k = 0; k < SCAN_PER; ++k) {
      uint32_t i = base + k;
      v[k] = i < P.table_total ? P.cell_count[i] : 0;
    }
  }
  for (int k = 0; k < SCAN_PER; ++k) s += v[k];
  uint32_t ex = block_excl_scan(s, ws, nullptr) + P.scan_tile_sum[tile];
  uint32_t st[SCAN_PER];
  for (int k = 0; k < SCAN_PER; ++k) {
    st[k] = ex;
    ex += v[k];
  }
  if (full) {
    // cell_start has table_total + 1 entries, so base need not be 16-byte aligned: plain stores
    uint4* s4 = reinterpret_cast<uint4*>(P.cell_start + base);  // base is a multiple of 16 entries
    for (int k = 0; k < SCAN_PER / 4; ++k) s4[k] = make_uint4(st[4 * k], st[4 * k + 1], st[4 * k + 2], st[4 * k + 3]);
    uint4* z4 = reinterpret_cast<uint4*>(P.cell_count + base);
    for (int k = 0; k < SCAN_PER / 4; ++k) z4[k] = make_uint4(0, 0, 0, 0);  // next step's counts
  } else {
    for (int k = 0; k < SCAN_PER; ++k) {
      uint32_t i = base + k;
      if (i < P.table_total) {
        P.cell_start[i] = st[k];
        P.cell_count[i] = 0;
      }
    }
  }
  if (tile == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) P.cell_start[P.table_total] = P.N;
}

// Node d's entry of the cell-sorted order (and, with candidate lists, its position image and key).
__device__ __forceinline__ void scatter_node(const Dev& P, uint32_t d) {
  const uint32_t at = P.cell_start[P.cell_key[d]] + P.cell_rank[d];
  P.sorted[at] = d;
  if (P.sorted_key) {
    const uint32_t g = P.node_grain[d];
    const uint32_t sub = P.node_sub[d];
    P.sorted_key[at] = ((unsigned long long)g << 32) | sub;
    if (P.dim == 2) {
      reinterpret_cast<float2*>(P.sorted_pos)[at] = reinterpret_cast<const float2*>(P.curf)[d];
    } else {
      reinterpret_cast<float4*>(P.sorted_pos)[at] = reinterpret_cast<const float4*>(P.curf)[d];
    }
  }
}

static __global__ void __launch_bounds__(256) k_scatter(const Dev P) {
  pdl_enter();
  if (grid_idle(P)) return;
  const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d < P.N) scatter_node(P, d);
}

// ---------------------------------------------------------------------------------------------
// Torque centroid: mean_CurrPos (particle2.h:89-98) in the reference's serial order.
// ---------------------------------------------------------------------------------------------
template <int D>
static __global__ void k_torque_center(const Dev P) {
  pdl_enter();
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= P.G) return;
  const GrainDev gr = P.grain[g];
  double m[D];
  for (int c = 0; c < D; ++c) m[c] = 0.0;
  for (uint32_t o = gr.node_begin; o < gr.node_end; ++o) {  // the input's node order
    double cu[D];
    ldv<D>(P.cur, at_of(P, o), cu);
    for (int c = 0; c < D; ++c) m[c] = m[c] + cu[c];
  }
  double n = (double)(gr.node_end - gr.node_begin);
  for (int c = 0; c < D; ++c) P.torque_c[(size_t)g * 3 + c] = m[c] / n;
}

template <int D>
__device__ __forceinline__ void grain_box(const Dev& P, uint32_t g, double (&mn)[D], double (&mx)[D]) {
  for (int c = 0; c < D; ++c) {
    mn[c] = ordered_to_dbl(P.bbox[(size_t)g * 2 * D + c]);
    mx[c] = ordered_to_dbl(P.bbox[(size_t)g * 2 * D + D + c]);
  }
}

// intersects_box_fext (contact.h:984-1020), written per axis: (min_i - c <= max_j) && (max_i + c >= min_j)
template <int D>
__device__ __forceinline__ bool boxes_touch(const double (&mni)[D], const double (&mxi)[D],
                                            const double (&mnj)[D], const double (&mxj)[D], double c) {
  bool r = true;
  for (int a = 0; a < D; ++a) r = r && ((mni[a] - c) <= mxj[a]) && ((mxi[a] + c) >= mnj[a]);
  return r;
}

// within_interior_fext (contact.h:1066-1080) applied to get_minmax() and RectWall::lrtb()
// arrays exactly as the reference indexes them (in 3D this reads the 6-entry arrays with the
// 2D index pattern, as the reference does).
template <int D>
__device__ __forceinline__ bool within_interior(const double (&mn)[D], const double (&mx)[D],
                                                const double* W, double c) {
  double A[4];
  if constexpr (D == 2) {
    A[0] = mn[0]; A[1] = mx[0]; A[2] = mx[1]; A[3] = mn[1];
  } else {
    A[0] = mn[0]; A[1] = mn[1]; A[2] = mn[2]; A[3] = mx[0];
  }
  double AL = A[0] - c, AR = A[1] + c, AT = A[2] + c, AB = A[3] - c;
  return (W[0] < AL) && (AR < W[1]) && (W[2] > AT) && (W[3] < AB);
}

template <int D>
__device__ __forceinline__ void insert_cand(unsigned long long (&keys)[MAX_CAND], uint32_t (&idx)[MAX_CAND],
                                            int& n, unsigned long long key, uint32_t q, const Dev& P) {
  if (n >= (int)P.max_cand) {
    set_status(P.status, PG_ECAPACITY);
    return;
  }
  int k = n++;
  while (k > 0 && keys[k - 1] > key) {
    keys[k] = keys[k - 1];
    idx[k] = idx[k - 1];
    --k;
  }
  keys[k] = key;
  idx[k] = q;
}

// ---------------------------------------------------------------------------------------------
// Per-instance end of a step (blocks 1.. of k_finalize, one warp per instance): wall move
// (timeloop.h:866-878); the instance's grid refitted to this step's bounding box for the next step
// (the grain boxes of the predict kernel folded by the warp, then reset for the next step).
constexpr uint32_t FINAL_BLOCK_INSTANCES = 64;  // up to this many instances: a block each, else a warp each

inline uint32_t finalize_blocks(uint32_t I) {
  return 1 + (I <= FINAL_BLOCK_INSTANCES ? I : (I + FINAL_THREADS / 32 - 1) / (FINAL_THREADS / 32));
}

template <int D>
__device__ __forceinline__ void finalize_instances(const Dev& P) {
  constexpr int NS = 2 * D;
  __shared__ unsigned long long red[2 * D][FINAL_THREADS / 32];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool per_block = P.I <= FINAL_BLOCK_INSTANCES;
  const uint32_t k = per_block ? blockIdx.x - 1 : (blockIdx.x - 1) * (blockDim.x >> 5) + warp;
  if (k >= P.I) return;
  InstDev* in = &P.inst[k];
  const uint32_t r = per_block ? threadIdx.x : lane, nr = per_block ? blockDim.x : 32u;
  if (r < (uint32_t)NS) in->wall[r] = in->wall[r] + in->wall_speed[r] * P.dt;
  unsigned long long mn[D], mx[D];
  for (int c = 0; c < D; ++c) {
    mn[c] = ~0ull;
    mx[c] = 0ull;
  }
  const uint32_t gb = in->grain_begin, ge = in->grain_end;
  for (uint32_t g = gb + r; g < ge; g += nr) {
    for (int c = 0; c < D; ++c) {
      const unsigned long long a = P.bbox[(size_t)g * NS + c], b = P.bbox[(size_t)g * NS + D + c];
      mn[c] = a < mn[c] ? a : mn[c];
      mx[c] = b > mx[c] ? b : mx[c];
      P.bbox[(size_t)g * NS + c] = ~0ull;
      P.bbox[(size_t)g * NS + D + c] = 0ull;
    }
  }
  for (int c = 0; c < D; ++c) {
    mn[c] = warp_min_u64(mn[c]);
    mx[c] = warp_max_u64(mx[c]);
  }
  if (per_block) {
    if (lane == 0)
      for (int c = 0; c < D; ++c) {
        red[c][warp] = mn[c];
        red[D + c][warp] = mx[c];
      }
    __syncthreads();
    if (warp != 0) return;
    const uint32_t nw = blockDim.x >> 5;
    for (int c = 0; c < D; ++c) {
      mn[c] = warp_min_u64(lane < nw ? red[c][lane] : ~0ull);
      mx[c] = warp_max_u64(lane < nw ? red[D + c][lane] : 0ull);
    }
  }
  if (lane == 0) {
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    bool ok = ge > gb;
    for (int c = 0; c < D; ++c) {
      lo[c] = ordered_to_dbl(mn[c]);
      hi[c] = ordered_to_dbl(mx[c]);
      ok = ok && isfinite(lo[c]) && isfinite(hi[c]);
    }
    if (ok) fit_grid(*in, D, lo, hi);
  }
}

// k_finalize, block 0: wall reactions in node order, pair log, step counter; blocks 1..: one warp
// per instance (finalize_instances).
// ---------------------------------------------------------------------------------------------
template <int D>
static __global__ void __launch_bounds__(FINAL_THREADS) k_finalize(const Dev P) {
  pdl_enter();
  if (blockIdx.x > 0) {
    finalize_instances<D>(P);
    return;
  }
  extern __shared__ unsigned long long skey[];
  constexpr int NS = 2 * D;
  const uint32_t tid = threadIdx.x;
  const uint32_t t = *P.step;
  const uint32_t R = *P.wrec_count;
  const uint32_t nrx = P.I * NS * D;
  for (uint32_t i = tid; i < nrx; i += blockDim.x) P.reaction[i] = 0.0;
  if (R > 0) {
    if (R > P.wrec_smem || R > P.wrec_cap) {
      if (tid == 0) set_status(P.status, PG_ECAPACITY);
    } else {
      // sort the records by (side, node in the reference's loop order); the index of the record
      // rides in the low bits
      double* sval = reinterpret_cast<double*>(skey + WREC_SMEM_CAP);  // [FIN_TILE][4]
      uint32_t n2 = 32;
      while (n2 < R) n2 <<= 1;
      for (uint32_t i = tid; i < n2; i += blockDim.x) {
        if (i < R) {
          const WallRec& r = P.wrec[i];
          skey[i] = ((unsigned long long)r.side << 60) | ((unsigned long long)r.gid << 14) | i;
        } else {
          skey[i] = ~0ull;
        }
      }
      __syncthreads();
      for (uint32_t k = 2; k <= n2; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
          for (uint32_t i = tid; i < n2; i += blockDim.x) {
            uint32_t l = i ^ j;
            if (l > i) {
              unsigned long long a = skey[i], b = skey[l];
              bool up = ((i & k) == 0);
              if ((a > b) == up) {
                skey[i] = b;
                skey[l] = a;
              }
            }
          }
          __syncthreads();
        }
      }
      // tiles of FIN_TILE sorted records: gather their terms into shared memory in parallel, then
      // one thread per (instance, side) subtracts its contiguous run in order (contact.h:339, :374,
      // :411-412, :428: normal, friction, damping; terms of absent branches are stored as 0, and
      // x - 0 == x)
      for (uint32_t base = 0; base < R; base += FIN_TILE) {
        const uint32_t m = min((uint32_t)FIN_TILE, R - base);
        for (uint32_t i = tid; i < m; i += blockDim.x) {
          const WallRec& w = P.wrec[skey[base + i] & 0x3fffu];
          sval[4 * i + 0] = w.a_normal;
          sval[4 * i + 1] = w.has_fric ? w.a_t1 : 0.0;
          sval[4 * i + 2] = w.has_fric ? w.a_t2 : 0.0;
          sval[4 * i + 3] = w.has_damp ? w.a_damp : 0.0;
        }
        __syncthreads();
        for (uint32_t p = tid; p < P.I * NS; p += blockDim.x) {
          const uint32_t inst = p / NS, side = p % NS;
          const unsigned long long lo_key =
              ((unsigned long long)side << 60) | ((unsigned long long)P.inst[inst].node_begin << 14);
          const unsigned long long hi_key =
              ((unsigned long long)side << 60) | ((unsigned long long)P.inst[inst].node_end << 14);
          uint32_t lo = base, hi = base + m;
          while (lo < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if (skey[mid] < lo_key) lo = mid + 1; else hi = mid;
          }
          uint32_t end = lo, top = base + m;
          while (end < top) {
            uint32_t mid = (end + top) >> 1;
            if (skey[mid] < hi_key) end = mid + 1; else top = mid;
          }
          if (end == lo) continue;
          const int dir = (D == 2) ? ((side == 0 || side == 1) ? 0 : 1) : (int)(side % 3);
          double* rp = P.reaction + ((size_t)inst * NS + side) * D;
          double r[3] = {0.0, 0.0, 0.0};
          for (int c = 0; c < D; ++c) r[c] = rp[c];
#pragma unroll 4
          for (uint32_t k = lo; k < end; ++k) {
            const double* v = sval + 4 * (k - base);
            r[dir] = r[dir] - v[0];
            if constexpr (D == 2) {
              r[(dir + 1) % 2] = r[(dir + 1) % 2] - v[1];
            } else {
              r[(dir + 1) % 3] = r[(dir + 1) % 3] - v[1];
              r[(dir + 2) % 3] = r[(dir + 2) % 3] - v[2];
            }
            r[dir] = r[dir] - v[3];
          }
          for (int c = 0; c < D; ++c) rp[c] = r[c];
        }
        __syncthreads();
      }
    }
  }
  __syncthreads();
  if (tid == 0) {
    if (P.record_pairs) {
      const uint32_t slot = (t - 1) % P.log_cap;
      P.log_count[slot] = P.pair_acc[0];
      P.log_hash[slot] = P.pair_acc[1];
      P.pair_acc[0] = 0;
      P.pair_acc[1] = 0;
    }
    *P.wrec_count = 0;
    *P.step = t + 1;
    if (P.cand_q) *P.rebuild = 0;
  }
}


inline uint32_t cdiv(uint32_t a, uint32_t b) { return (a + b - 1) / b; }
__device__ __forceinline__ uint32_t cdiv_dev(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

// ---------------------------------------------------------------------------------------------
// Contact candidate lists (Verlet lists with a skin): on rebuild steps the grid is recounted and
// every node's list rebuilt with radius R_c + skin; on the other steps the force kernels read the
// lists instead of searching the grid. A pair within R_c at step t was within R_c + skin at the
// last build while no node has moved more than skin/2 since (predict raises `rebuild` at 0.45 skin),
// so every pair the grid search would evaluate is in the list, in the same order.
// ---------------------------------------------------------------------------------------------
// grid keys of a rebuild step (the grid-search path computes them in the predict kernels)
template <int D>
static __global__ void __launch_bounds__(256) k_keys(const Dev P) {
  pdl_enter();
  if (!*P.rebuild) return;
  const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= P.N) return;
  const InstDev& in = P.inst[P.grain[P.node_grain[d]].inst];
  float rf[D];
  ldf<D>(P.curf, d, rf);
  int32_t ci[3] = {0, 0, 0};
  for (int c = 0; c < D; ++c) ci[c] = cell_coord(rf[c] + in.frame_off_f[c], in.inv_cell_f, in.dims[c]);
  const uint32_t key = in.table_off + ((uint32_t)ci[2] * in.dims[1] + (uint32_t)ci[1]) * in.dims[0] + (uint32_t)ci[0];
  P.cell_key[d] = key;
  P.cell_rank[d] = atomicAdd(&P.cell_count[key], 1u);
}

// Rebuild of node d's list: every node q of the 3x3 (3x3x3) cells within the FP32 radius pre_b that
// the contact rules could pair with d (same grain: self-contact; other grain: stoppable, or any in
// the worm loop; boundary nodes only when nl_bdry_only), sorted by the reference's visit order.
// The bounding-box prefilter is applied per step, not here. Also records the displacement.
template <int D>
__device__ __forceinline__ void cand_build_node(const Dev& P, uint32_t d) {
  const uint32_t lane = d & 31, chunk = d >> 5;
  constexpr uint32_t SF = (D == 2) ? 2 : 4;
  double dp[D];
  ldv<D>(P.disp, d, dp);
  for (int c = 0; c < D; ++c) P.disp_b[(size_t)d * SF + c] = (float)dp[c];
  const uint32_t g = P.node_grain[d];
  const GrainDev gr = P.grain[g];
  const bool mov = gr.flags & GF_MOVABLE;
  const bool p_bdry = !P.nl_bdry_only || P.bdry_rank[d] != NONE;
  const bool selfc = mov && P.enable_fracture && (gr.flags & GF_BREAKABLE) && P.self_contact;
  const bool other = mov && (P.worm || (gr.flags & GF_STOPPABLE));
  uint32_t n = 0;
  if ((selfc || other) && p_bdry) {
    const InstDev& in = P.inst[gr.inst];
    float pf[D];
    ldf<D>(P.curf, d, pf);
    int32_t cc[3] = {0, 0, 0};
    for (int c = 0; c < D; ++c) cc[c] = cell_coord(pf[c] + in.frame_off_f[c], in.inv_cell_f, in.dims[c]);
    const float thr2 = in.pre_b * in.pre_b;
    unsigned long long keys[CAND_CAP];
    uint32_t idx[CAND_CAP];
    const int z0 = (D == 3) ? max(cc[2] - 1, 0) : 0, z1 = (D == 3) ? min(cc[2] + 1, (int)in.dims[2] - 1) : 0;
    const int y0 = max(cc[1] - 1, 0), y1 = min(cc[1] + 1, (int)in.dims[1] - 1);
    const int x0 = max(cc[0] - 1, 0), x1 = min(cc[0] + 1, (int)in.dims[0] - 1);
    for (int z = z0; z <= z1; ++z)
      for (int y = y0; y <= y1; ++y) {
        const uint32_t row = in.table_off + ((uint32_t)z * in.dims[1] + (uint32_t)y) * in.dims[0];
        const uint32_t b0 = P.cell_start[row + x0], b1 = P.cell_start[row + x1 + 1];
        for (uint32_t b = b0; b < b1; ++b) {
          // the cell's entries are consecutive: index, position image and key without gathers
          const uint32_t q = P.sorted[b];
          float qf[D];
          ldf<D>(P.sorted_pos, b, qf);
          const unsigned long long qk = P.sorted_key[b];
          if (q == d) continue;
          float d2 = 0.f;
          for (int c = 0; c < D; ++c) {
            const float dd = qf[c] - pf[c];
            d2 += dd * dd;
          }
          if (d2 > thr2) continue;
          const uint32_t gq = (uint32_t)(qk >> 32), sub = (uint32_t)qk;
          const bool same = gq == g;
          if (same ? !selfc : !other) continue;
          if (P.nl_bdry_only && sub == NONE) continue;
          const unsigned long long key = ((unsigned long long)(same ? 0u : 1u) << 63) | qk;
          if (n >= P.cand_cap) {
            set_status(P.status, PG_ECAPACITY);
            continue;
          }
          int k = (int)n++;
          while (k > 0 && keys[k - 1] > key) {
            keys[k] = keys[k - 1];
            idx[k] = idx[k - 1];
            --k;
          }
          keys[k] = key;
          idx[k] = q;
        }
      }
    const size_t base = (size_t)chunk * P.cand_cap * 32 + lane;
    for (uint32_t k = 0; k < n; ++k) P.cand_q[base + (size_t)k * 32] = idx[k];
  }
  P.cand_n[d] = (uint8_t)n;
}

template <int D>
static __global__ void __launch_bounds__(128) k_cand_build(const Dev P) {
  pdl_enter();
  if (!*P.rebuild) return;
  const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d < P.N) cand_build_node<D>(P, d);
}

// ---------------------------------------------------------------------------------------------
// Cooperative grid build (candidate lists): keys and counts, scan of the counts, scatter and the
// candidate-list rebuild in one launch of co-resident blocks separated by grid barriers, so a step
// without a rebuild costs one idle launch here instead of five. The barrier waits are bounded: past GBAR_SPIN_LIMIT polls a
// block records PG_ETIMEOUT and returns (the step's status then reports it).
// ---------------------------------------------------------------------------------------------
constexpr uint32_t GBAR_SPIN_LIMIT = 1u << 22;  // polls of ~64 ns: about 0.3 s

__device__ __forceinline__ bool grid_barrier(const Dev& P, uint32_t* ok_smem) {
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t ok = 1;
    volatile uint32_t* gen = P.gbar + 1;
    const uint32_t g = *gen;
    __threadfence();
    if (atomicAdd(P.gbar, 1u) == gridDim.x - 1) {
      atomicExch(P.gbar, 0u);
      __threadfence();
      atomicAdd(P.gbar + 1, 1u);
    } else {
      uint32_t it = 0;
      while (*gen == g) {
        if (++it > GBAR_SPIN_LIMIT) {
          ok = 0;
          set_status(P.status, PG_ETIMEOUT);
          // the arrival count now holds this launch's stale arrivals: later launches of this
          // kernel must not use the barrier (an early release would let the scan read counts
          // before every key is in and the scatter write outside the sorted list)
          atomicExch(P.gbar + 2, 1u);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    *ok_smem = ok;
  }
  __syncthreads();
  return *ok_smem != 0;
}

// SCAN_PER consecutive cell counts from `base` (a multiple of SCAN_PER): four 16-byte loads when the
// run lies inside the table, element by element at its end (zeros past it).
__device__ __forceinline__ void load_counts(const Dev& P, uint32_t base, uint32_t (&v)[SCAN_PER]) {
  if (base + SCAN_PER <= P.table_total) {
    const uint4* q4 = reinterpret_cast<const uint4*>(P.cell_count + base);
    for (int k = 0; k < SCAN_PER / 4; ++k) {
      const uint4 q = q4[k];
      v[4 * k] = q.x;
      v[4 * k + 1] = q.y;
      v[4 * k + 2] = q.z;
      v[4 * k + 3] = q.w;
    }
  } else {
    for (int k = 0; k < SCAN_PER; ++k) v[k] = base + k < P.table_total ? P.cell_count[base + k] : 0u;
  }
}
// Cell starts of the run at `base`, and its counts cleared for the next build.
__device__ __forceinline__ void store_starts_clear_counts(const Dev& P, uint32_t base, const uint32_t (&st)[SCAN_PER]) {
  if (base + SCAN_PER <= P.table_total) {
    uint4* s4 = reinterpret_cast<uint4*>(P.cell_start + base);  // base is a multiple of 16 entries
    uint4* z4 = reinterpret_cast<uint4*>(P.cell_count + base);
    for (int k = 0; k < SCAN_PER / 4; ++k) {
      s4[k] = make_uint4(st[4 * k], st[4 * k + 1], st[4 * k + 2], st[4 * k + 3]);
      z4[k] = make_uint4(0u, 0u, 0u, 0u);
    }
  } else {
    for (int k = 0; k < SCAN_PER; ++k)
      if (base + k < P.table_total) {
        P.cell_start[base + k] = st[k];
        P.cell_count[base + k] = 0u;
      }
  }
}

template <int D>
static __global__ void __launch_bounds__(SCAN_THREADS) k_grid_coop(const Dev P) {
  pdl_enter();
  __shared__ uint32_t ws[32];
  __shared__ uint32_t ok;
  __shared__ bool last;
  if (!*P.rebuild) return;  // set by the predict kernel before this launch: the same for every block
  // a barrier of an earlier launch timed out: the handle is halted (the host refuses further steps
  // once it sees PG_ETIMEOUT; launches already enqueued return here)
  if (((volatile uint32_t*)P.gbar)[2]) return;
  const uint32_t nthr = gridDim.x * blockDim.x;
  // 1. grid keys and per-cell ranks
  for (uint32_t d = blockIdx.x * blockDim.x + threadIdx.x; d < P.N; d += nthr) {
    const InstDev& in = P.inst[P.grain[P.node_grain[d]].inst];
    float rf[D];
    ldf<D>(P.curf, d, rf);
    int32_t ci[3] = {0, 0, 0};
    for (int c = 0; c < D; ++c) ci[c] = cell_coord(rf[c] + in.frame_off_f[c], in.inv_cell_f, in.dims[c]);
    const uint32_t key = in.table_off + ((uint32_t)ci[2] * in.dims[1] + (uint32_t)ci[1]) * in.dims[0] + (uint32_t)ci[0];
    P.cell_key[d] = key;
    P.cell_rank[d] = atomicAdd(&P.cell_count[key], 1u);
  }
  if (!grid_barrier(P, &ok)) return;
  // 2. tile sums of the counts
  const uint32_t ntiles = cdiv_dev(P.table_total, SCAN_TILE);
  for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint32_t base = tile * SCAN_TILE + threadIdx.x * SCAN_PER;
    uint32_t v[SCAN_PER], sum = 0;
    load_counts(P, base, v);
    for (int k = 0; k < SCAN_PER; ++k) sum += v[k];
    uint32_t tot;
    block_excl_scan(sum, ws, &tot);
    if (threadIdx.x == 0) P.scan_tile_sum[tile] = tot;
    __syncthreads();
  }
  if (!grid_barrier(P, &ok)) return;
  // 3. exclusive scan of the tile sums (block 0)
  if (blockIdx.x == 0) {
    uint32_t carry = 0;
    for (uint32_t b0 = 0; b0 < ntiles; b0 += SCAN_THREADS) {
      const uint32_t i = b0 + threadIdx.x;
      const uint32_t v = i < ntiles ? ((volatile uint32_t*)P.scan_tile_sum)[i] : 0;
      uint32_t t2;
      const uint32_t ex = block_excl_scan(v, ws, &t2);
      __syncthreads();
      if (i < ntiles) P.scan_tile_sum[i] = carry + ex;
      carry += t2;
      __syncthreads();
    }
  }
  (void)last;
  if (!grid_barrier(P, &ok)) return;
  // 4. cell starts, counts cleared for the next build
  for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint32_t base = tile * SCAN_TILE + threadIdx.x * SCAN_PER;
    uint32_t v[SCAN_PER], sum = 0;
    load_counts(P, base, v);
    for (int k = 0; k < SCAN_PER; ++k) sum += v[k];
    uint32_t ex = block_excl_scan(sum, ws, nullptr) + ((volatile uint32_t*)P.scan_tile_sum)[tile];
    uint32_t st[SCAN_PER];
    for (int k = 0; k < SCAN_PER; ++k) {
      st[k] = ex;
      ex += v[k];
    }
    store_starts_clear_counts(P, base, st);
    __syncthreads();
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) P.cell_start[P.table_total] = P.N;
  if (!grid_barrier(P, &ok)) return;
  // 5. scatter
  for (uint32_t d = blockIdx.x * blockDim.x + threadIdx.x; d < P.N; d += nthr) scatter_node(P, d);
  if (!grid_barrier(P, &ok)) return;
  // 6. candidate lists
  for (uint32_t d = blockIdx.x * blockDim.x + threadIdx.x; d < P.N; d += nthr) cand_build_node<D>(P, d);
}

// Grid build shared by both precisions: exclusive scan of the bucket counts, then scatter; with
// candidate lists also the grid keys (before) and the list rebuild (after), all of them returning
// at once on steps that need no rebuild.
template <int D>
inline void launch_grid_build(const Dev& P, cudaStream_t s, uint64_t* launches, bool pdl = false) {
  const uint32_t ntiles = cdiv(P.table_total, SCAN_TILE);
  if (P.cand_q && P.coop_blocks) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(P.coop_blocks);
    cfg.blockDim = dim3(SCAN_THREADS);
    cfg.stream = s;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 2 : 1;
    cudaLaunchKernelEx(&cfg, k_grid_coop<D>, P);
    *launches += 1;
    return;
  }
  if (P.cand_q) {
    launch_k(k_keys<D>, cdiv(P.N, 256), 256, 0, s, pdl, P);
    *launches += 1;
  }
  launch_k(k_scan_reduce, ntiles, SCAN_THREADS, 0, s, pdl, P);
  launch_k(k_scan_final, ntiles, SCAN_THREADS, 0, s, pdl, P);
  launch_k(k_scatter, cdiv(P.N, 256), 256, 0, s, pdl, P);
  *launches += 3;
  if (P.cand_q) {
    launch_k(k_cand_build<D>, cdiv(P.N, 128), 128, 0, s, pdl, P);
    *launches += 1;
  }
}

}  // namespace pg
