// Device-side data layout and helpers of the GB300 PeriDEM engine.
//
// Layout in HBM (one handle, all instances):
//   * node vectors are stored AoS with a stride of S doubles per node, S = 2 (2D, one
//     double2 load) or 4 (3D, padded: two double2 loads);
//   * bonds use a warp-sliced ELL layout ("SELL-32"): the 32 nodes of warp chunk c own
//     chunk_deg[c] * 32 slots starting at chunk_slot[c]; bond k of node (32c + lane) sits in
//     slot chunk_slot[c] + 32k + lane, so the k-th bond of a whole warp is one coalesced
//     128-byte (col) / 256-byte (xi_norm) access. Row order within a node is the reference's
//     NbdArr order; padding slots are never alive;
//   * the alive set is one 32-bit word per (chunk, k): bit `lane` is bond k of that lane, so a
//     warp reads its alive bits with one broadcast load and writes them back with one ballot;
//   * the contact grid is a dense row-major uniform grid per instance (cell >= 1.0625 R_c), refitted
//     on the device every step to the instance's bounding box (plus two cells) and rebuilt by a
//     counting sort of the nodes by cell (one radix digit spanning all cells), whose exclusive scan
//     doubles as the cell-start table. Cell coordinates are clamped to the grid, so a node that
//     moves outside the box still lands in an edge cell and every pair within R_c is still found.
#pragma once
#include <cstdint>

#include "../../include/perigrain.h"

namespace pg {

constexpr uint32_t NONE = 0xffffffffu;
constexpr int MAX_CAND = 64;        // hard cap of contact candidates held per node
constexpr uint32_t CAND_CAP = 32;   // candidate-list entries per node (ECAPACITY beyond)
constexpr int FINAL_THREADS = 1024; // threads of the per-step finalize kernel
constexpr int WREC_SMEM_CAP = 16384;// wall-reaction records sorted in shared memory per step
constexpr int FIN_TILE = 2048;       // sorted wall records whose terms are staged in shared memory at once
// dynamic shared memory of k_finalize: sort keys + one tile of four terms per record
constexpr int FINAL_SMEM = WREC_SMEM_CAP * 8 + FIN_TILE * 4 * 8;
constexpr uint32_t ENT_NODE = 0x3fffffffu;  // partner bits of a recorded contact entry
// friction branch of a recorded contact entry; in 2D a sliding contact also records the sign of
// its tangential direction along perp(u) = (-u_y, u_x) (FR_SLIDE_NEG when negative)
constexpr uint32_t FR_SLIDE = 1u, FR_STICK = 2u, FR_SLIDE_NEG = 3u;

enum GrainFlag : uint32_t {
  GF_MOVABLE = 1u,
  GF_BREAKABLE = 2u,
  GF_STOPPABLE = 4u,
  GF_BREAK_BONDS = 8u,
};

struct GrainDev {
  uint32_t node_begin, node_end;
  uint32_t inst;
  uint32_t flags;
  double rho, one_over_rho, cnot, snot;
  double torque_val;
  uint32_t torque_axis;
  uint32_t pad;
  // per-grain contact parameters (normal stiffness, damping ratio, friction coefficient); used by
  // the force kernels only when Dev::grain_contact is set, always by the adjoint. A pair of
  // grains contacts with the arithmetic mean of the two grains' values, which is the reference's
  // global parameter when all grains carry the same value.
  double kn, zeta, mu;
  // FP32 copies of cnot, snot and 1/rho for the mixed kernels (set by set_grain_f whenever the
  // FP64 values change; an FP64 -> FP32 conversion per thread would run on the FP64 pipe)
  float cnot_f, snot_f, one_over_rho_f, pad_f;
};

inline void set_grain_f(GrainDev& g) {
  g.cnot_f = (float)g.cnot;
  g.snot_f = (float)g.snot;
  g.one_over_rho_f = (float)g.one_over_rho;
  g.pad_f = 0.f;
}

struct InstDev {
  double contact_rad, normal_stiffness, friction_coefficient, damping_ratio;
  double contact_s_max;  // sqrt_le_max(contact_rad): a squared distance above it rules contact out
  double origin[3];     // lower corner of this step's grid
  double xorigin[3];    // fixed origin of the FP32 hi/lo bond reference positions (mixed path)
  double cell;          // grid cell edge (>= 1.0625 contact_rad)
  double cell_min;      // smallest admissible cell edge
  float inv_cell_f;     // 1/cell in float (cell coordinates are computed in FP32)
  float cell_f;
  float pre_f;          // FP32 prefilter radius of contact candidates (1.0625 contact_rad)
  float pre_b;          // candidate lists: FP32 search radius at a build, 1.0625 (R_c + skin)
  float skin_lim2;      // candidate lists: squared displacement since the last build that forces
                        // a rebuild, (0.45 skin)^2 (the Verlet bound is skin/2; FP32 margin)
  uint32_t dims[3];     // cells per axis (dims[2] = 1 in 2D)
  // rel_frame != 0 (mixed path with candidate lists): the FP32 position images (curf) are
  // offsets from xorigin, which never moves, so the position update of a step does not depend on
  // the grid refit of the step before; frame_off_f = xorigin - origin turns them into offsets from
  // the grid origin for cell coordinates. Otherwise the images are offsets from origin, and 0.
  float frame_off_f[3];
  int32_t rel_frame;
  // the images' origin in FP32 (xorigin with rel_frame, else this step's grid origin): an image is
  // trunc_f32(CurrPos) - org_f, formed in FP32 (its error, ~1e-7 of the coordinates' size, is far
  // inside the 1/16 margin of the prefilter radius and the cell edge)
  float org_f[3];
  uint32_t table_off, table_cap;
  uint32_t node_begin, node_end, grain_begin, grain_end;
  int32_t allow_wall;
  double wall[6];
  double wall_speed[6];
};

// Fit the grid of one instance to the node bounding box [lo, hi] plus two cells on every side,
// with cells no smaller than cell_min and at most table_cap cells (coarser cells if needed).
__host__ __device__ inline void fit_grid(InstDev& in, int D, const double* lo, const double* hi) {
  // cell counts in FP32 (the grid only has to cover the box; the exact origin stays FP64) -- this
  // runs once per instance per step inside a single block, where FP64 division would be slow
  float cs = (float)in.cell_min;
  float ext[3] = {0.f, 0.f, 0.f};
  for (int a = 0; a < D; ++a) ext[a] = (float)(hi[a] - lo[a]);
  uint32_t n[3] = {1, 1, 1};
  for (int it = 0; it < 200; ++it) {
    const float inv = 1.f / cs;
    unsigned long long cells = 1;
    for (int a = 0; a < D; ++a) {
      n[a] = (uint32_t)(ext[a] * inv) + 5u;  // + two cells of margin on each side + rounding
      cells *= n[a];
    }
    if (cells <= in.table_cap) break;
    cs *= 1.25f;
  }
  in.cell = (double)cs;
  in.cell_f = cs;
  in.inv_cell_f = 1.f / cs;
  for (int a = 0; a < 3; ++a) {
    in.origin[a] = a < D ? lo[a] - 2.0 * (double)cs : 0.0;
    in.dims[a] = a < D ? n[a] : 1u;
    in.frame_off_f[a] = (in.rel_frame && a < D) ? (float)(in.xorigin[a] - in.origin[a]) : 0.f;
    in.org_f[a] = a < D ? (float)(in.rel_frame ? in.xorigin[a] : in.origin[a]) : 0.f;
  }
}

// Clamped cell coordinate of an FP32 offset from the grid origin.
__host__ __device__ inline int32_t cell_coord(float r, float inv_cell, uint32_t n) {
  float c = floorf(r * inv_cell);
  if (!(c >= 0.f)) return 0;  // also catches NaN
  if (c >= (float)(n - 1)) return (int32_t)(n - 1);
  return (int32_t)c;
}

// A wall interaction of one node with one wall side, kept so that the reaction sums can be
// replayed in the reference's serial node order (contact.h:339, :374, :411-412, :428).
struct WallRec {
  double a_normal;   // vol * c_sign * F            (subtracted from reaction[dir])
  double a_t1;       // vol * friction (tangent 1)  (subtracted from reaction[t1])
  double a_t2;       // vol * friction (tangent 2, 3D)
  double a_damp;     // vol * damping force         (subtracted from reaction[dir])
  uint32_t gid;
  uint16_t side;     // lrtb index
  uint8_t has_fric;
  uint8_t has_damp;
};

struct Dev {
  uint32_t dim, N, G, I;
  uint32_t n_chunks;
  uint32_t table_total;
  // node arrays
  double *xpos, *pos, *disp, *cur, *vel_in, *vel_out, *acc, *force, *extf, *vol;
  float* curf;  // float copy of (cur - origin) for the grid, stride SF
  uint32_t *node_grain, *bdry_rank;
  // node layout (pg_config::node_order): node_orig[d] = the input's global index of device node d,
  // node_at[o] = the device node of input node o; both null when the layout is the input order.
  // The reference's orders are kept through them: candidate visit order and wall-reaction order by
  // input index, the pair-log hash of input indices, sums over a grain in input order.
  uint32_t *node_orig, *node_at;
  // the low half of a node's candidate key in the reference's visit order: its rank in the
  // grain's nonlocal boundary list with nl_bdry_only (NONE for other nodes), else its input index
  // within its grain
  uint32_t* node_sub;
  uint8_t *clamped, *clamp_pending;
  // grid
  uint32_t *cell_key, *cell_rank, *cell_count, *cell_start, *sorted;
  // with candidate lists, beside `sorted`: each entry's FP32 position image (curf layout) and
  // candidate key (grain << 32 | rank in the reference's loop order, NONE for a node outside the
  // nonlocal boundary when nl_bdry_only), so a list rebuild reads a cell's nodes contiguously
  float* sorted_pos;
  unsigned long long* sorted_key;
  uint32_t *scan_tile_sum;
  uint32_t *scan_done;
  uint32_t* gbar;      // [3] grid barrier of the cooperative grid build: arrivals, generation,
                       // halted (set when a wait timed out; the build then returns at entry)
  uint32_t coop_blocks;  // blocks of that launch (all resident), 0 = separate grid kernels
  // bonds (SELL-32)
  uint32_t *chunk_slot, *chunk_deg, *chunk_word, *node_deg;
  uint32_t* bcol;
  double* bxin;
  uint32_t* alive;
  uint32_t* break_step;
  // grains / instances
  GrainDev* grain;
  unsigned long long* bbox;  // [G][2*dim] ordered keys: min..., max... (the step parity's buffer)
  double* torque_c;          // [G][3] centroid for torque
  InstDev* inst;
  double* reaction;          // [I][2*dim][dim]
  WallRec* wrec;
  uint32_t* wrec_count;
  uint32_t wrec_cap;
  uint32_t wrec_smem;  // wall records the finalize launch's shared memory holds (0 without walls)
  // pair log
  unsigned long long* pair_acc;  // [2]: count, hash
  unsigned long long *log_count, *log_hash;
  uint32_t log_cap;
  // control
  uint32_t* step;  // t of the step in flight
  int32_t* status;
  unsigned long long* too_close;
  // config
  double dt, hdt2, half_dt;
  int32_t enable_fracture, nl_bdry_only, allow_damping, allow_friction, self_contact;
  int32_t enable_torque, gradient_extforce, record_pairs;
  uint32_t extforce_maxstep;
  uint32_t max_cand;
  int32_t grain_contact;  // contact parameters from GrainDev (pair mean) instead of InstDev
  // contact candidate lists (Verlet lists with a skin; cand_q == null: grid search every step).
  // Node d's candidates are cand_q[(chunk * cand_cap + k) * 32 + lane], k < cand_n[d], in the
  // reference's visit order; disp_b holds the displacement at the last build (FP32, stride SF);
  // rebuild != 0 makes this step recount the grid and rebuild the lists.
  uint32_t* cand_q;
  uint8_t* cand_n;
  float* disp_b;
  uint32_t* rebuild;  // the step parity's flag (set by its position update, cleared by its finalize)
  uint32_t cand_cap;
  int32_t worm;           // run_timeloop_worm semantics (pg_config::timeloop == 1)
  // mask recording (force kernels instantiated with REC = true): per node of this step the
  // offset and count of its active contact entries in rec_ent (entry = partner | friction
  // branch << 30, FR_*) and the wall bits (4 per wall side in call order: in contact, friction
  // active, sticking, 2D sliding towards -t). rec_n counts entries appended so far. When rec_x is
  // set the kernel also writes the tape of the step: CurrPos and velocity its forces saw (stride
  // S), the wall positions [I][2D] and the step number.
  uint32_t *rec_off, *rec_ent, *rec_wall, *rec_n;
  uint8_t* rec_cnt;
  uint32_t rec_cap;
  double *rec_x, *rec_v, *rec_w;
  uint32_t* rec_t;
  float* rec_df;  // mixed precision: the step's displacement as FP32 hi/lo pairs (layout of bref's disp part)
  // mixed precision (PG_MIXED): FP32 hi/lo pairs (x = hi + lo to ~2^-47 |x|). `bref` interleaves,
  // per node, the pair of the FP64 displacement and the pair of the bond reference position
  // (relative to the instance's fixed origin) -- 4*SF floats, one 32-byte sector in 2D -- so a bond
  // gathers its neighbour's data from one sector. FP32 acceleration, force, external force and
  // volume.
  float* bref;
  float *acc_f, *force_f, *extf_f, *vol_f;
  float dt_f, hdt2_f, half_dt_f;
};

#ifdef __CUDACC__
// Warp-wide min / max of 64-bit keys with two 32-bit hardware reductions each (all 32 lanes).
__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long k) {
  const uint32_t hi = (uint32_t)(k >> 32), lo = (uint32_t)k;
  const uint32_t h = __reduce_min_sync(0xffffffffu, hi);
  const uint32_t l = __reduce_min_sync(0xffffffffu, hi == h ? lo : 0xffffffffu);
  return ((unsigned long long)h << 32) | l;
}
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long k) {
  const uint32_t hi = (uint32_t)(k >> 32), lo = (uint32_t)k;
  const uint32_t h = __reduce_max_sync(0xffffffffu, hi);
  const uint32_t l = __reduce_max_sync(0xffffffffu, hi == h ? lo : 0u);
  return ((unsigned long long)h << 32) | l;
}
#endif

__host__ __device__ inline unsigned long long dbl_to_ordered(double x) {
  unsigned long long b;
#ifdef __CUDA_ARCH__
  b = (unsigned long long)__double_as_longlong(x);
#else
  __builtin_memcpy(&b, &x, 8);
#endif
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ inline double ordered_to_dbl(unsigned long long k) {
  unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
  double x;
#ifdef __CUDA_ARCH__
  x = __longlong_as_double((long long)b);
#else
  __builtin_memcpy(&x, &b, 8);
#endif
  return x;
}

// Gait phase of run_timeloop_worm at step t (timeloop.h:1097-1107): 0 in the first of every three
// 1000-step periods (front nodes 0 and 3 held, external force on), 1 otherwise (back nodes 1, 2).
__host__ __device__ inline uint32_t worm_phase(uint32_t t) { return ((t / 1000u) % 3u == 0u) ? 0u : 1u; }

// The input's index of device node d, and the device node of input node o.
__host__ __device__ inline uint32_t orig_of(const Dev& P, uint32_t d) { return P.node_orig ? P.node_orig[d] : d; }
__host__ __device__ inline uint32_t at_of(const Dev& P, uint32_t o) { return P.node_at ? P.node_at[o] : o; }

__host__ __device__ inline uint64_t splitmix64(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

}  // namespace pg
