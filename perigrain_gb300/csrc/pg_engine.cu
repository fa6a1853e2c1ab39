// Host side of the GB300 PeriDEM engine: builds the device layout from a pg_setup_desc,
// drives the per-step kernels (captured into CUDA graphs) and implements the C ABI of
// include/perigrain.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "pg_device.cuh"
#include "pg_handle.h"
#include "pg_order.h"
#include "pg_sqrt_threshold.h"
#include "pg_kernels.h"
#include "pg_kernels_mixed.h"

using namespace pg;

static thread_local std::string g_err;

int pg_fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

static int fail(int code, const std::string& msg) { return pg_fail(code, msg); }

void set_vel(pg_handle* h, Dev& P, int parity) {
  P.vel_in = parity == 0 ? h->vel_a : h->vel_b;
  P.vel_out = parity == 0 ? h->vel_b : h->vel_a;
  P.bbox = h->bbox_pp[parity];
  P.rebuild = h->rebuild_pp[parity];
}

void enqueue_step(pg_handle* h, int parity, uint64_t* launches) {
  Dev P = h->P;
  set_vel(h, P, parity);
  if (h->precision == PG_MIXED) {
    launch_step_mixed(P, h->L, h->stream, launches);
  } else {
    launch_step(P, h->L, h->stream, launches);
  }
}

// Force a rebuild of the contact candidate lists at the next step (after host writes of state).
int request_list_rebuild(pg_handle* h) {
  if (!h->rebuild_pp[0]) return PG_OK;
  static const uint32_t one = 1;
  for (int p = 0; p < 2; ++p) CU(cudaMemcpyAsync(h->rebuild_pp[p], &one, 4, cudaMemcpyHostToDevice, h->stream));
  CU(cudaStreamSynchronize(h->stream));
  return PG_OK;
}

// GRAPH_STEPS mixed-precision steps from velocity parity `par` with each step's finalize on the
// side stream beside the next step's position update (which reads none of what finalize writes:
// the images are relative to the fixed frame, the grain boxes and rebuild flag are per parity);
// the next grid build waits for both. The last step ends with its finalize on the main stream.
static void enqueue_steps_overlapped(pg_handle* h, int par, uint64_t* n) {
  Dev P[pg_handle::GRAPH_STEPS];
  for (int k = 0; k < pg_handle::GRAPH_STEPS; ++k) {
    P[k] = h->P;
    set_vel(h, P[k], par ^ (k & 1));
  }
  launch_mixed_predict(P[0], h->stream, true, n);
  for (int k = 0; k < pg_handle::GRAPH_STEPS; ++k) {
    if (k > 0) cudaStreamWaitEvent(h->stream, h->ev_join, 0);
    launch_mixed_body(P[k], h->L, h->stream, true, n);
    if (k + 1 < pg_handle::GRAPH_STEPS) {
      cudaEventRecord(h->ev_fork, h->stream);
      cudaStreamWaitEvent(h->side, h->ev_fork, 0);
      launch_mixed_finalize(P[k], h->side, false, n);
      cudaEventRecord(h->ev_join, h->side);
      launch_mixed_predict(P[k + 1], h->stream, true, n);
    } else {
      launch_mixed_finalize(P[k], h->stream, true, n);
    }
  }
}

int build_graphs(pg_handle* h) {
  for (int par = 0; par < 2; ++par) {
    if (h->graph[par]) {
      cudaGraphExecDestroy(h->graph[par]);
      h->graph[par] = nullptr;
    }
    cudaGraph_t g = nullptr;
    CU(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    uint64_t n = 0;
    int p = par;
    if (h->overlap) {
      enqueue_steps_overlapped(h, par, &n);
    } else {
      for (int k = 0; k < pg_handle::GRAPH_STEPS; ++k) {
        enqueue_step(h, p, &n);
        p ^= 1;
      }
    }
    CU(cudaStreamEndCapture(h->stream, &g));
    cudaError_t e = cudaGraphInstantiate(&h->graph[par], g, 0);
    cudaGraphDestroy(g);
    CU(e);
    h->graph_launches_per = n;
  }
  return PG_OK;
}

// hi/lo FP32 image of FP64 vectors (hi = (float)x, lo = (float)(x - hi)), layout of ld_hl():
// 2D [hx, hy, lx, ly]; 3D [hx, hy, hz, 0, lx, ly, lz, 0]
static void pack_hl(const double* x, uint32_t N, uint32_t D, const std::vector<double>* origin_of_node,
                    std::vector<float>* out) {
  const uint32_t SF = (D == 2) ? 2 : 4;
  out->assign((size_t)N * 2 * SF, 0.f);
  for (uint32_t i = 0; i < N; ++i)
    for (uint32_t c = 0; c < D; ++c) {
      double v = x[(size_t)i * D + c] - (origin_of_node ? (*origin_of_node)[(size_t)i * 3 + c] : 0.0);
      float hi = (float)v;
      float lo = (float)(v - (double)hi);
      (*out)[(size_t)i * 2 * SF + c] = hi;
      (*out)[(size_t)i * 2 * SF + SF + c] = lo;
    }
}

static void pack_f(const double* x, uint32_t N, uint32_t D, std::vector<float>* out) {
  const uint32_t SF = (D == 2) ? 2 : 4;
  out->assign((size_t)N * SF, 0.f);
  for (uint32_t i = 0; i < N; ++i)
    for (uint32_t c = 0; c < D; ++c) (*out)[(size_t)i * SF + c] = (float)x[(size_t)i * D + c];
}

// FP32 images of the uploaded FP64 state for the mixed path (the host packing of pack_hl/pack_f,
// same conversions): bref = [disp hi, disp lo, (pos - xorigin) hi, lo] per node (2D record, 3D
// planes), acc, extforce and vol in FP32.
__global__ void k_mixed_images(const Dev P) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.N) return;
  const uint32_t D = P.dim, S = (D == 2) ? 2 : 4, SF = S, N = P.N;
  const InstDev& in = P.inst[P.grain[P.node_grain[i]].inst];
  for (uint32_t c = 0; c < D; ++c) {
    const double dv = P.disp[(size_t)i * S + c];
    const float dh = (float)dv, dl = (float)(dv - (double)dh);
    const double xv = P.pos[(size_t)i * S + c] - in.xorigin[c];
    const float xh = (float)xv, xl = (float)(xv - (double)xh);
    const float q4[4] = {dh, dl, xh, xl};
    for (uint32_t q = 0; q < 4; ++q) {
      if (D == 2) {
        P.bref[(size_t)i * 8 + q * 2 + c] = q4[q];
      } else {
        P.bref[(size_t)(q * D + c) * N + i] = q4[q];
      }
    }
    P.acc_f[(size_t)i * SF + c] = (float)P.acc[(size_t)i * S + c];
    P.extf_f[(size_t)i * SF + c] = (float)P.extf[(size_t)i * S + c];
  }
  P.vol_f[i] = (float)P.vol[i];
}

static int mixed_setup(pg_handle* h, const pg_setup_desc* s) {
  Dev& P = h->P;
  const uint32_t N = P.N, D = h->dim, SF = (D == 2) ? 2 : 4;
  // bref and vol_f padded to whole warp chunks: the mixed force kernel's lanes past the last node
  // gather their own (padding) index for bonds they never use
  const size_t NP = (size_t)P.n_chunks * 32;
  CU(h->dalloc(&P.bref, (NP - N) * 8 + (size_t)N * 4 * D));
  CU(h->dalloc(&P.acc_f, (size_t)N * SF));
  CU(h->dalloc(&P.force_f, (size_t)N * SF));
  CU(h->dalloc(&P.extf_f, (size_t)N * SF));
  CU(h->dalloc(&P.vol_f, NP));
  CU(cudaMemset(P.bref, 0, ((NP - N) * 8 + (size_t)N * 4 * D) * 4));
  CU(cudaMemset(P.vol_f, 0, NP * 4));
  P.dt_f = (float)P.dt;
  P.hdt2_f = (float)P.hdt2;
  P.half_dt_f = (float)P.half_dt;
  (void)s;
  CU(cudaMemset(P.acc_f, 0, (size_t)N * SF * 4));
  CU(cudaMemset(P.extf_f, 0, (size_t)N * SF * 4));
  CU(cudaMemset(P.force_f, 0, (size_t)N * SF * 4));
  if (N) {
    k_mixed_images<<<(N + 255) / 256, 256>>>(P);
    CU(cudaGetLastError());
  }
  return PG_OK;
}

// ---------------------------------------------------------------------------------------------
extern "C" {

int pg_version(void) { return 1; }

const char* pg_last_error(void) { return g_err.c_str(); }

const char* pg_status_string(int s) {
  switch (s) {
    case PG_OK: return "ok";
    case PG_EINVAL: return "invalid argument";
    case PG_ENOMEM: return "out of memory";
    case PG_ECUDA: return "CUDA error";
    case PG_ENAN: return "non-finite state";
    case PG_ETIMEOUT: return "device wait timed out";
    case PG_EIO: return "I/O error";
    case PG_ECAPACITY: return "device table capacity exceeded";
    case PG_ERANGE: return "node outside the resolvable coordinate range";
    case PG_ENODEV: return "no CUDA device";
  }
  return "unknown status";
}

int pg_device_count(int* count) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) {
    *count = 0;
    return fail(PG_ENODEV, cudaGetErrorString(e));
  }
  *count = n;
  return PG_OK;
}

int pg_select_device(int device) {
  CU(cudaSetDevice(device));
  return PG_OK;
}

void pg_config_default(pg_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->dt = 0.02 / 1e5;
  c->allow_damping = 1;
  c->allow_friction = 1;
  c->self_contact = 1;
  c->precision = PG_FP64;
  c->pair_log_capacity = 1024;
  c->first_step = 1;
  c->max_contacts = 48;
  c->contact_skin = 0.25;
  c->node_order = PG_ORDER_CELL;
}

// Host validation of a setup. With bonds_on_host the bond rows are checked here too (offsets
// non-decreasing, neighbours inside their grain); otherwise k_check_bonds checks them on the
// device from the uploaded copy before anything reads through them.
static int validate(const pg_setup_desc* s, const pg_config* c, bool bonds_on_host) {
  if (!s || !c) return fail(PG_EINVAL, "null setup or config");
  if (!(c->contact_skin >= 0) || !std::isfinite(c->contact_skin)) return fail(PG_EINVAL, "contact_skin must be >= 0");
  if (s->dim != 2 && s->dim != 3) return fail(PG_EINVAL, "dim must be 2 or 3");
  if (s->n_instances == 0 || s->n_grains == 0 || s->n_nodes == 0)
    return fail(PG_EINVAL, "empty setup");
  if (!s->grain_instance || !s->grain_node_offset || !s->pos || !s->vol || !s->disp || !s->vel ||
      !s->acc || !s->extforce || !s->bond_offset || !s->bdry_offset || !s->clamped_offset ||
      !s->delta || !s->rho || !s->cnot || !s->snot || !s->movable || !s->breakable ||
      !s->stoppable || !s->break_bonds || !s->contact_radius || !s->normal_stiffness ||
      !s->friction_coefficient || !s->damping_ratio || !s->allow_wall || !s->wall_geom ||
      !s->wall_speed)
    return fail(PG_EINVAL, "missing setup array");
  if (s->grain_node_offset[0] != 0 || s->grain_node_offset[s->n_grains] != s->n_nodes)
    return fail(PG_EINVAL, "grain_node_offset must start at 0 and end at n_nodes");
  for (uint32_t g = 0; g < s->n_grains; ++g) {
    if (s->grain_node_offset[g + 1] <= s->grain_node_offset[g])
      return fail(PG_EINVAL, "grain " + std::to_string(g) + " has no nodes");
    if (s->grain_instance[g] >= s->n_instances || (g && s->grain_instance[g] < s->grain_instance[g - 1]))
      return fail(PG_EINVAL, "grain_instance must be non-decreasing and < n_instances");
    if (c->enable_torque && s->dim == 2 && s->torque_axis && s->torque_axis[g] != 2)
      return fail(PG_EINVAL, "2D torque requires torque_axis = 2");
    if (c->enable_torque && (!s->torque_axis || !s->torque_val))
      return fail(PG_EINVAL, "enable_torque needs torque_axis and torque_val");
    if (c->enable_torque && s->torque_axis[g] > 2) return fail(PG_EINVAL, "torque_axis must be 0..2");
  }
  if (s->bond_offset[0] != 0) return fail(PG_EINVAL, "bond_offset[0] must be 0");
  if (s->bond_offset[s->n_nodes] >= (1ull << 31)) return fail(PG_EINVAL, "too many bonds");
  if (s->bond_offset[s->n_nodes] && !s->bond_local) return fail(PG_EINVAL, "missing bond_local");
  for (uint32_t g = 0; g < s->n_grains; ++g) {
    uint32_t n0 = s->grain_node_offset[g], n1 = s->grain_node_offset[g + 1];
    if (bonds_on_host) {
      for (uint32_t i = n0; i < n1; ++i)
        if (s->bond_offset[i + 1] < s->bond_offset[i]) return fail(PG_EINVAL, "bond_offset decreasing");
      // the grain's rows are one contiguous range: its largest local index decides, the offending
      // node is looked up only on failure
      uint32_t mx = 0;
      for (uint64_t b = s->bond_offset[n0]; b < s->bond_offset[n1]; ++b) mx = std::max(mx, s->bond_local[b]);
      if (s->bond_offset[n1] > s->bond_offset[n0] && mx >= n1 - n0) {
        for (uint32_t i = n0; i < n1; ++i)
          for (uint64_t b = s->bond_offset[i]; b < s->bond_offset[i + 1]; ++b)
            if (s->bond_local[b] >= n1 - n0)
              return fail(PG_EINVAL, "bond of node " + std::to_string(i) + " points outside its grain");
      }
    }
    for (uint32_t k = s->bdry_offset[g]; k < s->bdry_offset[g + 1]; ++k)
      if (s->bdry_nodes[k] >= n1 - n0) return fail(PG_EINVAL, "bdry node out of range");
    for (uint32_t k = s->clamped_offset[g]; k < s->clamped_offset[g + 1]; ++k)
      if (s->clamped_nodes[k] >= n1 - n0) return fail(PG_EINVAL, "clamped node out of range");
  }
  if (!(c->dt > 0)) return fail(PG_EINVAL, "dt must be positive");
  if (c->precision != PG_FP64 && c->precision != PG_MIXED) return fail(PG_EINVAL, "bad precision");
  return PG_OK;
}


static int create_impl(const pg_setup_desc* s, const pg_config* cfg_in, pg_handle** out);

// The project's autotuner: every (force-kernel block size, grid cells per node) candidate runs
// on a trial handle built from the same setup -- 3 warm-up steps, then 12 steps timed with CUDA
// events on the handle's stream -- and the fastest is kept; then the candidate-list skin and the
// node layout, each by the same kind of trial. The real handle starts from the untouched setup.
int pg_create(const pg_setup_desc* s, const pg_config* cfg_in, pg_handle** out) {
  if (!out || !cfg_in) return fail(PG_EINVAL, "null argument");
  if (!cfg_in->autotune) return create_impl(s, cfg_in, out);
  const uint32_t blocks[] = {64, 128};
  const uint32_t cells2[] = {2, 4, 8}, cells3[] = {4, 8, 16};
  const uint32_t* cells = (s && s->dim == 3) ? cells3 : cells2;
  double best_ms = 1e300;
  uint32_t best_b = 128, best_c = cells[1];
  for (uint32_t b : blocks)
    for (int ci = 0; ci < 3; ++ci) {
      pg_config c = *cfg_in;
      c.autotune = 0;
      c.block_size = b;
      c.cells_per_node = cells[ci];
      c.record_pairs = 0;
      pg_handle* t = nullptr;
      int rc = create_impl(s, &c, &t);
      if (rc) return rc;
      double ms = 0;
      rc = pg_step(t, 3);
      if (!rc) rc = pg_step_timed(t, 12, &ms);
      pg_destroy(t);
      if (rc) return rc;
      if (ms < best_ms) {
        best_ms = ms;
        best_b = b;
        best_c = cells[ci];
      }
    }
  // second stage: the candidate-list skin at the chosen launch shape (0 = grid search every step)
  double best_skin = cfg_in->contact_skin;
  {
    const double skins[] = {0.0, 0.25, 0.5, 1.0};
    double best_skin_ms = 1e300;
    for (double sk : skins) {
      pg_config c = *cfg_in;
      c.autotune = 0;
      c.block_size = best_b;
      c.cells_per_node = best_c;
      c.contact_skin = sk;
      c.record_pairs = 0;
      pg_handle* t = nullptr;
      int rc = create_impl(s, &c, &t);
      if (rc) return rc;
      double ms = 0;
      rc = pg_step(t, 3);
      if (!rc) rc = pg_step_timed(t, 24, &ms);
      pg_destroy(t);
      if (rc) return rc;
      if (ms < best_skin_ms) {
        best_skin_ms = ms;
        best_skin = sk;
      }
    }
  }
  // third stage: the node layout inside the grains, cell order or cell order grouped by bond count
  // over the whole grain or inside 256-node windows (fewer padded slots in the bond slab, less
  // coalesced neighbour gathers)
  int32_t best_order = cfg_in->node_order;
  if (cfg_in->node_order == PG_ORDER_CELL || cfg_in->node_order == PG_ORDER_CELL_DEGREE ||
      cfg_in->node_order == PG_ORDER_CELL_BLOCK_DEGREE) {
    const int32_t orders[] = {PG_ORDER_CELL, PG_ORDER_CELL_DEGREE, PG_ORDER_CELL_BLOCK_DEGREE};
    double best_order_ms = 1e300;
    for (int32_t od : orders) {
      pg_config c = *cfg_in;
      c.autotune = 0;
      c.block_size = best_b;
      c.cells_per_node = best_c;
      c.contact_skin = best_skin;
      c.node_order = od;
      c.record_pairs = 0;
      pg_handle* t = nullptr;
      int rc = create_impl(s, &c, &t);
      if (rc) return rc;
      // 96 timed steps: the layouts of one workload differ by a few percent of a step
      double ms = 0;
      rc = pg_step(t, 3);
      if (!rc) rc = pg_step_timed(t, 96, &ms);
      pg_destroy(t);
      if (rc) return rc;
      if (ms < best_order_ms) {
        best_order_ms = ms;
        best_order = od;
      }
    }
  }
  pg_config c = *cfg_in;
  c.autotune = 0;
  c.block_size = best_b;
  c.cells_per_node = best_c;
  c.contact_skin = best_skin;
  c.node_order = best_order;
  return create_impl(s, &c, out);
}

// out[i][c] = (double)f[i * S + c], c < D
__global__ void k_widen_field(const float* f, uint32_t S, uint32_t D, uint32_t N, double* out) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < N * D) out[k] = (double)f[(size_t)(k / D) * S + k % D];
}

// out[k] = a[k] + b[k]
__global__ void k_add_vec(const double* a, const double* b, double* out, uint32_t n) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) out[k] = a[k] + b[k];
}

// Bond rows of the uploaded CSR: offsets non-decreasing (and within the nb bonds), every neighbour
// inside its node's grain. The smallest (kind << 32 | node) found goes to *bad, kind 0 = offsets,
// 1 = neighbour; *bad stays ~0 for a valid setup.
__global__ void k_check_bonds(const uint64_t* off, const uint32_t* loc, const uint32_t* grain_node_offset,
                              const uint32_t* node_grain, uint32_t N, uint64_t nb, unsigned long long* bad) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const uint64_t lo = off[i], hi = off[i + 1];
  if (hi < lo || hi > nb) {
    atomicMin(bad, (unsigned long long)i);
    return;
  }
  const uint32_t g = node_grain[i];
  const uint32_t n = grain_node_offset[g + 1] - grain_node_offset[g];
  for (uint64_t b = lo; b < hi; ++b)
    if (loc[b] >= n) {
      atomicMin(bad, (1ull << 32) | i);
      return;
    }
}

// SELL-32 bond slab from the reference CSR, one warp per chunk of 32 nodes (lane = node): bond k of
// node 32c + lane goes to slot chunk_slot[c] + 32k + lane with its global neighbour index and
// xi_norm = |pos[j] - pos[i]| (gen_xi, particle2.h:236-252; the FP64 operations of the reference,
// this file is compiled without contraction); slots past a node's degree hold index 0 and norm 1;
// alive word (c, k) has bit lane set for k < degree.
__global__ void k_layout_bonds(const double* pos, uint32_t S, uint32_t D, uint32_t N, const uint64_t* off,
                               const uint32_t* loc, const uint32_t* grain_node_offset, const uint32_t* node_grain,
                               const uint32_t* chunk_slot, const uint32_t* chunk_word, const uint32_t* chunk_deg,
                               const uint32_t* node_orig, const uint32_t* node_at, uint32_t* bcol, double* bxin,
                               uint32_t* alive) {
  const uint32_t c = blockIdx.x, lane = threadIdx.x, i = c * 32 + lane;
  const bool act = i < N;
  // the row of device node i is the input's row of node_orig[i] (same grain), in its entry order;
  // neighbours are renumbered into the layout through node_at
  const uint32_t o = (act && node_orig) ? node_orig[i] : i;
  const uint32_t deg = act ? (uint32_t)(off[o + 1] - off[o]) : 0u;
  const uint32_t n0 = act ? grain_node_offset[node_grain[i]] : 0u;
  const uint32_t cd = chunk_deg[c];
  for (uint32_t k = 0; k < cd; ++k) {
    const size_t sl = chunk_slot[c] + (size_t)k * 32 + lane;
    const bool has = k < deg;
    uint32_t j = 0;
    double xn = 1.0;
    if (has) {
      j = n0 + loc[off[o] + k];
      if (node_at) j = node_at[j];
      double xi[3] = {0.0, 0.0, 0.0};
      for (uint32_t a = 0; a < D; ++a) xi[a] = pos[(size_t)j * S + a] - pos[(size_t)i * S + a];
      double n2 = xi[0] * xi[0];
      for (uint32_t a = 1; a < D; ++a) n2 = n2 + xi[a] * xi[a];
      xn = sqrt(n2);
    }
    bcol[sl] = j;
    bxin[sl] = xn;
    const uint32_t w = __ballot_sync(0xffffffffu, has);
    if (lane == 0) alive[chunk_word[c] + k] = w;
  }
}

// Phase times of pg_create on stderr (host wall clock) when the environment sets PERIGRAIN_TRACE.
struct CreateTrace {
  bool on = std::getenv("PERIGRAIN_TRACE") != nullptr;
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  void mark(const char* what) {
    if (!on) return;
    const auto n = std::chrono::steady_clock::now();
    std::fprintf(stderr, "pg_create %-22s %9.2f ms\n", what, std::chrono::duration<double, std::milli>(n - t).count());
    t = n;
  }
};

static int create_impl(const pg_setup_desc* s, const pg_config* cfg_in, pg_handle** out) {
  if (!out) return fail(PG_EINVAL, "null out");
  *out = nullptr;
  CreateTrace tr;
  pg_config cfg = *cfg_in;
  int ndev = 0;
  const bool have_dev = cudaGetDeviceCount(&ndev) == cudaSuccess && ndev > 0;
  // without a device everything is checked here (and the call ends with PG_ENODEV); with one the
  // bond rows are checked by the device on their uploaded copy
  int rc = validate(s, &cfg, !have_dev);
  if (rc) return rc;
  tr.mark("validate");
  if (!have_dev) return fail(PG_ENODEV, "no CUDA device");
  // node layout inside the grains (the device arrays follow `ord.perm`; outputs map back)
  NodeOrder ord;
  {
    std::string err;
    rc = make_node_order(s, cfg.node_order, &ord, &err);
    if (rc) return fail(rc, err);
  }
  const bool permuted = !ord.perm.empty();
  tr.mark("node order");
  if (cfg.pair_log_capacity == 0) cfg.pair_log_capacity = 1024;
  if (cfg.max_contacts == 0) cfg.max_contacts = 48;
  if (cfg.max_contacts > (uint32_t)MAX_CAND) cfg.max_contacts = MAX_CAND;
  if (cfg.first_step == 0) cfg.first_step = 1;

  CU(kernels_init());
  CU(kernels_mixed_init());

  std::unique_ptr<pg_handle> h(new pg_handle);
  CU(cudaGetDevice(&h->device));
  CU(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  tr.mark("context and stream");
  const uint32_t D = s->dim, S = (D == 2) ? 2 : 4, N = s->n_nodes, G = s->n_grains, I = s->n_instances;
  h->dim = D;
  h->S = S;
  h->precision = cfg.precision;
  h->next_t = cfg.first_step;
  if (cfg.block_size) h->L.force_block = std::min(128u, std::max(32u, (cfg.block_size / 32) * 32));
  h->L.cells_per_node = cfg.cells_per_node ? cfg.cells_per_node : ((s->dim == 2) ? 4 : 8);
  Dev& P = h->P;
  P.dim = D;
  P.N = N;
  P.G = G;
  P.I = I;
  P.n_chunks = (N + 31) / 32;
  P.dt = cfg.dt;
  P.hdt2 = (cfg.dt * cfg.dt) * 0.5;
  P.half_dt = 0.5 * cfg.dt;
  P.enable_fracture = cfg.enable_fracture;
  P.nl_bdry_only = cfg.nl_bdry_only;
  P.allow_damping = cfg.allow_damping;
  P.allow_friction = cfg.allow_friction;
  P.self_contact = cfg.self_contact;
  P.enable_torque = cfg.enable_torque;
  P.gradient_extforce = cfg.gradient_extforce;
  P.record_pairs = cfg.record_pairs;
  P.extforce_maxstep = cfg.extforce_maxstep;
  P.max_cand = cfg.max_contacts;
  if (cfg.timeloop != 0 && cfg.timeloop != 1) return fail(PG_EINVAL, "timeloop must be 0 or 1");
  P.worm = cfg.timeloop;

  h->grain_node_offset.assign(s->grain_node_offset, s->grain_node_offset + G + 1);
  h->bond_offset.assign(s->bond_offset, s->bond_offset + N + 1);

  h->node_order = cfg.node_order;
  if (permuted) {
    h->node_orig = ord.perm;
    CU(h->dalloc(&P.node_orig, N));
    CU(h->dalloc(&P.node_at, N));
    CU(cudaMemcpy(P.node_orig, ord.perm.data(), (size_t)N * 4, cudaMemcpyHostToDevice));
    CU(cudaMemcpy(P.node_at, ord.at.data(), (size_t)N * 4, cudaMemcpyHostToDevice));
  }

  // ---- node arrays (the layout's order; stride S) ----
  std::vector<double> tmp((size_t)N * S, 0.0);
  auto pack = [&](const double* src) {
    std::fill(tmp.begin(), tmp.end(), 0.0);
    for (uint32_t i = 0; i < N; ++i) {
      const size_t o = permuted ? ord.perm[i] : i;
      for (uint32_t c = 0; c < D; ++c) tmp[(size_t)i * S + c] = src[o * D + c];
    }
  };
  double** vecs[] = {&P.pos, &P.disp, &P.cur, &h->vel_a, &h->vel_b, &P.acc, &P.force, &P.extf};
  for (double** v : vecs) CU(h->dalloc(v, (size_t)N * S));
  P.xpos = P.pos;
  CU(h->dalloc(&P.vol, N));
  CU(h->dalloc(&P.curf, (size_t)N * S));
  // in 2D the stride is the dimension: straight uploads; in 3D through the padded host buffer
  auto upload = [&](double* dst, const double* src) -> cudaError_t {
    if (S == D && !permuted) return cudaMemcpy(dst, src, (size_t)N * D * 8, cudaMemcpyHostToDevice);
    pack(src);
    return cudaMemcpy(dst, tmp.data(), tmp.size() * 8, cudaMemcpyHostToDevice);
  };
  CU(upload(P.pos, s->pos));
  CU(upload(P.disp, s->disp));
  CU(upload(h->vel_a, s->vel));
  CU(cudaMemcpy(h->vel_b, h->vel_a, (size_t)N * S * 8, cudaMemcpyDeviceToDevice));
  CU(upload(P.acc, s->acc));
  CU(upload(P.extf, s->extforce));
  CU(cudaMemset(P.force, 0, (size_t)N * S * 8));
  // CurrPos before the first step is pos + disp (only used for the grid origin)
  if (N) {
    k_add_vec<<<(N * S + 255) / 256, 256>>>(P.pos, P.disp, P.cur, N * S);
    CU(cudaGetLastError());
  }
  if (permuted) {
    std::vector<double> v(N);
    for (uint32_t i = 0; i < N; ++i) v[i] = s->vol[ord.perm[i]];
    CU(cudaMemcpy(P.vol, v.data(), (size_t)N * 8, cudaMemcpyHostToDevice));
  } else {
    CU(cudaMemcpy(P.vol, s->vol, (size_t)N * 8, cudaMemcpyHostToDevice));
  }
  tr.mark("node vectors");

  // ---- per node metadata ----
  std::vector<uint32_t> node_grain(N), bdry_rank(N, NONE);
  std::vector<uint8_t> clamped(N, 0);
  const uint32_t* bdry_nodes = permuted ? ord.bdry_nodes.data() : s->bdry_nodes;
  const uint32_t* clamped_nodes = permuted ? ord.clamped_nodes.data() : s->clamped_nodes;
  for (uint32_t g = 0; g < G; ++g) {
    uint32_t n0 = s->grain_node_offset[g];
    for (uint32_t i = n0; i < s->grain_node_offset[g + 1]; ++i) node_grain[i] = g;
    for (uint32_t k = s->bdry_offset[g]; k < s->bdry_offset[g + 1]; ++k) {
      uint32_t nd = n0 + bdry_nodes[k];
      if (bdry_rank[nd] != NONE) return fail(PG_EINVAL, "duplicate entry in bdry_nodes of grain " + std::to_string(g));
      bdry_rank[nd] = k - s->bdry_offset[g];
    }
    for (uint32_t k = s->clamped_offset[g]; k < s->clamped_offset[g + 1]; ++k) clamped[n0 + clamped_nodes[k]] = 1;
  }
  CU(h->dalloc(&P.node_grain, N));
  CU(h->dalloc(&P.bdry_rank, N));
  CU(h->dalloc(&P.clamped, N));
  CU(h->dalloc(&P.clamp_pending, N));
  CU(cudaMemcpy(P.node_grain, node_grain.data(), N * 4, cudaMemcpyHostToDevice));
  {
    std::vector<uint32_t> sub(N);
    for (uint32_t i = 0; i < N; ++i) {
      const uint32_t o = permuted ? ord.perm[i] : i;  // same grain: grain node ranges are unchanged
      sub[i] = cfg.nl_bdry_only ? bdry_rank[i] : o - s->grain_node_offset[node_grain[i]];
    }
    CU(h->dalloc(&P.node_sub, N));
    CU(cudaMemcpy(P.node_sub, sub.data(), (size_t)N * 4, cudaMemcpyHostToDevice));
  }
  CU(cudaMemcpy(P.bdry_rank, bdry_rank.data(), N * 4, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(P.clamped, clamped.data(), N, cudaMemcpyHostToDevice));
  CU(cudaMemset(P.clamp_pending, 0, N));
  tr.mark("node classes");

  // ---- bonds: reference CSR -> SELL-32 ----
  const uint32_t NC = P.n_chunks;
  h->node_deg.resize(N);
  h->chunk_slot.resize(NC + 1);
  h->chunk_word.resize(NC + 1);
  std::vector<uint32_t> chunk_deg(NC, 0);
  for (uint32_t i = 0; i < N; ++i) {
    if (s->bond_offset[i + 1] < s->bond_offset[i]) return fail(PG_EINVAL, "bond_offset decreasing");
  }
  for (uint32_t i = 0; i < N; ++i) {
    const uint32_t o = permuted ? ord.perm[i] : i;
    h->node_deg[i] = (uint32_t)(s->bond_offset[o + 1] - s->bond_offset[o]);
    chunk_deg[i >> 5] = std::max<uint32_t>(chunk_deg[i >> 5], h->node_deg[i]);
  }
  uint64_t slots = 0, words = 0;
  for (uint32_t c = 0; c < NC; ++c) {
    h->chunk_slot[c] = (uint32_t)slots;
    h->chunk_word[c] = (uint32_t)words;
    slots += (uint64_t)chunk_deg[c] * 32;
    words += chunk_deg[c];
  }
  h->chunk_slot[NC] = (uint32_t)slots;
  h->chunk_word[NC] = (uint32_t)words;
  if (slots >= (1ull << 32)) return fail(PG_EINVAL, "bond slab too large");
  CU(h->dalloc(&P.chunk_slot, NC + 1));
  CU(h->dalloc(&P.chunk_word, NC + 1));
  CU(h->dalloc(&P.chunk_deg, NC));
  CU(h->dalloc(&P.node_deg, N));
  CU(h->dalloc(&P.bcol, slots));
  CU(h->dalloc(&P.bxin, slots));
  CU(h->dalloc(&P.alive, words));
  CU(h->dalloc(&P.break_step, slots));
  CU(cudaMemcpy(P.chunk_slot, h->chunk_slot.data(), (NC + 1) * 4, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(P.chunk_word, h->chunk_word.data(), (NC + 1) * 4, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(P.chunk_deg, chunk_deg.data(), NC * 4, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(P.node_deg, h->node_deg.data(), N * 4, cudaMemcpyHostToDevice));
  if (slots) {
    // the reference CSR goes up once; the SELL-32 slab, the alive words and xi_norm are built on
    // the device
    const uint64_t nb = s->bond_offset[N];
    uint64_t* d_off = nullptr;
    uint32_t* d_loc = nullptr;
    uint32_t* d_gno = nullptr;
    cudaError_t e = cudaMalloc((void**)&d_off, (size_t)(N + 1) * 8);
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_loc, (size_t)std::max<uint64_t>(nb, 1) * 4);
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_gno, (size_t)(G + 1) * 4);
    if (e == cudaSuccess) e = cudaMemcpy(d_off, s->bond_offset, (size_t)(N + 1) * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nb) e = cudaMemcpy(d_loc, s->bond_local, (size_t)nb * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_gno, s->grain_node_offset, (size_t)(G + 1) * 4, cudaMemcpyHostToDevice);
    // bond rows checked before anything reads through them
    unsigned long long bad = ~0ull, *d_bad = nullptr;
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_bad, 8);
    if (e == cudaSuccess) e = cudaMemcpy(d_bad, &bad, 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
      k_check_bonds<<<(N + 255) / 256, 256>>>(d_off, d_loc, d_gno, P.node_grain, N, nb, d_bad);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(&bad, d_bad, 8, cudaMemcpyDeviceToHost);
    if (d_bad) cudaFree(d_bad);
    if (e == cudaSuccess && bad != ~0ull) {
      cudaFree(d_off);
      cudaFree(d_loc);
      cudaFree(d_gno);
      const uint32_t node = (uint32_t)(bad & 0xffffffffu);
      if ((bad >> 32) == 0) return fail(PG_EINVAL, "bond_offset decreasing");
      return fail(PG_EINVAL, "bond of node " + std::to_string(node) + " points outside its grain");
    }
    if (e == cudaSuccess) {
      k_layout_bonds<<<NC, 32>>>(P.pos, S, D, N, d_off, d_loc, d_gno, P.node_grain, P.chunk_slot, P.chunk_word,
                                 P.chunk_deg, P.node_orig, P.node_at, P.bcol, P.bxin, P.alive);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemset(P.break_step, 0, slots * 4);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    cudaFree(d_off);
    cudaFree(d_loc);
    cudaFree(d_gno);
    CU(e);
  }
  tr.mark("bond layout");

  // ---- grains ----
  std::vector<GrainDev> grains(G);
  for (uint32_t g = 0; g < G; ++g) {
    GrainDev& gd = grains[g];
    gd.node_begin = s->grain_node_offset[g];
    gd.node_end = s->grain_node_offset[g + 1];
    gd.inst = s->grain_instance[g];
    gd.flags = (s->movable[g] ? GF_MOVABLE : 0) | (s->breakable[g] ? GF_BREAKABLE : 0) |
               (s->stoppable[g] ? GF_STOPPABLE : 0) | (s->break_bonds[g] ? GF_BREAK_BONDS : 0);
    gd.rho = s->rho[g];
    gd.one_over_rho = 1 / s->rho[g];
    gd.cnot = s->cnot[g];
    gd.snot = s->snot[g];
    gd.torque_axis = s->torque_axis ? s->torque_axis[g] : 2;
    gd.torque_val = s->torque_val ? s->torque_val[g] : 0.0;
    gd.pad = 0;
    // per-grain contact parameters start as the instance's (used once pg_set_grain_params sets them)
    gd.kn = s->normal_stiffness[s->grain_instance[g]];
    gd.zeta = s->damping_ratio[s->grain_instance[g]];
    gd.mu = s->friction_coefficient[s->grain_instance[g]];
    set_grain_f(gd);
  }
  CU(h->dalloc(&P.grain, G));
  CU(cudaMemcpy(P.grain, grains.data(), G * sizeof(GrainDev), cudaMemcpyHostToDevice));
  {
    std::vector<unsigned long long> bb((size_t)G * 2 * D);
    for (size_t i = 0; i < bb.size(); ++i) bb[i] = ((i % (2 * D)) < D) ? ~0ull : 0ull;
    for (int p = 0; p < 2; ++p) {
      CU(h->dalloc(&h->bbox_pp[p], (size_t)G * 2 * D));
      CU(cudaMemcpy(h->bbox_pp[p], bb.data(), bb.size() * 8, cudaMemcpyHostToDevice));
    }
    P.bbox = h->bbox_pp[0];
  }
  CU(h->dalloc(&P.torque_c, (size_t)G * 3));
  CU(cudaMemset(P.torque_c, 0, (size_t)G * 3 * 8));

  // ---- instances: contact parameters, wall, hashed grid ----
  h->inst_host.resize(I);
  uint64_t table_total = 0;
  for (uint32_t k = 0; k < I; ++k) {
    InstDev& in = h->inst_host[k];
    std::memset(&in, 0, sizeof(in));
    in.contact_rad = s->contact_radius[k];
    in.contact_s_max = pg::sqrt_le_max(in.contact_rad);
    in.normal_stiffness = s->normal_stiffness[k];
    in.friction_coefficient = s->friction_coefficient[k];
    in.damping_ratio = s->damping_ratio[k];
    in.allow_wall = s->allow_wall[k];
    for (uint32_t a = 0; a < 2 * D; ++a) {
      in.wall[a] = s->wall_geom[(size_t)k * 2 * D + a];
      in.wall_speed[a] = s->wall_speed[(size_t)k * 2 * D + a];
    }
    in.node_begin = NONE;
    in.node_end = 0;
    in.grain_begin = 0;
    in.grain_end = 0;
  }
  for (uint32_t g = 0; g < G; ++g) {
    InstDev& in = h->inst_host[s->grain_instance[g]];
    in.node_begin = std::min(in.node_begin, s->grain_node_offset[g]);
    in.node_end = std::max(in.node_end, s->grain_node_offset[g + 1]);
    if (in.grain_end == 0) in.grain_begin = g;
    in.grain_end = g + 1;
  }
  for (uint32_t k = 0; k < I; ++k) {
    InstDev& in = h->inst_host[k];
    if (in.node_begin == NONE) {  // instance without grains
      in.node_begin = in.node_end = 0;
      in.grain_begin = in.grain_end = 0;
    }
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (uint32_t a = 0; a < D; ++a) {
      lo[a] = INFINITY;
      hi[a] = -INFINITY;
    }
    for (uint32_t i = in.node_begin; i < in.node_end; ++i)
      for (uint32_t a = 0; a < D; ++a) {
        double x = s->pos[(size_t)i * D + a] + s->disp[(size_t)i * D + a];
        lo[a] = std::min(lo[a], x);
        hi[a] = std::max(hi[a], x);
      }
    double ext = 0;
    for (uint32_t a = 0; a < D; ++a) {
      if (!std::isfinite(lo[a]) || !std::isfinite(hi[a])) lo[a] = hi[a] = 0;
      in.xorigin[a] = 0.5 * (lo[a] + hi[a]);
      ext = std::max(ext, hi[a] - lo[a]);
    }
    double cmin = in.contact_rad * 1.0625;
    if (!(cmin > 0) || !std::isfinite(cmin)) cmin = std::max(ext, 1e-9) / 64;
    in.pre_f = (float)cmin;
    if (cfg.contact_skin > 0) {
      // candidate lists: cells cover the list radius R_c (1 + skin)
      cmin *= 1.0 + cfg.contact_skin;
      const double lim = 0.45 * cfg.contact_skin * in.contact_rad;
      in.skin_lim2 = (float)(lim * lim);
    }
    in.pre_b = (float)cmin;
    in.cell_min = cmin;
    in.rel_frame = (h->precision == PG_MIXED && cfg.contact_skin > 0) ? 1 : 0;
    const uint32_t nn = in.node_end - in.node_begin;
    in.table_cap = (uint32_t)std::max<uint64_t>(1024, (uint64_t)h->L.cells_per_node * nn);
    in.table_off = (uint32_t)table_total;
    table_total += in.table_cap;
    fit_grid(in, (int)D, lo, hi);
  }
  if (table_total >= (1ull << 31)) return fail(PG_EINVAL, "grid table too large");
  P.table_total = (uint32_t)table_total;
  CU(h->dalloc(&P.inst, I));
  CU(cudaMemcpy(P.inst, h->inst_host.data(), I * sizeof(InstDev), cudaMemcpyHostToDevice));
  CU(h->dalloc(&P.reaction, (size_t)I * 2 * D * D));
  CU(cudaMemset(P.reaction, 0, (size_t)I * 2 * D * D * 8));

  // ---- grid buffers ----
  CU(h->dalloc(&P.cell_key, N));
  CU(h->dalloc(&P.cell_rank, N));
  CU(h->dalloc(&P.sorted, N));
  CU(h->dalloc(&P.cell_count, table_total));
  CU(h->dalloc(&P.cell_start, table_total + 1));
  CU(cudaMemset(P.cell_count, 0, table_total * 4));
  const uint32_t ntiles = (uint32_t)((table_total + 4095) / 4096);
  CU(h->dalloc(&P.scan_tile_sum, ntiles));
  CU(h->dalloc(&P.scan_done, 1));
  CU(cudaMemset(P.scan_done, 0, 4));
  tr.mark("grains, grid");

  // ---- wall records, logs, control ----
  P.wrec_cap = (uint32_t)std::min<uint64_t>(WREC_SMEM_CAP, 2ull * D * N);
  {
    // the finalize kernel takes its large shared-memory buffer only when walls can make records
    bool any_wall = false;
    for (uint32_t k = 0; k < I; ++k) any_wall = any_wall || h->inst_host[k].allow_wall;
    P.wrec_smem = any_wall ? (uint32_t)WREC_SMEM_CAP : 0u;
  }
  CU(h->dalloc(&P.wrec, P.wrec_cap));
  CU(h->dalloc(&P.wrec_count, 1));
  CU(cudaMemset(P.wrec_count, 0, 4));
  P.log_cap = cfg.pair_log_capacity;
  CU(h->dalloc(&P.pair_acc, 2));
  CU(h->dalloc(&P.log_count, P.log_cap));
  CU(h->dalloc(&P.log_hash, P.log_cap));
  CU(cudaMemset(P.pair_acc, 0, 16));
  CU(cudaMemset(P.log_count, 0, (size_t)P.log_cap * 8));
  CU(cudaMemset(P.log_hash, 0, (size_t)P.log_cap * 8));
  CU(h->dalloc(&P.step, 1));
  uint32_t t0 = (uint32_t)h->next_t;
  CU(cudaMemcpy(P.step, &t0, 4, cudaMemcpyHostToDevice));
  CU(h->dalloc(&P.status, 1));
  CU(cudaMemset(P.status, 0, 4));
  CU(h->dalloc(&P.too_close, 1));
  CU(cudaMemset(P.too_close, 0, 8));
  tr.mark("logs and control");
  if (h->precision == PG_MIXED) {
    rc = mixed_setup(h.get(), s);
    if (rc) return rc;
    tr.mark("mixed images");
  }
  h->contact_skin = cfg.contact_skin;
  if (cfg.contact_skin > 0) {
    const uint32_t SF = (D == 2) ? 2 : 4;
    P.cand_cap = CAND_CAP;
    CU(h->dalloc(&P.cand_q, (size_t)P.n_chunks * 32 * CAND_CAP));
    CU(h->dalloc(&P.cand_n, N));
    CU(h->dalloc(&P.disp_b, (size_t)N * SF));
    CU(h->dalloc(&P.sorted_pos, (size_t)N * SF));
    CU(h->dalloc(&P.sorted_key, N));
    for (int p = 0; p < 2; ++p) CU(h->dalloc(&h->rebuild_pp[p], 1));
    P.rebuild = h->rebuild_pp[0];
    CU(h->dalloc(&P.gbar, 3));
    CU(cudaMemset(P.gbar, 0, 12));
    P.coop_blocks = grid_coop_blocks(P, h->device);
    CU(cudaMemset(P.cand_n, 0, N));
    CU(cudaMemset(P.disp_b, 0, (size_t)N * SF * 4));
    const uint32_t one = 1;
    for (int p = 0; p < 2; ++p) CU(cudaMemcpy(h->rebuild_pp[p], &one, 4, cudaMemcpyHostToDevice));
    if (h->precision == PG_MIXED) {
      h->overlap = true;
      CU(cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
      CU(cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
      CU(cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming));
    }
  }
  CU(cudaEventCreate(&h->ev_t0));
  CU(cudaEventCreate(&h->ev_t1));
  CU(cudaDeviceSynchronize());
  tr.mark("lists, sync");
  rc = build_graphs(h.get());
  if (rc) return rc;
  tr.mark("graphs");
  *out = h.release();
  return PG_OK;
}

int pg_destroy(pg_handle* h) {
  delete h;
  return PG_OK;
}

}  // extern "C"

int device_status_fail(int32_t st) {
  if (!st) return PG_OK;
  std::string m = "device reported: ";
  m += pg_status_string(st);
  if (st == PG_ECAPACITY) m += " (contact candidates per node, or wall records per step)";
  return fail(st, m);
}

int check_device_status(pg_handle* h) {
  int32_t st = 0;
  CU(cudaMemcpyAsync(&st, h->P.status, 4, cudaMemcpyDeviceToHost, h->stream));
  CU(cudaStreamSynchronize(h->stream));
  if (st == PG_ETIMEOUT) h->halted = true;
  return device_status_fail(st);
}

extern "C" {

int pg_step(pg_handle* h, uint32_t nsteps) {
  if (!h) return fail(PG_EINVAL, "null handle");
  // after a bounded device wait ran out, the grid build's barrier state is stale: no more steps
  if (h->halted) return fail(PG_ETIMEOUT, "handle halted: a device wait timed out in an earlier step");
  uint64_t launches = 0;
  if (h->timing) {
    // timed mode: plain launches with CUDA events around every force kernel
    if (h->ev.size() < 2 * (size_t)nsteps) {
      size_t old = h->ev.size();
      h->ev.resize(2 * (size_t)nsteps);
      for (size_t i = old; i < h->ev.size(); ++i) CU(cudaEventCreate(&h->ev[i]));
    }
    h->force_ms = 0;
    h->force_launches = 0;
    CU(cudaEventRecord(h->ev_t0, h->stream));
    for (uint32_t k = 0; k < nsteps; ++k) {
      Dev P = h->P;
      set_vel(h, P, h->vel_parity);
      if (h->precision == PG_MIXED) {
        launch_step_mixed(P, h->L, h->stream, &launches, h->ev[2 * k], h->ev[2 * k + 1]);
      } else {
        launch_step_timed(P, h->L, h->stream, &launches, h->ev[2 * k], h->ev[2 * k + 1]);
      }
      h->vel_parity ^= 1;
    }
    CU(cudaEventRecord(h->ev_t1, h->stream));
    CU(cudaEventSynchronize(h->ev_t1));
    for (uint32_t k = 0; k < nsteps; ++k) {
      float ms = 0;
      CU(cudaEventElapsedTime(&ms, h->ev[2 * k], h->ev[2 * k + 1]));
      h->force_ms += ms;
    }
    float tot = 0;
    CU(cudaEventElapsedTime(&tot, h->ev_t0, h->ev_t1));
    h->total_ms = tot;
    h->force_launches = nsteps;
  } else {
    uint32_t k = 0;
    while (k < nsteps) {
      if (nsteps - k >= (uint32_t)pg_handle::GRAPH_STEPS) {
        CU(cudaGraphLaunch(h->graph[h->vel_parity], h->stream));
        launches += h->graph_launches_per;
        k += pg_handle::GRAPH_STEPS;  // GRAPH_STEPS is even: parity unchanged
      } else {
        enqueue_step(h, h->vel_parity, &launches);
        h->vel_parity ^= 1;
        ++k;
      }
    }
    CU(cudaGetLastError());
  }
  h->next_t += nsteps;
  h->last_launches = launches;
  return PG_OK;
}

int pg_step_timed(pg_handle* h, uint32_t nsteps, double* elapsed_ms) {
  if (!h || !elapsed_ms) return fail(PG_EINVAL, "null argument");
  CU(cudaEventRecord(h->ev_t0, h->stream));
  int rc = pg_step(h, nsteps);
  if (rc) return rc;
  CU(cudaEventRecord(h->ev_t1, h->stream));
  CU(cudaEventSynchronize(h->ev_t1));
  float ms = 0;
  CU(cudaEventElapsedTime(&ms, h->ev_t0, h->ev_t1));
  *elapsed_ms = ms;
  return check_device_status(h);
}

int pg_synchronize(pg_handle* h) {
  if (!h) return fail(PG_EINVAL, "null handle");
  CU(cudaStreamSynchronize(h->stream));
  return check_device_status(h);
}

int pg_get_step(pg_handle* h, uint64_t* t) {
  if (!h || !t) return fail(PG_EINVAL, "null argument");
  *t = h->next_t;
  return PG_OK;
}

static double* field_ptr(pg_handle* h, int field) {
  switch (field) {
    case PG_FIELD_CURRPOS: return h->P.cur;
    case PG_FIELD_VEL: return h->vel_parity == 0 ? h->vel_a : h->vel_b;
    case PG_FIELD_ACC: return h->P.acc;
    case PG_FIELD_FORCE: return h->P.force;
    case PG_FIELD_DISP: return h->P.disp;
    case PG_FIELD_POS: return h->P.pos;
  }
  return nullptr;
}

int pg_get_field(pg_handle* h, int field, double* out) {
  if (!h || !out) return fail(PG_EINVAL, "null argument");
  double* src = field_ptr(h, field);
  if (!src) return fail(PG_EINVAL, "unknown field");
  int rc = pg_synchronize(h);
  if (rc) return rc;
  const uint32_t N = h->P.N, D = h->dim, S = h->S;
  if (h->precision == PG_MIXED && (field == PG_FIELD_ACC || field == PG_FIELD_FORCE)) {
    // the FP32 field widened on the device into [N][D] doubles, then one copy
    if (!h->field_scratch) CU(h->dalloc(&h->field_scratch, (size_t)N * D));
    if (N) {
      k_widen_field<<<(N * D + 255) / 256, 256, 0, h->stream>>>(
          field == PG_FIELD_ACC ? h->P.acc_f : h->P.force_f, S, D, N, h->field_scratch);
      CU(cudaGetLastError());
      if (h->node_orig.empty()) {
        CU(cudaMemcpyAsync(out, h->field_scratch, (size_t)N * D * 8, cudaMemcpyDeviceToHost, h->stream));
        CU(cudaStreamSynchronize(h->stream));
      } else {
        std::vector<double> tmp((size_t)N * D);
        CU(cudaMemcpyAsync(tmp.data(), h->field_scratch, tmp.size() * 8, cudaMemcpyDeviceToHost, h->stream));
        CU(cudaStreamSynchronize(h->stream));
        for (uint32_t i = 0; i < N; ++i)
          for (uint32_t c = 0; c < D; ++c) out[(size_t)h->node_orig[i] * D + c] = tmp[(size_t)i * D + c];
      }
    }
    return PG_OK;
  }
  if (S == D && h->node_orig.empty()) {
    CU(cudaMemcpy(out, src, (size_t)N * D * 8, cudaMemcpyDeviceToHost));
  } else {
    std::vector<double> tmp((size_t)N * S);
    CU(cudaMemcpy(tmp.data(), src, tmp.size() * 8, cudaMemcpyDeviceToHost));
    for (uint32_t i = 0; i < N; ++i)
      for (uint32_t c = 0; c < D; ++c) out[(size_t)h->orig(i) * D + c] = tmp[(size_t)i * S + c];
  }
  if (field == PG_FIELD_DISP) {
    std::vector<uint8_t> pend(N);
    CU(cudaMemcpy(pend.data(), h->P.clamp_pending, N, cudaMemcpyDeviceToHost));
    for (uint32_t i = 0; i < N; ++i)
      if (pend[i])
        for (uint32_t c = 0; c < D; ++c) out[(size_t)h->orig(i) * D + c] = 0.0;
  }
  return PG_OK;
}

int pg_set_field(pg_handle* h, int field, const double* in) {
  if (!h || !in) return fail(PG_EINVAL, "null argument");
  int rc = pg_synchronize(h);
  if (rc) return rc;
  const uint32_t N = h->P.N, D = h->dim, S = h->S;
  // the values in the layout's node order
  std::vector<double> in_layout;
  if (!h->node_orig.empty()) {
    in_layout.resize((size_t)N * D);
    for (uint32_t i = 0; i < N; ++i)
      for (uint32_t c = 0; c < D; ++c) in_layout[(size_t)i * D + c] = in[(size_t)h->node_orig[i] * D + c];
    in = in_layout.data();
  }
  if (field == PG_FIELD_POS && !h->xpos_separate) {
    // keep the bond reference positions (xi = pos[j] - pos[i] at load time) unchanged
    double* x = nullptr;
    CU(cudaMalloc((void**)&x, (size_t)N * S * 8));
    CU(cudaMemcpy(x, h->P.pos, (size_t)N * S * 8, cudaMemcpyDeviceToDevice));
    h->P.xpos = x;
    h->xpos_separate = true;
    rc = build_graphs(h);
    if (rc) return rc;
  }
  double* dst = nullptr;
  switch (field) {
    case PG_FIELD_POS: dst = h->P.pos; break;
    case PG_FIELD_DISP: dst = h->P.disp; break;
    case PG_FIELD_VEL: dst = h->vel_parity == 0 ? h->vel_a : h->vel_b; break;
    case PG_FIELD_ACC: dst = h->P.acc; break;
    default: return fail(PG_EINVAL, "field not writable");
  }
  std::vector<double> tmp((size_t)N * S, 0.0);
  for (uint32_t i = 0; i < N; ++i)
    for (uint32_t c = 0; c < D; ++c) tmp[(size_t)i * S + c] = in[(size_t)i * D + c];
  CU(cudaMemcpy(dst, tmp.data(), tmp.size() * 8, cudaMemcpyHostToDevice));
  if (field == PG_FIELD_DISP) CU(cudaMemset(h->P.clamp_pending, 0, N));
  rc = request_list_rebuild(h);
  if (rc) return rc;
  if (h->precision == PG_MIXED && (field == PG_FIELD_DISP || field == PG_FIELD_ACC)) {
    std::vector<float> tf;
    if (field == PG_FIELD_DISP) {
      const uint32_t SF = (D == 2) ? 2 : 4;
      pack_hl(in, N, D, nullptr, &tf);
      std::vector<float> ref((size_t)N * 4 * D);
      CU(cudaMemcpy(ref.data(), h->P.bref, ref.size() * 4, cudaMemcpyDeviceToHost));
      for (uint32_t i = 0; i < N; ++i)
        for (uint32_t c = 0; c < D; ++c) {
          const float hv = tf[(size_t)i * 2 * SF + c], lv = tf[(size_t)i * 2 * SF + SF + c];
          if (D == 2) {
            ref[(size_t)i * 8 + c] = hv;
            ref[(size_t)i * 8 + 2 + c] = lv;
          } else {
            ref[(size_t)c * N + i] = hv;
            ref[(size_t)(D + c) * N + i] = lv;
          }
        }
      CU(cudaMemcpy(h->P.bref, ref.data(), ref.size() * 4, cudaMemcpyHostToDevice));
    } else {
      pack_f(in, N, D, &tf);
      CU(cudaMemcpy(h->P.acc_f, tf.data(), tf.size() * 4, cudaMemcpyHostToDevice));
    }
  }
  return PG_OK;
}

int pg_get_bond_alive(pg_handle* h, uint8_t* out) {
  if (!h || !out) return fail(PG_EINVAL, "null argument");
  int rc = pg_synchronize(h);
  if (rc) return rc;
  const uint32_t N = h->P.N, NC = h->P.n_chunks;
  std::vector<uint32_t> words(h->chunk_word[NC]);
  if (!words.empty()) CU(cudaMemcpy(words.data(), h->P.alive, words.size() * 4, cudaMemcpyDeviceToHost));
  for (uint32_t i = 0; i < N; ++i) {
    const uint32_t c = i >> 5, lane = i & 31;
    for (uint32_t k = 0; k < h->node_deg[i]; ++k)
      out[h->bond_offset[h->orig(i)] + k] = (words[h->chunk_word[c] + k] >> lane) & 1u;
  }
  return PG_OK;
}

int pg_get_bond_break_step(pg_handle* h, uint32_t* out) {
  if (!h || !out) return fail(PG_EINVAL, "null argument");
  int rc = pg_synchronize(h);
  if (rc) return rc;
  const uint32_t N = h->P.N, NC = h->P.n_chunks;
  std::vector<uint32_t> bs(h->chunk_slot[NC]);
  if (!bs.empty()) CU(cudaMemcpy(bs.data(), h->P.break_step, bs.size() * 4, cudaMemcpyDeviceToHost));
  for (uint32_t i = 0; i < N; ++i) {
    const uint32_t c = i >> 5, lane = i & 31;
    for (uint32_t k = 0; k < h->node_deg[i]; ++k)
      out[h->bond_offset[h->orig(i)] + k] = bs[h->chunk_slot[c] + (size_t)k * 32 + lane];
  }
  return PG_OK;
}

int pg_set_bond_alive(pg_handle* h, const uint8_t* in) {
  if (!h || !in) return fail(PG_EINVAL, "null argument");
  int rc = pg_synchronize(h);
  if (rc) return rc;
  const uint32_t N = h->P.N, NC = h->P.n_chunks;
  std::vector<uint32_t> words(h->chunk_word[NC], 0);
  for (uint32_t i = 0; i < N; ++i) {
    const uint32_t c = i >> 5, lane = i & 31;
    for (uint32_t k = 0; k < h->node_deg[i]; ++k)
      if (in[h->bond_offset[h->orig(i)] + k]) words[h->chunk_word[c] + k] |= 1u << lane;
  }
  if (!words.empty()) CU(cudaMemcpy(h->P.alive, words.data(), words.size() * 4, cudaMemcpyHostToDevice));
  return PG_OK;
}

int pg_get_reaction(pg_handle* h, double* out) {
  if (!h || !out) return fail(PG_EINVAL, "null argument");
  int rc = pg_synchronize(h);
  if (rc) return rc;
  CU(cudaMemcpy(out, h->P.reaction, (size_t)h->P.I * 2 * h->dim * h->dim * 8, cudaMemcpyDeviceToHost));
  return PG_OK;
}

int pg_get_wall(pg_handle* h, double* out) {
  if (!h || !out) return fail(PG_EINVAL, "null argument");
  int rc = pg_synchronize(h);
  if (rc) return rc;
  std::vector<InstDev> in(h->P.I);
  CU(cudaMemcpy(in.data(), h->P.inst, in.size() * sizeof(InstDev), cudaMemcpyDeviceToHost));
  const uint32_t NS = 2 * h->dim;
  for (uint32_t k = 0; k < h->P.I; ++k)
    for (uint32_t a = 0; a < NS; ++a) out[(size_t)k * NS + a] = in[k].wall[a];
  return PG_OK;
}

int pg_set_wall(pg_handle* h, const double* geom) {
  if (!h || !geom) return fail(PG_EINVAL, "null argument");
  int rc = pg_synchronize(h);
  if (rc) return rc;
  std::vector<InstDev> in(h->P.I);
  CU(cudaMemcpy(in.data(), h->P.inst, in.size() * sizeof(InstDev), cudaMemcpyDeviceToHost));
  const uint32_t NS = 2 * h->dim;
  for (uint32_t k = 0; k < h->P.I; ++k)
    for (uint32_t a = 0; a < NS; ++a) in[k].wall[a] = geom[(size_t)k * NS + a];
  CU(cudaMemcpy(h->P.inst, in.data(), in.size() * sizeof(InstDev), cudaMemcpyHostToDevice));
  return PG_OK;
}

int pg_set_grain_flags(pg_handle* h, uint32_t grain, int32_t movable, int32_t stoppable) {
  if (!h || grain >= h->P.G) return fail(PG_EINVAL, "bad grain");
  int rc = pg_synchronize(h);
  if (rc) return rc;
  GrainDev gd;
  CU(cudaMemcpy(&gd, h->P.grain + grain, sizeof(gd), cudaMemcpyDeviceToHost));
  if (movable >= 0) gd.flags = movable ? (gd.flags | GF_MOVABLE) : (gd.flags & ~GF_MOVABLE);
  if (stoppable >= 0) gd.flags = stoppable ? (gd.flags | GF_STOPPABLE) : (gd.flags & ~GF_STOPPABLE);
  CU(cudaMemcpy(h->P.grain + grain, &gd, sizeof(gd), cudaMemcpyHostToDevice));
  return request_list_rebuild(h);
}

int pg_get_pair_log(pg_handle* h, uint32_t n, uint64_t* count, uint64_t* hash) {
  if (!h || !count || !hash) return fail(PG_EINVAL, "null argument");
  if (n > h->P.log_cap) return fail(PG_EINVAL, "n exceeds the pair log capacity");
  int rc = pg_synchronize(h);
  if (rc) return rc;
  std::vector<unsigned long long> c(h->P.log_cap), hs(h->P.log_cap);
  CU(cudaMemcpy(c.data(), h->P.log_count, c.size() * 8, cudaMemcpyDeviceToHost));
  CU(cudaMemcpy(hs.data(), h->P.log_hash, hs.size() * 8, cudaMemcpyDeviceToHost));
  // last completed step is next_t - 1; entry of step t sits at (t - 1) % cap
  for (uint32_t k = 0; k < n; ++k) {
    uint64_t t = h->next_t - n + k;
    if (t < 1) {
      count[k] = 0;
      hash[k] = 0;
      continue;
    }
    uint32_t slot = (uint32_t)((t - 1) % h->P.log_cap);
    count[k] = c[slot];
    hash[k] = hs[slot];
  }
  return PG_OK;
}

int pg_debug_grid_barrier(pg_handle* h, uint32_t arrivals) {
  if (!h) return fail(PG_EINVAL, "null handle");
  if (!h->P.gbar || !h->P.coop_blocks) return fail(PG_EINVAL, "no cooperative grid build on this handle");
  CU(cudaStreamSynchronize(h->stream));
  CU(cudaMemcpy(h->P.gbar, &arrivals, 4, cudaMemcpyHostToDevice));
  return PG_OK;
}

int pg_debug_ieee64(int32_t op, const double* a, const double* b, int64_t n, double* out) {
  if (op < PG_IEEE_DIV || op > PG_IEEE_WIDEN) return fail(PG_EINVAL, "unknown op");
  if (n < 0 || n > ((int64_t)1 << 26)) return fail(PG_EINVAL, "n out of range [0, 2^26]");
  if (n > 0 && (!a || !b || !out)) return fail(PG_EINVAL, "null array");
  if (n == 0) return PG_OK;
  const size_t bytes = (size_t)n * sizeof(double);
  double* buf = nullptr;
  CU(cudaMalloc(&buf, 3 * bytes));
  double *da = buf, *db = buf + n, *dout = buf + 2 * n;
  cudaError_t e = cudaMemcpy(da, a, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(db, b, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = pg::launch_ieee64_check(op, da, db, n, dout, 0);
  if (e == cudaSuccess) e = cudaMemcpy(out, dout, bytes, cudaMemcpyDeviceToHost);
  const cudaError_t ef = cudaFree(buf);
  if (e == cudaSuccess) e = ef;
  if (e != cudaSuccess) return fail(PG_ECUDA, std::string("pg_debug_ieee64: ") + cudaGetErrorString(e));
  return PG_OK;
}

int pg_get_device_status(pg_handle* h, int32_t* status, uint64_t* too_close) {
  if (!h) return fail(PG_EINVAL, "null handle");
  CU(cudaStreamSynchronize(h->stream));
  int32_t st = 0;
  unsigned long long tc = 0;
  CU(cudaMemcpy(&st, h->P.status, 4, cudaMemcpyDeviceToHost));
  CU(cudaMemcpy(&tc, h->P.too_close, 8, cudaMemcpyDeviceToHost));
  if (st == PG_ETIMEOUT) h->halted = true;
  if (status) *status = st;
  if (too_close) *too_close = tc;
  return PG_OK;
}

int pg_get_launch_config(pg_handle* h, uint32_t* block_size, uint32_t* cells_per_node) {
  if (!h) return fail(PG_EINVAL, "null handle");
  if (block_size) *block_size = h->L.force_block;
  if (cells_per_node) *cells_per_node = h->L.cells_per_node;
  return PG_OK;
}

int pg_get_node_order(pg_handle* h, int32_t* order, int32_t* permuted) {
  if (!h) return fail(PG_EINVAL, "null handle");
  if (order) *order = h->node_order;
  if (permuted) *permuted = h->node_orig.empty() ? 0 : 1;
  return PG_OK;
}

int pg_debug_node_order(const pg_setup_desc* s, int32_t order, uint32_t* perm, int32_t* permuted) {
  pg_config c;
  pg_config_default(&c);
  int rc = validate(s, &c, true);
  if (rc) return rc;
  if (!perm) return fail(PG_EINVAL, "null perm");
  NodeOrder ord;
  std::string err;
  rc = make_node_order(s, order, &ord, &err);
  if (rc) return fail(rc, err);
  for (uint32_t i = 0; i < s->n_nodes; ++i) perm[i] = ord.perm.empty() ? i : ord.perm[i];
  if (permuted) *permuted = ord.perm.empty() ? 0 : 1;
  return PG_OK;
}

int pg_get_contact_skin(pg_handle* h, double* skin) {
  if (!h || !skin) return fail(PG_EINVAL, "null argument");
  *skin = h->contact_skin;
  return PG_OK;
}

int pg_get_launch_count(pg_handle* h, uint64_t* n) {
  if (!h || !n) return fail(PG_EINVAL, "null argument");
  *n = h->last_launches;
  return PG_OK;
}

int pg_set_timing(pg_handle* h, int32_t enable) {
  if (!h) return fail(PG_EINVAL, "null handle");
  h->timing = enable != 0;
  return PG_OK;
}

int pg_get_kernel_times(pg_handle* h, double* force_ms, double* total_ms, uint64_t* force_launches) {
  if (!h) return fail(PG_EINVAL, "null handle");
  if (force_ms) *force_ms = h->force_ms;
  if (total_ms) *total_ms = h->total_ms;
  if (force_launches) *force_launches = h->force_launches;
  return PG_OK;
}

}  // extern "C"
